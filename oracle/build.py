"""Build recipe for the checkers (test infrastructure only).

* ``oracle/liboracle.so``  -- the plain-C FP64 restatement (mcpm_oracle.c).
* ``oracle/_ref/libref.so`` -- the reference's own translation units, compiled
  straight from the reference tree with empty MKL stand-in headers
  (``oracle/shim/``) plus ``ref_harness.cpp``; built only where the reference
  sources are present.  Nothing is copied out of the reference tree.

Both are built with ``-ffp-contract=off`` so that no multiply-add is fused:
the reference's arithmetic is then reproduced bit for bit on both x86-64 and
aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def default_ref_src():
    """The reference's source folder: $MCPM_REFERENCE_SRC, else the
    ``reference/src`` folder of a reference checkout beside this repository."""
    env = os.environ.get("MCPM_REFERENCE_SRC")
    if env:
        return env
    return os.path.join(os.path.dirname(REPO), "reference", "src")

# reference translation units the particle step reaches (main.cpp, the
# MKL-bound solver_pardiso.cpp, the dead solver.cpp demo and the rand()-based
# random_generator.cpp are replaced by ref_harness.cpp)
REF_TUS = ["Main_Functions", "Fokker_Planck", "Math_Func", "collisions", "FEM",
           "myIO", "hybrid", "dcones_BC", "my_Func", "ziggurat"]

CFLAGS = ["-O2", "-ffp-contract=off", "-fPIC"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build_oracle(force=False):
    src = os.path.join(HERE, "mcpm_oracle.c")
    out = os.path.join(HERE, "liboracle.so")
    deps = [src, os.path.join(HERE, "mcpm_oracle.h"), os.path.join(REPO, "include", "mcpm.h")]
    if force or _stale(out, deps):
        _run(["gcc", "-std=c11", *CFLAGS, "-shared", "-o", out, src, "-lm"])
    return out


def build_ref(ref_src=None, force=False):
    """Compile the reference into oracle/_ref/libref.so; returns the path or
    None when the reference sources are not available."""
    ref_src = ref_src or default_ref_src()
    if not os.path.isfile(os.path.join(ref_src, "cpp_headers.h")):
        return None
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    out = os.path.join(outdir, "libref.so")
    harness = os.path.join(HERE, "ref_harness.cpp")
    srcs = [os.path.join(ref_src, t + ".cpp") for t in REF_TUS]
    if not (force or _stale(out, srcs + [harness, os.path.join(REPO, "include", "mcpm.h")])):
        return out
    inc = ["-I" + os.path.join(HERE, "shim"), "-I" + ref_src]
    flags = ["-std=c++11", *CFLAGS, "-fopenmp", "-w", *inc]

    def cc(src):
        obj = os.path.join(outdir, os.path.splitext(os.path.basename(src))[0] + ".o")
        _run(["g++", *flags, "-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=os.cpu_count() or 4) as ex:
        objs = list(ex.map(cc, srcs + [harness]))
    _run(["g++", "-shared", "-fopenmp", "-o", out, *objs, "-lm"])
    return out


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
