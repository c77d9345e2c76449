"""Builds libmcpm.so (the C-ABI of include/mcpm.h) in-tree for sm_103a.

Each CUDA translation unit is compiled in parallel with nvcc, then linked into
one shared library next to this file.  The particle kernels are compiled with
``--fmad=false``: the FP64 path then rounds every multiply and add separately,
as the reference does (the FP32 kernels write their fused multiply-adds out;
the FP32 sessions' per-cell solve, ``mcpm_solve_fast.cu``, is the one unit
compiled with ``--fmad=true``);
host code is compiled with ``-ffp-contract=off`` for the same reason (aarch64
compilers contract by default).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmcpm.so")
# the reference's own routine signatures over the C-ABI (compat/reference_surface.cpp)
REF_LIB = os.path.join(HERE, "libmcpm_ref.so")
REF_SRC = [os.path.join(HERE, "compat", f) for f in ("reference_surface.cpp", "ref_layout.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-Xcompiler", "-fPIC,-O2,-ffp-contract=off",
           "-Xptxas", "-warn-spills", "--expt-relaxed-constexpr"]
SOURCES = ["mcpm_session.cu", "mcpm_kernels.cu", "mcpm_forces.cu", "mcpm_lr2d.cu", "mcpm_noalloc.cu",
           "mcpm_surrogate.cu", "mcpm_surrogate_tc.cu", "mcpm_settings.cu", "mcpm_dynamic.cu", "mcpm_output.cu",
           "mcpm_solve_fast.cu"]
# translation units whose FP64 multiply-adds may fuse (results of FP32
# sessions only); every other unit rounds each operation separately
FMAD_TRUE = {"mcpm_solve_fast.cu"}


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def _deps():
    out = [os.path.join(REPO, "include", "mcpm.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh")):
            out.append(os.path.join(CSRC, f))
    return out


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    hdrs = _deps()
    hdr_t = max(os.path.getmtime(h) for h in hdrs)
    objs, todo = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
            todo.append((s, o))
    cc = nvcc()
    logs = []

    def comp(so):
        s, o = so
        flags = [f.replace("--fmad=false", "--fmad=true") for f in NVFLAGS] \
            if os.path.basename(s) in FMAD_TRUE else NVFLAGS
        return _run([cc, *ARCH, *flags, "-c", s, "-o", o])

    if todo:
        with ThreadPoolExecutor(max_workers=len(todo)) as ex:
            logs = list(ex.map(comp, todo))
    if todo or not os.path.exists(LIB):
        _run([cc, *ARCH, "-shared", "-o", LIB, *objs])
    if (not os.path.exists(REF_LIB) or os.path.getmtime(REF_LIB) <
            max(os.path.getmtime(LIB), hdr_t, *(os.path.getmtime(f) for f in REF_SRC))):
        _run([os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-shared",
              "-o", REF_LIB, REF_SRC[0], "-L" + HERE, "-lmcpm", "-Wl,-rpath,$ORIGIN"])
    if verbose:
        for l in logs:
            if l.strip():
                print(l)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
