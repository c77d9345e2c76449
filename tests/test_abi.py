"""The C-ABI library without a GPU: it loads, exports every entry point that
include/mcpm.h declares, the ctypes view of mcpm_config matches the C layout,
and config derivation agrees between the library and the Python layer.
Also the counter-based RNG against the Philox4x32-10 known-answer vectors."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np

import mcpm
import oracle as O

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR = os.path.join(REPO, "include", "mcpm.h")


def declared_functions():
    src = open(HDR).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mcpm_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(mcpm.LIB_PATH)
    names = declared_functions()
    assert len(names) > 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_config_layout_matches_c(built, tmp_path):
    fields = [f for f, _ in mcpm.Config._fields_]
    prog = ["#include <stdio.h>", "#include <stddef.h>", '#include "mcpm.h"', "int main(void){",
            'printf("%zu\\n", sizeof(mcpm_config));']
    for f in fields:
        prog.append('printf("%%zu\\n", offsetof(mcpm_config, %s));' % f)
    prog.append("return 0;}")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(prog))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(REPO, "include"), str(c), "-o", str(exe)], check=True)
    out = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == C.sizeof(mcpm.Config)
    for f, off in zip(fields, out[1:]):
        assert getattr(mcpm.Config, f).offset == off, f


def test_config_derive_matches(built):
    lib = mcpm.load_library()
    c1 = mcpm.Config()
    c1.sigma, c1.m, c1.kb, c1.n = 1.0, 1.0, 1.0, 0.14
    c1.length[:] = (1.0, 100.0, 1.0)
    c2 = c1.copy()
    assert lib.mcpm_config_derive(C.byref(c1), 20000) == 0
    mcpm.derive(c2, 20000)
    for f in ("b", "T0", "visp", "mu", "Fn", "eqdist", "seed", "max_particles"):
        assert getattr(c1, f) == getattr(c2, f), f


def test_session_create_rejects_bad_config_without_gpu(built):
    lib = mcpm.load_library()
    c = mcpm.Config()
    h = C.c_void_p()
    c.n_cells[:] = (4, 4, 2)  # N2 must be 1
    assert lib.mcpm_session_create(C.byref(c), C.byref(h)) == mcpm.ERR_ARG


def _philox(ctr, key):
    L = O.oracle_lib()
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    L.orc_philox4x32_10(c, k, o)
    return list(o)


def test_philox_known_answers(built):
    # Philox4x32-10 known-answer vectors (Random123 distribution, kat_vectors)
    assert _philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert _philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert _philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_normals_are_standard(built):
    L = O.oracle_lib()
    z = np.zeros(4)
    vals = []
    for i in range(20000):
        L.orc_normals4(0x4D43504D, i, 7, 0, 0, z.ctypes.data_as(C.POINTER(C.c_double)))
        vals.extend(z[:3])
    v = np.array(vals)
    assert abs(v.mean()) < 0.02 and abs(v.std() - 1) < 0.02
