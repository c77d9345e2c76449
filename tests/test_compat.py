"""libmcpm_ref.so without a GPU: it loads, exports the reference's routines
under their C++ names (the names the reference's own objects bind, checked
against the reference's build where that is present), its struct layout is
the one the reference's compiler gives (re-measured from the reference's
header where that is present), the structs it allocates carry working
std::string members, and a gas.model outside the particle step stops the
program with exit status 1 as the reference's checks do."""
import ctypes as C
import os
import subprocess
import sys
import textwrap

import pytest

import compat_driver as D

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
COMPAT = os.path.join(REPO, "monte-carlo-particle-method_gb300", "compat")


@pytest.fixture(scope="module")
def lib(built):
    return D.load()


def _layout():
    out = {}
    with open(os.path.join(COMPAT, "ref_layout.h")) as fh:
        for line in fh:
            if line.startswith("#define MCPM_REF_"):
                _, name, val = line.split(None, 2)
                out[name[len("MCPM_REF_"):]] = tuple(int(v) for v in val.split(","))
    return out


def test_exports_reference_names(lib):
    for name, mangled in D.MANGLED.items():
        f = getattr(lib, mangled)
        assert C.cast(f, C.c_void_p).value == lib.mcpm_compat_routine(name.encode())
    assert lib.mcpm_compat_routine(b"no_such_routine") is None


def test_names_match_reference_build(lib):
    ref = os.path.join(REPO, "oracle", "_ref", "libref.so")
    if not os.path.exists(ref):
        pytest.skip("the reference's build is not present")
    R = C.CDLL(ref)
    for mangled in D.MANGLED.values():
        getattr(R, mangled)  # raises AttributeError when the reference defines no such symbol


def test_layout_table(lib):
    lay = _layout()
    sizes = {"GAS": lib.mcpm_compat_sizeof(0), "BOX": lib.mcpm_compat_sizeof(1), "CELLS": lib.mcpm_compat_sizeof(2)}
    assert lib.mcpm_compat_sizeof(3) == -1
    for t, n in sizes.items():
        assert n == lay["SIZEOF_" + t][0]
        spans = []
        for key, v in lay.items():
            if not key.startswith(t + "_"):
                continue
            sz = C.c_int64(0)
            off = lib.mcpm_compat_offset(("%s.%s" % (t, key[len(t) + 1:])).encode(), C.byref(sz))
            assert (off, sz.value) == v, key
            assert off % 4 == 0 and off + sz.value <= n, key
            spans.append((off, off + sz.value))
        spans.sort()
        for a, b in zip(spans, spans[1:]):
            assert a[1] <= b[0], (t, a, b)
    assert lib.mcpm_compat_offset(b"GAS.nothing", None) == -1


def test_layout_matches_reference_header():
    sys.path.insert(0, COMPAT)
    try:
        import make_layout
    finally:
        sys.path.remove(COMPAT)
    src = os.environ.get("MCPM_REFERENCE_SRC") or os.path.join(os.path.dirname(REPO), "reference", "src")
    if not os.path.isfile(os.path.join(src, "cpp_headers.h")):
        pytest.skip("the reference's header is not present")
    with open(os.path.join(COMPAT, "ref_layout.h")) as fh:
        assert fh.read() == make_layout.layout_text(src)


def test_structs_and_strings(lib):
    import mcpm
    import workloads as W
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=6, ppc=4)
    st = D.Structs(lib, cfg, len(parts["x2"]))
    assert st.get(st.gas, "GAS.N", C.c_long) == 24
    assert st.get(st.box, "BOX.N", C.c_int, 1) == 6 and st.get(st.box, "BOX.Len", C.c_double, 1) == 6.0
    assert st.get(st.gas, "GAS.delta_t") == cfg.dt
    assert st.get(st.cell(5), "CELLS.n_ratio", C.c_int) == 1
    assert st.list_of(0).size == 0
    lib.mcpm_compat_set_model(st.gas, b"a model name longer than the short-string buffer")
    lib.mcpm_compat_set_model(st.gas, b"FP_dense")
    st.close()
    assert mcpm.MODEL_FP_DENSE in D.MODEL_NAMES


def test_unsupported_model_exits(built):
    """gas.model "SPH" is outside the particle step: the first routine prints
    the reason and exits with status 1 before any device work."""
    code = textwrap.dedent("""
        import workloads as W
        from compat_driver import MainLoop
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=4, ppc=8)
        ml = MainLoop(cfg, parts)
        ml.L.mcpm_compat_set_model(ml.st.gas, b"SPH")
        ml.set_step(1)
        ml.cell_update()
        print("not reached")
    """)
    env = dict(os.environ, PYTHONPATH=os.pathsep.join(p for p in sys.path if p))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 1, r.stdout + r.stderr
    assert "outside the particle step" in r.stderr
    assert "not reached" not in r.stdout
