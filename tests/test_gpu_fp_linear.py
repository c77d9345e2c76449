"""The FP_linear model (Velocity_FP_linear, src/Fokker_Planck.cpp:1186-1283):
the Langevin relaxation M' <- A1 M' + A3 xi with the per-cell energy rescale
and no cubic drift, through the same kernels as Velocity_FP_parallel, against
the oracle's restatement (pinned to the reference by tests/golden/fp_linear_1d.npz).
FP64 within 1e-12 / 1e-10 (operation order as the reference's, no fused
multiply-adds); FP32 state within 5e-4 of the FP64 oracle after a step."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _linear(cfg):
    cfg.model = mcpm.MODEL_FP_LINEAR
    return cfg


def _pair(cfg, parts, seed=21, step=1, inject=True):
    s = mcpm.Session(cfg)
    s.upload(parts.get("x1"), parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg, parts)
    if inject:
        rng = np.random.default_rng(seed)
        xi = [rng.standard_normal(o.N) for _ in range(3)]
        s.inject_normals(*xi)
        o.inject_normals(*xi)
    s.set_step(step)
    o.set_step(step)
    return s, o


def _err(a, b):
    return np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))


def test_fp_linear_routines_fp64(cuda_ok):
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=30, ppc=120)
    s, o = _pair(_linear(cfg), parts)
    for x in (s, o):
        x.cell_update()
        x.random_generator()
    for a, b in zip(s.get_normals(), o.xi):
        assert _err(a, b) <= 1e-12
    # c and gamma are computed for FP_linear too (src/Main_Functions.cpp:2729)
    cg, co = s.get_cells(), o.cells()
    for f in ("C", "GAMMA"):
        b = mcpm.cell_field(co, f, True)
        assert np.max(np.abs(mcpm.cell_field(cg, f) - b)) <= 1e-9 * np.max(np.abs(b)), f
    s.velocity_update()
    o.velocity_fp()
    g = s.download()
    for k in ("U1", "U2", "U3"):
        assert _err(g[k], getattr(o.s, k)) <= 1e-12, k


@pytest.mark.parametrize("maker", ["relax", "uneven"])
def test_fp_linear_fused_step_philox_fp64(cuda_ok, maker):
    if maker == "relax":
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=25, ppc=80)
    else:
        cfg, parts = W.uneven_cells_2d(n_cells=(12, 10), precision=mcpm.FP64, hi=700)
    s, o = _pair(_linear(cfg), parts, inject=False)
    s.set_rng(mcpm.RNG_PHILOX)
    o.set_rng(mcpm.RNG_PHILOX)
    s.step(3)
    o.step(3)
    g = s.download()
    for k in ("x1", "x2", "U1", "U2", "U3"):
        assert _err(g[k], getattr(o.s, k)) <= 1e-10, k


def test_fp_linear_fused_step_fp32(cuda_ok):
    """FP32 state (slotted layout, drift-free per-cell records) against the FP64 oracle."""
    cfg64, parts = W.uneven_cells_2d(n_cells=(16, 16), precision=mcpm.FP64, hi=900)
    _linear(cfg64)
    cfg32 = cfg64.copy()
    cfg32.precision = mcpm.FP32
    s = mcpm.Session(cfg32)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg64, parts)
    s.set_step(1)
    o.set_step(1)
    s.step(1)
    o.step(1)
    g = s.download()
    for k in ("U1", "U2", "U3"):
        err = np.max(np.abs(g[k] - getattr(o.s, k)))
        assert err < 5e-4, (k, err)


def test_fp_linear_conserves_and_relaxes(cuda_ok):
    """1M particles, FP64: per-cell momentum and energy are unchanged by the
    update (centred noise, energy rescale, src/Fokker_Planck.cpp:1276-1283);
    the temperature anisotropy of the homogeneous box relaxes towards
    isotropy, and faster than nothing: T11 - T22 shrinks by about A1^2 per step."""
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=100, ppc=10000)
    _linear(cfg)
    cfg.direction[1] = 0  # streaming off: the cells keep their particles
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_rng(mcpm.RNG_PHILOX)
    s.set_step(1)
    s.cell_update()
    c0 = s.get_cells()
    s.random_generator()
    s.velocity_update()
    g = s.download()
    idx = s.get_index()
    C = s.C
    cnt = np.bincount(idx, minlength=C)
    for k, f in ((0, "U1"), (1, "U2"), (2, "U3")):
        sums = np.bincount(idx, weights=g[f], minlength=C)
        us = c0[mcpm.CF["U_SPACE"] + k]
        np.testing.assert_allclose(sums, us * cnt, rtol=0, atol=1e-9 * (1 + np.abs(us * cnt)).max())
    us = c0[mcpm.CF["U_SPACE"]:mcpm.CF["U_SPACE"] + 3][:, idx]
    e = np.bincount(idx, weights=((g["U1"] - us[0]) ** 2 + (g["U2"] - us[1]) ** 2 + (g["U3"] - us[2]) ** 2),
                    minlength=C)
    np.testing.assert_allclose(e, c0[mcpm.CF["DM2"]] * cnt, rtol=1e-10, atol=1e-12)
    d0 = np.var(parts["U1"]) - np.var(parts["U2"])
    d1 = np.var(g["U1"]) - np.var(g["U2"])
    assert 0 < d1 < d0
