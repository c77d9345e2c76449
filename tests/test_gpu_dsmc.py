"""The DSMC_VHS model (Collision_DSMC_VHS, src/collisions.cpp:2063-2141):
Bird's no-time-counter collisions inside each cell on the GPU against the
oracle's restatement (pinned statistically to the reference by
tests/test_oracle_reference.py, whose draws come from std::random_device).
With the GPU's in-cell order given to the oracle, FP64 candidates, pairs and
acceptances coincide: velocities and majorants within 1e-12.  FP32 state is
checked on >= 99 % of the particles (a float acceptance test may flip a
candidate whose sigma_T / crm lies within rounding of its uniform) and on
size-independent invariants at 1M particles."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _make(shape, prec):
    if shape[0] == 1:
        # (1, 8): 400 particles a cell, past the warp's 256-slot conflict
        # table (the candidates are then compared pairwise over the warp)
        ppc = 400 if shape[1] == 8 else 80
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=shape[1], ppc=ppc, precision=prec)
    else:
        cfg, parts = W.esmc_box_2d(n_cells=shape, ppc=60, precision=prec)
    return W.with_dsmc_vhs(cfg), parts


def _same_layout_pass(cfg, parts):
    cfg64 = cfg.copy()
    cfg64.precision = mcpm.FP64
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg64, parts)
    if cfg.precision == mcpm.FP32:
        for k in ("x1", "x2", "U1", "U2", "U3"):
            getattr(o.s, k)[:] = getattr(o.s, k).astype(np.float32).astype(np.float64)
    for x in (s, o):
        x.set_step(0)
        x.cell_update()
        x.init_omega_max()
        x.set_step(1)
        x.cell_update()
    pid, off = s.get_layout()
    o.set_layout(off, pid)
    om0 = mcpm.cell_field(o.cells(), "OMEGA_MAX", True).copy()
    s.velocity_update()
    o.dsmc()
    return s, o, om0


@pytest.mark.parametrize("shape", [(1, 30), (14, 12), (1, 8)])
def test_dsmc_fp64_same_layout(cuda_ok, shape):
    cfg, parts = _make(shape, mcpm.FP64)
    s, o, om0 = _same_layout_pass(cfg, parts)
    g = s.download()
    for k in ("U1", "U2", "U3"):
        a, b = g[k], getattr(o.s, k)
        assert np.max(np.abs(a - b)) <= 1e-12 * max(1.0, np.max(np.abs(b))), k
    # some pairs collided, and the majorant moved (src/collisions.cpp:2135)
    assert np.count_nonzero(g["U1"] != parts["U1"]) > 0.05 * len(g["U1"])
    cg, co = mcpm.cell_field(s.get_cells(), "OMEGA_MAX"), mcpm.cell_field(o.cells(), "OMEGA_MAX", True)
    assert np.max(np.abs(cg - co)) <= 1e-12 * np.max(co)
    assert not np.array_equal(co, om0)
    for k in ("U1", "U2", "U3"):
        assert abs(g[k].sum() - parts[k].sum()) < 1e-9 * len(g[k])
    e0 = sum((parts[k] ** 2).sum() for k in ("U1", "U2", "U3"))
    e1 = sum((g[k] ** 2).sum() for k in ("U1", "U2", "U3"))
    assert abs(e1 - e0) < 1e-12 * e0


def test_dsmc_fp32_same_layout(cuda_ok):
    cfg, parts = _make((14, 12), mcpm.FP32)
    s, o, _ = _same_layout_pass(cfg, parts)
    g = s.download()
    scale = np.sqrt(np.mean(o.s.U1 ** 2))
    ok = np.ones(len(g["U1"]), dtype=bool)
    for k in ("U1", "U2", "U3"):
        ok &= np.abs(g[k] - getattr(o.s, k)) <= 1e-4 * scale
    assert ok.mean() >= 0.99, ok.mean()


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_dsmc_conserves_and_relaxes_1m(cuda_ok, prec):
    """1M particles, streaming off, 3 fused steps: every cell keeps its
    momentum and energy (elastic pair collisions), and the anisotropic
    temperature relaxes towards isotropy."""
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=100, ppc=10000, precision=prec)
    W.with_dsmc_vhs(cfg)
    cfg.direction[1] = 0
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.step(3)
    g = s.download()
    # each particle's cell as the session binned it (streaming is off, so it
    # never changes): an FP32 session bins the float-rounded position, which
    # can lie across a face from the double one
    idx = s.get_index().astype(np.int64)
    C = cfg.n_cells[1]
    u0 = {k: parts[k].astype(np.float32).astype(np.float64) if prec == mcpm.FP32 else parts[k]
          for k in ("U1", "U2", "U3")}
    tol = 1e-10 if prec == mcpm.FP64 else 2e-4
    for k in ("U1", "U2", "U3"):
        a = np.bincount(idx, weights=g[k], minlength=C)
        b = np.bincount(idx, weights=u0[k], minlength=C)
        assert np.max(np.abs(a - b)) <= tol * 10000, k
    e0 = np.bincount(idx, weights=u0["U1"] ** 2 + u0["U2"] ** 2 + u0["U3"] ** 2, minlength=C)
    e1 = np.bincount(idx, weights=g["U1"] ** 2 + g["U2"] ** 2 + g["U3"] ** 2, minlength=C)
    assert np.max(np.abs(e1 - e0) / e0) <= tol
    d0 = np.var(parts["U1"]) - np.var(parts["U2"])
    d1 = np.var(g["U1"]) - np.var(g["U2"])
    assert 0 < d1 < 0.97 * d0
