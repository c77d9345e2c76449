"""Time sampling of the per-cell raw velocity sums (cell_poly_velocity,
src/Main_Functions.cpp:1918-1968) on the GPU against the oracle, whose
restatement tests/test_oracle_reference.py pins bit-exact to the reference.
The GPU sums each cell's particles in another order: within 1e-12 of each
field's scale."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _close(gpu, acc):
    """gpu: [SF_COUNT][C] from the session, acc: [C][SF_COUNT] from the oracle"""
    b = acc.T
    assert np.array_equal(gpu[mcpm.SF["WEIGHT"]], b[mcpm.SF["WEIGHT"]])
    for f, (lo, hi) in dict(M=(1, 4), MM=(4, 10), MMM=(10, 20), MMMM=(20, 26)).items():
        sc = max(np.max(np.abs(b[lo:hi])), 1e-300)
        assert np.max(np.abs(gpu[lo:hi] - b[lo:hi])) <= 1e-12 * sc, f


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_sample_cells_matches_oracle(cuda_ok, prec):
    cfg, parts = W.uneven_cells_2d(n_cells=(16, 12), precision=prec, hi=900)
    cfg64 = cfg.copy()
    cfg64.precision = mcpm.FP64
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg64, parts)
    if prec == mcpm.FP32:
        for k in ("x1", "x2", "U1", "U2", "U3"):
            getattr(o.s, k)[:] = getattr(o.s, k).astype(np.float32).astype(np.float64)
    rng = np.random.default_rng(31)
    xi = [rng.standard_normal(o.N) for _ in range(3)]
    s.inject_normals(*xi)
    o.inject_normals(*xi)
    s.set_step(2)
    o.set_step(2)
    acc = np.zeros((o.C, mcpm.SF_COUNT))
    for x in (s, o):
        x.cell_update()
    s.sample_cells()
    o.sample_cells(acc)
    _close(s.get_samples(), acc)
    if prec == mcpm.FP64:
        # a second sample after an FP velocity update adds to the first
        s.random_generator()
        s.velocity_update()
        o.random_generator()
        o.velocity_fp()
        for x in (s, o):
            x.cell_update()
        s.sample_cells()
        o.sample_cells(acc)
        _close(s.get_samples(), acc)
    s.reset_samples()
    assert not np.any(s.get_samples())


def test_sample_cells_after_fused_steps(cuda_ok):
    """1M particles, FP32 slotted steps, then cell_update + sample: the count
    field sums to N per sample and the first moments to the state's sums."""
    cfg, parts = W.uneven_cells_2d(n_cells=(64, 64), precision=mcpm.FP32, hi=2000)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    for _ in range(2):
        s.step(2)
        s.cell_update()
        s.sample_cells()
    smp = s.get_samples()
    g = s.download()
    assert smp[mcpm.SF["WEIGHT"]].sum() == 2 * len(g["U1"])
    # the last sample's first moments: the sums of the downloaded state
    s.reset_samples()
    s.cell_update()
    s.sample_cells()
    smp = s.get_samples()
    for j, k in enumerate(("U1", "U2", "U3")):
        tot = smp[mcpm.SF["M"] + j].sum()
        assert abs(tot - g[k].astype(np.float64).sum()) <= 1e-9 * np.abs(g[k]).sum(), k
