"""Slotted layouts of the FP32 fused step.

The particle pass writes each particle straight into its new cell's region of
the other buffer (capacity count + max(16, count / 4), rounded up to 8),
regions that fill up send the rest into overflow arrays, and the next scan's
repair pass packs those back.  The comparison is the same step with packed
layouts (MCPM_SLOTTED=0: keys, scan and the scatter pass) and the FP64
oracle; a converging flow that sends every particle of an 8 x 8 box into its
four central cells forces the overflow path on the first step (each of those
cells receives about 16 times its region's capacity).

Tolerances: FP32 state against the FP64 oracle, positions within 1e-4 of the
box size after free flights of up to half the box; slotted against packed,
1e-4 relative (the in-cell order differs, which reorders FP32 sums)."""
import os

import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _session(cfg, parts, slotted):
    old = os.environ.get("MCPM_SLOTTED")
    os.environ["MCPM_SLOTTED"] = "1" if slotted else "0"
    try:
        s = mcpm.Session(cfg)
    finally:
        if old is None:
            del os.environ["MCPM_SLOTTED"]
        else:
            os.environ["MCPM_SLOTTED"] = old
    s.upload(parts.get("x1"), parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(1)
    return s


def _converging_box(n=8, N=20000, seed=5):
    """Free flight (no collision model) in a closed 8 x 8 box of unit cells:
    every particle aimed at a point within 0.45 of the centre, so that after
    one step the four central cells hold all N particles."""
    cfg = W._base((n, n), (float(n), float(n), 1.0), (1, 1), mcpm.PROBLEM_CLOSED_BOX, mcpm.MODEL_NONE, mcpm.FP32,
                  n=0.1, T=1.0)
    rng = np.random.default_rng(seed)
    x1 = rng.uniform(0.05, n - 0.05, N)
    x2 = rng.uniform(0.05, n - 0.05, N)
    t1 = n / 2 + rng.uniform(-0.45, 0.45, N)
    t2 = n / 2 + rng.uniform(-0.45, 0.45, N)
    parts = dict(x1=x1, x2=x2, U1=(t1 - x1) / cfg.dt, U2=(t2 - x2) / cfg.dt, U3=rng.normal(0, 1, N))
    mcpm.derive(cfg, N)
    cfg.max_particles = N
    return cfg, parts


@pytest.mark.parametrize("steps", [1, 2, 5])
def test_overflowing_regions_are_repaired(cuda_ok, steps):
    cfg, parts = _converging_box()
    s = _session(cfg, parts, True)
    cfg64 = cfg.copy()
    cfg64.precision = mcpm.FP64
    o = Oracle(cfg64, parts)
    o.set_step(1)
    s.step(steps)
    o.step(steps)
    g = s.download()
    L = float(cfg.length[0])
    for k in ("x1", "x2"):
        err = np.max(np.abs(g[k] - getattr(o.s, k)))
        assert err <= 1e-4 * L, (k, err)
    for k in ("U1", "U2", "U3"):
        b = getattr(o.s, k)
        assert np.max(np.abs(g[k] - b)) <= 1e-5 * max(1.0, np.max(np.abs(b))), k
    # every particle once: the cell counts of the final positions
    s.cell_update()
    n_in = mcpm.cell_field(s.get_cells(), "NUM_INSIDE")
    assert int(n_in.sum()) == len(parts["x1"])
    if steps == 1:
        c = np.arange(64)
        centre = ((c % 8 == 3) | (c % 8 == 4)) & ((c // 8 == 3) | (c // 8 == 4))
        assert int(n_in[centre].sum()) == len(parts["x1"])


def test_slotted_steps_match_packed_steps(cuda_ok):
    """The benchmark's 2-D Enskog-Vlasov box (screened-Poisson force) at
    24 x 24 cells: nine fused steps (graph pairs and eager steps) with
    slotted and with packed layouts."""
    cfg, parts = W.vlasov_box_2d(n_cells=(24, 24), total=244 * 576, precision=mcpm.FP32,
                                 long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
    a, b = _session(cfg, parts, True), _session(cfg, parts, False)
    for s in (a, b):
        s.step(9)
    ga, gb = a.download(), b.download()
    for k in ("x1", "x2", "U1", "U2", "U3"):
        err = np.max(np.abs(ga[k] - gb[k])) / max(1.0, np.max(np.abs(gb[k])))
        assert err <= 1e-4, (k, err)
    for s in (a, b):
        s.cell_update()
    na = mcpm.cell_field(a.get_cells(), "NUM_INSIDE")
    nb = mcpm.cell_field(b.get_cells(), "NUM_INSIDE")
    assert na.sum() == nb.sum() == len(parts["x2"])
    # a particle within rounding of a face may bin either way
    assert np.abs(na - nb).sum() <= 4


def test_slotted_layout_survives_split_calls(cuda_ok):
    """Fused steps leave a slotted layout; the routines of the split loop
    body, the index and the download pack it first."""
    cfg, parts = W.vlasov_box_2d(n_cells=(12, 10), total=244 * 120, precision=mcpm.FP32,
                                 long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
    s = _session(cfg, parts, True)
    s.step(3)
    idx = s.get_index()  # the cell of every particle
    s.cell_update()
    n_in = mcpm.cell_field(s.get_cells(), "NUM_INSIDE")
    assert np.array_equal(np.bincount(idx, minlength=s.C), n_in)
    s.step(2)
    s.cell_update()
    s.random_generator()
    s.velocity_update()
    s.step(2)
    g = s.download()
    assert np.all(np.isfinite(g["U1"])) and np.all((g["x2"] >= 0) & (g["x2"] <= cfg.length[1]))


def test_slotted_layout_carries_old_positions(cuda_ok):
    """Diffuse (thermal) walls read each particle's position before its
    flight, which the slotted layout must move along with it: the FP_dense
    Couette box with a hot wall, four fused steps with slotted and with
    packed layouts.  The wall draws are keyed by particle id and step, so
    the two runs differ only by the in-cell order of FP32 sums."""
    cfg, parts = W.esmc_box_2d(n_cells=(12, 10), ppc=80, precision=mcpm.FP32)
    cfg.model = mcpm.MODEL_FP_DENSE
    a, b = _session(cfg, parts, True), _session(cfg, parts, False)
    for s in (a, b):
        s.step(4)
    ga, gb = a.download(), b.download()
    for k in ("x1", "x2", "U1", "U2", "U3"):
        err = np.max(np.abs(ga[k] - gb[k])) / max(1.0, np.max(np.abs(gb[k])))
        assert err <= 1e-4, (k, err)
    # the hot wall heated the gas near it in both runs alike
    assert np.all(np.isfinite(ga["U1"]))
