"""long_range 2, the density-expansion force (src/Main_Functions.cpp:1632-1653)
from the kernel-smoothed density of cell_update (:2378-2427), on the GPU
against the oracle (pinned bit-exact to the reference by
tests/test_oracle_reference.py and tests/golden/density_expansion_1d.npz).
The GPU sums each cell's Gaussian terms in a different order: FP64 fields
within 1e-12 of their scale, FP64 particles within 1e-10 after fused steps;
FP32 state within 5e-4 of the FP64 oracle after a step."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _case(shape, prec=mcpm.FP64):
    if shape == "1d":
        cfg, parts = W.vlasov_slab_1d(n_cells=80, mean_ppc=60, long_range=mcpm.LR_DENSITY_EXPANSION, precision=prec)
    else:
        cfg, parts = W.uneven_cells_2d(n_cells=(12, 10), precision=prec, hi=700)
        cfg.long_range, cfg.phi = mcpm.LR_DENSITY_EXPANSION, -1.0
    return cfg, parts


def _pair(cfg, parts, step=2):
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg, parts)
    s.set_step(step)
    o.set_step(step)
    return s, o


@pytest.mark.parametrize("shape", ["1d", "2d"])
def test_smoothing_fields_fp64(cuda_ok, shape):
    cfg, parts = _case(shape)
    s, o = _pair(cfg, parts)
    s.cell_update()
    o.cell_update()
    cg, co = s.get_cells(), o.cells()
    for f in ("N_SMOOTH", "DN2", "DN3"):
        a, b = mcpm.cell_field(cg, f), mcpm.cell_field(co, f, True)
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b)), f
    # the GPU's cell_update already forms the force velocity_update applies;
    # the oracle forms it in its long-range call
    o.long_range()
    a, b = mcpm.cell_field(cg, "F2"), mcpm.cell_field(o.cells(), "F2", True)
    assert np.max(np.abs(a - b)) <= 1e-11 * np.max(np.abs(b))
    N1 = cfg.n_cells[1]
    assert a[0] == 0.0 and a[N1 - 1] == 0.0  # no kick in cell 0 and cell N[1]-1


@pytest.mark.parametrize("shape", ["1d", "2d"])
def test_density_expansion_fused_step_fp64(cuda_ok, shape):
    cfg, parts = _case(shape)
    s, o = _pair(cfg, parts, step=1)
    s.set_rng(mcpm.RNG_PHILOX)
    o.set_rng(mcpm.RNG_PHILOX)
    s.step(3)
    o.step(3)
    g = s.download()
    for k in ("x2", "U1", "U2", "U3") if shape == "1d" else ("x1", "x2", "U1", "U2", "U3"):
        a, b = g[k], getattr(o.s, k)
        assert np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b))) <= 1e-10, k
    a, b = mcpm.cell_field(s.get_cells(), "F2"), mcpm.cell_field(o.cells(), "F2", True)
    assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b))


def test_density_expansion_fused_step_fp32(cuda_ok):
    cfg64, parts = _case("1d")
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
