"""A session with no particles: uploads, fused steps (eager, graph pairs and
the 2-D screened-Poisson force beside the moment pass), cell updates and
downloads all run, every cell is empty, nothing becomes NaN and no error is
raised -- as the oracle's step runs on an empty particle set.  (A cell of
one to three particles is not an edge the reference survives: its
temperature is zero or its 4x4 system singular and its positions become
NaN, which the step reports as MCPM_ERR_NAN, tests/test_gpu_parity.py.)"""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu

EMPTY = np.zeros(0)


def _empty():
    return dict(x1=EMPTY, x2=EMPTY, U1=EMPTY, U2=EMPTY, U3=EMPTY)


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
@pytest.mark.parametrize("maker", ["relax", "uneven", "vlasov2d"])
def test_no_particles(cuda_ok, prec, maker):
    if maker == "relax":
        cfg, _ = W.homogeneous_relaxation_1d(n_cells=20, ppc=10, precision=prec)
    elif maker == "uneven":
        cfg, _ = W.uneven_cells_2d(n_cells=(8, 6), precision=prec, hi=100)
    else:
        cfg, _ = W.vlasov_box_2d(n_cells=(8, 8), total=8 * 8 * 20, precision=prec,
                                 long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
    parts = _empty()
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(1)
    s.step(5)  # eager steps and graph pairs
    s.cell_update()
    g = s.download()
    assert all(len(g[k]) == 0 for k in ("x1", "x2", "U1", "U2", "U3"))
    cells = s.get_cells()
    assert np.all(mcpm.cell_field(cells, "NUM_INSIDE") == 0)
    for f in ("N", "T", "PIJ", "C", "GAMMA", "ALPHA", "BETA", "LAMBDA"):
        assert np.all(np.isfinite(mcpm.cell_field(cells, f))), f
    assert s.step_count == 6
    o = Oracle(cfg if prec == mcpm.FP64 else _fp64(cfg), parts)
    o.set_step(1)
    o.step(5)
    assert o.N == 0


def _fp64(cfg):
    c = cfg.copy()
    c.precision = mcpm.FP64
    return c
