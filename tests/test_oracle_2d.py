"""The CPU restatement of the 2-D rows against the reference's own build:
the nodal deposit n_n of cell_update (src/Main_Functions.cpp:2268-2364),
compute_Vlasov_2D (src/FEM.cpp:613-726) and compute_SP_2D
(src/FEM.cpp:249-610, with the dense LU standing in for PARDISO)."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(REPO, "monte-carlo-particle-method_gb300"))
sys.path.insert(0, os.path.join(REPO, "oracle"))

import mcpm  # noqa: E402
import workloads as W  # noqa: E402
from oracle import Oracle, Reference, ref_lib  # noqa: E402

needs_ref = pytest.mark.skipif(ref_lib() is None, reason="reference sources not present")


def _pair(lr, n_cells=(6, 5), ppc=30, seed=11):
    cfg, parts = W.vlasov_box_2d(n_cells=n_cells, total=ppc * n_cells[0] * n_cells[1], precision=mcpm.FP64,
                                 seed=seed, long_range=lr)
    return cfg, parts, Oracle(cfg, parts), Reference(cfg, parts)


@needs_ref
def test_node_density_bit_exact():
    cfg, parts, o, r = _pair(mcpm.LR_SCREENED_POISSON)
    o.cell_update()
    r.cell_update()
    assert np.array_equal(o.s.index, r.s.index)
    assert np.array_equal(o.node_density(), r.node_density())
    # every node's count of particles appears in each cell slot that shares it
    nn = o.node_density()
    assert np.all(nn >= 0) and nn.sum() > 0


# compute_Vlasov_2D's GL(100) table is a literal whose weights are accurate
# to about 1e-11 relative; the restatement computes the table to full double
# precision, so its kick agrees to ~1e-12 of the kick's size.  The GL(50)
# table of compute_SP_2D is the 8-decimal rounding, reproduced exactly, and
# that path agrees bit for bit.
TOL = {mcpm.LR_DIRECT: 1e-11, mcpm.LR_SCREENED_POISSON: 0.0}


@needs_ref
@pytest.mark.parametrize("lr", [mcpm.LR_DIRECT, mcpm.LR_SCREENED_POISSON])
def test_long_range_2d_matches_reference(lr):
    cfg, parts, o, r = _pair(lr)
    o.cell_update()
    r.cell_update()
    # all fields but the kernel-smoothing ones (computed for long_range 2 only)
    sm = mcpm.CF["N_SMOOTH"]
    assert np.array_equal(o.cells()[:, :sm], r.cells()[:, :sm])
    o.long_range()
    r.long_range()
    for k in ("U1", "U2"):
        a, b = getattr(o.s, k), getattr(r.s, k)
        d0 = b - parts[k]
        assert np.max(np.abs(d0)) > 0, "the force moved nothing"
        err = np.max(np.abs(a - b)) / np.max(np.abs(d0))
        assert err <= TOL[lr], "%s: kick differs from the reference by %.3e of its size" % (k, err)
    assert np.array_equal(o.s.U3, r.s.U3)
