"""The Vlasov force of 2-D boxes (node grid) on the GPU against the CPU
restatement: the nodal deposit n_n of cell_update (bit-exact in FP64), the
node potential of the direct quadrature (compute_Vlasov_2D) and of the
screened-Poisson FEM (compute_SP_2D, solved here by the sine transform,
there by dense LU), and the kick of the particles.

Tolerances (FP64): node potential within 1e-12 (direct) / 1e-10 (screened
Poisson) of its largest magnitude; kicked velocities within 1e-9 of the
kick's largest magnitude.  FP32: the kick within 1e-4 of its magnitude."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu

TOL_V = {mcpm.LR_DIRECT: 1e-12, mcpm.LR_SCREENED_POISSON: 1e-10}


def _box(lr, prec=mcpm.FP64, n_cells=(12, 10), ppc=40, model=mcpm.MODEL_NONE, seed=5, dx=1.0):
    return W.vlasov_box_2d(n_cells=n_cells, total=ppc * n_cells[0] * n_cells[1], precision=prec, seed=seed,
                           long_range=lr, model=model, dx=dx)


def _session(cfg, parts):
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    return s


@pytest.mark.parametrize("shape", [(12, 10), (5, 17)])
def test_node_density_bit_exact(cuda_ok, shape):
    cfg, parts = _box(mcpm.LR_SCREENED_POISSON, n_cells=shape)
    s, o = _session(cfg, parts), Oracle(cfg, parts)
    s.cell_update()
    o.cell_update()
    assert np.array_equal(s.get_node_density(), o.node_density())
    # the FP32 session takes count x Fn/volume instead of the running sum
    cfg32 = cfg.copy()
    cfg32.precision = mcpm.FP32
    s32 = _session(cfg32, parts)
    s32.cell_update()
    nn = o.node_density()
    assert np.max(np.abs(s32.get_node_density() - nn)) <= 1e-12 * np.max(nn)


@pytest.mark.parametrize("lr", [mcpm.LR_DIRECT, mcpm.LR_SCREENED_POISSON])
@pytest.mark.parametrize("shape,dx", [((12, 10), 1.0), ((7, 9), 1.0), ((16, 12), 0.5)])
def test_node_potential_and_kick_fp64(cuda_ok, lr, shape, dx):
    cfg, parts = _box(lr, n_cells=shape, dx=dx)
    s, o = _session(cfg, parts), Oracle(cfg, parts)
    s.cell_update()
    o.cell_update()
    s.velocity_update()  # model none: the long-range kick alone
    V = o.long_range()
    Vg = s.get_node_potential()
    assert np.max(np.abs(Vg - V)) <= TOL_V[lr] * np.max(np.abs(V))
    g = s.download()
    for k in ("U1", "U2"):
        kick = getattr(o.s, k) - parts[k]
        assert np.max(np.abs(kick)) > 0
        err = np.max(np.abs(g[k] - getattr(o.s, k))) / np.max(np.abs(kick))
        assert err <= 1e-9, (k, err)
    assert np.array_equal(g["U3"], parts["U3"])


@pytest.mark.parametrize("lr", [mcpm.LR_DIRECT, mcpm.LR_SCREENED_POISSON])
def test_kick_fp32(cuda_ok, lr):
    cfg, parts = _box(lr, n_cells=(24, 20))
    cfg32 = cfg.copy()
    cfg32.precision = mcpm.FP32
    s, o = _session(cfg32, parts), Oracle(cfg, parts)
    s.cell_update()
    o.cell_update()
    s.velocity_update()
    o.long_range()
    g = s.download()
    for k in ("U1", "U2"):
        kick = getattr(o.s, k) - parts[k]
        gk = g[k] - parts[k].astype(np.float32).astype(np.float64)
        err = np.max(np.abs(gk - kick)) / np.max(np.abs(kick))
        assert err <= 1e-4, (k, err)


def test_screened_poisson_larger_grid(cuda_ok):
    """the sine-transform solve against the dense LU on 33 x 25 nodes"""
    cfg, parts = _box(mcpm.LR_SCREENED_POISSON, n_cells=(32, 24), ppc=20)
    s, o = _session(cfg, parts), Oracle(cfg, parts)
    s.cell_update()
    o.cell_update()
    s.velocity_update()
    V = o.node_potential(mcpm.LR_SCREENED_POISSON)
    Vg = s.get_node_potential()
    assert np.max(np.abs(Vg - V)) <= 1e-10 * np.max(np.abs(V))


@pytest.mark.parametrize("lr", [mcpm.LR_DIRECT, mcpm.LR_SCREENED_POISSON])
def test_fused_step_fp_dense_2d_vlasov(cuda_ok, lr):
    """mcpm_step with FP_dense collisions and the 2-D force against orc_step
    (same Philox draws)"""
    cfg, parts = _box(lr, n_cells=(10, 8), ppc=50, model=mcpm.MODEL_FP_DENSE)
    s, o = _session(cfg, parts), Oracle(cfg, parts)
    s.set_step(1)
    o.set_step(1)
    s.step(2)
    o.step(2)
    g = s.download()
    for k in ("x1", "x2", "U1", "U2", "U3"):
        a, b = g[k], getattr(o.s, k)
        err = np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))
        assert err <= 1e-9, (k, err)


def test_fp32_quadrant_counts_after_fused_steps(cuda_ok):
    """FP32 sessions count cell quadrants against float thresholds (the
    smallest float at or above each cell centre).  After fused steps (a
    slotted layout) the deposit must equal a fresh session's from the same
    positions, and the FP64 session's exact comparison in double (counts x
    Fn/vol: equal up to the FP64 deposit's sequential sum)."""
    cfg, parts = _box(mcpm.LR_SCREENED_POISSON, prec=mcpm.FP32, n_cells=(24, 20), ppc=60, model=mcpm.MODEL_FP_DENSE)
    s = _session(cfg, parts)
    s.step(3)
    s.cell_update()
    after = s.get_node_density()
    g = s.download()
    r = _session(cfg, g)  # the same positions, binned and counted afresh
    r.cell_update()
    assert np.array_equal(after, r.get_node_density())
    cfg64 = cfg.copy()
    cfg64.precision = mcpm.FP64
    r64 = _session(cfg64, g)
    r64.cell_update()
    ref = r64.get_node_density()
    assert np.max(np.abs(after - ref)) <= 1e-12 * np.max(np.abs(ref))
