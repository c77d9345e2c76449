"""The learned 2-D Vlasov force on the GPU against its CPU oracle
(oracle/surrogate_oracle.py) and against the plain node-grid force.

Tolerances: the GPU sums in fp32 where the oracle sums in float64 at the same
bf16 rounding points, so a bf16 activation or gradient occasionally rounds
the other way; outputs agree within 5e-3 (relative L2), gradients within
3e-2 per layer; the tcgen05 and mma.sync forward paths within 3e-3."""
import os

import numpy as np
import pytest

import mcpm
import surrogate as S
import surrogate_oracle as SO
import workloads as W

pytestmark = pytest.mark.gpu


def _torch():
    torch = pytest.importorskip("torch")
    return torch


def _params(seed):
    rng = np.random.default_rng(seed)
    p = SO.init_params(seed).astype(np.float32)
    d = SO.unpack(p)
    for k in ("b1", "b2", "b3"):
        d[k][:] = rng.normal(0, 0.1, d[k].shape)
    d["b4"][:4] = rng.normal(0, 0.1, 4)
    return SO.pack(d)


def _inputs(seed, B, n1, n0):
    rng = np.random.default_rng(seed)
    x = np.zeros((B, n1, n0, 16), np.float32)
    x[..., :5] = rng.normal(0, 1, (B, n1, n0, 5))
    x[..., 5] = 1.0
    x[..., 6:11] = rng.normal(0, 0.004, (B, n1, n0, 5))
    return SO.bf16(x)


def _dev_bf16(torch, x):
    bits = SO.float_to_bf16_bits(x).reshape(x.shape[0], -1, 16)
    return torch.from_numpy(bits.view(np.int16)).cuda()


def _rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("shape", [(2, 13, 20), (1, 7, 130)])
def test_forward_mma_matches_oracle(cuda_ok, shape):
    torch = _torch()
    B, n1, n0 = shape
    p = _params(1)
    x = _inputs(2, B, n1, n0)
    sur = mcpm.Surrogate(n0, n1, B)
    sur.set_params(p, 1.0)
    sur.set_tensor_path(False)
    xd = _dev_bf16(torch, x)
    y = torch.zeros((B, n1 * n0, 4), dtype=torch.float32, device="cuda")
    sur.forward(xd.data_ptr(), B, y.data_ptr())
    yo, _ = SO.forward(p, x)
    assert _rel(y.cpu().numpy().reshape(yo.shape), yo) < 5e-3


@pytest.mark.parametrize("shape", [(2, 5, 256), (1, 9, 200), (3, 4, 32)])
def test_forward_tcgen05_matches_mma(cuda_ok, shape):
    torch = _torch()
    B, n1, n0 = shape
    p = _params(3)
    x = _inputs(4, B, n1, n0)
    sur = mcpm.Surrogate(n0, n1, B)
    sur.set_params(p, 1.0)
    xd = _dev_bf16(torch, x)
    out = []
    for tc in (False, True):
        sur.set_tensor_path(tc)
        y = torch.zeros((B, n1 * n0, 4), dtype=torch.float32, device="cuda")
        sur.forward(xd.data_ptr(), B, y.data_ptr())
        out.append(y.cpu().numpy())
    n_tc, on = sur.tensor_path()
    assert on and n_tc == 4, "all four layers ran on tcgen05"
    assert np.all(np.isfinite(out[1]))
    assert _rel(out[1], out[0]) < 3e-3
    yo, _ = SO.forward(p, x)
    assert _rel(out[1].reshape(yo.shape), yo) < 5e-3


@pytest.mark.parametrize("tc", [True, False])
def test_gradients_match_oracle(cuda_ok, tc):
    """Loss and all parameter gradients against the oracle's FP64 backward
    pass, on the tcgen05 path (forward and the three data-gradient
    convolutions: 7 tcgen05 launches per batch) and on mma.sync."""
    torch = _torch()
    B, n1, n0 = 2, 9, 14
    p = _params(5)
    x = _inputs(6, B, n1, n0)
    t = np.random.default_rng(7).normal(0, 1, (B, n1, n0, 4)).astype(np.float32)
    ts = 0.5
    sur = mcpm.Surrogate(n0, n1, B)
    sur.set_params(p, 1.0)
    sur.set_tensor_path(tc)
    xd = _dev_bf16(torch, x)
    td = torch.from_numpy(t.reshape(B, -1, 4)).cuda()
    n0_tc = sur.tensor_path()[0]
    g, loss = sur.gradients(xd.data_ptr(), td.data_ptr(), B, ts)
    assert sur.tensor_path() == ((n0_tc + 7, True) if tc else (n0_tc, False))
    lo, se, st, go = SO.loss_and_grad(p, x, t, ts)
    assert abs(loss[0] - se) <= 2e-3 * se and abs(loss[1] - st) <= 1e-6 * st
    dg, do = SO.unpack(g), SO.unpack(go)
    for name, _ in SO.SIZES:
        assert _rel(dg[name], do[name]) < 3e-2, name
    assert np.all(dg["W4"][4:] == 0) and np.all(dg["W1"][:, :, 11:] == 0)


def _sp_cfg(n, prec=mcpm.FP32, dx=1.0):
    return W.vlasov_box_2d(n_cells=(n, n), total=244 * n * n, precision=prec, long_range=mcpm.LR_SCREENED_POISSON,
                           model=mcpm.MODEL_FP_DENSE, dx=dx)


def test_snapshots_are_the_plain_force(cuda_ok):
    torch = _torch()
    cfg, _ = W.vlasov_box_2d(n_cells=(12, 10), total=244 * 120, precision=mcpm.FP64,
                             long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_NONE)
    s = mcpm.Session(cfg)
    C = s.C
    F = S.random_fields(np.random.default_rng(1), 3)
    x = torch.zeros((3, C, 16), dtype=torch.int16, device="cuda")
    y = torch.zeros((3, C, 4), dtype=torch.float32, device="cuda")
    s.vlasov_snapshots(F, S.N_WAVES, 99, x.data_ptr(), y.data_ptr())
    # the last snapshot's nodal data and potential are the session's now
    V = s.get_node_potential().reshape(cfg.n_cells[1] + 1, cfg.n_cells[0] + 1)
    d = np.stack([V[:-1, 1:] - V[:-1, :-1], V[1:, 1:] - V[1:, :-1], V[1:, :-1] - V[:-1, :-1],
                  V[1:, 1:] - V[:-1, 1:]], axis=-1).reshape(C, 4)
    yl = y[2].cpu().numpy()
    assert np.max(np.abs(yl - d)) <= 1e-6 * np.max(np.abs(d))
    nn = s.get_node_density()
    xl = SO.bf16_bits_to_float(x[2].cpu().numpy().view(np.uint16))
    v = 10.0 * (cfg.b * nn - 0.25)
    hi = SO.bf16(v.astype(np.float32))
    assert np.array_equal(xl[:, :4], hi)
    assert np.array_equal(xl[:, 6:10], SO.bf16((v - hi).astype(np.float32)))
    assert np.max(np.abs(xl[:, :4].astype(np.float64) + xl[:, 6:10] - v)) <= 2.0 ** -15 * np.max(np.abs(v))
    assert np.all(xl[:, 5] == 1.0) and np.all(xl[:, 11:] == 0.0)
    # the quadrant counts follow the field: mean packing fraction near the field's
    n_cell = s.get_cells()[mcpm.CF["N"]]
    assert abs(np.mean(n_cell * cfg.b) - np.mean(np.clip(F[2, 0], 0.05, 0.45))) < 0.03


def test_training_reduces_the_loss(cuda_ok):
    torch = _torch()
    cfg, _ = _sp_cfg(32)
    s = mcpm.Session(cfg)
    x, y = S.make_snapshots(s, 520, seed=3)
    params, scale, info = S.train(cfg, n_val=8, batch=8, epochs=6, lr=2e-3, seed=4, log=print, x=x, y=y,
                                  log_every=64)
    h = info["history"]
    print(h, info["val_kick_error"])
    assert h[-1][1] < 0.5 * h[0][1]
    assert info["val_kick_error"] < 0.5


def test_untrained_network_hands_over_to_the_plain_path(cuda_ok):
    """A network whose kick is far off is judged on the first step and the
    plain path takes over: the particles then evolve exactly as without it."""
    torch = _torch()
    cfg, parts = _sp_cfg(24)
    runs = []
    for attach in (False, True):
        s = mcpm.Session(cfg)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        sur = None
        if attach:
            sur = mcpm.Surrogate(24, 24, 1)
            sur.set_params(SO.init_params(9), 1.0)
            s.attach_surrogate(sur, judge_every=4, threshold=0.01)
        s.step(9)
        runs.append(s.download())
        if attach:
            st = s.surrogate_stats()
            assert st["judged"] == 3 and st["takeovers"] == 3 and st["active"] == 0
            assert st["plain_steps"] == 9 and st["surrogate_steps"] == 0 and st["last_error"] > 0.01
    # the binning's atomics order particles within a cell differently from
    # run to run, so sums round differently: equal to FP32 rounding, while
    # one kick of the untrained network would move U by O(0.1)
    for k in ("x1", "x2", "U1", "U2", "U3"):
        assert np.max(np.abs(runs[0][k] - runs[1][k])) < 1e-4 * max(1.0, np.max(np.abs(runs[0][k]))), k


@pytest.mark.parametrize("trained", [False, True])
def test_queued_steps_keep_the_judges_verdicts(cuda_ok, trained):
    """Queued steps (mcpm_step_async) read a judge step's verdict when the
    next step is queued: one step at a time without waiting gives the same
    judge record as the steps in one waiting call, and particles that differ
    from it no more than a second waiting run's do -- for a network that is
    kept in charge and for one the plain path takes over from."""
    if trained and not os.path.exists(S.WEIGHTS):
        pytest.skip("no trained weights")
    _torch()
    n = 128 if trained else 24
    cfg, parts = _sp_cfg(n)
    runs = []
    for wait in (True, True, False):
        s = mcpm.Session(cfg)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        if trained:
            sur = S.attach(s, judge_every=3, threshold=0.01)
        else:
            sur = mcpm.Surrogate(n, n, 1)
            sur.set_params(SO.init_params(9), 1.0)
            s.attach_surrogate(sur, judge_every=3, threshold=0.01)
        if wait:
            s.step(10)
        else:
            for _ in range(10):
                s.step(1, wait=False)
        st = s.surrogate_stats()  # reads the last judge step's verdict
        s.sync()
        s.check_status()
        runs.append((st, s.download()))
        sur.close()
    (sa, ga), (sr, gr), (sb, gb) = runs
    for key in ("judged", "takeovers", "surrogate_steps", "plain_steps", "active"):
        assert sa[key] == sb[key] == sr[key], (key, sa, sb)
    assert sa["judged"] == 4
    assert sa["takeovers"] == (0 if trained else 4)
    # the binning's atomics order the particles within a cell differently
    # from run to run, so FP32 sums round differently; now and then a
    # particle next to a cell face then bins into the neighbour, and the
    # two cells' particles take updates that differ by more than rounding.
    # Two waiting runs show how many such particles to expect.
    for k in ("x1", "x2", "U1", "U2", "U3"):
        tol = 1e-4 * max(1.0, np.max(np.abs(ga[k])))
        rep = np.mean(np.abs(ga[k] - gr[k]) >= tol)
        que = np.mean(np.abs(ga[k] - gb[k]) >= tol)
        assert que <= max(1e-5, 3 * rep), (k, que, rep)


@pytest.mark.skipif(not os.path.exists(S.WEIGHTS), reason="no trained weights")
def test_trained_network_gains_over_the_plain_path(cuda_ok):
    """The trained network's kick is within 1% of the plain path's on a live
    particle state, the judge keeps it in charge, and its force costs less
    device time per step than the plain path's."""
    torch = _torch()
    cfg, parts = _sp_cfg(128)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    sur = S.attach(s, judge_every=5, threshold=0.01)
    s.step(6)
    s.cell_update()
    s.eval_vlasov_2d(0)
    plain = s.get_kick_2d()
    s.eval_vlasov_2d(1)
    net = s.get_kick_2d()
    assert _rel(net, plain) < 0.01
    st = s.surrogate_stats()
    assert st["judged"] == 2 and st["takeovers"] == 0 and 0 <= st["last_error"] < 0.01
    s.profile(True)
    for _ in range(5):
        s.eval_vlasov_2d(0)
        s.eval_vlasov_2d(1)
    prof = s.profile_read()
    s.profile(False)
    assert prof["surrogate"][0] < prof["long_range"][0], prof
    sur.close()


@pytest.mark.skipif(not os.path.exists(S.WEIGHTS), reason="no trained weights")
def test_network_branch_reads_this_steps_densities(cuda_ok):
    """Between judge steps the network's branch (nodal deposit and network on
    a second stream) runs beside the moment pass and the per-cell solve,
    which writes the cell densities; the deposit kernel writes the network's
    input, the cell density from the layout's counts by the solve's own
    operations.  A profiled run executes every
    kernel in order on one stream and feeds the network the solve's
    densities: the two runs' kicks agree wherever the runs' particles bin
    alike (the in-cell order of the slotted passes reorders FP32 sums), so
    the branch's result does not depend on whether the solve has written the
    densities when the network reads its input."""
    cfg, parts = W.vlasov_box_2d(n_cells=(64, 64), total=244 * 64 * 64, precision=mcpm.FP32,
                                 long_range=mcpm.LR_SCREENED_POISSON, model=mcpm.MODEL_FP_DENSE)
    runs = []
    for profiled in (False, True):
        s = mcpm.Session(cfg)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        S.attach(s, judge_every=1000, threshold=1e9)  # in charge after the first (judge) step
        if profiled:
            s.profile(True)
        s.step(6)
        runs.append((s.get_kick_2d(), s.download()))
    (ka, ga), (kb, gb) = runs
    for k in ("x1", "x2", "U1", "U2", "U3"):
        err = np.max(np.abs(ga[k] - gb[k])) / max(1.0, np.max(np.abs(gb[k])))
        assert err <= 1e-4, (k, err)
    differ = np.any(ka != kb, axis=1)
    assert differ.mean() <= 0.02, differ.mean()
    assert np.linalg.norm(ka - kb) <= 1e-3 * np.linalg.norm(kb)
