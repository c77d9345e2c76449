"""The FP32 sessions' per-cell solves (mcpm_solve_fast.cu): the c/gamma 9x9
by FP32 LU with FP64 iterative refinement, alpha/beta by block elimination
of the three 4x4 systems.  Their coefficients must be the FP64 solutions of
the systems the reference builds (src/Fokker_Planck.cpp:200-804) from the
cell's own moments: rebuilt here from the exported CELLS fields and solved
by LAPACK in FP64, agreeing to 1e-9 of each cell's largest coefficient."""
import numpy as np
import pytest

import mcpm
import workloads as W

pytestmark = pytest.mark.gpu


def F(cells, name):
    f, w = mcpm.CF[name], mcpm.CF_WIDTH[name]
    return cells[f:f + w].T  # [C][w]


def cg_system(cells):
    P, Q, M3, M4, M5 = (F(cells, k) for k in ("PIJ", "Q", "M3", "M4", "M5"))
    DM2, DM4 = F(cells, "DM2")[:, 0], F(cells, "DM4")[:, 0]
    C = P.shape[0]
    A = np.zeros((C, 9, 9))
    A[:, 0, [0, 1, 2, 6]] = 2 * np.stack([P[:, 0], P[:, 1], P[:, 2], Q[:, 0]], 1)
    A[:, 1, [0, 1, 2, 3, 4, 6, 7]] = np.stack([P[:, 1], P[:, 0] + P[:, 3], P[:, 4], P[:, 1], P[:, 2], Q[:, 1],
                                               Q[:, 0]], 1)
    A[:, 2, [0, 1, 2, 4, 5, 6, 8]] = np.stack([P[:, 2], P[:, 4], P[:, 0] + P[:, 5], P[:, 1], P[:, 2], Q[:, 2],
                                               Q[:, 0]], 1)
    A[:, 3, [1, 3, 4, 7]] = 2 * np.stack([P[:, 1], P[:, 3], P[:, 4], Q[:, 1]], 1)
    A[:, 4, [1, 2, 3, 4, 5, 7, 8]] = np.stack([P[:, 2], P[:, 1], P[:, 4], P[:, 3] + P[:, 5], P[:, 4], Q[:, 2],
                                               Q[:, 1]], 1)
    A[:, 5, [2, 4, 5, 8]] = 2 * np.stack([P[:, 2], P[:, 4], P[:, 5], Q[:, 2]], 1)
    A[:, 6, :6] = np.stack([Q[:, 0] + 2 * M3[:, 0], Q[:, 1] + 4 * M3[:, 1], Q[:, 2] + 4 * M3[:, 2], 2 * M3[:, 3],
                            4 * M3[:, 4], 2 * M3[:, 5]], 1)
    A[:, 7, :6] = np.stack([2 * M3[:, 1], Q[:, 0] + 4 * M3[:, 3], 4 * M3[:, 4], Q[:, 1] + 2 * M3[:, 6],
                            Q[:, 2] + 4 * M3[:, 7], 2 * M3[:, 8]], 1)
    A[:, 8, :6] = np.stack([2 * M3[:, 2], 4 * M3[:, 4], Q[:, 0] + 4 * M3[:, 5], 2 * M3[:, 7],
                            Q[:, 1] + 4 * M3[:, 8], Q[:, 2] + 2 * M3[:, 9]], 1)
    sym = [[0, 1, 2], [1, 3, 4], [2, 4, 5]]
    for r in range(3):
        for q in range(3):
            A[:, 6 + r, 6 + q] = 2 * M4[:, sym[r][q]] - 2 * P[:, sym[r][q]] * DM2
        A[:, 6 + r, 6 + r] += DM4 - DM2 * DM2
    return A, (P, Q, M3, M4, M5, DM2, DM4)


def test_fp32_solves_are_the_fp64_solutions(cuda_ok):
    cfg, parts = W.vlasov_box_2d(n_cells=(48, 48), total=244 * 48 * 48, precision=mcpm.FP32,
                                 long_range=mcpm.LR_NONE, model=mcpm.MODEL_FP_DENSE)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(1)
    s.cell_update()  # step > 0: alpha/beta as well
    cells = s.get_cells()
    ncnt = F(cells, "NUM_INSIDE")[:, 0]
    ok = ncnt >= 2
    A, (P, Q, M3, M4, M5, DM2, DM4) = cg_system(cells)
    T, n = F(cells, "T")[:, 0], F(cells, "N")[:, 0]
    Lam, gst = F(cells, "LAMBDA")[:, 0], F(cells, "GAMMA_ST")[:, 0]
    nb = n * cfg.b
    Y = 1.0 + 0.625 * nb + 0.2869 * nb ** 2 + 0.115 * nb ** 3
    mu = cfg.mu * (T / cfg.T0) ** cfg.visp
    tau = 2.0 * mu / (n * cfg.kb * T)
    # c / gamma right-hand side (src/Fokker_Planck.cpp:590-804)
    rhs = np.zeros((len(T), 9))
    rhs[:, :6] = -2.0 * Lam[:, None] * M4
    PQ = np.stack([P[:, 0] * Q[:, 0] + P[:, 1] * Q[:, 1] + P[:, 2] * Q[:, 2],
                   P[:, 1] * Q[:, 0] + P[:, 3] * Q[:, 1] + P[:, 4] * Q[:, 2],
                   P[:, 2] * Q[:, 0] + P[:, 4] * Q[:, 1] + P[:, 5] * Q[:, 2]], 1)
    rhs[:, 6:] = (Y * (3.0 - 4.0 / 3.0) / tau)[:, None] * Q + Lam[:, None] * (-3.0 * M5 + DM2[:, None] * Q + 2.0 * PQ)
    x = np.linalg.solve(A[ok], rhs[ok][:, :, None])[:, :, 0]
    got = np.concatenate([F(cells, "C"), F(cells, "GAMMA")], 1)[ok]
    scale = np.max(np.abs(x), axis=1)
    err = np.max(np.abs(got - x), axis=1) / scale
    assert np.max(err) <= 1e-9, np.max(err)
    # alpha / beta: three 4x4 systems per cell (src/Fokker_Planck.cpp:200-587)
    trace = P[:, 0] + P[:, 3] + P[:, 5]
    dev = P.copy()
    for j in (0, 3, 5):
        dev[:, j] -= trace / 3.0
    ma, mb, mc = M3[:, 0] + M3[:, 3] + M3[:, 5], M3[:, 1] + M3[:, 6] + M3[:, 8], M3[:, 2] + M3[:, 7] + M3[:, 9]
    d = M4[:, 0] + M4[:, 3] + M4[:, 5] - DM2 * DM2
    nbY = nb * Y
    mu_crr, p_crr, k_crr = 1 + 2 * nbY / 5, 1 + nbY, 1 + 3 * nbY / 5
    w = (4.0 / 9.0) * np.sqrt(np.pi) * Y * n ** 2 * cfg.sigma ** 4 * np.sqrt(cfg.m * cfg.kb * T)
    div_U = F(cells, "DIVU")[:, 0]
    coeff_mu = 3 * 1.002 / 5 * nbY ** 2 / (1 + 2 * nbY / 5)
    coeff_k = 1.002 * nbY ** 2 / (1 + 3 * nbY / 5) / 5
    iso = (p_crr - 1) * trace / 3 - w * div_U / (cfg.m * n)
    r9 = np.stack([(mu_crr - 1) * dev[:, j] + coeff_mu * dev[:, j] - gst * M4[:, j] for j in range(6)], 1)
    for j in (0, 3, 5):
        r9[:, j] += iso
    rb = np.stack([(k_crr - 1) * m + coeff_k * m - gst * M5[:, i] + gst * DM2 * m for i, m in enumerate((ma, mb, mc))], 1)
    rows = [[0, 1, 2], [1, 3, 4], [2, 4, 5]]  # rhs of block b: P row entries of dev (r9 index)
    al, be = F(cells, "ALPHA"), F(cells, "BETA")
    for b, m3b in enumerate((ma, mb, mc)):
        A4 = np.zeros((len(T), 4, 4))
        A4[:, :3, :3] = P[:, [[0, 1, 2], [1, 3, 4], [2, 4, 5]]]
        A4[:, :3, 3] = m3b[:, None]
        A4[:, 3, :] = np.stack([ma, mb, mc, d], 1)
        r4 = np.concatenate([r9[:, rows[b]], rb[:, b:b + 1]], 1)
        x4 = np.linalg.solve(A4[ok], r4[ok][:, :, None])[:, :, 0]
        g4 = np.concatenate([al[ok][:, 3 * b:3 * b + 3], be[ok][:, b:b + 1]], 1)
        sc = np.max(np.abs(x4), axis=1)
        e4 = np.max(np.abs(g4 - x4), axis=1) / sc
        assert np.max(e4) <= 1e-9, (b, np.max(e4))
