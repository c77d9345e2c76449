"""Seeded synthetic workloads with the shapes of the five benchmark
configurations of the particle step.  The reference measures on no public
dataset; these generators stand in for its initialisation
(src/Main_Functions.cpp:4222-4814), which draws from an unseeded
std::random_device.

Units are reduced: sigma = m = kb = 1, b = 2 pi sigma^3 / 3, T0 = 1 (the
reference's T0 = 273 is an SI choice; mu(T) = mu(T0) (T/T0)^visp is the same
law).  The time step follows readSettingsFile (src/myIO.cpp:2851-2874):
dt = frac_mft * min(lambda, dy) / max(sqrt(kb T_wall_1 / m), U_wall_1, U_wall_2)
with frac_mft = 0.1 and the reference's mean free path (:2836-2844).
"""
from __future__ import annotations

import math

import numpy as np

from mcpm import (Config, derive, FP32, FP64, LR_DIRECT, LR_NONE, LR_SCREENED_POISSON, MODEL_DSMC_VHS, MODEL_ESMC,
                  MODEL_FP_DENSE, PROBLEM_CLOSED_BOX, PROBLEM_COUETTE, PROBLEM_PERIODIC)

BASE_SEED = 0x4D43504D
B_HS = 2.0 * math.pi / 3.0                   # b for sigma = 1
SIGMA_AR = 3.405e-10                         # the reference's argon sigma (src/myIO.cpp:2631)
EPS_AR = 119.8 * 1.38064852e-23              # its epsilon, 119.8 kb (src/myIO.cpp:2236)
AST_SI, BST_SI = -1.64835851e-28, 6.91304716e09  # src/myIO.cpp:2891-2892, fitted to phi = -4 eps
BST_RED = BST_SI * SIGMA_AR                  # b* = b sigma_Ar
AST_RED_4EPS = AST_SI / (EPS_AR * SIGMA_AR)  # a* = a / (eps sigma_Ar), for phi = -4 eps


def mean_free_path(n, T, mu, visp=0.5, nualpha=1.0, m=1.0, kb=1.0):
    """src/myIO.cpp:2836-2844"""
    lam = 4.0 * nualpha * (5.0 - 2.0 * visp) * (7.0 - 2.0 * visp)
    lam = lam / (5.0 * (nualpha + 1.0) * (nualpha + 2.0))
    return lam * math.sqrt(m / (2.0 * math.pi * kb * T)) * mu / (m * n)


def _base(n_cells, length, direction, problem, model, precision, n, T, frac_mft=0.1, Tw=None, seed=0):
    c = Config()
    c.n_cells[:] = (n_cells[0], n_cells[1], 1)
    c.direction[:] = (direction[0], direction[1], 0)
    c.length[:] = length
    c.problem, c.model, c.long_range, c.precision = problem, model, LR_NONE, precision
    c.sigma, c.m, c.kb, c.n = 1.0, 1.0, 1.0, n
    c.T0, c.visp = 1.0, 0.5
    tw = Tw if Tw is not None else (T, T, T, T)
    c.T_wall[:] = tw
    c.U_wall[:] = (0.0, 0.0, 0.0, 0.0)
    c.seed = seed or BASE_SEED
    c.mu = 5.0 / (16.0 * c.sigma ** 2) * math.sqrt(c.m * c.kb * c.T0 / math.pi)
    lam = mean_free_path(n, T, c.mu)
    dy = length[1] / n_cells[1]
    c.dt = frac_mft * min(lam, dy) / max(math.sqrt(c.kb * tw[0] / c.m), 0.0)
    return c


def _fill_cells(rng, counts, n_cells, length, lo_y=0.0, hi_y=None):
    """Uniform positions inside each cell, `counts[c]` particles in cell c."""
    N0, N1 = n_cells
    dx, dy = length[0] / N0, length[1] / N1
    cell = np.repeat(np.arange(N0 * N1, dtype=np.int64), counts)
    j, k = cell % N0, cell // N0
    x1 = (j + rng.random(cell.size)) * dx
    x2 = (k + rng.random(cell.size)) * dy
    if hi_y is not None:
        x2 = np.clip(x2, lo_y + 1e-9, hi_y - 1e-9)
    return x1, x2


def homogeneous_relaxation_1d(n_cells=100, ppc=200, precision=FP64, seed=BASE_SEED, nb=0.3):
    """Plain Enskog-FP homogeneous relaxation: 1-D periodic box of unit cells,
    200 particles per cell, n b = 0.3, anisotropic Maxwellian T_x = 2,
    T_y = T_z = 0.5, no long-range force (100 steps on the CPU)."""
    rng = np.random.default_rng(seed)
    L = (1.0, float(n_cells), 1.0)
    c = _base((1, n_cells), L, (0, 1), PROBLEM_PERIODIC, MODEL_FP_DENSE, precision, nb / B_HS, 1.0, seed=seed)
    N = n_cells * ppc
    x1, x2 = _fill_cells(rng, np.full(n_cells, ppc), (1, n_cells), L)
    U1 = rng.normal(0.0, math.sqrt(2.0), N)
    U2 = rng.normal(0.0, math.sqrt(0.5), N)
    U3 = rng.normal(0.0, math.sqrt(0.5), N)
    derive(c, N)
    return c, dict(x1=x1, x2=x2, U1=U1, U2=U2, U3=U3)


def vlasov_slab_1d(n_cells=1000, mean_ppc=1000, precision=FP64, seed=BASE_SEED + 1, T=0.8, dy=0.25,
                   long_range=LR_SCREENED_POISSON, eps=1.0):
    """1-D Enskog-Vlasov liquid-vapour slab: density n b = 0.25 + 0.20 tanh((y - L/2) / 4 sigma)
    (0.05 .. 0.45), Sutherland attraction phi(r) = -eps (sigma/r)^6, kT = 0.8,
    specular walls, Vlasov force by the screened-Poisson Green's-function path."""
    rng = np.random.default_rng(seed)
    L1 = n_cells * dy
    L = (1.0, L1, 1.0)
    yc = (np.arange(n_cells) + 0.5) * dy
    nb = 0.25 + 0.20 * np.tanh((yc - L1 / 2) / 4.0)
    counts = np.maximum(1, np.rint(mean_ppc * nb / nb.mean())).astype(np.int64)
    N = int(counts.sum())
    n_mean = float(nb.mean()) / B_HS
    c = _base((1, n_cells), L, (0, 1), PROBLEM_CLOSED_BOX, MODEL_FP_DENSE, precision, n_mean, T, seed=seed)
    c.long_range = long_range
    c.phi = -eps
    c.eqdist = 1.0
    c.bst = BST_RED
    c.ast = AST_RED_4EPS * (eps / 4.0)
    x1, x2 = _fill_cells(rng, counts, (1, n_cells), L)
    s = math.sqrt(T)
    U1, U2, U3 = rng.normal(0, s, N), rng.normal(0, s, N), rng.normal(0, s, N)
    derive(c, N)
    return c, dict(x1=x1, x2=x2, U1=U1, U2=U2, U3=U3)


def esmc_box_2d(n_cells=(256, 256), ppc=100, precision=FP32, seed=BASE_SEED + 2, nb=0.2, T=1.0, T_hot=1.5):
    """ESMC hard spheres in a 2-D box of unit cells, 100 particles per cell,
    n b = 0.2, Maxwellian T = 1, diffuse walls (BC_thermal_wall_3D) with the
    y = sigma wall at T = 1.5 and the others at T = 1."""
    rng = np.random.default_rng(seed)
    N0, N1 = n_cells
    L = (float(N0), float(N1), 1.0)
    c = _base(n_cells, L, (1, 1), PROBLEM_COUETTE, MODEL_ESMC, precision, nb / B_HS, T,
              Tw=(T_hot, T, T, T), seed=seed)
    counts = np.full(N0 * N1, ppc, dtype=np.int64)
    counts[:N0] = 0            # y in [0, sigma) lies behind the wall at y = sigma
    counts[(N1 - 1) * N0:] = 0  # and y in (L - sigma, L]
    N = int(counts.sum())
    x1, x2 = _fill_cells(rng, counts, n_cells, L, lo_y=1.0, hi_y=L[1] - 1.0)
    s = math.sqrt(T)
    U1, U2, U3 = rng.normal(0, s, N), rng.normal(0, s, N), rng.normal(0, s, N)
    derive(c, N)
    return c, dict(x1=x1, x2=x2, U1=U1, U2=U2, U3=U3)


def with_dsmc_vhs(cfg, T=1.0):
    """The same box with Bird's DSMC (Collision_DSMC_VHS) as the collision
    model; crref = sqrt(kb T / m) of the initial temperature, as
    readSettingsFile sets it (src/myIO.cpp:2242)."""
    cfg.model = MODEL_DSMC_VHS
    cfg.crref = math.sqrt(cfg.kb * T / cfg.m)
    return cfg


def lognormal_counts(n_cells, seed, median=100, lo=10, hi=5000, target=None, s=None):
    """Per-cell occupancy ~ LogNormal(ln median, s) clipped to [lo, hi]; s is
    bisected so that the total is `target` (16.0M for 65,536 cells) to 0.5%."""
    C = n_cells[0] * n_cells[1]
    z = np.random.default_rng(seed).standard_normal(C)
    if target is None:
        target = int(round(16_000_000 * C / 65536))

    def counts_for(sig):
        return np.clip(np.rint(median * np.exp(sig * z)), lo, hi).astype(np.int64)

    if s is None:
        a, b = 0.5, 2.5
        for _ in range(60):
            m = 0.5 * (a + b)
            if counts_for(m).sum() < target:
                a = m
            else:
                b = m
        s = 0.5 * (a + b)
    return counts_for(s), s


def uneven_cells_2d(n_cells=(256, 256), precision=FP32, seed=BASE_SEED + 3, streaming=True, nb_max=0.45,
                    hi=5000, T=1.0):
    """Batched uneven cells: 65,536 cells (256 x 256, unit cells) with
    log-normal occupancy (median 100, clipped 10..5000, total 16.0M), Maxwellian
    T = 1 in every cell, Enskog-FP (FP_dense), FP32 velocities.  The mean
    density is set so that the fullest cell has n b = nb_max.  streaming=True
    is the variant with free flight and specular walls; False keeps the
    particles in place so the uneven occupancy persists."""
    rng = np.random.default_rng(seed)
    N0, N1 = n_cells
    L = (float(N0), float(N1), 1.0)
    counts, s = lognormal_counts(n_cells, seed, hi=hi)
    N = int(counts.sum())
    n_cell_max = nb_max / B_HS
    Fn = n_cell_max / counts.max()  # unit cell volume
    n_mean = Fn * N / (N0 * N1)
    c = _base(n_cells, L, (1, 1) if streaming else (0, 0), PROBLEM_CLOSED_BOX, MODEL_FP_DENSE, precision,
              n_mean, T, seed=seed)
    x1, x2 = _fill_cells(rng, counts, n_cells, L)
    sT = math.sqrt(T)
    U1, U2, U3 = rng.normal(0, sT, N), rng.normal(0, sT, N), rng.normal(0, sT, N)
    derive(c, N)
    return c, dict(x1=x1, x2=x2, U1=U1, U2=U2, U3=U3, sigma_lognormal=s)


def density_field(rng, n_cells, length, K=6, nbar=None):
    """One seeded 2-D packing-fraction field n b(x, y) at the cell centres:
    nbar + sum_{k=1..K} a_k sin(2 pi (kx x / L0 + ky y / L1) + phi_k), with
    nbar ~ U[0.15, 0.35], sum |a_k| ~ U[0.05, 0.1], integer wave vectors of
    norm 1..8, clipped to [0.05, 0.45]."""
    N0, N1 = n_cells
    xc = (np.arange(N0) + 0.5) * (length[0] / N0)
    yc = (np.arange(N1) + 0.5) * (length[1] / N1)
    X, Y = np.meshgrid(xc, yc)  # [N1][N0]
    nb = np.full(X.shape, rng.uniform(0.15, 0.35) if nbar is None else nbar)
    amp = rng.uniform(0.0, 1.0, K)
    amp *= rng.uniform(0.05, 0.1) / max(amp.sum(), 1e-12)
    for a in amp:
        while True:
            kx, ky = rng.integers(-8, 9, 2)
            if 1.0 <= math.hypot(kx, ky) <= 8.0:
                break
        ph = rng.uniform(0.0, 2.0 * math.pi)
        nb += a * np.sin(2.0 * math.pi * (kx * X / length[0] + ky * Y / length[1]) + ph)
    return np.clip(nb, 0.05, 0.45).reshape(-1)


def vlasov_box_2d(n_cells=(256, 256), total=16_000_000, precision=FP32, seed=BASE_SEED + 4, T=0.8,
                  long_range=LR_SCREENED_POISSON, eps=1.0, model=MODEL_FP_DENSE, dx=1.0, particles=True):
    """2-D Enskog-Vlasov box: square cells of side dx, particles per cell in
    proportion to a density_field (at least one per cell, `total` in all),
    Maxwellian kT = T, specular walls, Sutherland attraction
    phi(r) = -eps (sigma/r)^6 through the 2-D Vlasov force (long_range 1:
    direct node quadrature; 3: screened-Poisson FEM with Green's-function
    wall values)."""
    rng = np.random.default_rng(seed)
    N0, N1 = n_cells
    L = (N0 * dx, N1 * dx, 1.0)
    nb = density_field(rng, n_cells, L)
    counts = np.maximum(1, np.rint(total * nb / nb.sum())).astype(np.int64)
    N = int(counts.sum())
    n_mean = float(nb.mean()) / B_HS
    c = _base(n_cells, L, (1, 1), PROBLEM_CLOSED_BOX, model, precision, n_mean, T, seed=seed)
    c.long_range = long_range
    c.phi = -eps
    c.eqdist = 1.0
    c.bst = BST_RED
    c.ast = AST_RED_4EPS * (eps / 4.0)
    if not particles:  # the configuration alone
        derive(c, N)
        return c, None
    x1, x2 = _fill_cells(rng, counts, n_cells, L)
    s = math.sqrt(T)
    U1, U2, U3 = rng.normal(0, s, N), rng.normal(0, s, N), rng.normal(0, s, N)
    derive(c, N)
    return c, dict(x1=x1, x2=x2, U1=U1, U2=U2, U3=U3)
