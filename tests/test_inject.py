"""Injected uniforms on the oracle (no GPU): the face jitter of a particle
exactly on a face (src/Main_Functions.cpp:2238-2247) follows the injected
word, and a diffuse re-emission at the wall (BC_wall,
src/Main_Functions.cpp:4816-4914) takes the injected Rayleigh factor and
normals -- known answers computed here from the same uniforms.  The GPU
kernels read the same rows (tests/test_gpu_inject.py)."""
import math

import numpy as np

import mcpm
import workloads as W
from oracle import Oracle

SCALE = 4294967296.0


def grid_u(w):
    """the uniform the FP64 kernels see for the word w: (w + 1/2) 2^-32"""
    return (np.asarray(w, dtype=np.float64) + 0.5) / SCALE


def face_case(precision=mcpm.FP64):
    cfg, _ = W.homogeneous_relaxation_1d(n_cells=10, ppc=2, precision=precision)
    cfg.problem = mcpm.PROBLEM_CLOSED_BOX
    N = 8
    x2 = np.array([3.0, 3.0, 5.0, 5.0, 7.0, 7.0, 2.5, 8.5])
    parts = dict(x1=np.full(N, 0.5), x2=x2, U1=np.zeros(N), U2=np.zeros(N), U3=np.zeros(N))
    cfg.max_particles = N
    # word 0 >= 2^31 moves the particle up by 1e-14, below moves it down
    up = np.array([1, 0, 1, 0, 1, 0, 1, 0], dtype=bool)
    u = np.full((N, 4), 0.5)
    u[:, 0] = np.where(up, grid_u(3 << 30), grid_u(1 << 30))
    want = np.where(up, np.floor(x2), np.floor(x2) - 1).astype(np.int32)
    want[6:] = np.floor(x2[6:])  # not on a face: no draw
    return cfg, parts, u, want


def test_oracle_face_jitter_follows_injection():
    cfg, parts, u, want = face_case()
    o = Oracle(cfg, parts)
    o.inject_uniforms(mcpm.RS["BIN"], u)
    o.set_step(1)
    o.cell_update()
    assert np.array_equal(o.s.index, want)
    # the opposite words move every face particle the other way
    u2 = u.copy()
    u2[:, 0] = grid_u(SCALE - 1) - u[:, 0] + grid_u(0)
    o.inject_uniforms(mcpm.RS["BIN"], u2)
    o.cell_update()
    flip = want.copy()
    flip[:6] = np.where(want[:6] == np.floor(parts["x2"][:6]), want[:6] - 1, want[:6] + 1)
    assert np.array_equal(o.s.index, flip)


def wall_case():
    cfg, _ = W.vlasov_slab_1d(n_cells=10, mean_ppc=4, long_range=mcpm.LR_NONE)
    cfg.problem = mcpm.PROBLEM_WALL
    cfg.T_wall[0] = 1.7
    cfg.U_wall[0] = 0.3
    N = 6
    L1 = cfg.length[1]
    x2 = np.array([0.01, 0.3 * L1, 0.02, 0.5 * L1, 0.6 * L1, 0.005])
    U2 = np.array([-0.5, 0.1, -0.9, -0.1, 0.2, -0.3]) / cfg.dt * 0.1
    parts = dict(x1=np.full(N, 0.5), x2=x2, U1=np.full(N, 0.2), U2=U2, U3=np.full(N, -0.1))
    cfg.max_particles = N
    rng = np.random.default_rng(5)
    w = rng.integers(1 << 20, (1 << 32) - (1 << 20), size=(N, 4))
    w = (w >> 9 << 9) + 256  # on the FP32 kernels' 2^-23 grid as well
    u = grid_u(w)
    hits = x2 + U2 * cfg.dt <= 0.0
    return cfg, parts, u, hits


def expected_wall(cfg, u):
    """BC_wall's re-emission (src/Main_Functions.cpp:4816-4914) for the
    draws u of one row: Rayleigh normal speed, Maxwellian tangential"""
    kb, m, T, Uw = cfg.kb, cfg.m, cfg.T_wall[0], cfg.U_wall[0]
    ray = math.sqrt(-math.log(u[0]))
    a = math.sqrt(-2.0 * math.log(u[1]))
    z0, z1 = a * math.cos(2 * math.pi * u[2]), a * math.sin(2 * math.pi * u[2])
    return (math.sqrt(kb * T / m) * z0 + Uw, math.sqrt(2.0 * kb * T / m) * ray, math.sqrt(kb * T / m) * z1)


def test_oracle_wall_draw_follows_injection():
    cfg, parts, u, hits = wall_case()
    assert hits.sum() == 3
    o = Oracle(cfg, parts)
    o.inject_uniforms(mcpm.RS["BC"], u)
    o.set_step(1)
    o.cell_update()
    o.store_old_positions()
    o.stream()
    o.apply_bc(0)
    for i in np.flatnonzero(hits):
        e = expected_wall(cfg, u[i])
        got = (o.s.U1[i], o.s.U2[i], o.s.U3[i])
        assert np.allclose(got, e, rtol=1e-13, atol=0), (i, got, e)
        assert 0 < o.s.x2[i] < cfg.length[1]
    for i in np.flatnonzero(~hits):
        assert o.s.U2[i] == parts["U2"][i]
