"""CUDA path (libmcpm.so through the C-ABI) against the FP64 CPU restatement
on identical inputs and draws.

Tolerances (FP64 path): cell indices and counts bit-exact; moments within
1e-12 of the natural scale of each field (velocity^k for a k-th moment);
velocities and positions within 1e-12 of max(1, |value|); the per-cell
drift coefficients (outputs of ill-conditioned 9x9 / 12x12 solves) within
1e-9 of their field's largest magnitude.  FP32 path: 2e-5 of the same scales.
"""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu

VEL_POW = dict(U_SPACE=1, MP=1, PIJ=2, DM2=2, M3=3, Q=3, M4=4, DM4=4, M5=5)


def _pair(cfg, parts, seed=11, step=1, inject=True):
    s = mcpm.Session(cfg)
    s.upload(parts.get("x1"), parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg, parts)
    if inject:
        rng = np.random.default_rng(seed)
        xi = [rng.standard_normal(o.N) for _ in range(3)]
        s.inject_normals(*xi)
        o.inject_normals(*xi)
    s.set_step(step)
    o.set_step(step)
    return s, o


def _close_particles(g, o, tol, keys=("x1", "x2", "U1", "U2", "U3")):
    for k in keys:
        a, b = g[k], getattr(o.s, k)
        err = np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))
        assert err <= tol, "%s: %.3e > %.1e" % (k, err, tol)


def _close_cells(cg, co, tol, tol_coef):
    """cg: [CF][C] from the GPU, co: [C][CF] from the oracle."""
    n = mcpm.cell_field(co, "NUM_INSIDE", True)
    assert np.array_equal(mcpm.cell_field(cg, "NUM_INSIDE"), n)
    vs = np.sqrt(max(np.max(mcpm.cell_field(co, "DM2", True)), 1e-300))
    for f, p in VEL_POW.items():
        a, b = mcpm.cell_field(cg, f), mcpm.cell_field(co, f, True)
        assert np.max(np.abs(a - b)) <= tol * vs ** p, f
    for f in ("T", "N", "GAMMA_ST", "LAMBDA"):
        a, b = mcpm.cell_field(cg, f), mcpm.cell_field(co, f, True)
        m = n > 1
        sc = np.max(np.abs(b[m])) if m.any() else 1.0
        assert np.max(np.abs(a[m] - b[m])) <= tol * sc, f
    for f in ("C", "GAMMA", "ALPHA", "BETA"):
        a, b = mcpm.cell_field(cg, f), mcpm.cell_field(co, f, True)
        sc = max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) <= tol_coef * sc, f


# ------------------------------------------------------------- binning
@pytest.mark.parametrize("maker", ["relax", "uneven"])
def test_binning_bit_exact(cuda_ok, maker):
    cfg, parts = (W.homogeneous_relaxation_1d(n_cells=37, ppc=53) if maker == "relax"
                  else W.uneven_cells_2d(n_cells=(19, 23), hi=400, precision=mcpm.FP64))
    s, o = _pair(cfg, parts)
    o.cell_update()
    s.cell_update()
    assert np.array_equal(s.get_index(), o.s.index)
    assert np.array_equal(mcpm.cell_field(s.get_cells(), "NUM_INSIDE"), mcpm.cell_field(o.cells(), "NUM_INSIDE", True))
    pid, off = s.get_layout()
    assert off[-1] == o.N and np.all(np.diff(off) >= 0)
    assert np.array_equal(np.sort(pid), np.arange(o.N))


def _face_positions(n, d, L, rng, count):
    """float32 positions in [0, L]: uniform ones, every face k d rounded to
    float and its two float neighbours, 0 and L."""
    f = np.arange(n + 1) * d
    x = np.concatenate([rng.random(count) * L, f, np.nextafter(f.astype(np.float32), np.float32(np.inf)),
                        np.nextafter(f.astype(np.float32), np.float32(-np.inf)), [0.0, L]])
    top = np.float32(L)
    if float(top) > L:  # the largest float inside the box
        top = np.nextafter(top, np.float32(-np.inf))
    x = np.clip(x.astype(np.float32), np.float32(0.0), top).astype(np.float64)
    return rng.permutation(x)


@pytest.mark.parametrize("shape,d", [((1, 37), 0.3), ((1, 40), 1.0), ((19, 23), 0.7)])
def test_binning_fp32_bit_exact(cuda_ok, shape, d):
    """FP32 sessions bin the float position by the reference's rule,
    floor(x / dx) in double (src/Main_Functions.cpp:2232-2266), face jitter
    included (a float lying on a face of unit cells, :2238-2247): the cell
    index equals the oracle's on the same float-rounded positions, for
    positions on every face, one float either side of it, 0 and Len; then
    again after a fused step, whose particle pass bins the new positions."""
    rng = np.random.default_rng(17)
    N0, N1 = shape
    cfg, _ = W.homogeneous_relaxation_1d(n_cells=N1, ppc=4, precision=mcpm.FP32)
    cfg.n_cells[0] = N0
    cfg.length[0] = N0 * d if N0 > 1 else 1.0
    cfg.length[1] = N1 * d
    cfg.direction[0] = 1 if N0 > 1 else 0
    x2 = _face_positions(N1, d, cfg.length[1], rng, 40 * N0 * N1)
    n = len(x2)
    x1 = (_face_positions(N0, d, cfg.length[0], rng, n)[:n] if N0 > 1 else rng.random(n))
    x1 = np.resize(x1, n)
    U = [rng.normal(0.0, 1.0, n).astype(np.float32).astype(np.float64) for _ in range(3)]
    parts = dict(x1=x1, x2=x2, U1=U[0], U2=U[1], U3=U[2])
    mcpm.derive(cfg, n)
    cfg.max_particles = n
    s, o = _pair(cfg, parts, step=3)
    o.cell_update()
    s.cell_update()
    idx = s.get_index()
    assert np.array_equal(idx, o.s.index), np.count_nonzero(idx != o.s.index)
    # the faces of unit cells are floats: some particles took the jitter branch
    if d == 1.0:
        on = (x2 == np.floor(x2)) & (x2 > 1.0) & (x2 < N1 - 1)
        assert on.sum() > 10
        assert np.any(o.s.index[on] == x2[on].astype(np.int64) - 1)
    s.step(1)
    g = s.download()
    o2 = Oracle(cfg, g)
    o2.set_step(s.step_count)
    o2.cell_update()
    assert np.array_equal(s.get_index(), o2.s.index)


def test_binning_edges_and_out_of_box(cuda_ok):
    """Particles on the far wall bin into the last cell; a particle outside
    the box raises MCPM_ERR_OUT_OF_BOX (the reference exits)."""
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=8, ppc=16)
    parts = {k: v.copy() for k, v in parts.items()}
    parts["x2"][0] = cfg.length[1]          # exactly on the wall
    parts["x2"][1] = 0.0
    s, o = _pair(cfg, parts)
    s.cell_update()
    o.cell_update()
    idx = s.get_index()
    assert idx[0] == 7 and idx[1] == 0
    assert np.array_equal(idx, o.s.index)
    s.check_status()
    bad = {k: v.copy() for k, v in parts.items()}
    bad["x2"][5] = cfg.length[1] + 0.5
    s2 = mcpm.Session(cfg)
    s2.upload(bad["x1"], bad["x2"], bad["U1"], bad["U2"], bad["U3"])
    with pytest.raises(mcpm.MCPMError) as e:
        s2.check_status()
    assert e.value.code & mcpm.ERR_OUT_OF_BOX


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_nan_velocity_raises(cuda_ok, prec):
    """A NaN velocity spreads through its cell's moments into the FP update,
    which raises MCPM_ERR_NAN (the reference prints the cell and exits,
    src/Fokker_Planck.cpp:1137-1148); the other cells step on."""
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=8, ppc=16, precision=prec)
    bad = {k: v.copy() for k, v in parts.items()}
    bad["U2"][3] = np.nan
    s = mcpm.Session(cfg)
    s.upload(bad["x1"], bad["x2"], bad["U1"], bad["U2"], bad["U3"])
    s.check_status()
    with pytest.raises(mcpm.MCPMError) as e:
        s.step(1)
        s.check_status()
    assert e.value.code & mcpm.ERR_NAN
    g = s.download()
    # only the NaN particle's cell (16 of 128 particles) is lost
    assert np.count_nonzero(np.isfinite(g["U1"])) >= len(g["U1"]) - 16


# -------------------------------------------------------- cell update
@pytest.mark.parametrize("step", [0, 1])
def test_cell_update_fp64(cuda_ok, step):
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=40, ppc=150)
    s, o = _pair(cfg, parts, step=step)
    o.cell_update()
    s.cell_update()
    _close_cells(s.get_cells(), o.cells(), 1e-12, 1e-9)


def test_cell_update_fp64_uneven_2d(cuda_ok):
    """log-normal occupancy: both the warp-per-cell and block-per-cell paths"""
    cfg, parts = W.uneven_cells_2d(n_cells=(24, 20), precision=mcpm.FP64, hi=1500)
    s, o = _pair(cfg, parts, step=3)
    o.cell_update()
    s.cell_update()
    _close_cells(s.get_cells(), o.cells(), 1e-12, 1e-9)


def test_cell_update_fp32(cuda_ok):
    cfg, parts = W.uneven_cells_2d(n_cells=(16, 16), precision=mcpm.FP32, hi=1200)
    s, o = _pair(cfg, parts, step=2)
    # the FP32 path stores float velocities: give the oracle the rounded state
    for k in ("U1", "U2", "U3"):
        getattr(o.s, k)[:] = getattr(o.s, k).astype(np.float32).astype(np.float64)
    o.cell_update()
    s.cell_update()
    cg, co = s.get_cells(), o.cells()
    vs = np.sqrt(np.max(mcpm.cell_field(co, "DM2", True)))
    for f, p in VEL_POW.items():
        if f == "MP":
            continue
        assert np.max(np.abs(mcpm.cell_field(cg, f) - mcpm.cell_field(co, f, True))) <= 2e-5 * vs ** p, f


# ------------------------------------------- random generator + FP update
def test_random_generator_and_velocity_fp64(cuda_ok):
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=30, ppc=120)
    s, o = _pair(cfg, parts)
    o.cell_update()
    o.random_generator()
    o.velocity_fp()
    s.cell_update()
    s.random_generator()
    xg = s.get_normals()
    for a, b in zip(xg, o.xi):
        assert np.max(np.abs(a - b)) <= 1e-12 * max(1.0, np.max(np.abs(b)))
    s.velocity_update()
    _close_particles(s.download(), o, 1e-12, keys=("U1", "U2", "U3"))


def test_fp_update_conserves_cell_momentum_and_energy(cuda_ok):
    """Size-independent invariants of Velocity_FP_parallel on a 1M-particle
    uneven box: per-cell sum of U and sum |U - U_cell|^2 are unchanged
    (centred noise, src/Fokker_Planck.cpp:109-114; energy rescale :1169-1172)."""
    cfg, parts = W.uneven_cells_2d(n_cells=(64, 64), precision=mcpm.FP64, hi=2000)
    s, _ = _pair(cfg, parts, inject=False)
    s.set_rng(mcpm.RNG_PHILOX)
    s.cell_update()
    c0 = s.get_cells()
    s.random_generator()
    s.velocity_update()
    g = s.download()
    idx = s.get_index()
    C = s.C
    cnt = np.bincount(idx, minlength=C)
    for k, f in ((0, "U1"), (1, "U2"), (2, "U3")):
        sums = np.bincount(idx, weights=g[f], minlength=C)
        us = c0[mcpm.CF["U_SPACE"] + k]
        np.testing.assert_allclose(sums, us * cnt, rtol=0, atol=1e-9 * (1 + np.abs(us * cnt)).max())
    us = c0[mcpm.CF["U_SPACE"]:mcpm.CF["U_SPACE"] + 3][:, idx]
    e = np.bincount(idx, weights=((g["U1"] - us[0]) ** 2 + (g["U2"] - us[1]) ** 2 + (g["U3"] - us[2]) ** 2),
                    minlength=C)
    e0 = c0[mcpm.CF["DM2"]] * cnt
    np.testing.assert_allclose(e, e0, rtol=1e-10, atol=1e-12)


# ------------------------------------------------------------ full step
def test_loop_body_routines_fp64(cuda_ok):
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=20, ppc=100)
    s, o = _pair(cfg, parts)
    for _ in range(3):
        rng = np.random.default_rng(o.step_count)
        xi = [rng.standard_normal(o.N) for _ in range(3)]
        s.inject_normals(*xi)
        o.inject_normals(*xi)
        s.loop_body()
        o.step(1)
    _close_particles(s.download(), o, 1e-11, keys=("x2", "U1", "U2", "U3"))


@pytest.mark.parametrize("maker", ["relax", "slab_gf", "slab_direct", "uneven"])
def test_fused_step_philox_fp64(cuda_ok, maker):
    """mcpm_step (fused kernels) against orc_step, both drawing the same
    Philox streams keyed by particle id and step."""
    if maker == "relax":
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=25, ppc=80)
    elif maker == "slab_gf":
        cfg, parts = W.vlasov_slab_1d(n_cells=80, mean_ppc=60, long_range=mcpm.LR_SCREENED_POISSON)
    elif maker == "slab_direct":
        cfg, parts = W.vlasov_slab_1d(n_cells=80, mean_ppc=60, long_range=mcpm.LR_DIRECT)
    else:
        cfg, parts = W.uneven_cells_2d(n_cells=(12, 10), precision=mcpm.FP64, hi=700)
    s, o = _pair(cfg, parts, inject=False)
    s.set_rng(mcpm.RNG_PHILOX)
    o.set_rng(mcpm.RNG_PHILOX)
    s.step(3)
    o.step(3)
    _close_particles(s.download(), o, 1e-10)
    cg, co = s.get_cells(), o.cells()
    if cfg.long_range:
        a, b = mcpm.cell_field(cg, "F2"), mcpm.cell_field(co, "F2", True)
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b))


def test_fused_step_fp32_tolerance(cuda_ok):
    cfg64, parts = W.uneven_cells_2d(n_cells=(16, 16), precision=mcpm.FP64, hi=900)
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
    # moment error of the FP32 step against FP64: the 1% bar of the benchmark
    T32 = mcpm.cell_field(s.get_cells(), "T")
    s64 = mcpm.Session(cfg64)
    s64.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s64.set_step(1)
    s64.step(1)
    s.cell_update()
    s64.cell_update()
    T32, T64 = mcpm.cell_field(s.get_cells(), "T"), mcpm.cell_field(s64.get_cells(), "T")
    assert np.max(np.abs(T32 - T64) / T64) < 1e-3


# --------------------------------------------------------------- walls
@pytest.mark.parametrize("problem", [mcpm.PROBLEM_COUETTE, mcpm.PROBLEM_WALL])
def test_diffuse_walls_fp64(cuda_ok, problem):
    if problem == mcpm.PROBLEM_COUETTE:
        cfg, parts = W.esmc_box_2d(n_cells=(12, 12), ppc=40, precision=mcpm.FP64)
        cfg.model = mcpm.MODEL_FP_DENSE
    else:
        cfg, parts = W.vlasov_slab_1d(n_cells=30, mean_ppc=40, long_range=mcpm.LR_NONE)
        cfg.problem = mcpm.PROBLEM_WALL
        cfg.T_wall[0] = 1.3
    parts = {k: v.copy() for k, v in parts.items()}
    parts["U2"] *= 5.0  # many wall hits
    if problem == mcpm.PROBLEM_COUETTE:
        parts["U1"] *= 5.0
    s, o = _pair(cfg, parts, inject=False)
    s.set_rng(mcpm.RNG_PHILOX)
    o.set_rng(mcpm.RNG_PHILOX)
    s.step(2)
    o.step(2)
    _close_particles(s.download(), o, 1e-10, keys=("x2", "U1", "U2", "U3") if problem == mcpm.PROBLEM_WALL
                     else ("x1", "x2", "U1", "U2", "U3"))


# ---------------------------------------------------------------- ESMC
@pytest.mark.parametrize("shape", [(1, 30), (14, 12), (1, 8)])
def test_esmc_fp64_same_layout(cuda_ok, shape):
    """ESMC with the GPU's in-cell order given to the oracle: candidate picks,
    directions, partners and acceptances then coincide.  (1, 8): 400
    particles a cell, past the warp's 256-slot conflict table (the candidates
    are then compared pairwise over the warp)."""
    if shape[0] == 1:
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=shape[1], ppc=400 if shape[1] == 8 else 80)
        cfg.model = mcpm.MODEL_ESMC
    else:
        cfg, parts = W.esmc_box_2d(n_cells=shape, ppc=60, precision=mcpm.FP64)
    s, o = _pair(cfg, parts, inject=False)
    s.set_step(0)
    o.set_step(0)
    s.cell_update()
    o.cell_update()
    s.init_omega_max()
    o.init_omega_max()
    s.set_step(1)
    o.set_step(1)
    s.cell_update()
    o.cell_update()
    pid, off = s.get_layout()
    o.set_layout(off, pid)
    s.velocity_update()
    o.esmc()
    _close_particles(s.download(), o, 1e-12, keys=("U1", "U2", "U3"))
    om_g = mcpm.cell_field(s.get_cells(), "OMEGA_MAX")
    om_o = mcpm.cell_field(o.cells(), "OMEGA_MAX", True)
    assert np.max(np.abs(om_g - om_o)) <= 1e-12 * np.max(om_o)
    # collisions conserve momentum and energy
    g = s.download()
    assert abs(g["U1"].sum() - parts["U1"].sum()) < 1e-8 * len(g["U1"])


def test_esmc_fused_step_runs_fp32(cuda_ok):
    """ESMC with diffuse walls in FP32: positions rounding onto a wall must
    not stall the re-flight loop (MCPM_ERR_BC_LOOP)."""
    cfg, parts = W.esmc_box_2d(n_cells=(64, 64), ppc=100, precision=mcpm.FP32)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.cell_update()
    s.init_omega_max()
    s.step(20)
    g = s.download()
    assert np.all(np.isfinite(g["U1"]))
    assert np.all((g["x2"] > 0) & (g["x2"] < cfg.length[1]))


def test_autotune_restores_state(cuda_ok):
    """The autotuner times steps on the session's own particles and must hand
    back exactly the state it was given.  Different warp/block splits change
    only the summation order; trajectories then diverge (a rounding-level
    change can move a particle into the neighbouring cell), so the check
    across splits is on an invariant: the FP update rescales each cell to its
    own kinetic energy and specular walls conserve it, so the total kinetic
    energy agrees to FP32 rounding."""
    cfg, parts = W.uneven_cells_2d(n_cells=(20, 20), precision=mcpm.FP32, hi=1500)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.step(2)
    before = s.download()
    w = s.autotune(2)
    assert 128 <= w <= 768 and s.wcap == w
    after = s.download()
    for k in before:
        assert np.array_equal(before[k], after[k]), k
    s.step(1)
    g1 = s.download()
    s2 = mcpm.Session(cfg)
    s2.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s2.set_wcap(128 if w != 128 else 384)
    s2.step(3)
    g2 = s2.download()
    e0 = np.sum(parts["U1"] ** 2 + parts["U2"] ** 2 + parts["U3"] ** 2)
    e1 = np.sum(g1["U1"] ** 2 + g1["U2"] ** 2 + g1["U3"] ** 2)
    e2 = np.sum(g2["U1"] ** 2 + g2["U2"] ** 2 + g2["U3"] ** 2)
    assert abs(e1 - e0) < 1e-5 * e0 and abs(e2 - e0) < 1e-5 * e0


@pytest.mark.parametrize("maker", ["relax", "vlasov2d"])
def test_graph_replay_matches_eager_steps(cuda_ok, maker):
    """mcpm_step(n) replays pairs of steps as a CUDA graph; the same steps one
    call at a time run eagerly.  Same kernels, same draws: the results agree
    to rounding (the in-cell order of the reorder is not deterministic, which
    only reorders sums for the FP models; ESMC picks its pairs by slot, so its
    trajectories are compared statistically elsewhere)."""
    if maker == "relax":
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=20, ppc=60)
    else:
        cfg, parts = W.vlasov_box_2d(n_cells=(10, 8), total=4000, precision=mcpm.FP64,
                                     long_range=mcpm.LR_SCREENED_POISSON)
    a, b = mcpm.Session(cfg), mcpm.Session(cfg)
    for s in (a, b):
        s.upload(parts.get("x1"), parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        s.set_step(1)
    l0 = a.kernel_launches
    a.step(7)
    for _ in range(7):
        b.step(1)
    assert a.step_count == b.step_count == 8
    ga, gb = a.download(), b.download()
    for k in ("x2", "U1", "U2", "U3"):
        err = np.max(np.abs(ga[k] - gb[k])) / max(1.0, np.max(np.abs(gb[k])))
        assert err <= 1e-9, (k, err)
    assert a.kernel_launches - l0 >= 7 * 6


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_queued_steps_match_and_report_status(cuda_ok, prec):
    """mcpm_step_async queues the same steps as mcpm_step: a loop of queued
    uploads, steps and downloads (the host never waiting) gives the arrays
    of the same loop run call by call, and a NaN raised on the device is
    reported by the next check_status, not by the queued step."""
    cfg, parts = W.homogeneous_relaxation_1d(n_cells=20, ppc=60, precision=prec)
    a, b = mcpm.Session(cfg), mcpm.Session(cfg)
    outs = {}
    for s, wait in ((a, True), (b, False)):
        res = []
        for i in range(3):
            out = {k: np.zeros(len(parts["x2"])) for k in ("x1", "x2", "U1", "U2", "U3")}
            s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"], wait=wait)
            s.set_step(1 + 2 * i)
            s.step(2, wait=wait)
            s.download_into(out, wait=wait)
            res.append(out)
        s.sync()
        s.check_status()
        outs[wait] = res
    tol = 1e-9 if prec == mcpm.FP64 else 1e-5
    for ra, rb in zip(outs[True], outs[False]):
        for k in ("x2", "U1", "U2", "U3"):
            err = np.max(np.abs(ra[k] - rb[k])) / max(1.0, np.max(np.abs(ra[k])))
            assert err <= tol, (k, err)
    bad = {k: v.copy() for k, v in parts.items()}
    bad["U2"][3] = np.nan
    b.upload(bad["x1"], bad["x2"], bad["U1"], bad["U2"], bad["U3"])
    b.check_status()
    b.step(1, wait=False)
    with pytest.raises(mcpm.MCPMError) as e:
        b.check_status()
    assert e.value.code & mcpm.ERR_NAN


def _ragged_box(prec):
    """12 cells with very uneven occupancy -- an empty cell, small, warp-,
    block- and beyond-staging-sized cells (20 to 4,000) -- Maxwellian T = 1.
    (Cells of 1 to 3 particles are left out: there the reference's own
    formulas divide by a zero temperature or solve a singular 4x4 system and
    its positions become NaN, which the GPU step reports as the reference
    would exit.)"""
    cfg, _ = W.uneven_cells_2d(n_cells=(4, 3), precision=prec, streaming=True)
    counts = np.array([4000, 3500, 60, 20, 0, 200, 3100, 100, 40, 2000, 800, 30])
    rng = np.random.default_rng(21)
    cell = np.repeat(np.arange(12), counts)
    x1 = (cell % 4 + rng.random(cell.size)) * 1.0
    x2 = (cell // 4 + rng.random(cell.size)) * 1.0
    N = cell.size
    parts = dict(x1=x1, x2=x2, U1=rng.normal(0, 1, N), U2=rng.normal(0, 1, N), U3=rng.normal(0, 1, N))
    mcpm.derive(cfg, N)
    cfg.max_particles = N
    return cfg, parts


def test_ragged_cells_fused_steps(cuda_ok):
    """Cells from empty to 4,000 particles (past the shared staging of the
    particle pass, which then recomputes its draws): two fused FP64 steps
    against the oracle drawing the same Philox streams, one FP32 step within
    its tolerance."""
    cfg, parts = _ragged_box(mcpm.FP64)
    s, o = _pair(cfg, parts, inject=False)
    s.set_rng(mcpm.RNG_PHILOX)
    o.set_rng(mcpm.RNG_PHILOX)
    s.step(2)
    o.step(2)
    _close_particles(s.download(), o, 1e-10)
    cfg32 = cfg.copy()
    cfg32.precision = mcpm.FP32
    s32 = mcpm.Session(cfg32)
    s32.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o1 = Oracle(cfg, parts)
    for x in (s32, o1):
        x.set_rng(mcpm.RNG_PHILOX)
        x.set_step(1)
        x.step(1)
    g = s32.download()
    for k in ("U1", "U2", "U3"):
        err = np.max(np.abs(g[k] - getattr(o1.s, k)))
        assert err < 5e-4, (k, err)
