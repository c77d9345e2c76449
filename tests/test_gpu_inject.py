"""mcpm_inject_uniforms on the GPU: the face jitter and the diffuse wall take
the injected draws (known answers computed from the uniforms, and the oracle
reading the same rows), ESMC with injected candidate, acceptance and count
draws matches the oracle given the same in-cell order, removing the table
restores the Philox stream, and a step pair captured as a graph before the
injection is re-recorded after it."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle
from test_inject import expected_wall, face_case, grid_u, wall_case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_face_jitter_follows_injection(cuda_ok, prec):
    cfg, parts, u, want = face_case(prec)
    s = mcpm.Session(cfg)
    s.inject_uniforms("BIN", u)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(1)
    s.cell_update()
    assert np.array_equal(s.get_index(), want)
    o = Oracle(cfg, parts)
    o.inject_uniforms(mcpm.RS["BIN"], u)
    o.set_step(1)
    o.cell_update()
    assert np.array_equal(s.get_index(), o.s.index)


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_wall_draw_follows_injection(cuda_ok, prec):
    cfg, parts, u, hits = wall_case()
    cfg.precision = prec
    s = mcpm.Session(cfg)
    s.inject_uniforms("BC", u)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(1)
    s.cell_update()
    s.store_old_positions()
    s.stream_particles()
    s.apply_BC()
    g = s.download()
    rtol = 1e-13 if prec == mcpm.FP64 else 2e-5
    for i in np.flatnonzero(hits):
        e = expected_wall(cfg, u[i])
        got = (g["U1"][i], g["U2"][i], g["U3"][i])
        assert np.allclose(got, e, rtol=rtol, atol=rtol * 1e-3), (i, got, e)
        assert 0 < g["x2"][i] < cfg.length[1]
    if prec == mcpm.FP64:
        o = Oracle(cfg, parts)
        o.inject_uniforms(mcpm.RS["BC"], u)
        o.set_step(1)
        o.cell_update()
        o.store_old_positions()
        o.stream()
        o.apply_bc(0)
        for k in ("x2", "U1", "U2", "U3"):
            assert np.max(np.abs(g[k] - getattr(o.s, k))) <= 1e-13 * np.max(np.abs(getattr(o.s, k))), k


def test_esmc_injected_draws_match_oracle(cuda_ok):
    cfg, parts = W.esmc_box_2d(n_cells=(12, 12), ppc=40, precision=mcpm.FP64)
    rng = np.random.default_rng(9)
    tables = {st: grid_u(rng.integers(0, 1 << 32, size=(257, 4))) for st in ("ESMC", "ESMC_ACC", "ESMC_M")}
    res = []
    for inject in (True, False):
        s = mcpm.Session(cfg)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        o = Oracle(cfg, parts)
        if inject:
            for st, u in tables.items():
                s.inject_uniforms(st, u)
                o.inject_uniforms(mcpm.RS[st], u)
        for x in (s, o):
            x.set_step(0)
            x.cell_update()
            x.init_omega_max()
            x.set_step(1)
            x.cell_update()
        pid, off = s.get_layout()
        o.set_layout(off, pid)
        s.velocity_update()
        o.esmc()
        g = s.download()
        for k in ("U1", "U2", "U3"):
            assert np.max(np.abs(g[k] - getattr(o.s, k))) <= 1e-12 * max(1.0, np.max(np.abs(getattr(o.s, k)))), k
        assert np.count_nonzero(g["U1"] != parts["U1"]) > 0
        res.append(g["U1"])
    # the injected draws pick other pairs than the Philox stream
    assert not np.array_equal(res[0], res[1])


def test_removing_injection_restores_philox(cuda_ok):
    cfg, parts = W.vlasov_slab_1d(n_cells=30, mean_ppc=40, long_range=mcpm.LR_NONE)
    cfg.problem = mcpm.PROBLEM_WALL
    parts = {k: v.copy() for k, v in parts.items()}
    parts["U2"] *= 5.0
    u = grid_u(np.random.default_rng(4).integers(1 << 20, (1 << 32) - (1 << 20), size=(len(parts["x2"]), 4)))
    out = []
    for inject in (True, False):
        s = mcpm.Session(cfg)
        if inject:
            s.inject_uniforms("BC", u)
            s.inject_uniforms("BC", None)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        s.set_step(1)
        s.step(2)
        out.append(s.download())
    for k in ("x2", "U1", "U2", "U3"):
        a, b = out[0][k], out[1][k]
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b)), k


def test_graph_rerecorded_after_injection(cuda_ok):
    """two graph-replayed step pairs with an injection between them equal the
    same calls made eagerly (profiling on: no graphs)"""
    cfg, parts = W.vlasov_slab_1d(n_cells=30, mean_ppc=40, long_range=mcpm.LR_NONE)
    cfg.problem = mcpm.PROBLEM_WALL
    parts = {k: v.copy() for k, v in parts.items()}
    parts["U2"] *= 5.0
    u = grid_u(np.random.default_rng(3).integers(1 << 20, (1 << 32) - (1 << 20), size=(len(parts["x2"]), 4)))
    out = []
    for eager in (False, True):
        s = mcpm.Session(cfg)
        s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
        if eager:
            s.profile(True)
        s.set_step(1)
        s.step(4)
        s.inject_uniforms("BC", u)
        s.step(4)
        out.append(s.download())
    for k in ("x2", "U1", "U2", "U3"):
        a, b = out[0][k], out[1][k]
        assert np.max(np.abs(a - b)) <= 1e-10 * np.max(np.abs(b)), k
