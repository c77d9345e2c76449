"""The interface problems on the GPU against the oracle restatement (itself
pinned against the reference in tests/test_dynamic.py): the thermostat
(src/Main_Functions.cpp:1674-1869) and the weighted-particle split / merge
that changes N (inverted_addremove_particles, :1206-1450) -- deletions and
copies drawn from the shared Philox stream, so FP64 states agree to 1e-12
(only the order of a per-cell sum differs); FP32 to 2e-5 of the velocity
scale.  Then fused steps run on the new particle count, and a split that
would exceed max_particles is refused with the state unchanged."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _slab(prec, flow=3.0, n_cells=16, ppc=200, g=4):
    cfg, parts = W.vlasov_slab_1d(n_cells=n_cells, mean_ppc=ppc, long_range=mcpm.LR_NONE, precision=prec)
    parts = {k: v.copy() for k, v in parts.items()}
    parts["U1"] = parts["U1"] + flow
    if prec == mcpm.FP32:
        for k in ("x1", "x2", "U1", "U2", "U3"):
            parts[k] = parts[k].astype(np.float32).astype(np.float64)
    cfg.max_particles = len(parts["x2"]) * g
    return cfg, parts


def _tol(prec, ref):
    return (1e-12 if prec == mcpm.FP64 else 2e-5) * max(1.0, float(np.max(np.abs(ref))))


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_thermostat_matches_oracle(cuda_ok, prec):
    cfg, parts = _slab(prec)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg, parts)
    L1 = cfg.length[1]
    for x in (s, o):
        x.set_step(2)
        x.cell_update()
        x.thermostat(0.55, 1.3, 0.2 * L1, 0.3 * L1)
    g = s.download()
    for k in ("U1", "U2", "U3"):
        ref = getattr(o.s, k)
        assert np.max(np.abs(g[k] - ref)) <= _tol(prec, ref), k
    assert not np.allclose(g["U2"], parts["U2"])
    s.close()


@pytest.mark.parametrize("prec", [mcpm.FP64, mcpm.FP32])
def test_addremove_matches_oracle(cuda_ok, prec):
    g = 4
    cfg, parts = _slab(prec, g=g)
    N = len(parts["x2"])
    rng = np.random.default_rng(21)
    C = cfg.n_cells[1]
    cw = np.where(np.arange(C) < C // 2, 1, g).astype(np.int32)
    w = rng.choice([1, g], size=N).astype(np.int32)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    o = Oracle(cfg, parts)
    for x in (s, o):
        x.set_step(5)
        x.cell_update()
    s.set_particle_weights(w)
    s.set_cell_weights(cw)
    assert np.array_equal(s.get_particle_weights(), w)
    n = s.addremove_particles(g)
    out, wout, flag = o.addremove(w, cw, g)
    assert n == len(out["U1"]) and n != N
    assert (flag == -1).any() and (flag == 1).any()
    got = s.download()
    assert np.array_equal(got["x2"], out["x2"])
    for k in ("U1", "U2", "U3"):
        assert np.max(np.abs(got[k] - out[k])) <= _tol(prec, out[k]), k
    assert np.array_equal(s.get_particle_weights(), wout)
    # the fused steps go on with the new particle count
    e0 = sum(np.sum(got[k] ** 2) for k in ("U1", "U2", "U3"))
    s.step(4)
    s.check_status()
    g2 = s.download()
    assert len(g2["U1"]) == n and np.all(np.isfinite(g2["U1"]))
    e1 = sum(np.sum(g2[k] ** 2) for k in ("U1", "U2", "U3"))
    assert abs(e1 / e0 - 1.0) < 0.2
    s.close()


def test_addremove_refuses_beyond_capacity(cuda_ok):
    g = 4
    cfg, parts = _slab(mcpm.FP64, g=g)
    N = len(parts["x2"])
    cfg.max_particles = N
    C = cfg.n_cells[1]
    cw = np.full(C, 1, dtype=np.int32)
    w = np.full(N, g, dtype=np.int32)  # every particle heavy: N (g - 1) copies
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_step(1)
    s.cell_update()
    s.set_particle_weights(w)
    s.set_cell_weights(cw)
    before = s.download()
    with pytest.raises(mcpm.MCPMError) as e:
        s.addremove_particles(g)
    assert e.value.code == mcpm.ERR_CAPACITY
    assert s.N == N
    after = s.download()
    for k in ("x2", "U1", "U2", "U3"):
        assert np.array_equal(before[k], after[k])
    # weights equal to the cells': nothing to split or delete, N stays
    s.set_particle_weights(np.ones(N, dtype=np.int32))
    assert s.addremove_particles(g) == N
    s.close()


def test_weighted_cell_density_matches_oracle(cuda_ok):
    """cells[].n_ratio in the cell density n = n_ratio Fn N / V
    (src/Main_Functions.cpp:2588) and what is built on it (Y, gamma*, the
    drift coefficients)"""
    cfg, parts = _slab(mcpm.FP64)
    C = cfg.n_cells[1]
    cw = np.where(np.arange(C) < C // 2, 3, 1).astype(np.int32)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_cell_weights(cw)
    o = Oracle(cfg, parts)
    o.set_cell_weights(cw)
    for x in (s, o):
        x.set_step(2)
        x.cell_update()
    cg, co = s.get_cells(), o.cells()
    for f in ("N", "T", "GAMMA_ST"):
        a, b = mcpm.cell_field(cg, f), mcpm.cell_field(co, f, True)
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b)), f
    for f in ("C", "GAMMA", "ALPHA", "BETA"):
        a, b = mcpm.cell_field(cg, f), mcpm.cell_field(co, f, True)
        assert np.max(np.abs(a - b)) <= 1e-9 * max(np.max(np.abs(b)), 1e-300), f
    n = mcpm.cell_field(cg, "N")
    assert n[0] > 0 and np.all(n[: C // 2] > 0)
    s.close()
