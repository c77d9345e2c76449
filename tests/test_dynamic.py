"""The interface problems' thermostat and weighted-particle split / merge
(src/Main_Functions.cpp:1674-1869, :1206-1450): the oracle restatement
against the reference compiled from its own sources (oracle/_ref).

thermostat is deterministic: bit for bit.  inverted_addremove_particles
draws its deletions and its copies' velocity perturbations from
std::random_device, so the comparison is by what is fixed and by
statistics: the reference's kept particles are read off its output (they
keep their velocities exactly, in id order), the oracle's per-cell spread h
for exactly those flags is computed, and the reference's copies, taken as
parent + h z, must give z standard normal (mean and variance within 4
standard errors); deletions follow Binomial(light particles, 1 - 1/n_ratio)
within 4 sigma; every weight afterwards is its cell's.  The workload has a
mean flow, under which the reference's assigning "mean" loop (:1300-1306)
gives a spread far from the one a true mean would: the statistics pin it."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle, Reference, ref_lib


def _slab(flow=3.0, n_cells=24, ppc=120):
    cfg, parts = W.vlasov_slab_1d(n_cells=n_cells, mean_ppc=ppc, long_range=mcpm.LR_NONE)
    parts = {k: v.copy() for k, v in parts.items()}
    parts["U1"] = parts["U1"] + flow
    return cfg, parts


def _need_ref():
    if ref_lib() is None:
        pytest.skip("reference sources not present")


def test_weighted_cell_density_bit_exact_against_reference():
    """cells[].n_ratio enters the cell density, n = n_ratio Fn N / V
    (src/Main_Functions.cpp:2588), and every quantity built on it"""
    _need_ref()
    cfg, parts = _slab()
    cw = np.where(np.arange(cfg.n_cells[1]) < 10, 3, 1).astype(np.int32)
    o, r = Oracle(cfg, parts), Reference(cfg, parts)
    for x in (o, r):
        x.set_cell_weights(cw)
        x.set_step(2)
        x.cell_update()
    # every field but the kernel smoothing, which the oracle forms for its
    # one consumer (long_range 2) only
    ns = mcpm.CF["N_SMOOTH"]
    assert np.array_equal(o.cells()[:, :ns], r.cells()[:, :ns])
    o1 = Oracle(cfg, parts)
    o1.set_step(2)
    o1.cell_update()
    n, n1 = mcpm.cell_field(o.cells(), "N", True), mcpm.cell_field(o1.cells(), "N", True)
    assert np.allclose(n / n1, cw, rtol=1e-15)


def test_thermostat_bit_exact_against_reference():
    _need_ref()
    cfg, parts = _slab()
    o, r = Oracle(cfg, parts), Reference(cfg, parts)
    for x in (o, r):
        x.set_step(2)
        x.cell_update()
    L1 = cfg.length[1]
    for x in (o, r):
        x.thermostat(0.55, 1.3, 0.2 * L1, 0.3 * L1)
    for k in ("U1", "U2", "U3"):
        assert np.array_equal(getattr(o.s, k), getattr(r.s, k)), k
    assert not np.array_equal(o.s.U2, parts["U2"])


def _weights(cfg, parts, rng, g):
    C = cfg.n_cells[1]
    cw = np.where(np.arange(C) < C // 2, 1, g).astype(np.int32)  # liquid half light, vapour heavy
    w = rng.choice([1, g], size=len(parts["x2"])).astype(np.int32)
    return w, cw


def test_addremove_against_reference_statistics():
    _need_ref()
    g = 4
    cfg, parts = _slab(n_cells=16, ppc=400)
    rng = np.random.default_rng(21)
    w, cw = _weights(cfg, parts, rng, g)
    o, r = Oracle(cfg, parts), Reference(cfg, parts)
    for x in (o, r):
        x.set_step(5)
        x.cell_update()
    N = o.N
    out, wout = r.addremove(w, cw, g, cap=N * g)
    idx = o.s.index
    heavy = w > cw[idx]
    light = w < cw[idx]
    # the reference's kept particles: the first entries, their velocities
    # unchanged, in id order
    kept = np.zeros(N, dtype=bool)
    j = 0
    for i in range(N):
        if j < len(out["U1"]) and out["U1"][j] == o.s.U1[i] and out["U2"][j] == o.s.U2[i]:
            kept[i] = True
            j += 1
    n_kept = j
    assert np.all(kept[heavy]) and np.all(kept[~heavy & ~light])
    n_light, n_del = int(light.sum()), int((light & ~kept).sum())
    p = 1.0 - 1.0 / g
    assert abs(n_del - n_light * p) <= 4.0 * np.sqrt(n_light * p * (1 - p)) + 1
    assert len(out["U1"]) == n_kept + (g - 1) * int(heavy.sum())
    assert np.all(wout == cw[np.floor(out["x2"] / (cfg.length[1] / cfg.n_cells[1])).astype(int)])
    # the copies: parents ordered by cell, then id (src/Main_Functions.cpp:1337-1358)
    flag = np.where(heavy, 1, np.where(light & ~kept, -1, np.where(light, 2, 0))).astype(np.int8)
    h = o.addremove_widths(w, cw, g, flag)
    parents = sorted(np.nonzero(heavy)[0], key=lambda i: (idx[i], i))
    z = []
    for a, i in enumerate(parents):
        for c in range(g - 1):
            e = n_kept + a * (g - 1) + c
            assert out["x2"][e] == o.s.x2[i]
            for k in ("U1", "U2", "U3"):
                z.append((out[k][e] - getattr(o.s, k)[i]) / h[idx[i]])
    z = np.asarray(z)
    n = len(z)
    assert abs(z.mean()) <= 4.0 / np.sqrt(n), z.mean()
    assert abs(z.var() - 1.0) <= 4.0 * np.sqrt(2.0 / n), z.var()
    # a true weighted cell mean would give a much smaller spread under the
    # flow: the statistics above tell the two apart
    keep = flag != -1
    weff = np.where(flag == 2, cw[idx], w).astype(float)
    C = cfg.n_cells[1]
    Wc = np.bincount(idx[keep], weights=weff[keep], minlength=C)
    m = [np.bincount(idx[keep], weights=(getattr(o.s, k) * weff)[keep], minlength=C) / Wc for k in ("U1", "U2", "U3")]
    e = sum((getattr(o.s, k) - m[a][idx]) ** 2 for a, k in enumerate(("U1", "U2", "U3")))
    sig_true = np.sqrt(np.bincount(idx[keep], weights=(e * weff)[keep], minlength=C) / Wc)
    cells = np.nonzero(h > 0)[0]
    h_true = 1.06 * sig_true[cells] * (np.bincount(idx[keep & (flag != 1)], minlength=C)[cells] + g) ** -0.2
    assert np.median(h[cells] / h_true) > 1.5


def test_addremove_oracle_counts_and_order():
    g = 3
    cfg, parts = _slab(n_cells=12, ppc=100)
    rng = np.random.default_rng(5)
    w, cw = _weights(cfg, parts, rng, g)
    o = Oracle(cfg, parts)
    o.set_step(7)
    o.cell_update()
    out, wout, flag = o.addremove(w, cw, g)
    kept = flag != -1
    n_kept = int(kept.sum())
    assert len(out["U1"]) == n_kept + (g - 1) * int((flag == 1).sum())
    assert np.array_equal(out["U1"][:n_kept], o.s.U1[kept])
    assert np.array_equal(wout, cw[np.concatenate([o.s.index[kept], np.repeat(o.s.index[flag == 1], g - 1)])])
    # nothing heavy or light: nothing changes
    out2, w2, f2 = o.addremove(cw[o.s.index], cw, g)
    assert np.all(f2 == 0) and len(out2["U1"]) == o.N and np.array_equal(w2, cw[o.s.index])
