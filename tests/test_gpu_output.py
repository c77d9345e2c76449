"""Pressure sampling and the post-processing file on the GPU: p_m of
measure_pressure (src/Main_Functions.cpp:13-34) from the routine-by-routine
loop and from fused steps against the oracle (itself bit-exact against the
reference, tests/test_output.py) with the shared Philox draws -- FP64 within
1e-12 of the largest value (only the order of the per-cell additions
differs); and the session's .dat file equal byte for byte to the host writer
fed with the session's own fields."""
import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle

pytestmark = pytest.mark.gpu


def _slab(prec=mcpm.FP64):
    cfg, parts = W.vlasov_slab_1d(n_cells=30, mean_ppc=60, long_range=mcpm.LR_NONE, precision=prec)
    cfg.dt = cfg.dt * 4.0
    return cfg, parts


def test_measure_pressure_routine_matches_oracle(cuda_ok):
    cfg, parts = _slab()
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_pressure_sampling(True)
    o = Oracle(cfg, parts)
    for x in (s, o):
        x.set_step(3)
        x.cell_update()
    s.store_old_positions()
    s.stream_particles()
    s.apply_BC()
    s.measure_pressure()
    o.store_old_positions()
    o.stream()
    o.apply_bc(1)
    p = np.zeros(o.C)
    o.measure_pressure(p)
    g = s.get_pressure()
    assert np.count_nonzero(p) > o.C // 2
    assert np.max(np.abs(g - p)) <= 1e-12 * np.max(p)


def test_pressure_in_fused_steps_matches_oracle(cuda_ok):
    cfg, parts = _slab()
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_pressure_sampling(True)
    s.set_step(1)
    s.step(4)
    o = Oracle(cfg, parts)
    o.set_step(1)
    p = np.zeros(o.C)
    for _ in range(4):
        o.step(1)
        o.measure_pressure(p)
    g = s.get_pressure()
    assert np.max(np.abs(g - p)) <= 1e-10 * np.max(p)
    s.reset_pressure()
    assert not np.any(s.get_pressure())
    s.close()


def test_pressure_fp32_fused_totals(cuda_ok):
    cfg, parts = _slab(mcpm.FP32)
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_pressure_sampling(True)
    s.set_step(1)
    s.step(4)
    cfg64 = cfg.copy()
    cfg64.precision = mcpm.FP64
    o = Oracle(cfg64, {k: (v.astype(np.float32).astype(np.float64) if k in ("x1", "x2", "U1", "U2", "U3") else v)
                       for k, v in parts.items()})
    o.set_step(1)
    p = np.zeros(o.C)
    for _ in range(4):
        o.step(1)
        o.measure_pressure(p)
    g = s.get_pressure()
    assert abs(g.sum() / p.sum() - 1.0) < 2e-3
    s.close()


def test_session_post_processing_file(cuda_ok, tmp_path):
    cfg, parts = _slab()
    s = mcpm.Session(cfg)
    s.upload(parts["x1"], parts["x2"], parts["U1"], parts["U2"], parts["U3"])
    s.set_pressure_sampling(True)
    s.set_step(1)
    s.step(3)
    s.cell_update()
    s.sample_cells()
    path = s.write_post_processing(4, 0.5, str(tmp_path), "slab")
    host = tmp_path / "host"
    host.mkdir()
    ref = mcpm.post_processing_write(cfg, 4, 0.5, str(host), "slab", s.get_cells(), samples=s.get_samples(),
                                     p_m=s.get_pressure())
    assert open(path, "rb").read() == open(ref, "rb").read()
    lines = open(path).read().splitlines()
    assert len(lines) == 1 + cfg.n_cells[1] + 1 and len(lines[1].split()) == 121
    s.close()
