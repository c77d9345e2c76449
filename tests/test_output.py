"""The sampling and output row: measure_pressure (src/Main_Functions.cpp:
13-34) restated in the oracle, bit for bit against the reference compiled
from its own sources; the PostProc .dat file of write_post_processing
(src/myIO.cpp:597-934) written by the library from the reference's own cell
data, byte for byte equal to the file the reference writes; and the console
lines of post_processing (src/myIO.cpp:945-965), character for character."""
import os

import numpy as np
import pytest

import mcpm
import workloads as W
from oracle import Oracle, Reference, ref_lib

KEYS = ("x1", "x2", "U1", "U2", "U3")


def _need_ref():
    if ref_lib() is None:
        pytest.skip("reference sources not present")


def _stepped(n_cells=30, ppc=60, dt_scale=4.0):
    """a 1-D slab after one flight: old positions, new positions, the cells
    of cell_update at the old state, particles crossing faces"""
    cfg, parts = W.vlasov_slab_1d(n_cells=n_cells, mean_ppc=ppc, long_range=mcpm.LR_NONE)
    cfg.dt = cfg.dt * dt_scale
    return cfg, parts


def _flight(x):
    """cell_update, store_old_positions, stream_particles, apply_BC (the
    walls bring every particle back into the box)"""
    x.set_step(3)
    x.cell_update()
    x.store_old_positions()
    x.stream()
    if isinstance(x, Oracle):
        x.apply_bc(1)
    else:
        x.apply_bc()


def test_measure_pressure_bit_exact_against_reference():
    _need_ref()
    cfg, parts = _stepped()
    o, r = Oracle(cfg, parts), Reference(cfg, parts)
    for x in (o, r):
        _flight(x)
    p = np.zeros(o.C)
    o.measure_pressure(p)
    pr = r.measure_pressure()
    assert np.array_equal(p, pr)
    assert np.count_nonzero(p) > o.C // 2


def _ref_cells_field_major(r):
    return np.ascontiguousarray(r.cells().T)


def test_post_processing_file_matches_reference(tmp_path):
    _need_ref()
    cfg, parts = _stepped()
    cfg.model = mcpm.MODEL_FP_DENSE
    r = Reference(cfg, parts)
    _flight(r)
    r.set_step(4)
    r.cell_update()
    acc = np.zeros((r.C, mcpm.SF_COUNT))
    r.sample_cells(acc)
    pm = r.measure_pressure()
    (tmp_path / "ref" / "PostProc").mkdir(parents=True)
    (tmp_path / "ours").mkdir()
    r.write_post(7, 0.125, str(tmp_path / "ref"), "slab")
    ref_file = tmp_path / "ref" / "PostProc" / "slab_noatt_7.dat"
    assert ref_file.exists()
    path = mcpm.post_processing_write(cfg, 7, 0.125, str(tmp_path / "ours"), "slab", _ref_cells_field_major(r),
                                      samples=np.ascontiguousarray(acc.T), p_m=pm)
    assert os.path.basename(path) == "slab_noatt_7.dat"
    a, b = ref_file.read_bytes(), open(path, "rb").read()
    assert a == b, (len(a), len(b))


def test_post_processing_text_matches_reference():
    _need_ref()
    cfg, parts = _stepped()
    r = Reference(cfg, parts)
    r.set_step(2)
    r.cell_update()
    ref = [l for l in r.post_text(2).splitlines() if not l.startswith("post-proc took")]
    ours = mcpm.post_processing_text(cfg, _ref_cells_field_major(r)).splitlines()
    assert ours == ref
    # the 1-D-box form
    cfg1, parts1 = W.homogeneous_relaxation_1d(n_cells=1, ppc=500)
    r1 = Reference(cfg1, parts1)
    r1.set_step(2)
    r1.cell_update()
    ref1 = [l for l in r1.post_text(2).splitlines() if not l.startswith("post-proc took")]
    assert mcpm.post_processing_text(cfg1, _ref_cells_field_major(r1)).splitlines() == ref1
