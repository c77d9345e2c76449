"""The reference's own routine signatures (libmcpm_ref.so,
compat/reference_surface.cpp) driven in the order of the reference's main
loop (src/main.cpp:392-514) on caller-owned arrays and the reference's
GAS / BOX / CELLS structs.

FP models: three iterations against the oracle's loop on the same seeded
particles -- positions and velocities within 1e-9 (the moment sums run in
another order), the index[] and the per-cell lists (cells[].indices_inside,
ascending ids) exactly, the CELLS moments within 1e-9 and the pressure
count (cells[].p_m) within 1e-9.  Pair models (ESMC, DSMC_VHS), whose pairs
follow the in-cell order of the device layout (the oracle is handed that
order after each cell_update): the same, with the majorant the reference
keeps in cells[].omega_max / cells[].crm within 1e-12."""
import ctypes

import numpy as np
import pytest

import mcpm
import workloads as W
from compat_driver import SEED, MainLoop
from oracle import Oracle

pytestmark = pytest.mark.gpu

K = 3
CELL_FIELDS = [("U_space", "U_SPACE", 3), ("PIJ", "PIJ", 6), ("M3", "M3", 10), ("T", "T", 1), ("n", "N", 1),
               ("Q", "Q", 3), ("alpha", "ALPHA", 9), ("beta", "BETA", 3), ("gamma", "GAMMA", 3), ("c", "C", 6),
               ("Lambda", "LAMBDA", 1), ("gamma_st", "GAMMA_ST", 1), ("DM2", "DM2", 1)]


def _fp64(cfg, N):
    c = cfg.copy()
    c.precision = mcpm.FP64
    c.seed = SEED
    c.max_particles = N
    return c


def _case(name):
    if name == "slab_poisson":
        cfg, parts = W.vlasov_slab_1d(n_cells=30, mean_ppc=40, precision=mcpm.FP64)
    elif name == "couette_fp":
        cfg, parts = W.esmc_box_2d(n_cells=(12, 12), ppc=40, precision=mcpm.FP64)
        cfg.model = mcpm.MODEL_FP_DENSE
        parts = {k: v.copy() for k, v in parts.items()}
        parts["U1"] *= 5.0
        parts["U2"] *= 5.0
    elif name == "wall_fp":
        cfg, parts = W.vlasov_slab_1d(n_cells=30, mean_ppc=40, long_range=mcpm.LR_NONE, precision=mcpm.FP64)
        cfg.problem = mcpm.PROBLEM_WALL
        cfg.T_wall[0] = 1.3
        parts = {k: v.copy() for k, v in parts.items()}
        parts["U2"] *= 5.0
    elif name == "periodic_ideal":
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=30, ppc=80, precision=mcpm.FP64)
        cfg.model = mcpm.MODEL_FP_IDEAL_GAS
    elif name == "esmc_couette":
        cfg, parts = W.esmc_box_2d(n_cells=(10, 10), ppc=40, precision=mcpm.FP64)
    elif name == "dsmc_periodic":
        cfg, parts = W.homogeneous_relaxation_1d(n_cells=30, ppc=80, precision=mcpm.FP64)
        W.with_dsmc_vhs(cfg)
    else:
        raise KeyError(name)
    return _fp64(cfg, len(parts["x2"])), parts


def _check_lists(ml):
    idx = ml.index
    for c in range(ml.st.C):
        assert np.array_equal(ml.st.list_of(c), np.flatnonzero(idx == c)), c


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(1.0, np.max(np.abs(b)))


@pytest.mark.parametrize("name", ["slab_poisson", "couette_fp", "wall_fp", "periodic_ideal"])
def test_reference_loop_fp_vs_oracle(cuda_ok, name):
    cfg, parts = _case(name)
    pressure = name == "slab_poisson"
    ml = MainLoop(cfg, parts)
    o = Oracle(cfg, parts)
    o.set_step(1)
    p_o = np.zeros(ml.st.C)
    try:
        for step in range(1, K + 1):
            ml.iteration(step, pressure=pressure)
            o.step(1)
            if pressure:
                o.measure_pressure(p_o)
            assert np.array_equal(ml.index, o.s.index), step
            _check_lists(ml)
            co = o.cells()
            for ref_name, cf, w in CELL_FIELDS:
                a = ml.st.field(ref_name, w)
                b = co[:, mcpm.CF[cf]:mcpm.CF[cf] + w]
                assert _rel(a, b) <= 1e-9, (step, ref_name)
            n_in = np.array([ml.st.get(ml.st.cell(c), "CELLS.num_inside", ctypes.c_int) for c in range(ml.st.C)])
            assert np.array_equal(n_in, np.bincount(o.s.index, minlength=ml.st.C))
        keys = ("x2", "U1", "U2", "U3") if cfg.direction[0] == 0 else ("x1", "x2", "U1", "U2", "U3")
        for k in keys:
            assert _rel(getattr(ml, k), getattr(o.s, k)) <= 1e-9, k
        if cfg.problem in (mcpm.PROBLEM_COUETTE, mcpm.PROBLEM_WALL):
            assert _rel(ml.x2o, o.s.x2o) <= 1e-9
        if pressure:
            p = ml.st.field("p_m")[:, 0]
            assert np.any(p != 0.0)
            assert _rel(p, p_o) <= 1e-9
    finally:
        ml.close()


@pytest.mark.parametrize("name", ["esmc_couette", "dsmc_periodic"])
def test_reference_loop_pairs_vs_oracle(cuda_ok, name):
    cfg, parts = _case(name)
    ml = MainLoop(cfg, parts)
    o = Oracle(cfg, parts)
    # the majorant the reference's main sets before its loop (src/main.cpp:236-269)
    o.set_step(0)
    o.cell_update()
    o.init_omega_max()
    om = mcpm.cell_field(o.cells(), "OMEGA_MAX", True).copy()
    field = "crm" if cfg.model == mcpm.MODEL_DSMC_VHS else "omega_max"
    p_o = np.zeros(ml.st.C)
    try:
        for c in range(ml.st.C):
            ml.st.put(ml.st.cell(c), "CELLS." + field, ctypes.c_double, float(om[c]))

        for step in range(1, K + 1):
            def oracle_cell_update():
                # the oracle's pairs follow the device's in-cell order
                pid, off = ml.layout()
                o.set_step(step)
                o.cell_update()
                o.set_layout(off, pid)
                if step == 1:
                    o.set_cell_field(mcpm.CF["OMEGA_MAX"], om)

            ml.iteration(step, pressure=True, after_cell_update=oracle_cell_update)
            (o.esmc if cfg.model == mcpm.MODEL_ESMC else o.dsmc)()
            o.apply_bc(0)
            o.store_old_positions()
            o.stream()
            o.apply_bc(1)
            o.measure_pressure(p_o)
            o.apply_bc(2)
            for k in ("x1", "x2", "U1", "U2", "U3"):
                if k == "x1" and cfg.direction[0] == 0:
                    continue
                assert _rel(getattr(ml, k), getattr(o.s, k)) <= 1e-10, (step, k)
            if cfg.problem == mcpm.PROBLEM_COUETTE:
                assert _rel(ml.x1o, o.s.x1o) <= 1e-10 and _rel(ml.x2o, o.s.x2o) <= 1e-10
            assert np.array_equal(ml.index, o.s.index), step
            _check_lists(ml)
            co = o.cells()
            for ref_name, cf, w in CELL_FIELDS:
                assert _rel(ml.st.field(ref_name, w), co[:, mcpm.CF[cf]:mcpm.CF[cf] + w]) <= 1e-9, (step, ref_name)
            om_o = mcpm.cell_field(co, "OMEGA_MAX", True)
            assert np.max(np.abs(ml.st.field(field)[:, 0] - om_o)) <= 1e-12 * max(1.0, np.max(om_o)), step
        assert _rel(ml.st.field("p_m")[:, 0], p_o) <= 1e-9
        # the collisions moved velocities
        assert np.count_nonzero(ml.U1 != parts["U1"]) > 0.05 * ml.N
    finally:
        ml.close()
