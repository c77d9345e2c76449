"""Drives libmcpm_ref.so -- the reference's own routine signatures
(cell_update, velocity_update, apply_BC, ... of src/cpp_headers.h) over the
C-ABI -- the way the reference's main loop (src/main.cpp:389-514) calls
them: caller-owned double arrays and the reference's GAS / BOX / CELLS
structs, allocated and filled here through the library's layout helpers
(mcpm_compat_offset / mcpm_compat_new), since Python has no copy of the
reference's header."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import mcpm

REF_LIB = os.path.join(os.path.dirname(mcpm.LIB_PATH), "libmcpm_ref.so")
# the session seed the routines key their draws with (no field of GAS / BOX carries one)
SEED = 0x4D43504D
GAS, BOX, CELLS = 0, 1, 2
MODEL_NAMES = {mcpm.MODEL_FP_DENSE: "FP_dense", mcpm.MODEL_FP_IDEAL_GAS: "FP_ideal_gas", mcpm.MODEL_ESMC: "ESMC",
               mcpm.MODEL_FP_LINEAR: "FP_linear", mcpm.MODEL_DSMC_VHS: "DSMC_VHS", mcpm.MODEL_NONE: "none"}
# Itanium C++ names of the reference's prototypes (src/cpp_headers.h:362-501)
MANGLED = {
    "cell_update": "_Z11cell_updatePdS_S_S_S_P3GASP5CELLSP3BOXPiPS_S_S6_",
    "random_generator": "_Z16random_generatorPdS_S_S_S_S_P5CELLSP3BOXP3GASPi",
    "velocity_update": "_Z15velocity_updatePdS_S_S_S_S_P3GASP3BOXP5CELLSPiP9CollisionS_S_S_S_S_S_S_S_S_S_S_S6_",
    "DFP_extra_streaming": "_Z19DFP_extra_streamingPdS_S_S_S_P3GASP3BOXP5CELLSPid",
    "apply_BC": "_Z8apply_BCPdS_S_S_S_S_S_S_S_P3GASP3BOXP5CELLSPiS6_S_S_S_S_S_S_S_S_S_S_",
    "store_old_positions": "_Z19store_old_positionsPdS_S_S_S_S_P3GASP3BOX",
    "stream_particles": "_Z16stream_particlesPdS_S_S_S_S_S_S_S_P3GASP3BOXP5CELLSPi",
    "measure_pressure": "_Z16measure_pressurePdS_S_P3GASP3BOXP5CELLS",
}
# argument counts (all pointers, but DFP_extra_streaming's trailing double dt)
NARGS = {"cell_update": 12, "random_generator": 10, "velocity_update": 23, "DFP_extra_streaming": 10,
         "apply_BC": 24, "store_old_positions": 8, "stream_particles": 13, "measure_pressure": 6}


def load():
    L = C.CDLL(REF_LIB)
    L.mcpm_compat_sizeof.restype = C.c_int64
    L.mcpm_compat_sizeof.argtypes = [C.c_int32]
    L.mcpm_compat_offset.restype = C.c_int64
    L.mcpm_compat_offset.argtypes = [C.c_char_p, C.POINTER(C.c_int64)]
    L.mcpm_compat_new.restype = C.c_void_p
    L.mcpm_compat_new.argtypes = [C.c_int32, C.c_int64]
    L.mcpm_compat_delete.restype = None
    L.mcpm_compat_delete.argtypes = [C.c_int32, C.c_void_p, C.c_int64]
    L.mcpm_compat_set_model.restype = None
    L.mcpm_compat_set_model.argtypes = [C.c_void_p, C.c_char_p]
    L.mcpm_compat_routine.restype = C.c_void_p
    L.mcpm_compat_routine.argtypes = [C.c_char_p]
    L.mcpm_compat_session.restype = C.c_void_p
    L.mcpm_compat_reset.restype = None
    return L


def routine(L, name):
    """The routine bound by its C++ name, the way the reference's objects bind it."""
    addr = C.cast(getattr(L, MANGLED[name]), C.c_void_p).value
    assert addr == L.mcpm_compat_routine(name.encode())
    args = [C.c_void_p] * NARGS[name]
    if name == "DFP_extra_streaming":
        args[-1] = C.c_double
    return C.CFUNCTYPE(None, *args)(addr)


class Structs:
    """One GAS, one BOX and the CELLS array, laid out as the reference's
    compiler lays them out, filled from an mcpm config."""

    def __init__(self, L, cfg, N):
        self.L, self.N = L, N
        self.C = cfg.n_cells[0] * cfg.n_cells[1] * cfg.n_cells[2]
        self.gas = L.mcpm_compat_new(GAS, 1)
        self.box = L.mcpm_compat_new(BOX, 1)
        self.cells = L.mcpm_compat_new(CELLS, self.C)
        self.cell_size = L.mcpm_compat_sizeof(CELLS)
        g = self.put
        g(self.gas, "GAS.N", C.c_long, N)
        for f in ("sigma", "m", "kb", "n", "Fn", "T0", "mu", "visp", "b", "phi", "eqdist", "ast", "bst", "crref"):
            g(self.gas, "GAS." + f, C.c_double, getattr(cfg, f))
        g(self.gas, "GAS.delta_t", C.c_double, cfg.dt)
        g(self.gas, "GAS.long_range", C.c_int, cfg.long_range)
        L.mcpm_compat_set_model(self.gas, MODEL_NAMES[cfg.model].encode())
        for i in range(3):
            g(self.box, "BOX.N", C.c_int, cfg.n_cells[i], i)
            g(self.box, "BOX.direction", C.c_int, cfg.direction[i], i)
            g(self.box, "BOX.Len", C.c_double, cfg.length[i], i)
        g(self.box, "BOX.problem", C.c_int, cfg.problem)
        for i in range(4):
            g(self.box, "BOX.T_wall_%d" % (i + 1), C.c_double, cfg.T_wall[i])
            g(self.box, "BOX.U_wall_%d" % (i + 1), C.c_double, cfg.U_wall[i])
        for c in range(self.C):
            self.put(self.cell(c), "CELLS.n_ratio", C.c_int, 1)

    def close(self):
        if self.gas:
            self.L.mcpm_compat_delete(GAS, self.gas, 1)
            self.L.mcpm_compat_delete(BOX, self.box, 1)
            self.L.mcpm_compat_delete(CELLS, self.cells, self.C)
            self.gas = self.box = self.cells = None

    def __del__(self):
        self.close()

    def _addr(self, base, name, ctype, i):
        sz = C.c_int64(0)
        off = self.L.mcpm_compat_offset(name.encode(), C.byref(sz))
        assert off >= 0, name
        assert (i + 1) * C.sizeof(ctype) <= sz.value, name
        return base + off + i * C.sizeof(ctype)

    def put(self, base, name, ctype, v, i=0):
        ctype.from_address(self._addr(base, name, ctype, i)).value = v

    def get(self, base, name, ctype=C.c_double, i=0):
        return ctype.from_address(self._addr(base, name, ctype, i)).value

    def cell(self, c):
        return self.cells + c * self.cell_size

    def field(self, name, width=1):
        """[C][width] of a CELLS double field"""
        out = np.empty((self.C, width))
        for c in range(self.C):
            for j in range(width):
                out[c, j] = self.get(self.cell(c), "CELLS." + name, C.c_double, j)
        return out

    def list_of(self, c):
        n = self.get(self.cell(c), "CELLS.num_inside", C.c_int)
        p = C.c_void_p.from_address(self._addr(self.cell(c), "CELLS.indices_inside", C.c_void_p, 0)).value
        return np.ctypeslib.as_array((C.c_int * n).from_address(p)).copy() if n else np.zeros(0, np.int32)


class MainLoop:
    """The particle part of one iteration of src/main.cpp:389-514, through
    the routines of libmcpm_ref.so on arrays owned here."""

    def __init__(self, cfg, parts):
        self.L = load()
        self.cfg = cfg
        N = len(parts["x2"])
        self.N = N
        self.st = Structs(self.L, cfg, N)
        f = lambda k: np.ascontiguousarray(parts.get(k, np.zeros(N)), dtype=np.float64).copy()  # noqa: E731
        self.x1, self.x2, self.U1, self.U2, self.U3 = f("x1"), f("x2"), f("U1"), f("U2"), f("U3")
        self.x3 = np.zeros(N)
        self.x1o, self.x2o, self.x3o = self.x1.copy(), self.x2.copy(), self.x3.copy()
        self.index = np.zeros(N, dtype=np.int32)
        self.flag = np.zeros(N, dtype=np.int32)
        self.scratch = [np.zeros(N) for _ in range(12)]
        self.T = np.zeros(self.st.C)
        self.T_ptr = C.c_void_p(self.T.ctypes.data)
        self.r = {k: routine(self.L, k) for k in MANGLED}

    def close(self):
        self.st.close()
        self.L.mcpm_compat_reset()

    def _p(self, a):
        return a.ctypes.data

    def set_step(self, step):
        self.st.put(self.st.box, "BOX.step", C.c_int, step)

    def cell_update(self):
        p, s = self._p, self.st
        self.r["cell_update"](p(self.x1), p(self.x2), p(self.U1), p(self.U2), p(self.U3), s.gas, s.cells, s.box,
                              p(self.index), C.addressof(self.T_ptr), p(self.scratch[0]), p(self.flag))

    def random_generator(self):
        p, s, x = self._p, self.st, self.scratch
        self.r["random_generator"](p(x[0]), p(x[1]), p(x[2]), p(x[3]), p(x[4]), p(x[5]), s.cells, s.box, s.gas,
                                   p(self.index))

    def velocity_update(self):
        p, s, x = self._p, self.st, self.scratch
        self.r["velocity_update"](p(self.U1), p(self.U2), p(self.U3), p(self.x1), p(self.x2), p(self.x3), s.gas,
                                  s.box, s.cells, p(self.index), None, p(x[3]), p(x[4]), p(x[5]), p(x[6]), p(x[7]),
                                  p(x[8]), p(x[9]), p(x[10]), p(x[11]), p(x[0]), p(self.T), p(self.flag))

    def DFP_extra_streaming(self):
        p, s = self._p, self.st
        self.r["DFP_extra_streaming"](p(self.U1), p(self.U2), p(self.U3), p(self.x1), p(self.x2), s.gas, s.box,
                                      s.cells, p(self.index), self.cfg.dt)

    def apply_BC(self):
        p, s, x = self._p, self.st, self.scratch
        self.r["apply_BC"](p(self.U1), p(self.U2), p(self.U3), p(self.x1), p(self.x2), p(self.x3), p(self.x1o),
                           p(self.x2o), p(self.x3o), s.gas, s.box, s.cells, p(self.index), p(self.flag), p(x[0]),
                           p(x[1]), p(x[2]), p(x[3]), p(x[4]), p(x[5]), p(x[6]), p(x[7]), p(x[8]), p(self.T))

    def store_old_positions(self):
        p, s = self._p, self.st
        self.r["store_old_positions"](p(self.x1), p(self.x2), p(self.x3), p(self.x1o), p(self.x2o), p(self.x3o),
                                      s.gas, s.box)

    def stream_particles(self):
        p, s = self._p, self.st
        self.r["stream_particles"](p(self.U1), p(self.U2), p(self.U3), p(self.x1), p(self.x2), p(self.x3),
                                   p(self.x1o), p(self.x2o), p(self.x3o), s.gas, s.box, s.cells, p(self.index))

    def measure_pressure(self):
        p, s = self._p, self.st
        self.r["measure_pressure"](p(self.U2), p(self.x2), p(self.x2o), s.gas, s.box, s.cells)

    def layout(self):
        """(pid_by_slot, off) of the session behind the routines: the in-cell
        order of its last cell_update"""
        lib = mcpm.load_library()
        pid = np.empty(self.N, dtype=np.int32)
        off = np.empty(self.st.C + 1, dtype=np.int32)
        rc = lib.mcpm_get_layout(self.L.mcpm_compat_session(), pid.ctypes.data_as(C.POINTER(C.c_int32)),
                                 off.ctypes.data_as(C.POINTER(C.c_int32)))
        assert rc == 0, rc
        return pid, off

    def iteration(self, step, pressure=False, after_cell_update=None):
        """src/main.cpp:392-514 for the particle step (no shock / hybrid
        branches): cell_update, the FP draws, velocity_update,
        DFP_extra_streaming, apply_BC, store_old_positions,
        stream_particles, apply_BC, measure_pressure, apply_BC."""
        m = self.cfg.model
        self.set_step(step)
        self.cell_update()
        if after_cell_update is not None:
            after_cell_update()
        if m in (mcpm.MODEL_FP_DENSE, mcpm.MODEL_FP_IDEAL_GAS):
            self.random_generator()
        self.velocity_update()
        if m == mcpm.MODEL_FP_DENSE:
            self.DFP_extra_streaming()
        self.apply_BC()
        self.store_old_positions()
        self.stream_particles()
        self.apply_BC()
        if pressure:
            self.measure_pressure()
        self.apply_BC()

    def particles(self):
        return dict(x1=self.x1, x2=self.x2, U1=self.U1, U2=self.U2, U3=self.U3)

