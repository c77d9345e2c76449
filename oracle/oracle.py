"""ctypes bindings of the checkers (TEST INFRASTRUCTURE ONLY).

* :class:`Oracle` -- liboracle.so, the plain-C FP64 restatement of the
  reference step (mcpm_oracle.c).
* :class:`Reference` -- oracle/_ref/libref.so, the reference's own routines
  compiled from its sources (available only where the reference tree was
  present at build time).

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU baseline use
this module.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
PKG = os.path.join(REPO, "monte-carlo-particle-method_gb300")
if PKG not in sys.path:
    sys.path.insert(0, PKG)
from mcpm import CF_COUNT, LR_DENSITY_EXPANSION, Config  # noqa: E402

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int32)


def _dp(a):
    return a.ctypes.data_as(dp) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ip) if a is not None else None


def _load_oracle():
    from build import build_oracle  # oracle/build.py
    path = build_oracle()
    L = C.CDLL(path)
    vp = C.c_void_p
    sig = {
        "orc_create": (vp, [C.POINTER(Config), C.c_int64]),
        "orc_destroy": (None, [vp]),
        "orc_num_cells": (C.c_int, [vp]),
        "orc_set_cell_weights": (None, [vp, ip]),
        "orc_get_cells": (None, [vp, dp]),
        "orc_set_cell_field": (None, [vp, C.c_int, dp]),
        "orc_get_step": (C.c_int, [vp]),
        "orc_set_step": (None, [vp, C.c_int]),
        "orc_status": (C.c_int, [vp]),
        "orc_inject_normals": (None, [vp, dp, dp, dp]),
        "orc_set_rng": (None, [vp, C.c_int]),
        "orc_inject_uniforms": (None, [vp, C.c_int, C.c_int64, dp]),
        "orc_cell_update": (None, [vp, dp, dp, dp, dp, dp, ip]),
        "orc_random_generator": (None, [vp, dp, dp, dp]),
        "orc_velocity_fp": (None, [vp, dp, dp, dp, dp, dp, dp]),
        "orc_esmc": (None, [vp, dp, dp, dp, dp, dp]),
        "orc_dsmc_vhs": (None, [vp, dp, dp, dp]),
        "orc_sample_cells": (None, [vp, dp, dp, dp, dp]),
        "orc_long_range": (None, [vp, dp]),
        "orc_dfp_extra_streaming": (None, [vp, dp, dp, dp, dp, dp]),
        "orc_apply_bc": (None, [vp, C.c_int, dp, dp, dp, dp, dp, dp, dp]),
        "orc_store_old_positions": (None, [vp, dp, dp, dp, dp]),
        "orc_stream": (None, [vp, dp, dp, dp, dp, dp]),
        "orc_init_omega_max": (None, [vp]),
        "orc_step": (None, [vp, dp, dp, dp, dp, dp, dp, dp, ip]),
        "orc_set_layout": (None, [vp, ip, ip]),
        "orc_philox4x32_10": (None, [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]),
        "orc_normals4": (None, [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, dp]),
        "orc_gauss_jordan": (None, [dp, dp, C.c_int, dp]),
        "orc_gl_table": (None, [C.c_int, dp, dp]),
        "orc_vlasov_face_potential": (None, [vp, dp]),
        "orc_poisson_faces": (None, [vp, dp]),
        "orc_get_node_density": (None, [vp, dp]),
        "orc_vlasov2d_nodes": (None, [vp, dp]),
        "orc_sp2d_nodes": (None, [vp, dp]),
        "orc_long_range_2d": (None, [vp, dp, dp, dp, dp, dp]),
        "orc_thermostat": (None, [vp, dp, dp, dp, C.c_double, C.c_double, C.c_double, C.c_double]),
        "orc_addremove_flags": (None, [vp, ip, ip, C.c_int, C.POINTER(C.c_int8), C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)]),
        "orc_measure_pressure": (None, [vp, dp, dp, dp, dp]),
        "orc_addremove_widths": (None, [vp, dp, dp, dp, ip, ip, C.c_int, C.POINTER(C.c_int8), dp]),
        "orc_addremove_apply": (None, [vp, dp, dp, dp, dp, dp, dp, dp, ip, ip, C.c_int, C.POINTER(C.c_int8),
                                       dp, dp, dp, dp, dp, dp, dp, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    return L


_OL = None


def oracle_lib():
    global _OL
    if _OL is None:
        sys.path.insert(0, HERE)
        try:
            _OL = _load_oracle()
        finally:
            sys.path.remove(HERE)
    return _OL


class State:
    """Particle arrays in the reference's layout (indexed by particle id)."""

    def __init__(self, parts, N):
        self.x1 = np.ascontiguousarray(parts.get("x1", np.zeros(N)), dtype=np.float64).copy()
        self.x2 = np.ascontiguousarray(parts["x2"], dtype=np.float64).copy()
        self.U1 = np.ascontiguousarray(parts["U1"], dtype=np.float64).copy()
        self.U2 = np.ascontiguousarray(parts["U2"], dtype=np.float64).copy()
        self.U3 = np.ascontiguousarray(parts["U3"], dtype=np.float64).copy()
        self.x1o = self.x1.copy()
        self.x2o = self.x2.copy()
        self.index = np.zeros(N, dtype=np.int32)

    def as_dict(self):
        return dict(x1=self.x1, x2=self.x2, U1=self.U1, U2=self.U2, U3=self.U3)


class Oracle:
    """The FP64 CPU restatement, one instance per particle system."""

    def __init__(self, cfg: Config, parts):
        self.L = oracle_lib()
        self.cfg = cfg.copy()
        self.N = len(parts["x2"])
        self.C = cfg.n_cells[0] * cfg.n_cells[1]
        self.h = self.L.orc_create(C.byref(self.cfg), self.N)
        self.s = State(parts, self.N)
        self.xi = [np.zeros(self.N), np.zeros(self.N), np.zeros(self.N)]

    def __del__(self):
        try:
            self.L.orc_destroy(self.h)
        except Exception:
            pass

    @property
    def step_count(self):
        return self.L.orc_get_step(self.h)

    def set_step(self, k):
        self.L.orc_set_step(self.h, k)

    def status(self):
        return self.L.orc_status(self.h)

    def inject_normals(self, a, b, c):
        self._inj = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c)]
        self.L.orc_inject_normals(self.h, *[_dp(v) for v in self._inj])

    def set_rng(self, mode):
        self.L.orc_set_rng(self.h, mode)

    def inject_uniforms(self, stream, u):
        """u: [rows][4] uniforms for the stream (None restores Philox)"""
        if u is None:
            self.L.orc_inject_uniforms(self.h, int(stream), 0, None)
            return
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 4)
        self.L.orc_inject_uniforms(self.h, int(stream), len(u), _dp(u))

    def cells(self):
        out = np.empty((self.C, CF_COUNT))
        self.L.orc_get_cells(self.h, _dp(out))
        return out

    def set_cell_field(self, f, v):
        v = np.ascontiguousarray(v, dtype=np.float64)
        self.L.orc_set_cell_field(self.h, f, _dp(v))

    def set_layout(self, off, pid_by_slot):
        """Use a given in-cell order (e.g. the GPU's) instead of ascending ids."""
        self._lay = (np.ascontiguousarray(off, dtype=np.int32), np.ascontiguousarray(pid_by_slot, dtype=np.int32))
        self.L.orc_set_layout(self.h, _ip(self._lay[0]), _ip(self._lay[1]))

    def cell_update(self):
        s = self.s
        self.L.orc_cell_update(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U1), _dp(s.U2), _dp(s.U3), _ip(s.index))

    def random_generator(self):
        self.L.orc_random_generator(self.h, *[_dp(v) for v in self.xi])

    def velocity_fp(self):
        s = self.s
        self.L.orc_velocity_fp(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), *[_dp(v) for v in self.xi])

    def esmc(self):
        s = self.s
        self.L.orc_esmc(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U1), _dp(s.U2), _dp(s.U3))

    def sample_cells(self, acc):
        """cell_poly_velocity into acc, [C][SF_COUNT] (added to)"""
        s = self.s
        self.L.orc_sample_cells(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(acc))

    def dsmc(self):
        """Collision_DSMC_VHS (src/collisions.cpp:2063-2141)"""
        s = self.s
        self.L.orc_dsmc_vhs(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3))

    def long_range(self):
        """velocity_update's long-range kick: the 1-D face paths, or the 2-D
        node paths when the box is 2-D (returns the node potential then)."""
        s = self.s
        if self.cfg.direction[0] == 1 and self.cfg.long_range != LR_DENSITY_EXPANSION:
            V = np.empty((self.cfg.n_cells[0] + 1) * (self.cfg.n_cells[1] + 1))
            self.L.orc_long_range_2d(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U1), _dp(s.U2), _dp(V))
            return V
        self.L.orc_long_range(self.h, _dp(s.U2))
        return None

    def node_density(self):
        out = np.empty((self.C, 4))
        self.L.orc_get_node_density(self.h, _dp(out))
        return out

    def node_potential(self, mode):
        V = np.empty((self.cfg.n_cells[0] + 1) * (self.cfg.n_cells[1] + 1))
        (self.L.orc_vlasov2d_nodes if mode == 1 else self.L.orc_sp2d_nodes)(self.h, _dp(V))
        return V

    def dfp_extra_streaming(self):
        s = self.s
        self.L.orc_dfp_extra_streaming(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2))

    def apply_bc(self, call_no):
        s = self.s
        self.L.orc_apply_bc(self.h, call_no, _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o), _dp(s.U1), _dp(s.U2),
                            _dp(s.U3))

    def store_old_positions(self):
        s = self.s
        self.L.orc_store_old_positions(self.h, _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o))

    def stream(self):
        s = self.s
        self.L.orc_stream(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U1), _dp(s.U2), _dp(s.U3))

    def init_omega_max(self):
        self.L.orc_init_omega_max(self.h)

    def set_cell_weights(self, cw):
        """cells[].n_ratio (the weight in the cell density)"""
        self._cw = np.ascontiguousarray(cw, dtype=np.int32)
        self.L.orc_set_cell_weights(self.h, _ip(self._cw))

    def measure_pressure(self, p_m):
        """measure_pressure (src/Main_Functions.cpp:13-34) added into p_m [C]"""
        s = self.s
        self.L.orc_measure_pressure(self.h, _dp(s.U2), _dp(s.x2), _dp(s.x2o), _dp(p_m))

    def thermostat(self, Tc, Th, thermc, thermh):
        """thermostat (src/Main_Functions.cpp:1674-1869) on the lists of the
        last cell_update"""
        s = self.s
        self.L.orc_thermostat(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), Tc, Th, thermc, thermh)

    def addremove(self, w, cw, n_ratio):
        """inverted_addremove_particles (src/Main_Functions.cpp:1206-1450)
        against the cells of the last cell_update: returns (parts, weights,
        flags) of the new state; the oracle itself is left as it was (build a
        new one on the returned particles to go on)."""
        w = np.ascontiguousarray(w, dtype=np.int32)
        cw = np.ascontiguousarray(cw, dtype=np.int32)
        flag = np.zeros(self.N, dtype=np.int8)
        nk, nn = C.c_int64(0), C.c_int64(0)
        i8 = lambda a: a.ctypes.data_as(C.POINTER(C.c_int8))  # noqa: E731
        self.L.orc_addremove_flags(self.h, _ip(w), _ip(cw), int(n_ratio), i8(flag), C.byref(nk), C.byref(nn))
        n = nk.value + nn.value if (nn.value or nk.value != self.N) else self.N
        out = {k: np.zeros(n) for k in ("x1", "x2", "x1o", "x2o", "U1", "U2", "U3")}
        wo = np.zeros(n, dtype=np.int32)
        s = self.s
        self.L.orc_addremove_apply(self.h, _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o), _dp(s.U1), _dp(s.U2),
                                   _dp(s.U3), _ip(w), _ip(cw), int(n_ratio), i8(flag),
                                   *[_dp(out[k]) for k in ("x1", "x2", "x1o", "x2o", "U1", "U2", "U3")], _ip(wo))
        if n == self.N and not nn.value:
            out = {k: getattr(s, k).copy() for k in ("x1", "x2", "x1o", "x2o", "U1", "U2", "U3")}
        return out, wo, flag

    def addremove_widths(self, w, cw, n_ratio, flag):
        """per-cell velocity spread h of the copies for the given flags"""
        w = np.ascontiguousarray(w, dtype=np.int32)
        cw = np.ascontiguousarray(cw, dtype=np.int32)
        flag = np.ascontiguousarray(flag, dtype=np.int8)
        h = np.zeros(self.C)
        s = self.s
        self.L.orc_addremove_widths(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _ip(w), _ip(cw), int(n_ratio),
                                    flag.ctypes.data_as(C.POINTER(C.c_int8)), _dp(h))
        return h

    def step(self, n=1):
        s = self.s
        for _ in range(n):
            self.L.orc_step(self.h, _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o), _dp(s.U1), _dp(s.U2), _dp(s.U3),
                            _ip(s.index))

    def face_potential(self, mode):
        V = np.empty(self.cfg.n_cells[1] + 1)
        if mode == 1:
            self.L.orc_vlasov_face_potential(self.h, _dp(V))
        else:
            self.L.orc_poisson_faces(self.h, _dp(V))
        return V


# ------------------------------------------------------------- reference
def ref_lib_path():
    return os.path.join(HERE, "_ref", "libref.so")


_RL = None


def ref_lib(build=True):
    """libref.so, building it when the reference sources are present; None
    when they are not."""
    global _RL
    if _RL is not None:
        return _RL
    path = ref_lib_path()
    if build:
        sys.path.insert(0, HERE)
        try:
            from build import build_ref
            p = build_ref()
        finally:
            sys.path.remove(HERE)
        if p:
            path = p
    if not os.path.exists(path):
        return None
    L = C.CDLL(path)
    vp = C.c_void_p
    sig = {
        "ref_create": (vp, [C.POINTER(Config), C.c_long]),
        "ref_read_settings": (None, [C.c_char_p, C.POINTER(C.c_long), C.POINTER(C.c_double)]),
        "ref_initialize": (None, [C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_double),
                                  C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_long]),
        "ref_destroy": (None, [vp]),
        "ref_set_step": (None, [vp, C.c_int]),
        "ref_inject_normals": (None, [dp, dp, dp, C.c_long]),
        "ref_cell_update": (None, [vp, dp, dp, dp, dp, dp, ip]),
        "ref_random_generator": (None, [vp, ip, dp, dp, dp]),
        "ref_velocity_fp": (None, [vp, dp, dp, dp, ip, dp, dp, dp]),
        "ref_long_range": (None, [vp, dp, dp, dp, ip]),
        "ref_dfp_extra_streaming": (None, [vp, dp, dp, dp, dp, dp, ip]),
        "ref_apply_bc": (None, [vp, dp, dp, dp, dp, dp, dp, dp, ip]),
        "ref_store_old_positions": (None, [vp, dp, dp, dp, dp]),
        "ref_stream": (None, [vp, dp, dp, dp, dp, dp, dp, dp, ip]),
        "ref_esmc": (None, [vp, dp, dp, dp, dp, dp, ip]),
        "ref_dsmc_vhs": (None, [vp, dp, dp, dp, dp, dp]),
        "ref_sample_cells": (None, [vp, dp, dp, dp, ip, dp]),
        "ref_init_omega_max": (None, [vp]),
        "ref_get_cells": (None, [vp, dp]),
        "ref_long_range_2d": (None, [vp, dp, dp, dp, dp, ip]),
        "ref_get_node_density": (None, [vp, dp]),
        "ref_measure_pressure": (None, [vp, dp, dp, dp, dp]),
        "ref_set_cell_weights": (None, [vp, ip]),
        "ref_write_post": (None, [vp, C.c_int, C.c_double, C.c_char_p, C.c_char_p, dp, dp, dp, dp, dp, dp, ip]),
        "ref_post_text": (C.c_long, [vp, C.c_int, dp, dp, dp, dp, dp, dp, ip, C.c_char_p, C.c_long]),
        "ref_thermostat": (None, [vp, dp, dp, dp, dp, ip, C.c_double, C.c_double, C.c_double, C.c_double]),
        "ref_addremove": (C.c_long, [vp, dp, dp, dp, dp, dp, dp, dp, ip, ip, ip, C.c_int, C.c_long,
                                     dp, dp, dp, dp, dp, dp, dp, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _RL = L
    return L


class Reference:
    """The reference's own routines on caller arrays (oracle/_ref)."""

    def __init__(self, cfg: Config, parts):
        self.L = ref_lib()
        if self.L is None:
            raise RuntimeError("reference build not available")
        self.cfg = cfg.copy()
        self.N = len(parts["x2"])
        self.C = cfg.n_cells[0] * cfg.n_cells[1]
        self.h = self.L.ref_create(C.byref(self.cfg), self.N)
        self.s = State(parts, self.N)
        self.xi = [np.zeros(self.N), np.zeros(self.N), np.zeros(self.N)]

    def __del__(self):
        try:
            self.L.ref_destroy(self.h)
        except Exception:
            pass

    def set_step(self, k):
        self.L.ref_set_step(self.h, k)

    def inject_normals(self, a, b, c):
        self._inj = [np.ascontiguousarray(v, dtype=np.float64) for v in (a, b, c)]
        self.L.ref_inject_normals(*[_dp(v) for v in self._inj], self.N)

    def cells(self):
        out = np.empty((self.C, CF_COUNT))
        self.L.ref_get_cells(self.h, _dp(out))
        return out

    def cell_update(self):
        s = self.s
        self.L.ref_cell_update(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U1), _dp(s.U2), _dp(s.U3), _ip(s.index))

    def random_generator(self):
        self.L.ref_random_generator(self.h, _ip(self.s.index), *[_dp(v) for v in self.xi])

    def velocity_fp(self):
        s = self.s
        self.L.ref_velocity_fp(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _ip(s.index), *[_dp(v) for v in self.xi])

    def long_range(self):
        s = self.s
        if self.cfg.direction[0] == 1 and self.cfg.long_range != LR_DENSITY_EXPANSION:
            self.L.ref_long_range_2d(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U1), _dp(s.U2), _ip(s.index))
        else:
            self.L.ref_long_range(self.h, _dp(s.x1), _dp(s.x2), _dp(s.U2), _ip(s.index))

    def node_density(self):
        out = np.empty((self.C, 4))
        self.L.ref_get_node_density(self.h, _dp(out))
        return out

    def dfp_extra_streaming(self):
        s = self.s
        self.L.ref_dfp_extra_streaming(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2), _ip(s.index))

    def apply_bc(self):
        s = self.s
        self.L.ref_apply_bc(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o),
                            _ip(s.index))

    def store_old_positions(self):
        s = self.s
        self.L.ref_store_old_positions(self.h, _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o))

    def stream(self):
        s = self.s
        self.L.ref_stream(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o),
                          _ip(s.index))

    def esmc(self):
        s = self.s
        self.L.ref_esmc(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2), _ip(s.index))

    def set_cell_weights(self, cw):
        self._cw = np.ascontiguousarray(cw, dtype=np.int32)
        self.L.ref_set_cell_weights(self.h, _ip(self._cw))

    def measure_pressure(self):
        """the reference's measure_pressure; returns its cells' p_m (cumulative)"""
        s = self.s
        out = np.empty(self.C)
        self.L.ref_measure_pressure(self.h, _dp(s.U2), _dp(s.x2), _dp(s.x2o), _dp(out))
        return out

    def write_post(self, step, t_post, directory, name):
        """the reference's write_post_processing into directory/PostProc"""
        s = self.s
        self.L.ref_write_post(self.h, int(step), float(t_post), os.fsencode(directory), name.encode(), _dp(s.U1),
                              _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2), _dp(s.x2o), _ip(s.index))

    def post_text(self, step):
        """the console lines of the reference's post_processing"""
        s = self.s
        buf = C.create_string_buffer(1 << 16)
        n = self.L.ref_post_text(self.h, int(step), _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2),
                                 _dp(s.x2o), _ip(s.index), buf, 1 << 16)
        return buf.value.decode() if n >= 0 else None

    def thermostat(self, Tc, Th, thermc, thermh):
        s = self.s
        self.L.ref_thermostat(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x2), _ip(s.index), Tc, Th, thermc, thermh)

    def addremove(self, w, cw, n_ratio, cap):
        """the reference's inverted_addremove_particles; returns (parts,
        weights) of its new state (the reference object keeps its own)"""
        s = self.s
        w = np.ascontiguousarray(w, dtype=np.int32)
        cw = np.ascontiguousarray(cw, dtype=np.int32)
        out = {k: np.zeros(cap) for k in ("x1", "x2", "x1o", "x2o", "U1", "U2", "U3")}
        wo = np.zeros(cap, dtype=np.int32)
        m = self.L.ref_addremove(self.h, _dp(s.x1), _dp(s.x2), _dp(s.x1o), _dp(s.x2o), _dp(s.U1), _dp(s.U2),
                                 _dp(s.U3), _ip(s.index), _ip(w), _ip(cw), int(n_ratio), int(cap),
                                 *[_dp(out[k]) for k in ("x1", "x2", "x1o", "x2o", "U1", "U2", "U3")], _ip(wo))
        if m < 0:
            raise RuntimeError("reference addremove: more than %d particles" % cap)
        return {k: v[:m] for k, v in out.items()}, wo[:m]

    def sample_cells(self, acc):
        """the reference's cell_poly_velocity; acc receives its running sums"""
        s = self.s
        self.L.ref_sample_cells(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _ip(s.index), _dp(acc))

    def dsmc(self):
        s = self.s
        self.L.ref_dsmc_vhs(self.h, _dp(s.U1), _dp(s.U2), _dp(s.U3), _dp(s.x1), _dp(s.x2))

    def init_omega_max(self):
        self.L.ref_init_omega_max(self.h)


def ref_read_settings(path):
    """The reference's readSettingsFile on path: (ints, doubles) in the order
    of ref_read_settings in ref_harness.cpp; None without the reference."""
    L = ref_lib()
    if L is None:
        return None
    iv = np.zeros(10, dtype=np.int64)
    dv = np.zeros(28)
    L.ref_read_settings(os.fsencode(path), iv.ctypes.data_as(C.POINTER(C.c_long)),
                        dv.ctypes.data_as(C.POINTER(C.c_double)))
    return iv, dv[:26]


def ref_initialize(path, N):
    """The reference's initialization after readSettingsFile: dict of its N
    initial particles; None without the reference."""
    L = ref_lib()
    if L is None:
        return None
    out = {k: np.zeros(N) for k in ("x1", "x2", "U1", "U2", "U3")}
    dp = C.POINTER(C.c_double)
    L.ref_initialize(os.fsencode(path), *[out[k].ctypes.data_as(dp) for k in ("x1", "x2", "U1", "U2", "U3")], N)
    return out


def ref_src_dir():
    """The reference's source directory when present (the sources oracle/build.py
    compiles), else None."""
    sys.path.insert(0, HERE)
    try:
        from build import default_ref_src
    finally:
        sys.path.remove(HERE)
    d = default_ref_src()
    return d if os.path.isdir(d) else None
