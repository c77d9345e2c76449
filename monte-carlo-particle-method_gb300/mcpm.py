"""Python mirror of the reference's particle-loop routine surface over the
C-ABI in include/mcpm.h (libmcpm.so, built in-tree by build.py).

The reference drives its particle step from src/main.cpp:389-669 with free
functions on caller-owned ``double*`` arrays; :class:`Session` keeps the same
routine names and call order (``cell_update``, ``random_generator``,
``velocity_update``, ``DFP_extra_streaming``, ``apply_BC``,
``store_old_positions``, ``stream_particles``) over a device-resident state.
There is no CPU fallback: constructing a Session without the compiled library
raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcpm.so")

# ---- enums (include/mcpm.h) -------------------------------------------------
OK = 0
ERR_ARG, ERR_CUDA, ERR_OUT_OF_BOX, ERR_NAN, ERR_CAPACITY, ERR_BC_LOOP, ERR_ITER_LIMIT, ERR_STATE = (
    1, 2, 4, 8, 16, 32, 64, 128)
PROBLEM_CLOSED_BOX, PROBLEM_COUETTE, PROBLEM_WALL, PROBLEM_PERIODIC = 1, 2, 11, 100
MODEL_NONE, MODEL_FP_DENSE, MODEL_FP_IDEAL_GAS, MODEL_ESMC, MODEL_FP_LINEAR, MODEL_DSMC_VHS = 0, 1, 2, 3, 4, 5
LR_NONE, LR_DIRECT, LR_DENSITY_EXPANSION, LR_SCREENED_POISSON = 0, 1, 2, 3
FP64, FP32 = 0, 1
RNG_PHILOX, RNG_INJECTED = 0, 1
# enum mcpm_rng_stream
RS = dict(FP=0, BC=1, ESMC=2, BIN=3, ESMC_ACC=4, ESMC_M=5, DSMC=6, DSMC_ACC=7, DSMC_M=8, ADDREM_DEL=9,
          ADDREM_NEW=10)

CF = dict(NUM_INSIDE=0, U_SPACE=1, PIJ=4, M3=10, M4=20, M5=26, Q=29, DM2=32, DM4=33, MP=34, T=37, N=38,
          GAMMA_ST=39, LAMBDA=40, C=41, GAMMA=47, ALPHA=50, BETA=59, PHI=62, F2=65, OMEGA_MAX=66, DIVU=67,
          N_SMOOTH=68, DN2=69, DN3=70)
CF_COUNT = 71
# enum mcpm_sample_field: cell_poly_velocity's accumulators
SF = dict(WEIGHT=0, M=1, MM=4, MMM=10, MMMM=20)
SF_COUNT = 26
K_NAMES = ["bin", "scan", "scatter", "moments", "solve", "esmc", "long_range", "update", "surrogate"]
K_COUNT = len(K_NAMES)
# (field, width) of every exported per-cell quantity
CF_WIDTH = dict(NUM_INSIDE=1, U_SPACE=3, PIJ=6, M3=10, M4=6, M5=3, Q=3, DM2=1, DM4=1, MP=3, T=1, N=1,
                GAMMA_ST=1, LAMBDA=1, C=6, GAMMA=3, ALPHA=9, BETA=3, PHI=3, F2=1, OMEGA_MAX=1, DIVU=1,
                N_SMOOTH=1, DN2=1, DN3=1)


class Config(C.Structure):
    """mcpm_config: the subset of GAS/BOX (src/cpp_headers.h:145-269) the step reads."""
    _fields_ = [
        ("n_cells", C.c_int32 * 3), ("direction", C.c_int32 * 3), ("length", C.c_double * 3),
        ("problem", C.c_int32), ("model", C.c_int32), ("long_range", C.c_int32), ("precision", C.c_int32),
        ("sigma", C.c_double), ("m", C.c_double), ("kb", C.c_double), ("n", C.c_double), ("Fn", C.c_double),
        ("T0", C.c_double), ("mu", C.c_double), ("visp", C.c_double), ("b", C.c_double), ("dt", C.c_double),
        ("phi", C.c_double), ("eqdist", C.c_double), ("ast", C.c_double), ("bst", C.c_double),
        ("T_wall", C.c_double * 4), ("U_wall", C.c_double * 4), ("seed", C.c_uint64),
        ("max_particles", C.c_int64), ("crref", C.c_double),
    ]

    def copy(self):
        c = Config()
        C.pointer(c)[0] = self
        return c

    def as_dict(self):
        out = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            out[name] = list(v) if hasattr(v, "__len__") else v
        return out


def config_from_settings(path: str):
    """readSettingsFile (src/myIO.cpp:1756-3016) through the library: the
    reference's settings file as (Config, N) for problems 1, 2 and 11."""
    L = load_library()
    cfg, n = Config(), C.c_int64(0)
    msg = C.create_string_buffer(512)
    rc = L.mcpm_config_from_settings(os.fsencode(path), C.byref(cfg), C.byref(n), msg, 512)
    if rc:
        raise MCPMError(rc, msg.value.decode())
    return cfg, n.value


def initialize_from_settings(path: str, seed: int, n_particles: int):
    """initialization (src/Main_Functions.cpp:4222-4814) for a settings file's
    closed-box or Couette run: dict of the N initial particles."""
    L = load_library()
    out = {k: np.zeros(n_particles) for k in ("x1", "x2", "U1", "U2", "U3")}
    msg = C.create_string_buffer(512)
    rc = L.mcpm_initialize_from_settings(os.fsencode(path), seed, *[_dp(out[k]) for k in ("x1", "x2", "U1", "U2", "U3")],
                                         n_particles, msg, 512)
    if rc:
        raise MCPMError(rc, msg.value.decode())
    return out


def derive(cfg: Config, n_particles: int) -> Config:
    """Derived GAS fields as readSettingsFile fills them (src/myIO.cpp:2217-2233,
    :2828-2830); identical to mcpm_config_derive in the library."""
    cfg.b = 2 * math.pi * cfg.sigma ** 3 / 3.0
    if not cfg.T0 > 0:
        cfg.T0 = 273.0
    if not cfg.visp > 0:
        cfg.visp = 0.5
    if not cfg.mu > 0:
        cfg.mu = 5.0 / (16.0 * cfg.sigma * cfg.sigma) * math.sqrt(cfg.m * cfg.kb * cfg.T0 / math.acos(-1.0))
    vol = cfg.length[0] * cfg.length[1] * cfg.length[2]
    if n_particles > 0:
        cfg.Fn = cfg.n * vol / n_particles
    if not cfg.eqdist > 0:
        cfg.eqdist = cfg.sigma
    if cfg.seed == 0:
        cfg.seed = 0x4D43504D
    if cfg.max_particles < n_particles:
        cfg.max_particles = n_particles
    return cfg


class SurrogateStats(C.Structure):
    """mcpm_surrogate_stats: what the judge of the learned force saw."""
    _fields_ = [("last_error", C.c_double), ("judged", C.c_int64), ("takeovers", C.c_int64),
                ("surrogate_steps", C.c_int64), ("plain_steps", C.c_int64), ("active", C.c_int32)]


SUR_IN, SUR_OUT, SUR_NPARAM = 16, 4, 92368


class MCPMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("mcpm error %d: %s" % (code, msg))
        self.code = code


_lib = None


def load_library(path: str | None = None):
    """Loads libmcpm.so; raises if it is missing (there is no fallback path)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise MCPMError(ERR_STATE, "libmcpm.so is not built (%s); run __graft_entry__.build()" % p)
    L = C.CDLL(p)
    vp, i64, i32, dp, ip = C.c_void_p, C.c_int64, C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_int32)
    sig = {
        "mcpm_config_derive": (C.c_int, [C.POINTER(Config), i64]),
        "mcpm_config_from_settings": (C.c_int, [C.c_char_p, C.POINTER(Config), C.POINTER(i64), C.c_char_p, i32]),
        "mcpm_initialize_from_settings": (C.c_int, [C.c_char_p, C.c_uint64, dp, dp, dp, dp, dp, i64, C.c_char_p, i32]),
        "mcpm_session_create": (C.c_int, [C.POINTER(Config), C.POINTER(vp)]),
        "mcpm_session_destroy": (C.c_int, [vp]),
        "mcpm_last_error": (C.c_char_p, [vp]),
        "mcpm_sync": (C.c_int, [vp]),
        "mcpm_check_status": (C.c_int, [vp]),
        "mcpm_upload_particles": (C.c_int, [vp, i64, dp, dp, dp, dp, dp]),
        "mcpm_download_particles": (C.c_int, [vp, i64, dp, dp, dp, dp, dp]),
        "mcpm_download_particles_async": (C.c_int, [vp, i64, dp, dp, dp, dp, dp]),
        "mcpm_upload_particles_async": (C.c_int, [vp, i64, dp, dp, dp, dp, dp]),
        "mcpm_set_old_positions": (C.c_int, [vp, dp, dp]),
        "mcpm_get_old_positions": (C.c_int, [vp, dp, dp]),
        "mcpm_cell_update": (C.c_int, [vp]),
        "mcpm_random_generator": (C.c_int, [vp]),
        "mcpm_velocity_update": (C.c_int, [vp]),
        "mcpm_dfp_extra_streaming": (C.c_int, [vp]),
        "mcpm_apply_bc": (C.c_int, [vp]),
        "mcpm_store_old_positions": (C.c_int, [vp]),
        "mcpm_stream_particles": (C.c_int, [vp]),
        "mcpm_end_step": (C.c_int, [vp]),
        "mcpm_step": (C.c_int, [vp, i32]),
        "mcpm_step_async": (C.c_int, [vp, i32]),
        "mcpm_inject_normals": (C.c_int, [vp, i64, dp, dp, dp]),
        "mcpm_set_rng": (C.c_int, [vp, i32]),
        "mcpm_inject_uniforms": (C.c_int, [vp, i32, i64, dp]),
        "mcpm_get_cells": (C.c_int, [vp, dp]),
        "mcpm_sample_cells": (C.c_int, [vp]),
        "mcpm_get_samples": (C.c_int, [vp, dp]),
        "mcpm_reset_samples": (C.c_int, [vp]),
        "mcpm_get_index": (C.c_int, [vp, ip]),
        "mcpm_post_processing_write": (C.c_int, [C.POINTER(Config), i32, C.c_double, C.c_char_p, C.c_char_p, dp, dp,
                                                 dp, ip, C.c_char_p, i32]),
        "mcpm_write_post_processing": (C.c_int, [vp, i32, C.c_double, C.c_char_p, C.c_char_p, C.c_char_p, i32]),
        "mcpm_post_processing_text": (C.c_int, [C.POINTER(Config), dp, C.c_char_p, i32]),
        "mcpm_set_pressure_sampling": (C.c_int, [vp, i32]),
        "mcpm_measure_pressure": (C.c_int, [vp]),
        "mcpm_get_pressure": (C.c_int, [vp, dp]),
        "mcpm_reset_pressure": (C.c_int, [vp]),
        "mcpm_set_particle_weights": (C.c_int, [vp, ip]),
        "mcpm_get_particle_weights": (C.c_int, [vp, ip]),
        "mcpm_set_cell_weights": (C.c_int, [vp, ip]),
        "mcpm_thermostat": (C.c_int, [vp, C.c_double, C.c_double, C.c_double, C.c_double]),
        "mcpm_addremove_particles": (C.c_int, [vp, i32, C.POINTER(i64)]),
        "mcpm_get_normals": (C.c_int, [vp, dp, dp, dp]),
        "mcpm_get_node_density": (C.c_int, [vp, dp]),
        "mcpm_get_node_potential": (C.c_int, [vp, dp]),
        "mcpm_get_layout": (C.c_int, [vp, ip, ip]),
        "mcpm_get_step": (i32, [vp]),
        "mcpm_set_step": (C.c_int, [vp, i32]),
        "mcpm_set_cell_field": (C.c_int, [vp, i32, dp]),
        "mcpm_init_omega_max": (C.c_int, [vp]),
        "mcpm_kernel_launches": (i64, [vp]),
        "mcpm_set_stream": (C.c_int, [vp, vp]),
        "mcpm_profile": (C.c_int, [vp, i32]),
        "mcpm_profile_read": (C.c_int, [vp, dp, C.POINTER(C.c_int64), i32]),
        "mcpm_poisson_force_1d_noalloc": (C.c_int, [vp, i32, C.POINTER(Config), vp, vp]),
        "mcpm_set_wcap": (C.c_int, [vp, i32]),
        "mcpm_get_wcap": (i32, [vp]),
        "mcpm_autotune": (C.c_int, [vp, i32, C.POINTER(i32)]),
        "mcpm_surrogate_create": (C.c_int, [i32, i32, i32, C.POINTER(vp)]),
        "mcpm_surrogate_destroy": (C.c_int, [vp]),
        "mcpm_surrogate_last_error": (C.c_char_p, [vp]),
        "mcpm_surrogate_set_params": (C.c_int, [vp, C.POINTER(C.c_float), i64, C.c_double]),
        "mcpm_surrogate_get_params": (C.c_int, [vp, C.POINTER(C.c_float), i64]),
        "mcpm_surrogate_set_tensor_path": (C.c_int, [vp, i32]),
        "mcpm_surrogate_launches": (C.c_int, [vp, C.POINTER(C.c_int64), C.POINTER(i32)]),
        "mcpm_surrogate_forward": (C.c_int, [vp, vp, i32, vp]),
        "mcpm_surrogate_gradients": (C.c_int, [vp, vp, vp, i32, C.c_double, C.POINTER(C.c_float), dp]),
        "mcpm_surrogate_train_step": (C.c_int, [vp, vp, vp, i32, C.c_double, C.c_double, i32, dp]),
        "mcpm_surrogate_sync": (C.c_int, [vp]),
        "mcpm_vlasov_snapshots": (C.c_int, [vp, i32, dp, i32, C.c_uint64, vp, vp]),
        "mcpm_attach_surrogate": (C.c_int, [vp, vp, i32, C.c_double]),
        "mcpm_get_surrogate_stats": (C.c_int, [vp, C.POINTER(SurrogateStats)]),
        "mcpm_eval_vlasov_2d": (C.c_int, [vp, i32]),
        "mcpm_get_kick_2d": (C.c_int, [vp, C.POINTER(C.c_float)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    if path is None:
        _lib = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _f64(a, n):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (n,):
        raise ValueError("expected %d values" % n)
    return a


class Session:
    """One device-resident particle system; methods follow the reference's
    routines (file:line in include/mcpm.h)."""

    def __init__(self, cfg: Config):
        self.lib = load_library()
        self.cfg = cfg.copy()
        self.C = cfg.n_cells[0] * cfg.n_cells[1] * cfg.n_cells[2]
        h = C.c_void_p()
        rc = self.lib.mcpm_session_create(C.byref(self.cfg), C.byref(h))
        if rc != OK:
            raise MCPMError(rc, "session_create failed (configuration rejected or no device)")
        self.h = h
        self.N = 0

    # -- plumbing
    def _ck(self, rc, what):
        if rc != OK:
            msg = self.lib.mcpm_last_error(self.h)
            raise MCPMError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if getattr(self, "h", None):
            self.lib.mcpm_session_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- particles
    def upload(self, x1, x2, U1, U2, U3, wait=True):
        """Copy the caller's arrays to the device; with wait=False the copies
        are queued (mcpm_upload_particles_async) and the arrays must stay
        unchanged until sync() returns."""
        n = len(x2)
        self._keep = [_f64(x1, n) if x1 is not None else None, _f64(x2, n), _f64(U1, n), _f64(U2, n), _f64(U3, n)]
        k = self._keep
        fn = self.lib.mcpm_upload_particles if wait else self.lib.mcpm_upload_particles_async
        self._ck(fn(self.h, n, _dp(k[0]) if k[0] is not None else None, _dp(k[1]), _dp(k[2]), _dp(k[3]), _dp(k[4])),
                 "upload_particles")
        self.N = n

    def download(self):
        n = self.N
        out = {k: np.empty(n) for k in ("x1", "x2", "U1", "U2", "U3")}
        if self._keep[0] is not None:
            out["x1"][:] = self._keep[0]  # kept when the device does not track x1
        else:
            out["x1"][:] = 0.0
        self._ck(self.lib.mcpm_download_particles(self.h, n, _dp(out["x1"]), _dp(out["x2"]), _dp(out["U1"]),
                                                  _dp(out["U2"]), _dp(out["U3"])), "download_particles")
        return out

    def set_old_positions(self, x1_old, x2_old):
        """The reference's x1_old / x2_old into the session (the walls and the
        pressure count read them)."""
        n = self.N
        self._old = [_f64(x1_old, n) if x1_old is not None else None, _f64(x2_old, n)]
        a, b = self._old
        self._ck(self.lib.mcpm_set_old_positions(self.h, _dp(a) if a is not None else None, _dp(b)),
                 "set_old_positions")

    def get_old_positions(self):
        n = self.N
        out = {"x1_old": np.zeros(n), "x2_old": np.empty(n)}
        self._ck(self.lib.mcpm_get_old_positions(self.h, _dp(out["x1_old"]), _dp(out["x2_old"])),
                 "get_old_positions")
        return out

    # -- the reference routines
    def cell_update(self):
        self._ck(self.lib.mcpm_cell_update(self.h), "cell_update")

    def random_generator(self):
        self._ck(self.lib.mcpm_random_generator(self.h), "random_generator")

    def velocity_update(self):
        self._ck(self.lib.mcpm_velocity_update(self.h), "velocity_update")

    def DFP_extra_streaming(self):
        self._ck(self.lib.mcpm_dfp_extra_streaming(self.h), "DFP_extra_streaming")

    def apply_BC(self):
        self._ck(self.lib.mcpm_apply_bc(self.h), "apply_BC")

    def store_old_positions(self):
        self._ck(self.lib.mcpm_store_old_positions(self.h), "store_old_positions")

    def stream_particles(self):
        self._ck(self.lib.mcpm_stream_particles(self.h), "stream_particles")

    def end_step(self):
        self._ck(self.lib.mcpm_end_step(self.h), "end_step")

    def loop_body(self):
        """One iteration of src/main.cpp:389-669 through the individual routines."""
        self.cell_update()
        self.random_generator()
        self.velocity_update()
        self.DFP_extra_streaming()
        self.apply_BC()
        self.store_old_positions()
        self.stream_particles()
        self.apply_BC()
        self.apply_BC()
        self.end_step()
        self.check_status()

    def step(self, n=1, wait=True):
        """n fused steps; with wait=False they are only queued, and the
        device status is read by check_status (or the next waiting step)."""
        fn = self.lib.mcpm_step if wait else self.lib.mcpm_step_async
        self._ck(fn(self.h, int(n)), "step")

    # -- hooks
    def check_status(self):
        st = self.lib.mcpm_check_status(self.h)
        if st != OK:
            self._ck(st, "device status")

    def sync(self):
        self._ck(self.lib.mcpm_sync(self.h), "sync")

    def inject_normals(self, xi1, xi2, xi3):
        n = self.N
        self._inj = [_f64(xi1, n), _f64(xi2, n), _f64(xi3, n)]
        self._ck(self.lib.mcpm_inject_normals(self.h, n, *[_dp(a) for a in self._inj]), "inject_normals")

    def inject_uniforms(self, stream, u):
        """u: [rows][4] uniforms in place of the stream's draws (name or
        number of enum mcpm_rng_stream); None restores Philox."""
        st = RS[stream] if isinstance(stream, str) else int(stream)
        if u is None:
            self._ck(self.lib.mcpm_inject_uniforms(self.h, st, 0, None), "inject_uniforms")
            return
        u = np.ascontiguousarray(u, dtype=np.float64).reshape(-1, 4)
        self._ck(self.lib.mcpm_inject_uniforms(self.h, st, len(u), _dp(u)), "inject_uniforms")

    def set_rng(self, mode):
        self._ck(self.lib.mcpm_set_rng(self.h, int(mode)), "set_rng")

    def get_cells(self):
        out = np.empty((CF_COUNT, self.C))
        self._ck(self.lib.mcpm_get_cells(self.h, _dp(out)), "get_cells")
        return out

    def sample_cells(self):
        """cell_poly_velocity (src/Main_Functions.cpp:1918-1968) into the session's accumulators."""
        self._ck(self.lib.mcpm_sample_cells(self.h), "sample_cells")

    def get_samples(self):
        out = np.empty((SF_COUNT, self.C))
        self._ck(self.lib.mcpm_get_samples(self.h, _dp(out)), "get_samples")
        return out

    def reset_samples(self):
        self._ck(self.lib.mcpm_reset_samples(self.h), "reset_samples")

    def get_index(self):
        out = np.empty(self.N, dtype=np.int32)
        self._ck(self.lib.mcpm_get_index(self.h, _ip(out)), "get_index")
        return out

    # -- post-processing output (src/myIO.cpp:597-965)
    def write_post_processing(self, step, t_post, directory, output_name):
        """The reference's .dat file of the current cell fields; returns its path."""
        buf = C.create_string_buffer(4096)
        self._ck(self.lib.mcpm_write_post_processing(self.h, int(step), float(t_post), os.fsencode(directory),
                                                     output_name.encode(), buf, 4096), "write_post_processing")
        return buf.value.decode()

    # -- pressure sampling (measure_pressure, src/Main_Functions.cpp:13-34)
    def set_pressure_sampling(self, on=True):
        self._ck(self.lib.mcpm_set_pressure_sampling(self.h, 1 if on else 0), "set_pressure_sampling")

    def measure_pressure(self):
        self._ck(self.lib.mcpm_measure_pressure(self.h), "measure_pressure")

    def get_pressure(self):
        out = np.empty(self.C)
        self._ck(self.lib.mcpm_get_pressure(self.h, _dp(out)), "get_pressure")
        return out

    def reset_pressure(self):
        self._ck(self.lib.mcpm_reset_pressure(self.h), "reset_pressure")

    # -- interface problems (the reference's problem inverted)
    def set_particle_weights(self, w):
        """n_ratio[] of the reference, particle-id order."""
        w = np.ascontiguousarray(w, dtype=np.int32)
        self._ck(self.lib.mcpm_set_particle_weights(self.h, _ip(w)), "set_particle_weights")

    def get_particle_weights(self):
        out = np.empty(self.N, dtype=np.int32)
        self._ck(self.lib.mcpm_get_particle_weights(self.h, _ip(out)), "get_particle_weights")
        return out

    def set_cell_weights(self, w):
        """cells[].n_ratio of the reference, cell order."""
        w = np.ascontiguousarray(w, dtype=np.int32)
        self._ck(self.lib.mcpm_set_cell_weights(self.h, _ip(w)), "set_cell_weights")

    def thermostat(self, Tc, Th, thermc, thermh):
        """thermostat (src/Main_Functions.cpp:1674-1869)."""
        self._ck(self.lib.mcpm_thermostat(self.h, Tc, Th, thermc, thermh), "thermostat")

    def addremove_particles(self, n_ratio):
        """inverted_addremove_particles (src/Main_Functions.cpp:1206-1450);
        returns the new particle count."""
        n = C.c_int64(0)
        self._ck(self.lib.mcpm_addremove_particles(self.h, int(n_ratio), C.byref(n)), "addremove_particles")
        if n.value != self.N:
            self.N = n.value
            # x1 of the caller no longer lines up with the new ids
            if self._keep and self._keep[0] is not None and not self.cfg.direction[0]:
                self._keep[0] = np.zeros(self.N)
        return self.N

    def get_normals(self):
        a, b, c = np.empty(self.N), np.empty(self.N), np.empty(self.N)
        self._ck(self.lib.mcpm_get_normals(self.h, _dp(a), _dp(b), _dp(c)), "get_normals")
        return a, b, c

    def get_node_density(self):
        """n_n of the last cell_update, [C][4] (2-D screened-Poisson sessions)."""
        out = np.empty((self.C, 4))
        self._ck(self.lib.mcpm_get_node_density(self.h, _dp(out)), "get_node_density")
        return out

    def get_node_potential(self):
        """Node potential of the last 2-D Vlasov force, (N0+1)(N1+1) values."""
        n = (self.cfg.n_cells[0] + 1) * (self.cfg.n_cells[1] + 1)
        out = np.empty(n)
        self._ck(self.lib.mcpm_get_node_potential(self.h, _dp(out)), "get_node_potential")
        return out

    def get_layout(self):
        pid = np.empty(self.N, dtype=np.int32)
        off = np.empty(self.C + 1, dtype=np.int32)
        self._ck(self.lib.mcpm_get_layout(self.h, _ip(pid), _ip(off)), "get_layout")
        return pid, off

    @property
    def step_count(self):
        return int(self.lib.mcpm_get_step(self.h))

    def set_step(self, step):
        self._ck(self.lib.mcpm_set_step(self.h, int(step)), "set_step")

    def set_cell_field(self, field, values):
        v = _f64(values, self.C)
        self._ck(self.lib.mcpm_set_cell_field(self.h, CF[field], _dp(v)), "set_cell_field")

    def init_omega_max(self):
        self._ck(self.lib.mcpm_init_omega_max(self.h), "init_omega_max")

    def set_stream(self, stream_handle):
        """Launch on an external cudaStream_t (e.g. torch's current stream)."""
        self._ck(self.lib.mcpm_set_stream(self.h, C.c_void_p(stream_handle or None)), "set_stream")

    def autotune(self, steps=3):
        """Pick the warp/block split by timing steps on this state (state restored)."""
        ch = C.c_int32()
        self._ck(self.lib.mcpm_autotune(self.h, int(steps), C.byref(ch)), "autotune")
        return ch.value

    def set_wcap(self, wcap):
        self._ck(self.lib.mcpm_set_wcap(self.h, int(wcap)), "set_wcap")

    @property
    def wcap(self):
        return int(self.lib.mcpm_get_wcap(self.h))

    def profile(self, enable=True):
        self._ck(self.lib.mcpm_profile(self.h, 1 if enable else 0), "profile")

    def profile_read(self):
        ms = np.zeros(K_COUNT)
        n = np.zeros(K_COUNT, dtype=np.int64)
        self._ck(self.lib.mcpm_profile_read(self.h, _dp(ms), n.ctypes.data_as(C.POINTER(C.c_int64)), K_COUNT),
                 "profile_read")
        return {name: (float(ms[i]), int(n[i])) for i, name in enumerate(K_NAMES)}

    def download_into(self, out, wait=True):
        """Download into caller arrays (e.g. pinned host buffers); with
        wait=False the copies are queued and the arrays are written once
        sync() returns (mcpm_download_particles_async)."""
        fn = self.lib.mcpm_download_particles if wait else self.lib.mcpm_download_particles_async
        self._ck(fn(self.h, self.N, _dp(out["x1"]), _dp(out["x2"]), _dp(out["U1"]), _dp(out["U2"]), _dp(out["U3"])),
                 "download_particles")

    @property
    def kernel_launches(self):
        return int(self.lib.mcpm_kernel_launches(self.h))

    # -- learned 2-D Vlasov force (no counterpart in the reference)
    def vlasov_snapshots(self, fields, n_waves, seed, x_ptr, y_ptr):
        """Training snapshots of the plain force into device buffers x
        ([n][C][16] bf16) and y ([n][C][4] fp32); fields [n][1 + 4 n_waves]."""
        f = np.ascontiguousarray(fields, dtype=np.float64)
        n = f.shape[0]
        if f.shape[1] != 1 + 4 * n_waves:
            raise ValueError("fields must be [n][1 + 4 n_waves]")
        self._ck(self.lib.mcpm_vlasov_snapshots(self.h, n, _dp(f), int(n_waves), C.c_uint64(seed), C.c_void_p(x_ptr),
                                                C.c_void_p(y_ptr)), "vlasov_snapshots")

    def attach_surrogate(self, sur, judge_every=10, threshold=0.01):
        self._ck(self.lib.mcpm_attach_surrogate(self.h, sur.h if sur is not None else None, int(judge_every),
                                                float(threshold)), "attach_surrogate")
        self._sur = sur

    def surrogate_stats(self):
        st = SurrogateStats()
        self._ck(self.lib.mcpm_get_surrogate_stats(self.h, C.byref(st)), "surrogate_stats")
        return {k: getattr(st, k) for k, _ in SurrogateStats._fields_}

    def eval_vlasov_2d(self, method):
        """Re-evaluate the kick of the current cell state: 0 plain path, 1 network."""
        self._ck(self.lib.mcpm_eval_vlasov_2d(self.h, int(method)), "eval_vlasov_2d")

    def get_kick_2d(self):
        out = np.empty((self.C, 4), dtype=np.float32)
        self._ck(self.lib.mcpm_get_kick_2d(self.h, out.ctypes.data_as(C.POINTER(C.c_float))), "get_kick_2d")
        return out


class Surrogate:
    """mcpm_surrogate: the learned 2-D Vlasov force network (include/mcpm.h).
    Device buffers are passed as raw pointers (e.g. torch tensors' data_ptr())."""

    def __init__(self, n0, n1, max_batch=1):
        self.lib = load_library()
        h = C.c_void_p()
        rc = self.lib.mcpm_surrogate_create(int(n0), int(n1), int(max_batch), C.byref(h))
        if rc != OK:
            raise MCPMError(rc, "surrogate_create failed")
        self.h = h
        self.n0, self.n1, self.max_batch = int(n0), int(n1), int(max_batch)
        self.C = self.n0 * self.n1

    def _ck(self, rc, what):
        if rc != OK:
            msg = self.lib.mcpm_surrogate_last_error(self.h)
            raise MCPMError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    def close(self):
        if getattr(self, "h", None):
            self.lib.mcpm_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params, out_scale):
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.shape != (SUR_NPARAM,):
            raise ValueError("expected %d parameters" % SUR_NPARAM)
        self._ck(self.lib.mcpm_surrogate_set_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), SUR_NPARAM,
                                                    float(out_scale)), "surrogate_set_params")

    def get_params(self):
        p = np.empty(SUR_NPARAM, dtype=np.float32)
        self._ck(self.lib.mcpm_surrogate_get_params(self.h, p.ctypes.data_as(C.POINTER(C.c_float)), SUR_NPARAM),
                 "surrogate_get_params")
        return p

    def set_tensor_path(self, tcgen05):
        self._ck(self.lib.mcpm_surrogate_set_tensor_path(self.h, 1 if tcgen05 else 0), "surrogate_set_tensor_path")

    def tensor_path(self):
        """(tcgen05 launches so far, tcgen05 path on)"""
        n, on = C.c_int64(), C.c_int32()
        self._ck(self.lib.mcpm_surrogate_launches(self.h, C.byref(n), C.byref(on)), "surrogate_launches")
        return int(n.value), bool(on.value)

    def forward(self, x_ptr, batch, y_ptr):
        self._ck(self.lib.mcpm_surrogate_forward(self.h, C.c_void_p(x_ptr), int(batch), C.c_void_p(y_ptr)),
                 "surrogate_forward")

    def gradients(self, x_ptr, t_ptr, batch, target_scale):
        g = np.empty(SUR_NPARAM, dtype=np.float32)
        loss = np.zeros(2)
        self._ck(self.lib.mcpm_surrogate_gradients(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), int(batch),
                                                   float(target_scale), g.ctypes.data_as(C.POINTER(C.c_float)),
                                                   _dp(loss)), "surrogate_gradients")
        return g, loss

    def train_step(self, x_ptr, t_ptr, batch, target_scale, lr, t, want_loss=False):
        loss = np.zeros(2) if want_loss else None
        self._ck(self.lib.mcpm_surrogate_train_step(self.h, C.c_void_p(x_ptr), C.c_void_p(t_ptr), int(batch),
                                                    float(target_scale), float(lr), int(t),
                                                    _dp(loss) if want_loss else None), "surrogate_train_step")
        return loss

    def sync(self):
        self._ck(self.lib.mcpm_surrogate_sync(self.h), "surrogate_sync")


def cell_field(cells, name, cell_major=False):
    """Slice one named field out of a [CF_COUNT][C] (or [C][CF_COUNT]) array."""
    o, w = CF[name], CF_WIDTH[name]
    if cell_major:
        v = cells[:, o:o + w]
        return v[:, 0] if w == 1 else v
    v = cells[o:o + w]
    return v[0] if w == 1 else v.T


def post_processing_write(cfg, step, t_post, directory, output_name, cells, samples=None, p_m=None,
                          cell_weights=None):
    """write_post_processing (src/myIO.cpp:597-934) of host arrays: cells
    [CF_COUNT][C], samples [SF_COUNT][C], p_m [C], cell weights [C]; returns
    the file's path."""
    L = load_library()
    buf = C.create_string_buffer(4096)

    def arr(a, dt):
        return None if a is None else np.ascontiguousarray(a, dtype=dt)
    cells, samples, p_m, cw = arr(cells, np.float64), arr(samples, np.float64), arr(p_m, np.float64), arr(cell_weights, np.int32)
    rc = L.mcpm_post_processing_write(C.byref(cfg), int(step), float(t_post), os.fsencode(directory),
                                      output_name.encode(), _dp(cells), None if samples is None else _dp(samples),
                                      None if p_m is None else _dp(p_m), None if cw is None else _ip(cw), buf, 4096)
    if rc:
        raise MCPMError(rc, "post_processing_write failed")
    return buf.value.decode()


def post_processing_text(cfg, cells):
    """The console summary of post_processing (src/myIO.cpp:945-965)."""
    L = load_library()
    buf = C.create_string_buffer(1 << 14)
    cells = np.ascontiguousarray(cells, dtype=np.float64)
    n = L.mcpm_post_processing_text(C.byref(cfg), _dp(cells), buf, 1 << 14)
    if n < 0:
        raise MCPMError(-n, "post_processing_text failed")
    return buf.value.decode()
