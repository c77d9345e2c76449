/*
 * mcpm.h -- C-ABI of the GB300 particle time step (Enskog-Fokker-Planck /
 * ESMC / Enskog-Vlasov particle method).
 *
 * The reference is a serial C++ program whose particle loop is a set of free
 * functions taking raw `double*` SoA particle arrays plus GAS/BOX/CELLS structs
 * (prototypes in src/cpp_headers.h:360-730, driven by src/main.cpp:389-669).
 * This header replaces that routine surface with one device-resident session:
 *
 *   reference (file:line)                                   replacement
 *   ------------------------------------------------------  -------------------------------
 *   GAS/BOX/CELLS setup, src/myIO.cpp:1756 + :1094          mcpm_session_create
 *   caller-owned double* x1,x2,U1,U2,U3 (src/main.cpp:104)  mcpm_upload/download_particles
 *   cell_update          src/Main_Functions.cpp:2138        mcpm_cell_update
 *   random_generator     src/Fokker_Planck.cpp:20           mcpm_random_generator
 *   velocity_update      src/Main_Functions.cpp:1538        mcpm_velocity_update
 *     Velocity_FP_parallel src/Fokker_Planck.cpp:1065         (model FP_dense / FP_ideal_gas)
 *     Collision_ESMC_new3  src/collisions.cpp:583             (model ESMC)
 *     vlasov_taking_the_integral src/Main_Functions.cpp:3582  (long_range 1, 1-D)
 *     poisson_solver       src/Main_Functions.cpp:3285        (long_range 3, 1-D)
 *     compute_Vlasov_2D    src/FEM.cpp:613                    (long_range 1, 2-D)
 *     compute_SP_2D        src/FEM.cpp:249                    (long_range 3, 2-D)
 *   cells[].n_n (cell_update) src/Main_Functions.cpp:2268   mcpm_get_node_density
 *   DFP_extra_streaming  src/Fokker_Planck.cpp:904          mcpm_dfp_extra_streaming
 *   apply_BC             src/Main_Functions.cpp:1451        mcpm_apply_bc
 *   store_old_positions  src/Main_Functions.cpp:5736        mcpm_store_old_positions
 *   stream_particles     src/Main_Functions.cpp:1494        mcpm_stream_particles
 *   one iteration of the loop src/main.cpp:389-669          mcpm_step
 *
 * Conventions
 *  - Every call returns an int status (MCPM_OK == 0).  Nothing calls exit();
 *    where the reference printed and exited (out-of-box particle
 *    src/Main_Functions.cpp:2248-2263, NaN velocity src/Fokker_Planck.cpp:1137-1149)
 *    the device raises a bit in a status word and the call returns the code.
 *    mcpm_last_error() gives the message.
 *  - Host arrays stay caller-owned and are copied; device state is owned by
 *    the session.  Particle arrays are indexed by the caller's particle id, in
 *    the order they were uploaded, exactly like the reference's arrays.
 *  - A session is bound to one CUDA stream; calls are asynchronous unless they
 *    return host data (download/get_*), which synchronise.  One session per
 *    host thread.
 */
#ifndef MCPM_H_INCLUDED
#define MCPM_H_INCLUDED

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MCPM_ABI_VERSION 1

/* ---- status codes (bit flags may be OR-ed in the device status word) ---- */
enum mcpm_status {
  MCPM_OK = 0,
  MCPM_ERR_ARG = 1,          /* invalid argument / configuration            */
  MCPM_ERR_CUDA = 2,         /* CUDA runtime error                           */
  MCPM_ERR_OUT_OF_BOX = 4,   /* particle outside the box at binning          */
  MCPM_ERR_NAN = 8,          /* NaN velocity or position                     */
  MCPM_ERR_CAPACITY = 16,    /* more particles or cells than allocated       */
  MCPM_ERR_BC_LOOP = 32,     /* wall re-flight did not converge (>20 loops)  */
  MCPM_ERR_ITER_LIMIT = 64,  /* a bounded device wait gave up                */
  MCPM_ERR_STATE = 128       /* call out of order (e.g. no particles)        */
};

/* ---- problem (boundary treatment), names follow src/cpp_headers.h:24-35 --- */
enum mcpm_problem {
  MCPM_PROBLEM_CLOSED_BOX = 1,  /* BC_specular_reflection, src/Main_Functions.cpp:6399 */
  MCPM_PROBLEM_COUETTE = 2,     /* BC_thermal_wall_3D, src/Main_Functions.cpp:4917     */
  MCPM_PROBLEM_WALL = 11,       /* BC_wall (diffuse lower, specular upper) :4816       */
  MCPM_PROBLEM_PERIODIC = 100   /* x <- x - L*floor(x/L) in every active direction;
                                   the reference has no generic periodic BC, this
                                   is the wrap the homogeneous relaxation case needs */
};

/* ---- collision model, the gas.model strings of the reference ------------- */
enum mcpm_model {
  MCPM_MODEL_NONE = 0,          /* "none"                                       */
  MCPM_MODEL_FP_DENSE = 1,      /* "FP_dense"   (Enskog-Fokker-Planck)          */
  MCPM_MODEL_FP_IDEAL_GAS = 2,  /* "FP_ideal_gas"                               */
  MCPM_MODEL_ESMC = 3           /* "ESMC" (Enskog DSMC, Collision_ESMC_new3)    */
};

/* ---- long-range (Vlasov) force, gas.long_range (src/Main_Functions.cpp:1612) */
enum mcpm_long_range {
  MCPM_LR_NONE = 0,
  MCPM_LR_DIRECT = 1,           /* 1-D vlasov_taking_the_integral               */
  MCPM_LR_SCREENED_POISSON = 3  /* 1-D poisson_solver (Green's-function BC)     */
};

enum mcpm_precision {
  MCPM_FP64 = 0,                /* particle state and sums in double            */
  MCPM_FP32 = 1                 /* particle state float, compensated sums,
                                   per-cell solves still in double              */
};

enum mcpm_rng {
  MCPM_RNG_PHILOX = 0,          /* counter-based Philox4x32-10 keyed by seed,
                                   particle id and step                          */
  MCPM_RNG_INJECTED = 1         /* normals from mcpm_inject_normals (tests)     */
};

/* Plain-data configuration: the subset of GAS/BOX (src/cpp_headers.h:145-269)
   the particle step reads.  Units are whatever the caller uses consistently
   (the reference mixes SI and reduced units; mcpm does no unit conversion). */
typedef struct mcpm_config {
  int32_t n_cells[3];     /* box.N[0..2]; n_cells[2] must be 1                  */
  int32_t direction[3];   /* box.direction: 1 = streaming in that direction;
                             direction[2] must be 0                             */
  double  length[3];      /* box.Len[0..2]                                      */
  int32_t problem;        /* enum mcpm_problem                                  */
  int32_t model;          /* enum mcpm_model                                    */
  int32_t long_range;     /* enum mcpm_long_range                               */
  int32_t precision;      /* enum mcpm_precision                                */
  double  sigma;          /* gas.sigma  hard-sphere diameter                    */
  double  m;              /* gas.m      particle mass                           */
  double  kb;             /* gas.kb     Boltzmann constant                      */
  double  n;              /* gas.n      mean number density                     */
  double  Fn;             /* gas.Fn     real particles per simulation particle  */
  double  T0;             /* gas.T0     viscosity reference temperature         */
  double  mu;             /* gas.mu     viscosity at T0                         */
  double  visp;           /* gas.visp   viscosity exponent mu ~ T^visp          */
  double  b;              /* gas.b      2*pi*sigma^3/3                          */
  double  dt;             /* gas.delta_t                                        */
  double  phi;            /* gas.phi    attraction strength (direct Vlasov)     */
  double  eqdist;         /* gas.eqdist inner radius of the direct quadrature   */
  double  ast;            /* gas.ast    screened-Poisson amplitude              */
  double  bst;            /* gas.bst    screened-Poisson inverse range          */
  double  T_wall[4];      /* box.T_wall_1..4                                    */
  double  U_wall[4];      /* box.U_wall_1..4                                    */
  uint64_t seed;          /* Philox key                                         */
  int64_t max_particles;  /* capacity of the device particle arrays             */
} mcpm_config;

/* Per-cell quantities exported by mcpm_get_cells as a [MCPM_CF_COUNT][C]
   array of doubles (C = n_cells[0]*n_cells[1]); field names are the CELLS
   members of src/cpp_headers.h:271-347. */
enum mcpm_cell_field {
  MCPM_CF_NUM_INSIDE = 0,
  MCPM_CF_U_SPACE = 1,    /* 3 */
  MCPM_CF_PIJ = 4,        /* 6: 11 12 13 22 23 33 */
  MCPM_CF_M3 = 10,        /* 10: 111 112 113 122 123 133 222 223 233 333 */
  MCPM_CF_M4 = 20,        /* 6 */
  MCPM_CF_M5 = 26,        /* 3 */
  MCPM_CF_Q = 29,         /* 3 */
  MCPM_CF_DM2 = 32,
  MCPM_CF_DM4 = 33,
  MCPM_CF_MP = 34,        /* 3 */
  MCPM_CF_T = 37,
  MCPM_CF_N = 38,
  MCPM_CF_GAMMA_ST = 39,
  MCPM_CF_LAMBDA = 40,
  MCPM_CF_C = 41,         /* 6 */
  MCPM_CF_GAMMA = 47,     /* 3 */
  MCPM_CF_ALPHA = 50,     /* 9 */
  MCPM_CF_BETA = 59,      /* 3 */
  MCPM_CF_PHI = 62,       /* 3 */
  MCPM_CF_F2 = 65,        /* long-range force per cell (y component)     */
  MCPM_CF_OMEGA_MAX = 66, /* ESMC majorant                                */
  MCPM_CF_DIVU = 67,
  MCPM_CF_COUNT = 68
};

typedef struct mcpm_session mcpm_session;

/* Fill derived GAS fields the way readSettingsFile does
   (src/myIO.cpp:2217-2233, :2828-2830): b = 2 pi sigma^3/3, T0 = 273,
   mu = 5/(16 sigma^2) sqrt(m kb T0/pi), Fn = n*Volume/N, eqdist = sigma. */
int mcpm_config_derive(mcpm_config* cfg, int64_t n_particles);

int mcpm_session_create(const mcpm_config* cfg, mcpm_session** out);
int mcpm_session_destroy(mcpm_session* s);
const char* mcpm_last_error(const mcpm_session* s);
int mcpm_sync(mcpm_session* s);
/* Pending device status bits (enum mcpm_status); clears them. Synchronises. */
int mcpm_check_status(mcpm_session* s);

/* Copies caller arrays (reference layout, double, indexed by particle id) to
   the device, bins them (cell_update's binning) and sorts the device copy by
   cell.  x1 may be NULL when direction[0] == 0.  Resets the step counter. */
int mcpm_upload_particles(mcpm_session* s, int64_t n, const double* x1,
                          const double* x2, const double* U1, const double* U2,
                          const double* U3);
/* Copies the device state back into caller arrays, in particle-id order.
   When x1 never changes (direction[0] == 0 and not ESMC) the device does not
   keep it and the caller's x1 is left untouched. */
int mcpm_download_particles(mcpm_session* s, int64_t n, double* x1, double* x2,
                            double* U1, double* U2, double* U3);

/* cell_update (src/Main_Functions.cpp:2138-2749): binning, per-cell moments,
   Lambda, alpha/beta (FP_dense, step > 0), c/gamma, phi. */
int mcpm_cell_update(mcpm_session* s);
/* random_generator (src/Fokker_Planck.cpp:20-145): 3 normals per particle,
   centred and normalised per cell; kept on the device for the next
   mcpm_velocity_update. */
int mcpm_random_generator(mcpm_session* s);
/* velocity_update (src/Main_Functions.cpp:1538-1672): FP Langevin update or
   ESMC collisions, then the long-range force kick. */
int mcpm_velocity_update(mcpm_session* s);
int mcpm_dfp_extra_streaming(mcpm_session* s);
int mcpm_apply_bc(mcpm_session* s);
int mcpm_store_old_positions(mcpm_session* s);
int mcpm_stream_particles(mcpm_session* s);
/* Advances the box step counter (box.step++ / t += dt, src/main.cpp:667). */
int mcpm_end_step(mcpm_session* s);

/* n_steps iterations of the main loop body (src/main.cpp:389-669) for the
   in-scope models: cell_update, random_generator, velocity_update,
   DFP_extra_streaming, apply_BC, store_old_positions, stream_particles,
   apply_BC.  The particle-side stages run fused in one kernel per step;
   once the cell layout is in its steady state, pairs of steps are replayed
   as one CUDA graph (not in profiling mode). */
int mcpm_step(mcpm_session* s, int32_t n_steps);

/* ---- test and diagnostic hooks ---------------------------------------- */
/* Raw (un-whitened) normals for the next random_generator, per particle id
   (the three arrays random_generator fills with generateGaussianNoise,
   src/Fokker_Planck.cpp:85-90).  Switches the session to MCPM_RNG_INJECTED. */
int mcpm_inject_normals(mcpm_session* s, int64_t n, const double* xi1,
                        const double* xi2, const double* xi3);
int mcpm_set_rng(mcpm_session* s, int32_t mode);
/* [MCPM_CF_COUNT][C] doubles, see enum mcpm_cell_field. */
int mcpm_get_cells(mcpm_session* s, double* out);
/* Cell index of every particle, in particle-id order (cell_update's index[]). */
int mcpm_get_index(mcpm_session* s, int32_t* index);
/* Nodal densities n_n of the last cell_update, [C][4] doubles (cell-major,
   corner 0 lower left, 1 lower right, 2 upper left, 3 upper right), as
   cell_update deposits them (src/Main_Functions.cpp:2268-2364).  Computed
   only by sessions whose Vlasov force is the 2-D screened-Poisson one
   (their only consumer, src/FEM.cpp:285-288); MCPM_ERR_STATE otherwise. */
int mcpm_get_node_density(mcpm_session* s, double* out);
/* Node potential of the last 2-D Vlasov force evaluation, (N0+1)(N1+1)
   doubles, node (i, j) at j (N0+1) + i: the direct quadrature
   (compute_Vlasov_2D, src/FEM.cpp:675-701) or the screened-Poisson FEM
   solution after the near-field correction (compute_SP_2D, :458-546). */
int mcpm_get_node_potential(mcpm_session* s, double* out);
/* Whitened normals last produced by random_generator, per particle id. */
int mcpm_get_normals(mcpm_session* s, double* xi1, double* xi2, double* xi3);
int32_t mcpm_get_step(const mcpm_session* s);
int mcpm_set_step(mcpm_session* s, int32_t step);
/* Overwrite one cell field (e.g. omega_max) for all cells from host data. */
int mcpm_set_cell_field(mcpm_session* s, int32_t field, const double* values);
/* Slot layout of the device copy: particle id held by every slot and the
   first slot of every cell (C+1 entries); valid after mcpm_cell_update. */
int mcpm_get_layout(mcpm_session* s, int32_t* pid_by_slot, int32_t* off);
/* ESMC majorant from the current cell T and n (src/main.cpp:250-269). */
int mcpm_init_omega_max(mcpm_session* s);
/* Launch on the caller's CUDA stream (cudaStream_t) instead of the
   session's own; NULL restores the session stream. */
int mcpm_set_stream(mcpm_session* s, void* stream);
/* Kernel classes timed by the profiling mode, in mcpm_profile_read order. */
enum mcpm_kernel_class {
  MCPM_K_BIN = 0, MCPM_K_SCAN, MCPM_K_SCATTER, MCPM_K_MOMENTS, MCPM_K_SOLVE,
  MCPM_K_ESMC, MCPM_K_LONG_RANGE, MCPM_K_UPDATE, MCPM_K_COUNT
};
/* enable != 0: bracket every kernel launch with CUDA events on the launch
   stream and accumulate device time per kernel class. */
int mcpm_profile(mcpm_session* s, int32_t enable);
/* Synchronises; per class: total milliseconds and launches since the last
   read (n <= MCPM_K_COUNT entries each). */
int mcpm_profile_read(mcpm_session* s, double* ms, int64_t* launches, int32_t n);
/* ---- work split between warps and blocks -------------------------------- */
/* Cells with at most wcap particles are processed by one warp each, larger
   cells by a 256-thread block; wcap <= 768 (FP32) / 384 (FP64). */
int mcpm_set_wcap(mcpm_session* s, int32_t wcap);
int32_t mcpm_get_wcap(const mcpm_session* s);
/* Times `steps` fused steps per candidate wcap on the session's particles,
   restoring the state after each trial, and keeps the fastest (written to
   *chosen).  Leaves the particle and cell state as it found it. */
int mcpm_autotune(mcpm_session* s, int32_t steps, int32_t* chosen);

/* ---- allocation-free entry point -------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
   memory (a host framework that owns the GPU allocator, code running between
   CUDA-graph replays, plugins handed only their input and output buffers):
   the screened-Poisson Vlasov force of poisson_solver for a 1-D column of
   cells, from n_cell[n_cells] (device, cell number densities) into
   F2[n_cells] (device, per-cell force), with the geometry and constants taken
   from cfg (length[1], sigma, eqdist, bst, ast, m).  It allocates nothing:
   its scratch is a fixed array of the library that every GPU loading the
   library holds until exit.  n_cells above MCPM_NOALLOC_MAX_CELLS returns
   MCPM_ERR_CAPACITY.  The first call on a device resolves the scratch's
   device address (call it once before any stream capture).  All calls share
   the scratch, so calls that overlap on the GPU race.  stream may be NULL.
   Synchronises the stream before returning. */
#define MCPM_NOALLOC_MAX_CELLS 6999
int mcpm_poisson_force_1d_noalloc(const double* n_cell, int32_t n_cells,
                                  const mcpm_config* cfg, double* F2,
                                  void* stream);
/* Number of kernel launches the session issued since creation. */
int64_t mcpm_kernel_launches(const mcpm_session* s);

#ifdef __cplusplus
}
#endif
#endif /* MCPM_H_INCLUDED */
