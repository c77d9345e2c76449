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
 *     Velocity_FP_linear   src/Fokker_Planck.cpp:1186         (model FP_linear)
 *     Collision_ESMC_new3  src/collisions.cpp:583             (model ESMC)
 *     Collision_DSMC_VHS   src/collisions.cpp:2063            (model DSMC_VHS)
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

#define MCPM_ABI_VERSION 2

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
  MCPM_MODEL_ESMC = 3,          /* "ESMC" (Enskog DSMC, Collision_ESMC_new3)    */
  MCPM_MODEL_FP_LINEAR = 4,     /* "FP_linear" (Velocity_FP_linear: Langevin
                                   relaxation without the cubic drift,
                                   src/Fokker_Planck.cpp:1186-1283)             */
  MCPM_MODEL_DSMC_VHS = 5       /* "DSMC_VHS" (Collision_DSMC_VHS: Bird's
                                   no-time-counter DSMC with variable hard
                                   spheres, src/collisions.cpp:2063-2141)       */
};

/* ---- long-range (Vlasov) force, gas.long_range (src/Main_Functions.cpp:1612) */
enum mcpm_long_range {
  MCPM_LR_NONE = 0,
  MCPM_LR_DIRECT = 1,           /* 1-D vlasov_taking_the_integral               */
  MCPM_LR_DENSITY_EXPANSION = 2, /* density-gradient force from the kernel-
                                   smoothed density (src/Main_Functions.cpp:1632-1653) */
  MCPM_LR_SCREENED_POISSON = 3  /* 1-D poisson_solver (Green's-function BC)     */
};

enum mcpm_precision {
  MCPM_FP64 = 0,                /* particle state and sums in double            */
  MCPM_FP32 = 1                 /* particle state and moment sums float
                                   (per-lane runs combined pairwise), per-cell
                                   solves still in double                       */
};

enum mcpm_rng {
  MCPM_RNG_PHILOX = 0,          /* counter-based Philox4x32-10 keyed by seed,
                                   particle id and step                          */
  MCPM_RNG_INJECTED = 1         /* normals from mcpm_inject_normals (tests)     */
};

/* The draw streams of the particle step (the Philox counter's third word);
   mcpm_inject_uniforms replaces one stream's draws.  The key of a draw is
   the particle id for FP, BC, BIN and the ADDREM streams (the parent's id
   for ADDREM_NEW) and the cell for the collision streams; the counter is 0
   except for BC ((apply_BC call of the step << 8) | re-flight loop), the
   candidate number for ESMC / ESMC_ACC / DSMC / DSMC_ACC and the copy
   number for ADDREM_NEW. */
enum mcpm_rng_stream {
  MCPM_RNG_STREAM_FP = 0,          /* random_generator's normals (4 words)     */
  MCPM_RNG_STREAM_BC = 1,          /* diffuse re-emission (BC_thermal_wall_3D,
                                      BC_wall): Rayleigh factor, two normals   */
  MCPM_RNG_STREAM_ESMC = 2,        /* ESMC candidate pair and direction        */
  MCPM_RNG_STREAM_BIN = 3,         /* cell_update's face jitter (word 0 >= 2^31:
                                      +1e-14, else -1e-14)                     */
  MCPM_RNG_STREAM_ESMC_ACC = 4,    /* ESMC acceptance                          */
  MCPM_RNG_STREAM_ESMC_M = 5,      /* ESMC candidate count rounding            */
  MCPM_RNG_STREAM_DSMC = 6,        /* DSMC_VHS candidate pair and direction    */
  MCPM_RNG_STREAM_DSMC_ACC = 7,    /* DSMC_VHS acceptance                      */
  MCPM_RNG_STREAM_DSMC_M = 8,      /* DSMC_VHS candidate count rounding        */
  MCPM_RNG_STREAM_ADDREM_DEL = 9,  /* merge: deletion test                     */
  MCPM_RNG_STREAM_ADDREM_NEW = 10, /* split: the copies' velocity normals      */
  MCPM_RNG_STREAM_COUNT = 11
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
  double  crref;          /* gas.crref  VHS reference speed sqrt(kb T / m) of
                             the initial temperature (src/myIO.cpp:2242);
                             DSMC_VHS only, must then be > 0                    */
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
  MCPM_CF_F2 = 65,        /* long-range force per cell (y component); for
                             long_range 2 the kick -dummyF of
                             src/Main_Functions.cpp:1647, 0 in the
                             first cell and in cell N[1]-1               */
  MCPM_CF_OMEGA_MAX = 66, /* ESMC majorant omega_max; for DSMC_VHS the
                             cell's majorant relative speed crm          */
  MCPM_CF_DIVU = 67,
  MCPM_CF_N_SMOOTH = 68,  /* kernel-smoothed density and its first and
                             third y-derivative sums (cell_update,
                             src/Main_Functions.cpp:2378-2427); computed
                             when long_range is 2, the only consumer,
                             else 0                                      */
  MCPM_CF_DN2 = 69,
  MCPM_CF_DN3 = 70,
  MCPM_CF_COUNT = 71
};

typedef struct mcpm_session mcpm_session;

/* Fill derived GAS fields the way readSettingsFile does
   (src/myIO.cpp:2217-2233, :2828-2830): b = 2 pi sigma^3/3, T0 = 273,
   mu = 5/(16 sigma^2) sqrt(m kb T0/pi), Fn = n*Volume/N, eqdist = sigma. */
int mcpm_config_derive(mcpm_config* cfg, int64_t n_particles);

/* readSettingsFile (src/myIO.cpp:1756-3016) for the problems the particle
   step covers, closed_box (1), couette_flow (2), wall (11) and injection
   (12, run between the closed box's specular walls): reads the reference's
   settings file ("keyword values..." per line, '#' comment lines) and
   derives the configuration as the reference does (cell sizes, Fn, sigma and
   crref from mu for hard or variable hard spheres, b, mu(T0), dt from the
   mean free path and frac_mft, phi from epsilon; SI constants where the
   reference fixes them; for wall the liquid slab between vapour layers:
   sigma of argon, densities in sigma^-3, Fn = 1e13, N and the box height
   from the layers, the liquid's temperature; for injection a droplet of
   extra particles in a gas at rest, box and densities in units of argon's
   sigma).  *n_particles receives gas.N.  Keywords the
   reference does not know, other problems and models outside the step
   return MCPM_ERR_ARG; msg (optional, msg_len bytes) receives the reason.
   The result is an FP64 configuration; change precision before creating
   the session for an FP32 one. */
int mcpm_config_from_settings(const char* path, mcpm_config* out, int64_t* n_particles, char* msg,
                              int32_t msg_len);
/* initialization (src/Main_Functions.cpp:4222-4814) for the same problems:
   fills n_particles (= gas.N as derived) host particles, uniform along the
   streaming directions and mid-box along the others (wall: x2 uniform
   within the lower vapour layer, the liquid slab and the upper vapour layer
   in id order, as the reference places them; injection: the gas over the
   box, then the droplet's particles over the central disc), velocities Maxwellian
   about U0 at T = max(gas.T, max(T_wall_1 + T_wall_2, T_wall_3 + T_wall_4)/2).
   The reference seeds from std::random_device; seed makes a run repeatable. */
int mcpm_initialize_from_settings(const char* path, uint64_t seed, double* x1, double* x2, double* U1, double* U2,
                                  double* U3, int64_t n_particles, char* msg, int32_t msg_len);
int mcpm_session_create(const mcpm_config* cfg, mcpm_session** out);
int mcpm_session_destroy(mcpm_session* s);
const char* mcpm_last_error(const mcpm_session* s);
int mcpm_sync(mcpm_session* s);
/* Pending device status bits (enum mcpm_status); clears them. Synchronises. */
int mcpm_check_status(mcpm_session* s);

/* Copies caller arrays (reference layout, double, indexed by particle id) to
   the device and bins them (cell_update's binning, which also reports
   particles outside the box); the device copy is sorted by cell at the
   first cell_update or step.  x1 may be NULL when direction[0] == 0.
   Resets the step counter to 0.  Returns once the caller's arrays have been
   read; the copies run on a stream of their own and overlap the copies of
   a download still in flight (mcpm_download_particles_async). */
int mcpm_upload_particles(mcpm_session* s, int64_t n, const double* x1,
                          const double* x2, const double* U1, const double* U2,
                          const double* U3);
/* The same without waiting for the copies: the caller's arrays must stay
   unchanged until mcpm_sync returns.  With pinned host arrays the copies
   run while the session's earlier work (steps, a download's copies) is
   still in flight. */
int mcpm_upload_particles_async(mcpm_session* s, int64_t n, const double* x1,
                                const double* x2, const double* U1,
                                const double* U2, const double* U3);
/* The positions before the last flight (the reference's x1_old, x2_old,
   particle-id order), for sessions with diffuse walls, which read them:
   an upload starts them as the positions themselves.  x1_old may be NULL
   when direction[0] == 0.  No effect where nothing reads them. */
int mcpm_set_old_positions(mcpm_session* s, const double* x1_old, const double* x2_old);
/* The positions before the last flight as the walls left them (diffuse
   walls move them to the wall crossing), particle-id order; sessions that
   keep them only (diffuse walls, pressure sampling). */
int mcpm_get_old_positions(mcpm_session* s, double* x1_old, double* x2_old);
/* Copies the device state back into caller arrays, in particle-id order.
   When x1 never changes (direction[0] == 0 and not ESMC) the device does not
   keep it and the caller's x1 is left untouched. */
int mcpm_download_particles(mcpm_session* s, int64_t n, double* x1, double* x2,
                            double* U1, double* U2, double* U3);
/* The same without waiting: the conversions are queued on the session's
   stream and the copies on a stream of their own; the caller's arrays are
   written once mcpm_sync returns (or a later synchronous download).  The
   state may be stepped or replaced by an upload meanwhile: the copies read
   a staging buffer, not the state.  With pinned host arrays the copies of a
   download overlap those of the next upload (the host link carries both
   directions at once). */
int mcpm_download_particles_async(mcpm_session* s, int64_t n, double* x1,
                                  double* x2, double* U1, double* U2,
                                  double* U3);

/* cell_update (src/Main_Functions.cpp:2138-2749): binning, per-cell moments,
   Lambda, alpha/beta (FP_dense, step > 0), c/gamma, phi. */
int mcpm_cell_update(mcpm_session* s);
/* random_generator (src/Fokker_Planck.cpp:20-145): 3 normals per particle,
   centred and normalised per cell; kept on the device for the next
   mcpm_velocity_update.  Draws for the models the routine serves
   (FP_dense, FP_ideal_gas, FP_linear, :22); a no-op for the others. */
int mcpm_random_generator(mcpm_session* s);
/* velocity_update (src/Main_Functions.cpp:1538-1672): FP Langevin update
   (Velocity_FP_parallel, or Velocity_FP_linear for FP_linear) or ESMC
   collisions, then the long-range force kick. */
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
   apply_BC.  FP_linear steps draw their normals with random_generator:
   the reference's loop calls it for FP_dense and FP_ideal_gas only
   (src/main.cpp:442), which leaves Velocity_FP_linear reading noise arrays
   that nothing filled (malloc'd at :129).  The particle-side stages run fused in one kernel per step;
   once the cell layout is in its steady state, pairs of steps are replayed
   as one CUDA graph (not in profiling mode).  Returns once the steps have
   run, with the device status bits (mcpm_check_status). */
int mcpm_step(mcpm_session* s, int32_t n_steps);
/* The same steps, returning once they are queued: the host goes on (an
   upload or download of the next batch, mcpm_*_async) while the device
   steps.  The status bits stay on the device until mcpm_check_status or a
   synchronous step reads them.  After a judge step of an attached learned
   force the verdict is read (the host waits for the judge step) when the
   next step is queued, or by mcpm_sync or mcpm_get_surrogate_stats. */
int mcpm_step_async(mcpm_session* s, int32_t n_steps);

/* ---- test and diagnostic hooks ---------------------------------------- */
/* Raw (un-whitened) normals for the next random_generator, per particle id
   (the three arrays random_generator fills with generateGaussianNoise,
   src/Fokker_Planck.cpp:85-90).  Switches the session to MCPM_RNG_INJECTED. */
int mcpm_inject_normals(mcpm_session* s, int64_t n, const double* xi1,
                        const double* xi2, const double* xi3);
int mcpm_set_rng(mcpm_session* s, int32_t mode);
/* Uniform draws in place of one stream's Philox words (tests that need a
   known draw: a wall re-emission, the face jitter of a particle exactly on
   a face, a chosen collision candidate).  u holds n_rows rows of four
   uniforms in [0, 1); a draw with key q and counter c reads row
   (q + c) mod n_rows, at every step, as the four 32-bit words
   floor(u 2^32) (clamped to [0, 2^32 - 1]).  The FP64 kernels turn a word w
   into the uniform (w + 1/2) 2^-32, so u = (w + 1/2) 2^-32 comes back
   exactly; the FP32 kernels take the top 23 bits, (floor(w / 2^9) + 1/2) 2^-23.
   Integer uses (a candidate picked among n) take floor(w n / 2^32).
   n_rows = 0 (or u = NULL) restores the Philox stream. */
int mcpm_inject_uniforms(mcpm_session* s, int32_t stream, int64_t n_rows, const double* u);
/* Time-sampled raw velocity sums per cell, the CELLS members that
   cell_poly_velocity accumulates (src/Main_Functions.cpp:1918-1968, called by
   post_processing once the run passes its averaging start, src/myIO.cpp:968-971):
   particle count, sum U_i, sum U_i U_j (11 12 13 22 23 33), sum
   U1^m U2^n U3^(3-m-n) in the order m = 0..3, n = 0..3-m, and
   sum U_i U_j |U|^2 (11 12 13 22 23 33). */
enum mcpm_sample_field {
  MCPM_SF_WEIGHT = 0,
  MCPM_SF_M = 1,     /* 3  */
  MCPM_SF_MM = 4,    /* 6  */
  MCPM_SF_MMM = 10,  /* 10 */
  MCPM_SF_MMMM = 20, /* 6  */
  MCPM_SF_COUNT = 26
};
/* cell_poly_velocity: adds the current particles' sums to the session's
   sample accumulators (FP64, zero at creation).  Needs the layout of a
   preceding mcpm_cell_update, as the reference samples right after it. */
int mcpm_sample_cells(mcpm_session* s);
/* [MCPM_SF_COUNT][C] doubles, see enum mcpm_sample_field. */
int mcpm_get_samples(mcpm_session* s, double* out);
/* Sets the sample accumulators back to zero. */
int mcpm_reset_samples(mcpm_session* s);
/* [MCPM_CF_COUNT][C] doubles, see enum mcpm_cell_field. */
int mcpm_get_cells(mcpm_session* s, double* out);
/* Cell index of every particle, in particle-id order (cell_update's index[]). */
int mcpm_get_index(mcpm_session* s, int32_t* index);

/* ---- pressure sampling -------------------------------------------------- */
/* measure_pressure (src/Main_Functions.cpp:13-34, called src/main.cpp:490-492
   once step > times * after): every particle whose cell row changed over
   the step adds Fn m |U2| to p_m of each row index it crossed.  Switching
   sampling on keeps the positions before the flight (sessions without
   diffuse walls otherwise do not) and makes every fused step add its
   crossings after the flight and the walls; mcpm_measure_pressure adds
   those of the current state once (the routine-by-routine loop, after
   store_old_positions / stream_particles / apply_BC).  p_m accumulates until
   reset; mcpm_get_pressure copies its C values (cells[].p_m). */
int mcpm_set_pressure_sampling(mcpm_session* s, int32_t on);
int mcpm_measure_pressure(mcpm_session* s);
int mcpm_get_pressure(mcpm_session* s, double* p_m);
int mcpm_reset_pressure(mcpm_session* s);

/* ---- post-processing output ------------------------------------------- */
/* write_post_processing (src/myIO.cpp:597-934): the file
   <dir>/<output_name>_<lr>_<step>.dat (lr: noatt / direct / denexp /
   screened-Poisson) in the reference's layout -- a header of 122 names,
   then per cell (x outer, y inner, a blank line after each column) 121
   values: geometry, t_post, dt, U_space, T, n, the cell_poly_velocity sums,
   the interface face sums (0 here), volume, n_smooth, num_inside, the
   Enskog pressure with attraction, n_ratio Fn, model / xx / UU.. (0 here),
   P_12 ... the FP coefficients, p_m and the Enskog pressure.  The reference
   writes it into PostProc/ when step > times * after and step % every == 0
   or at its first step; the caller decides.  cells: [MCPM_CF_COUNT][C]
   (mcpm_get_cells); samples [MCPM_SF_COUNT][C], p_m [C], cell_weights [C]
   may be NULL (0, 0, 1).  path receives the file name. */
int mcpm_post_processing_write(const mcpm_config* cfg, int32_t step, double t_post,
                               const char* dir, const char* output_name,
                               const double* cells, const double* samples,
                               const double* p_m, const int32_t* cell_weights,
                               char* path, int32_t path_len);
/* The same from a session's cell fields, sample sums, p_m and cell weights. */
int mcpm_write_post_processing(mcpm_session* s, int32_t step, double t_post,
                               const char* dir, const char* output_name,
                               char* path, int32_t path_len);
/* The console summary of post_processing (src/myIO.cpp:945-965: T, N,
   n sigma^3 and p of cells 0, 1, 2, N[1]/2, N[1]-2, N[1]-1, their mean T,
   Fn; the 1-D-box form when N[1] == 1) into buf; returns its length. */
int mcpm_post_processing_text(const mcpm_config* cfg, const double* cells,
                              char* buf, int32_t len);

/* ---- interface problems: thermostat and weighted particles ------------ */
/* Per-particle weights (the reference's n_ratio[], particle-id order, N
   values) and per-cell weights (cells[].n_ratio, C values, set by make_cells
   from the problem's liquid / vapour regions, src/myIO.cpp:1486-1526).  Until
   set, every particle and cell weighs 1.  The particle weights follow the
   ids through uploads only by being set again. */
int mcpm_set_particle_weights(mcpm_session* s, const int32_t* w);
int mcpm_get_particle_weights(mcpm_session* s, int32_t* w);
int mcpm_set_cell_weights(mcpm_session* s, const int32_t* w);
/* thermostat (src/Main_Functions.cpp:1674-1869, the live branch, problem
   inverted): every cell num < N[1] whose centre lies below thermc is
   rescaled to temperature Tc and every one above Len[1] - thermh to Th,
   U <- sqrt(T_target / T) (U - U_space) + U_space, with T and U_space of
   the last cell_update (cells with T > 0).  Call cell_update first, as the
   reference's loop does (src/main.cpp:429-436). */
int mcpm_thermostat(mcpm_session* s, double Tc, double Th, double thermc, double thermh);
/* inverted_addremove_particles (src/Main_Functions.cpp:1206-1450): against
   the cells of the last binning, a particle heavier than its cell is split
   into n_ratio particles (itself and n_ratio - 1 copies with velocities
   U + h z, z standard normals, h = 1.06 sig (numb_rem + n_ratio)^(-1/5));
   a lighter one is deleted with probability 1 - 1/n_ratio or takes the
   cell's weight.  When any particle was split or deleted the state is
   rebuilt: the kept particles in their id order, then the copies (by the
   rank of the split particle's id, copy j inner), every weight set to its
   cell's, N updated (*n_out); the next cell_update or step bins it.  The
   draws are Philox, keyed by particle id and the session's step number (the
   reference draws from std::random_device).  MCPM_ERR_CAPACITY when the new
   N would exceed max_particles (the state is then unchanged). */
int mcpm_addremove_particles(mcpm_session* s, int32_t n_ratio, int64_t* n_out);
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
/* The step number the draws are keyed by (the reference's loop counter).
   Setting another number re-draws the binning's face jitter
   (src/Main_Functions.cpp:2238-2247) at the next cell_update or step, as the
   reference's cell_update at that step would. */
int32_t mcpm_get_step(const mcpm_session* s);
int mcpm_set_step(mcpm_session* s, int32_t step);
/* Overwrite one cell field (e.g. omega_max) for all cells from host data. */
int mcpm_set_cell_field(mcpm_session* s, int32_t field, const double* values);
/* Slot layout of the device copy: particle id held by every slot and the
   first slot of every cell (C+1 entries); valid after mcpm_cell_update. */
int mcpm_get_layout(mcpm_session* s, int32_t* pid_by_slot, int32_t* off);
/* Collision majorants from the current cell T and n (src/main.cpp:250-269):
   omega_max for ESMC, crm = 10 sqrt(kb T / m) for DSMC_VHS.  mcpm_step calls
   it before its first step for those two models. */
int mcpm_init_omega_max(mcpm_session* s);
/* Launch on the caller's CUDA stream (cudaStream_t) instead of the
   session's own; NULL restores the session stream. */
int mcpm_set_stream(mcpm_session* s, void* stream);
/* Kernel classes timed by the profiling mode, in mcpm_profile_read order
   (MCPM_K_SCATTER: the keyed reorder of packed layouts, or the overflow
   repair of the slotted layouts FP32 sessions keep between fused steps). */
enum mcpm_kernel_class {
  MCPM_K_BIN = 0, MCPM_K_SCAN, MCPM_K_SCATTER, MCPM_K_MOMENTS, MCPM_K_SOLVE,
  MCPM_K_ESMC, MCPM_K_LONG_RANGE, MCPM_K_UPDATE, MCPM_K_SURROGATE, MCPM_K_COUNT
};
/* enable != 0: bracket every kernel launch with CUDA events on the launch
   stream and accumulate device time per kernel class. */
int mcpm_profile(mcpm_session* s, int32_t enable);
/* Synchronises; per class: total milliseconds and launches since the last
   read (n <= MCPM_K_COUNT entries each). */
int mcpm_profile_read(mcpm_session* s, double* ms, int64_t* launches, int32_t n);
/* ---- work split between warps and blocks -------------------------------- */
/* Cells with at most wcap particles are processed by one warp each, larger
   cells by a 256-thread block; wcap <= 384 (the shared-memory staging of a
   warp in the particle pass). */
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
   MCPM_ERR_CAPACITY.  The first call on a device, with that device current,
   looks up the scratch's device address and sets the force kernel's
   shared-memory limit; make that first call before any stream capture on
   the device begins.  All calls on one device share its scratch, so calls
   whose work overlaps on that GPU (two streams, or two host threads) race;
   calls on different devices do not share it, and no host-side buffer is
   shared.  stream may be NULL.  The work is queued on the stream and the
   call returns without waiting: F2 is ready once the stream has reached it. */
#define MCPM_NOALLOC_MAX_CELLS 6999
int mcpm_poisson_force_1d_noalloc(const double* n_cell, int32_t n_cells,
                                  const mcpm_config* cfg, double* F2,
                                  void* stream);
/* ---- learned Vlasov force of a 2-D box --------------------------------- */
/* No counterpart in the reference (its only learned model, the hybrid NN/GPR
   of src/hybrid.cpp, is not on the particle path).  A 4-layer convolutional
   operator on the N1 x N0 cell grid maps the nodal and cell densities that
   the node-grid force reads (compute_SP_2D / compute_Vlasov_2D inputs,
   src/FEM.cpp:249, :613) to the corner-potential differences of every cell
   that the kick applies (src/FEM.cpp:567-578, :703-714):
     input  [cells][MCPM_SUR_IN] bf16 (raw uint16 bits): v_k = 10 (b n_n[k] - 0.25)
            for the 4 corner nodal densities and v_4 = 10 (b n - 0.25), each
            as hi = bf16(v_k) in channel k and lo = bf16(v_k - hi) in channel
            6 + k; channel 5 = 1; channels 11..15 = 0;
     conv3x3 16->64, ReLU, 64->64, ReLU, 64->64, ReLU, 64->16 (zero padding);
     output [cells][MCPM_SUR_OUT] fp32 = (V1-V0, V3-V2, V2-V0, V3-V1) / out_scale.
   Parameters: MCPM_SUR_NPARAM floats, conv weights [co][tap][ci] with
   tap = 3 (dy + 1) + (dx + 1) followed by the biases, per layer:
   W1[64][9][16] b1[64] W2[64][9][64] b2[64] W3[64][9][64] b3[64]
   W4[16][9][64] b4[16] (input channels 11..15 and outputs 4..15 unused).
   Forward, backward and the Adam step run on the GPU in BF16 with FP32
   accumulation.  Device pointers below are on the surrogate's device; the
   standalone calls run on the surrogate's own stream and synchronise. */
typedef struct mcpm_surrogate mcpm_surrogate;
#define MCPM_SUR_IN 16
#define MCPM_SUR_OUT 4
#define MCPM_SUR_NPARAM 92368
/* Network for batches of up to max_batch grids of n1 x n0 cells. */
int mcpm_surrogate_create(int32_t n0, int32_t n1, int32_t max_batch, mcpm_surrogate** out);
int mcpm_surrogate_destroy(mcpm_surrogate* m);
const char* mcpm_surrogate_last_error(const mcpm_surrogate* m);
/* Sets the parameters (host, MCPM_SUR_NPARAM floats) and the output scale,
   and clears the Adam moments. */
int mcpm_surrogate_set_params(mcpm_surrogate* m, const float* params, int64_t n, double out_scale);
int mcpm_surrogate_get_params(mcpm_surrogate* m, float* params, int64_t n);
/* tcgen05 != 0: the 64->64 layers of inference (forward, and the step's
   force) run on the tcgen05 tensor cores; 0: on mma.sync, the path the
   backward pass differentiates.  Default 1. */
int mcpm_surrogate_set_tensor_path(mcpm_surrogate* m, int32_t tcgen05);
/* tcgen05 launches so far and whether that path is on (it turns itself off,
   with a message in mcpm_surrogate_last_error, if a TMA descriptor is
   refused). */
int mcpm_surrogate_launches(const mcpm_surrogate* m, int64_t* tcgen05_launches, int32_t* tcgen05_on);
/* y[batch][cells][MCPM_SUR_OUT] = network(x[batch][cells][MCPM_SUR_IN]),
   device pointers, outputs in units of out_scale. */
int mcpm_surrogate_forward(mcpm_surrogate* m, const uint16_t* x, int32_t batch, float* y);
/* Loss L = mean over cells and outputs of (y - target_scale target)^2 and
   its gradient with respect to every parameter (host grad[MCPM_SUR_NPARAM],
   may be NULL); loss[2] = (sum of squared errors, sum of squared scaled
   targets), may be NULL. */
int mcpm_surrogate_gradients(mcpm_surrogate* m, const uint16_t* x, const float* target, int32_t batch,
                             double target_scale, float* grad, double* loss);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8, step number t >= 1) on the
   loss of mcpm_surrogate_gradients.  loss may be NULL (no synchronisation). */
int mcpm_surrogate_train_step(mcpm_surrogate* m, const uint16_t* x, const float* target, int32_t batch,
                              double target_scale, double lr, int32_t t, double* loss);
int mcpm_surrogate_sync(mcpm_surrogate* m);

/* Training snapshots from the plain node-grid force of a 2-D long-range
   session: for snapshot i the packing fraction
     n b(x, y) = f[0] + sum_w f[1+4w] sin(2 pi (f[2+4w] x / L0 + f[3+4w] y / L1) + f[4+4w]),
   clipped to [0.05, 0.45] (f = fields + i (1 + 4 n_waves)), gives quadrant
   counts round(lambda + sqrt(lambda) z) per cell quadrant (lambda =
   n vol / 4 / Fn, z a Philox normal keyed by seed, i, quadrant), from which
   the nodal densities, the cell densities and the session's plain force
   (long_range 1 or 3) are computed; x[i] (device, [cells][MCPM_SUR_IN]) gets
   the network input and y[i] (device, [cells][4]) the corner-potential
   differences.  Overwrites the session's cell densities and nodal data
   (mcpm_get_node_density / mcpm_get_node_potential then describe the last
   snapshot). */
int mcpm_vlasov_snapshots(mcpm_session* s, int32_t n_snap, const double* fields, int32_t n_waves, uint64_t seed,
                          uint16_t* x, float* y);
/* Attaches a trained network (m NULL detaches) to an FP32 2-D long-range
   session of the same grid: mcpm_step then takes the Vlasov kick from the
   network, and every judge_every steps (the first step included) runs the
   plain path as the judge, compares the two kicks and keeps the plain one
   for that step; while the relative L2 error of the kick coefficients of
   the last judge step exceeds threshold the plain path supplies the force.
   The network's buffers are used on the session's stream. */
int mcpm_attach_surrogate(mcpm_session* s, mcpm_surrogate* m, int32_t judge_every, double threshold);
typedef struct mcpm_surrogate_stats {
  double last_error;        /* relative L2 kick error of the last judge step (-1: none yet) */
  int64_t judged;           /* judge steps                                   */
  int64_t takeovers;        /* judge steps whose error exceeded the threshold */
  int64_t surrogate_steps;  /* steps whose force came from the network        */
  int64_t plain_steps;      /* steps whose force came from the plain path     */
  int32_t active;           /* the network supplies the force now             */
} mcpm_surrogate_stats;
int mcpm_get_surrogate_stats(mcpm_session* s, mcpm_surrogate_stats* out);
/* Re-evaluates the 2-D Vlasov kick of the last cell_update (or step) with
   the plain path (method 0) or the attached network (method 1) into the
   session's per-cell kick coefficients. */
int mcpm_eval_vlasov_2d(mcpm_session* s, int32_t method);
/* The per-cell kick coefficients of an FP32 2-D long-range session,
   [cells][4] floats (LA1, LB1, LA2, LB2: U1 -= LA1 + LB1 eta,
   U2 -= LA2 + LB2 xi, xi/eta the particle's bilinear coordinates). */
int mcpm_get_kick_2d(mcpm_session* s, float* out);

/* Number of kernel launches the session issued since creation. */
int64_t mcpm_kernel_launches(const mcpm_session* s);

#ifdef __cplusplus
}
#endif
#endif /* MCPM_H_INCLUDED */
