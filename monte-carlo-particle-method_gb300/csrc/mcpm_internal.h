// mcpm_internal.h -- session state and kernel launchers shared by the
// translation units of libmcpm.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/mcpm.h"

namespace mcpm {

// Internal per-cell fields stored after the exported ones (enum mcpm_cell_field).
enum {
  CFI_Y = MCPM_CF_COUNT,  // Y(n)
  CFI_A1,                 // exp(-dt/tau)
  CFI_A2,                 // (1 - exp(-dt/tau)) tau
  CFI_A3,                 // sqrt((1 - exp(-2 dt/tau)) kT/m)
  CFI_3KT,                // 3 kb T / m
  CFI_RAW,                // 29 raw central-moment sums from the moments kernel:
                          // Mp(3) PIJ(6) M3(10) M4(6) M5(3) DM2(1), finalised by k_solve
  CF_DEV_COUNT = CFI_RAW + 29
};

// Packed FP32 per-cell record the FP32 update kernel reads (written by the
// solve and long-range kernels), so that the particle pass runs no FP64.
enum {
  PF_US0, PF_US1, PF_US2, PF_A1, PF_A2, PF_A3, PF_EQ, PF_LAM,
  PF_C0, PF_C1, PF_C2, PF_C3, PF_C4, PF_C5, PF_G0, PF_G1, PF_G2, PF_Q0, PF_Q1, PF_Q2,
  PF_AL0, PF_AL1, PF_AL2, PF_AL3, PF_AL4, PF_AL5, PF_BE0, PF_BE1, PF_GST,
  PF_HQ0, PF_HQ1,          // M3[0]+M3[3]+M3[5], M3[1]+M3[6]+M3[8] (DFP heat-flux terms)
  PF_PH0, PF_PH1, PF_F2DT, PF_N,
  PF_E2,                   // sum over the cell of |M'|^2 (the moment pass's energy sum)
  // 2-D Vlasov kick: U1 -= LA1 + LB1 eta, U2 -= LA2 + LB2 xi (xi, eta the
  // particle's bilinear coordinates in its cell), one float4 of its own
  PF_LA1 = 36, PF_LB1, PF_LA2, PF_LB2,
  PF_STRIDE = 40
};
static_assert(PF_E2 < PF_LA1 && PF_LA1 % 4 == 0 && PF_STRIDE % 4 == 0, "packed record: float4 groups");

// Stages of the fused per-cell particle pass (update kernel).
enum : uint32_t {
  ST_RNG = 1u << 0,       // draw + whiten normals (random_generator)
  ST_STORE_XI = 1u << 1,  // keep whitened normals in the session (split mode)
  ST_LOAD_XI = 1u << 2,   // take whitened normals from the session (split mode)
  ST_FP = 1u << 3,        // Velocity_FP_parallel
  ST_LR = 1u << 4,        // long-range kick U2 += F2 dt
  ST_DFP = 1u << 5,       // DFP_extra_streaming
  ST_BC1 = 1u << 6,       // apply_BC before store_old_positions
  ST_OLD = 1u << 7,       // store_old_positions
  ST_STREAM = 1u << 8,    // free flight
  ST_BC2 = 1u << 9,       // apply_BC after streaming
  ST_BC3 = 1u << 10,      // the third apply_BC of the loop body
  ST_KEY = 1u << 11       // bin the new positions for the next cell_update
};

// Counter-stream ids for the Philox draws (third counter word).
enum : uint32_t { RNG_FP = MCPM_RNG_STREAM_FP, RNG_BC = MCPM_RNG_STREAM_BC, RNG_ESMC = MCPM_RNG_STREAM_ESMC,
                  RNG_BIN = MCPM_RNG_STREAM_BIN, RNG_ESMC_ACC = MCPM_RNG_STREAM_ESMC_ACC,
                  RNG_ESMC_M = MCPM_RNG_STREAM_ESMC_M, RNG_DSMC = MCPM_RNG_STREAM_DSMC,
                  RNG_DSMC_ACC = MCPM_RNG_STREAM_DSMC_ACC, RNG_DSMC_M = MCPM_RNG_STREAM_DSMC_M,
                  RNG_ADDREM_DEL = MCPM_RNG_STREAM_ADDREM_DEL, RNG_ADDREM_NEW = MCPM_RNG_STREAM_ADDREM_NEW,
                  RNG_COUNT = MCPM_RNG_STREAM_COUNT };

struct DevConsts {
  int N0, N1, C;
  int dir0, dir1;
  int problem, model, long_range;
  double dx, dy, dz, L0, L1;
  double sigma, m, kb, n, Fn, T0, mu, visp, b, dt, phi, eqdist, ast, bst;
  double Tw[4], Uw[4];
  uint64_t seed;
  // the Philox key of each of the ten rounds for this seed (formed once on
  // the host: the draws then read the round keys from the parameter bank)
  uint32_t rk[20];
  // wall offset of the diffuse walls, max(1e-15, 4 ulp(Len)) per direction
  double eps_x, eps_y;
  // 2-D long range: 1 when the Vlasov force acts on the node grid of a 2-D
  // box; its coefficient (phi for the direct path, ast for screened Poisson)
  int lr2d;
  double lr_coef;
  // quotients of constants for the FP32 sessions' per-cell solve (formed
  // once on the host): m/(3 kb), m/kb, kb/m, 1/dy, 1/m
  double q_T, q_m_kb, q_kb_m, q_idy, q_im;
  // DSMC_VHS: exponent 2 - 2 visp of the relative speed and the factor
  // crref^(2 visp - 1) of sigma_T (src/collisions.cpp:2102)
  double vhs_e, vhs_cr;
  // density expansion: pow(sigma 2^(1/6), 3) (src/Main_Functions.cpp:1647),
  // sqrt(2 pi) and pow(1/h/h, 2) with h = dy/2 of the kernel smoothing (:2380-2393)
  double de_p, de_s2p, de_s2h2;
  // float copies for the FP32 kernels
  float f_dx, f_dy, f_L0, f_L1, f_dt, f_sigma, f_m, f_kb, f_Tw[4], f_Uw[4], f_idx, f_idy, f_eps_x, f_eps_y;
  // FP32 binning.  f_face_x[j] (j = 0..N0) is the smallest float x with
  // floor((double)x / dx) >= j, +inf at j = N0 + 1; f_face_y likewise over
  // dy.  f_bin_wx / f_bin_wy: where the fraction of x * (1/dx) in float lies
  // within this distance of an integer, the float quotient may sit on the
  // wrong side of a face (or within the reference's 1e-15 jitter band), and
  // the cell is taken from the face table instead.
  const float* f_face_x;
  const float* f_face_y;
  float f_bin_wx, f_bin_wy;
  // the cells' weights (cells[].n_ratio) once set, else null (weight 1): the
  // cell density is n_ratio Fn N / V (src/Main_Functions.cpp:2588)
  const int32_t* cell_w;
  // injected draws per stream (mcpm_inject_uniforms): rng_inj_rows[st] rows
  // of four words in place of the Philox output, null for Philox
  const uint4* rng_inj[RNG_COUNT];
  uint32_t rng_inj_rows[RNG_COUNT];
};

// One set of device particle arrays (SoA).  real is float or double.
struct PBuf {
  void *x1, *x2, *U1, *U2, *U3, *x1o, *x2o;
  int32_t* pid;
};

// Work-list bookkeeping written by the scan kernel.
enum { WL_NSMALL = 0, WL_NBIG = 1, WL_MAXCNT = 2, WL_N = 3, WL_COUNT = 4 };
// Work counters used by the persistent kernels (reset by the scan kernel).
enum { WK_MOM_BIG = 0, WK_MOM_SMALL, WK_UPD_BIG, WK_UPD_SMALL, WK_COUNT };

struct Tuning {
  int wcap;         // cells with more particles than this go to the block path
  int block;        // threads per block of the persistent kernels
  int bcap;         // particles per cell staged in shared memory (block path)
  int grid_mom;     // persistent grid sizes
  int grid_upd;
};

struct LR2D;          // 2-D long-range tables and buffers (mcpm_lr2d.cu)
struct SurrogateNet;  // learned 2-D Vlasov force (mcpm_surrogate.cu)

struct Session {
  mcpm_config cfg{};
  DevConsts k{};
  int prec = MCPM_FP64;
  size_t rsz = 8;  // sizeof(real)
  int64_t N = 0, cap = 0;
  int C = 0;
  bool need_old = false;  // diffuse walls read positions before the last flight
  bool need_x1 = false;
  PBuf P[2]{};
  int cur = 0;
  int32_t* key = nullptr;       // cell of each slot, current layout
  int32_t* cnt = nullptr;       // [C] particles per cell, current layout
  int32_t* cnt_next = nullptr;  // [C] counts accumulated for the next layout
  int32_t* off = nullptr;       // [C+1] first slot of each cell, current layout
  int32_t* cursor = nullptr;    // [C]
  // Slotted layouts (FP32 fused steps): the particle pass writes each
  // particle straight into its new cell's region of the other buffer, a
  // region of capacity doff[c+1] - doff[c] with slack over the cell's count,
  // slots handed out by dcur; a region that fills up sends the rest to the
  // overflow arrays, and the repair after the next scan moves such cells,
  // overflow included, to spare slots past the layout
  int64_t slots = 0;            // slots per particle array (>= cap)
  int32_t* doff = nullptr;      // [C+1] region bases of the destination layout
  int32_t* noff = nullptr;      // [C+1] packed offsets of the totals (repair / compaction)
  int32_t* dcur = nullptr;      // [C] slots taken per destination region (= particles binned there)
  PBuf ovf{};                   // overflow particles (cap each)
  int32_t* ovf_key = nullptr;   // [cap] their cells
  int32_t* ovf_n = nullptr;     // [4] overflow counts (alternating between steps), spare cursor
  int ovf_par = 0;              // the overflow counter the next slotted pass uses
  bool use_slotted = false;     // the session writes slotted layouts (FP32)
  bool slotted = false;         // P[cur] holds a slotted layout (off = doff of that pass,
                                // counts in dcur): the next scan finalises it
  int32_t* list_small = nullptr;
  int32_t* list_big = nullptr;
  int32_t* wl = nullptr;        // [WL_COUNT]
  int32_t* work = nullptr;      // [WK_COUNT]
  int32_t* scan_blk = nullptr;  // [4][C/1024 + 1] block totals / bases of the scan
  double* cell = nullptr;       // [CF_DEV_COUNT][C]
  float* pcell = nullptr;       // [C][PF_STRIDE] packed FP32 record, then [2][C]: the cells'
                                // Y(n) and n as floats (the FP32 ESMC acceptance test)
  double* xi = nullptr;         // [3][cap] whitened normals, slot order
  double* inj = nullptr;        // [3][cap] injected raw normals, particle-id order
  uint4* rng_inj[RNG_COUNT] = {};  // injected words per stream (k.rng_inj points here)
  uint32_t rng_inj_gen = 0;        // bumped by every injection (captured steps are re-recorded)
  double* stage = nullptr;      // [5][cap] host<->device staging (double)
  double* faces = nullptr;      // [4][N1+1] long-range face scratch
  float* bin_faces = nullptr;   // [N0+2 + N1+2] FP32 binning face tables (DevConsts f_face_x/y)
  void* lr_tab = nullptr;       // long-range tables (stencil / PCR coefficients)
  alignas(16) char lr_host[160];  // the kernel's view of lr_tab
  LR2D* lr2d = nullptr;         // 2-D long range (node grid), when configured
  bool nodes_valid = false;     // nodal densities describe the last cell_update
  uint32_t* status = nullptr;
  int32_t* dstep = nullptr;     // device copy of the step number the kernels read
  int dstep_val = -1;           // the value it holds once queued work has run (-1: unknown)
  cudaStream_t stream = nullptr;
  // the learned force's branch of a fused step (nodal deposit + network)
  // runs on a stream of its own, beside the moment pass and the solves
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // on a judge step the branch runs the network on a stream of its own
  // beside the plain path (side2), joined before the comparison
  cudaStream_t side2 = nullptr;
  cudaEvent_t ev_fork2 = nullptr, ev_net = nullptr;
  // host transfers: uploads copy into stage_in on h2d, downloads copy out of
  // stage on d2h, so that a download's copies overlap the next upload's
  // (the host link runs both directions at once); the events order the
  // staging buffers' reuse and each field's conversion against its copy
  double* stage_in = nullptr;   // [5][cap] upload staging (double)
  cudaStream_t h2d = nullptr, d2h = nullptr;
  cudaEvent_t ev_in_free = nullptr, ev_out_free = nullptr, ev_up[5] = {}, ev_dn[5] = {};
  int step = 0;
  int bc_calls = 0;             // apply_BC calls in the current step (split mode)
  int rng_mode = MCPM_RNG_PHILOX;
  bool keys_current = false;    // key/cnt_next describe the current positions
  bool sorted = false;          // layout is sorted by key, cnt/off/lists valid
  bool needs_rebin = false;     // positions moved since the last binning
  bool have_particles = false;
  double* samples = nullptr;    // [MCPM_SF_COUNT][C] cell_poly_velocity accumulators
  // particle weights (the reference's n_ratio[]) in particle-id order, the
  // cells' weights (cells[].n_ratio), and the split / merge scratch
  int32_t* pw = nullptr;        // [cap]
  int32_t* pw_alt = nullptr;    // [cap] the weights in the new id order
  int32_t* cw = nullptr;        // [C]
  int8_t* ar_flag = nullptr;    // [cap] per particle id: 1 split, -1 deleted, 2 re-weighted, 0 kept
  int32_t* ar_ci = nullptr;     // [4][C] split, kept, kept weight, last kept id per cell
  double* ar_h = nullptr;       // [C] velocity spread of the copies
  int32_t* ar_newid = nullptr;  // [cap]
  int32_t* ar_srank = nullptr;  // [cap]
  int32_t* ar_tiles = nullptr;  // [2][tiles of the scan]
  unsigned long long* ar_tot = nullptr;  // [2] split, deleted
  double* p_m = nullptr;        // [C] measure_pressure accumulators (cells[].p_m)
  bool press = false;           // fused steps add their crossings to p_m
  bool omega_init = false;      // ESMC / DSMC majorant initialised (src/main.cpp:250-269)
  int num_sms = 0;
  Tuning tune{};
  int64_t launches = 0;
  cudaStream_t own_stream = nullptr;
  // profiling mode: CUDA-event pairs per launch, by kernel class
  bool prof = false;
  struct ProfRec { cudaEvent_t a, b; int cls; int n; };
  std::vector<ProfRec> prof_recs;
  std::vector<cudaEvent_t> prof_pool;
  // graph of two fused steps (the buffer pair returns to its start), replayed
  // by mcpm_step; rebuilt when its signature (stream, layout parity, stages,
  // tuning) changes
  cudaGraphExec_t graph = nullptr;
  uint64_t graph_sig = 0;
  int graph_launches = 0;
  bool use_graphs = true;
  // learned 2-D Vlasov force: attached network (not owned), the plain path
  // re-run as judge every sur_every steps, taking over while the relative
  // kick error exceeds sur_thr
  SurrogateNet* sur = nullptr;
  int sur_every = 10;
  double sur_thr = 0.01;
  bool sur_active = true;       // the network supplies the force
  bool sur_judge_now = false;   // this step runs both paths and compares
  bool sur_xin_ready = false;   // the nodal deposit also wrote the network input
  double* sur_err = nullptr;    // device [2]: sum |kick_net - kick_plain|^2, sum |kick_plain|^2
  double* sur_err_h = nullptr;  // pinned host copy
  cudaEvent_t ev_judge = nullptr;  // recorded after the verdict's copy to sur_err_h
  bool judge_pending = false;      // a judge step's verdict not yet read on the host
  double sur_last_err = -1.0;
  int64_t sur_judged = 0, sur_takeovers = 0, sur_steps = 0, sur_plain_steps = 0;
  std::string err;
};

// ------------------------------------------------------------- launchers
// (defined in mcpm_kernels.cu / mcpm_forces.cu; each returns the number of
// kernels it launched)
int launch_bin(Session& s, int bin_step);
int launch_scan(Session& s);
int launch_scatter(Session& s);
// slotted layouts: the scan that finalises one (counts from dcur, packed
// offsets, the next destination layout), the overflow repair (two launches
// that return at once when nothing overflowed; force: compact the layout
// into the other buffer instead, host-side)
int launch_scan_slotted(Session& s);
int launch_repair(Session& s);
int launch_compact(Session& s);
int launch_moments(Session& s);
int launch_solve(Session& s, int with_alpha);
// the FP32 sessions' variant (mcpm_solve_fast.cu, FP64 multiply-adds fused)
int launch_solve_fast(Session& s, int with_alpha, int fp_model);
// threads per block of the solves (fewer for grids with few cells)
int solve_block(const Session& s);
// slotted: write the new state into the slotted layout of the other buffer
// (FP32 passes that bin the new positions)
int launch_update(Session& s, uint32_t stages, int bc_call_base, bool slotted = false);
int launch_esmc(Session& s);
int launch_dsmc_vhs(Session& s);
int launch_smoothing(Session& s);
int launch_sample(Session& s);
int launch_long_range(Session& s);
int launch_init_omega(Session& s);
// 2-D long range (mcpm_lr2d.cu): set-up / release, the nodal deposit of
// cell_update, the node potential + kick coefficients, device views
int lr2d_setup(Session& s);
void lr2d_free(Session& s);
// count_density: also the cell densities from the layout's counts
// (lr2d_count_density), for a force that runs beside the per-cell solve
int launch_node_density(Session& s, bool count_density = false);
// n: the cell densities the force reads (null: the cell array's, which the
// per-cell solve writes)
int launch_long_range_2d(Session& s, const double* n = nullptr);
// the cell densities the last nodal deposit with count_density formed from
// the layout's counts (the per-cell solve's values)
const double* lr2d_count_density(const Session& s);
int launch_node_density_from(Session& s, const int32_t* qc);
int32_t* lr2d_quadrants(Session& s);
double* lr2d_node_density_mut(Session& s);
const double* lr2d_potential(const Session& s);
const double* lr2d_node_density(const Session& s);
int lr2d_num_nodes(const Session& s);
// the device step number made equal to s.step (a one-thread kernel when it
// differs); returns the launches it made
int sync_dstep(Session& s);
// the interface problems (mcpm_dynamic.cu): thermostat, and the split /
// merge of weighted particles -- flags and counts, then the move into the
// other buffer in the new id order, or the in-place re-weighting when
// nothing was split or deleted
int launch_thermostat(Session& s, double Tc, double Th, double thermc, double thermh);
int launch_addremove_flags(Session& s, int g, int step);
int launch_addremove_move(Session& s, int g, int step, int64_t n_kept);
int launch_addremove_reweight(Session& s);
int addremove_tiles(int64_t n);
// measure_pressure on the current state (x2, x2_old, U2) into p_m
int launch_pressure(Session& s);
// one staged upload field (0..4: x1 x2 U1 U2 U3; field 2 also sets the ids)
// on stream st
int launch_convert_field(Session& s, int field, int64_t n, cudaStream_t st);
// a staged field in particle-id order (doubles) into dst, a field of the
// current packed layout's slots
int launch_gather_field(Session& s, void* dst, const double* src);
// one download field (0..4: x1 x2 U1 U2 U3, 5..6: x1_old x2_old) into
// particle-id order in the stage, from the
// current layout (packed or slotted)
int launch_convert_out_field(Session& s, int field, int64_t n);
// the staging of a download straight from a slotted layout (FP32 sessions)

}  // namespace mcpm
