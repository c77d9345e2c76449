// mcpm_session.cu -- the C-ABI of include/mcpm.h: session lifetime, host
// copies, and the order in which the step's kernels run.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "mcpm_internal.h"
#include "mcpm_surrogate.h"

// particles per block staged in shared memory by the FP32 particle pass
// (bcap / 8 per warp): 36 KB per block, so that 6 blocks fit in an SM
#ifndef MCPM_UPD_BCAP
#define MCPM_UPD_BCAP 3072
#endif

namespace mcpm {
SurrogateNet* sur_net(mcpm_surrogate* m);
size_t update_smem_bytes(const Session& s);
int update_occupancy(const Session& s);
int moments_occupancy(const Session& s);
int long_range_setup(Session& s);
cudaError_t pcr_set_smem(int nf);
cudaError_t update_set_smem_max();

// ------------------------------------------------------- small kernels
__global__ void k_unpermute3(const double* src, const int32_t* pid, double* dst, int64_t n, int64_t cap) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int q = pid[i];
    dst[q] = src[i];
    dst[cap + q] = src[cap + i];
    dst[2 * cap + q] = src[2 * cap + i];
  }
}
// cell of every particle from the sorted segments (binary search in off)
__global__ void k_index(const int32_t* off, int C, const int32_t* pid, int32_t* out, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = C;  // find c with off[c] <= i < off[c+1]
    while (hi - lo > 1) {
      int mid = (lo + hi) >> 1;
      if (off[mid] <= i) lo = mid; else hi = mid;
    }
    out[pid[i]] = lo;
  }
}
__global__ void k_set_step(int32_t* dstep, int v) { *dstep = v; }
__global__ void k_step_advance(int32_t* dstep) { *dstep += 1; }

int sync_dstep(Session& s) {
  if (s.dstep_val == s.step) return 0;
  k_set_step<<<1, 1, 0, s.stream>>>(s.dstep, s.step);
  s.dstep_val = s.step;
  return 1;
}
}  // namespace mcpm

using namespace mcpm;

struct mcpm_session : public Session {};

static int fail(mcpm_session* s, int code, const char* msg) {
  if (s) s->err = msg;
  return code;
}

static int cuda_check(mcpm_session* s, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return MCPM_OK;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", where, cudaGetErrorString(e));
  s->err = buf;
  return MCPM_ERR_CUDA;
}

static int after_launch(mcpm_session* s, int n, const char* where) {
  s->launches += n;
  return cuda_check(s, cudaGetLastError(), where);
}

static cudaEvent_t prof_event(mcpm_session* s) {
  if (!s->prof_pool.empty()) {
    cudaEvent_t e = s->prof_pool.back();
    s->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}

// runs launcher f (which returns its launch count) inside an event pair
template <typename F> static int timed(mcpm_session* s, int cls, F f) {
  if (!s->prof) return f();
  cudaEvent_t a = prof_event(s), b = prof_event(s);
  cudaEventRecord(a, s->stream);
  int n = f();
  cudaEventRecord(b, s->stream);
  s->prof_recs.push_back({a, b, cls, n});
  return n;
}
#define T_BIN(x) timed(s, MCPM_K_BIN, [&] { return (x); })
#define T_SCAN(x) timed(s, MCPM_K_SCAN, [&] { return (x); })
#define T_SCAT(x) timed(s, MCPM_K_SCATTER, [&] { return (x); })
#define T_MOM(x) timed(s, MCPM_K_MOMENTS, [&] { return (x); })
#define T_SOLVE(x) timed(s, MCPM_K_SOLVE, [&] { return (x); })
#define T_ESMC(x) timed(s, MCPM_K_ESMC, [&] { return (x); })
#define T_LR(x) timed(s, MCPM_K_LONG_RANGE, [&] { return (x); })
#define T_UPD(x) timed(s, MCPM_K_UPDATE, [&] { return (x); })
#define T_SUR(x) timed(s, MCPM_K_SURROGATE, [&] { return (x); })

// FP32 binning.  face[c], c = 0..n: the smallest float x whose cell by the
// reference's rule, floor((double)x / d), is at least c; face[n + 1] = +inf.
// Division by a positive d is monotone, so the float cell of any x is the
// number of faces at or below it.
static void bin_face_table(float* face, int n, double d) {
  for (int c = 0; c <= n; ++c) {
    float f = (float)((double)c * d);
    const float lo = -INFINITY, hi = INFINITY;
    while (floor((double)nextafterf(f, lo) / d) >= c) f = nextafterf(f, lo);
    while (floor((double)f / d) < c) f = nextafterf(f, hi);
    face[c] = f;
  }
  face[n + 1] = INFINITY;
}

// Half-width of the band around an integer in which the fraction of the
// float quotient x * fl(1/d) is not trusted: its error is below 2^-23 of the
// quotient (two float roundings), at most n for a particle in the box; the
// band also covers the reference's face-jitter band of 1e-15 / d, plus a
// margin for the rounding of 1 - w in float.
static float bin_window(int n, double d) {
  const double w = 2.0 * ldexp(1.0, -23) * (n + 1) + 2e-15 / d + ldexp(1.0, -22);
  return (float)fmin(w, 0.5);
}

// the models random_generator and the FP velocity update serve
// (src/Fokker_Planck.cpp:22, src/Main_Functions.cpp:1565-1570)
static inline bool is_fp_model(int m) {
  return m == MCPM_MODEL_FP_DENSE || m == MCPM_MODEL_FP_IDEAL_GAS || m == MCPM_MODEL_FP_LINEAR;
}

extern "C" {
static int long_range_force(mcpm_session* s, bool branch = false);
static int read_judge(mcpm_session* s);

int mcpm_config_derive(mcpm_config* c, int64_t n_particles) {
  if (!c) return MCPM_ERR_ARG;
  const double pi = acos(-1.0);
  c->b = 2 * pi * pow(c->sigma, 3) / (3.0);  // src/myIO.cpp:2828
  if (!(c->T0 > 0)) c->T0 = 273.0;           // :2234
  if (!(c->visp > 0)) c->visp = 0.5;
  if (!(c->mu > 0)) c->mu = 5.0 / (16.0 * c->sigma * c->sigma) * sqrt(c->m * c->kb * c->T0 / acos(-1.0));  // :2829
  double vol = c->length[0] * c->length[1] * c->length[2];
  if (n_particles > 0) c->Fn = c->n * vol / n_particles;  // :2225
  if (!(c->eqdist > 0)) c->eqdist = c->sigma;
  if (c->seed == 0) c->seed = 0x4D43504Dull;
  if (c->max_particles < n_particles) c->max_particles = n_particles;
  return MCPM_OK;
}

int mcpm_session_create(const mcpm_config* cfg, mcpm_session** out) {
  if (!cfg || !out) return MCPM_ERR_ARG;
  *out = nullptr;
  const mcpm_config& c = *cfg;
  if (c.n_cells[0] < 1 || c.n_cells[1] < 1 || c.n_cells[2] != 1) return MCPM_ERR_ARG;
  if (c.direction[2] != 0 || c.max_particles < 1) return MCPM_ERR_ARG;
  if ((int64_t)c.n_cells[0] * c.n_cells[1] > (1 << 24)) return MCPM_ERR_ARG;
  if (c.max_particles > ((int64_t)1 << 31) - 1) return MCPM_ERR_ARG;
  if (c.precision != MCPM_FP64 && c.precision != MCPM_FP32) return MCPM_ERR_ARG;
  if (c.model < MCPM_MODEL_NONE || c.model > MCPM_MODEL_DSMC_VHS) return MCPM_ERR_ARG;
  if (c.model == MCPM_MODEL_DSMC_VHS && !(c.crref > 0)) return MCPM_ERR_ARG;
  if (c.problem != MCPM_PROBLEM_CLOSED_BOX && c.problem != MCPM_PROBLEM_COUETTE && c.problem != MCPM_PROBLEM_WALL &&
      c.problem != MCPM_PROBLEM_PERIODIC)
    return MCPM_ERR_ARG;
  if (c.long_range != MCPM_LR_NONE && c.long_range != MCPM_LR_DIRECT && c.long_range != MCPM_LR_SCREENED_POISSON &&
      c.long_range != MCPM_LR_DENSITY_EXPANSION)
    return MCPM_ERR_ARG;
  // the density-expansion force works per column of cells in any box
  if (c.long_range != MCPM_LR_NONE && c.long_range != MCPM_LR_DENSITY_EXPANSION) {
    if (c.direction[0] == 1) {
      // 2-D: the node-grid paths of src/FEM.cpp; the screened-Poisson solve
      // needs interior nodes and keeps two dense DST matrices of order <= 2047
      if (c.n_cells[0] > 2048 || c.n_cells[1] > 2048) return MCPM_ERR_ARG;
      if (c.long_range == MCPM_LR_SCREENED_POISSON && (c.n_cells[0] < 2 || c.n_cells[1] < 2)) return MCPM_ERR_ARG;
      if (c.long_range == MCPM_LR_SCREENED_POISSON && !(c.bst > 0)) return MCPM_ERR_ARG;
    } else if (c.n_cells[0] != 1 || c.n_cells[1] + 1 > 7000) {
      // the 1-D Vlasov routines index cells by row (src/Main_Functions.cpp:3772)
      return MCPM_ERR_ARG;
    }
  }
  if (!(c.sigma > 0 && c.m > 0 && c.kb > 0 && c.dt > 0 && c.mu > 0 && c.T0 > 0)) return MCPM_ERR_ARG;
  for (int i = 0; i < 2; ++i)
    if (!(c.length[i] > 0)) return MCPM_ERR_ARG;

  mcpm_session* s = new (std::nothrow) mcpm_session();
  if (!s) return MCPM_ERR_ARG;
  s->cfg = c;
  s->prec = c.precision;
  s->rsz = c.precision == MCPM_FP32 ? 4 : 8;
  s->cap = c.max_particles;
  s->C = c.n_cells[0] * c.n_cells[1];
  DevConsts& k = s->k;
  k.N0 = c.n_cells[0]; k.N1 = c.n_cells[1]; k.C = s->C;
  k.dir0 = c.direction[0]; k.dir1 = c.direction[1];
  k.problem = c.problem; k.model = c.model; k.long_range = c.long_range;
  k.dx = c.length[0] / c.n_cells[0]; k.dy = c.length[1] / c.n_cells[1]; k.dz = c.length[2] / c.n_cells[2];
  k.L0 = c.length[0]; k.L1 = c.length[1];
  k.sigma = c.sigma; k.m = c.m; k.kb = c.kb; k.n = c.n; k.Fn = c.Fn; k.T0 = c.T0; k.mu = c.mu; k.visp = c.visp;
  k.b = c.b; k.dt = c.dt; k.phi = c.phi; k.eqdist = c.eqdist; k.ast = c.ast; k.bst = c.bst;
  for (int i = 0; i < 4; ++i) { k.Tw[i] = c.T_wall[i]; k.Uw[i] = c.U_wall[i]; }
  k.seed = c.seed;
  for (int r = 0; r < 10; ++r) {
    k.rk[2 * r] = (uint32_t)c.seed + (uint32_t)r * 0x9E3779B9u;
    k.rk[2 * r + 1] = (uint32_t)(c.seed >> 32) + (uint32_t)r * 0xBB67AE85u;
  }
  k.lr2d = (c.long_range != MCPM_LR_NONE && c.long_range != MCPM_LR_DENSITY_EXPANSION && c.direction[0] == 1) ? 1 : 0;
  // 4 pi (sigma 2^(1/6))^3 of the density-expansion force, the pow factor
  // formed once as src/Main_Functions.cpp:1647 forms it
  k.de_p = pow(c.sigma * pow(2.0, 1.0 / 6.0), 3.0);
  k.de_s2p = sqrt(2.0 * acos(-1.0));
  {
    const double h = 2.0 * k.dy / 4.0;
    k.de_s2h2 = pow(1.0 / h / h, 2.0);
  }
  k.lr_coef = c.long_range == MCPM_LR_DIRECT ? c.phi : c.ast;
  k.q_T = c.m / (3.0 * c.kb);
  k.q_m_kb = c.m / c.kb;
  k.q_kb_m = c.kb / c.m;
  k.q_idy = 1.0 / k.dy;
  k.q_im = 1.0 / c.m;
  k.vhs_e = 2.0 - 2.0 * c.visp;
  k.vhs_cr = pow(c.crref, 2.0 * c.visp - 1.0);
  k.f_dx = (float)k.dx; k.f_dy = (float)k.dy; k.f_L0 = (float)k.L0; k.f_L1 = (float)k.L1;
  k.f_dt = (float)k.dt; k.f_sigma = (float)k.sigma; k.f_m = (float)k.m; k.f_kb = (float)k.kb;
  for (int i = 0; i < 4; ++i) { k.f_Tw[i] = (float)k.Tw[i]; k.f_Uw[i] = (float)k.Uw[i]; }
  k.f_idx = (float)(1.0 / k.dx); k.f_idy = (float)(1.0 / k.dy);
  // The reference offsets re-emitted particles by epsilon = 1e-15 from a
  // diffuse wall (src/Main_Functions.cpp:4933), an absolute length meant for
  // SI boxes; where 1e-15 is below the resolution of the box length the
  // offset is 4 ulp(Len) instead, in the precision of the particle state.
  k.eps_x = fmax(1e-15, 4.0 * (nextafter(k.L0, 2.0 * k.L0 + 1.0) - k.L0));
  k.eps_y = fmax(1e-15, 4.0 * (nextafter(k.L1, 2.0 * k.L1 + 1.0) - k.L1));
  k.f_eps_x = fmaxf(1e-15f, 4.0f * (nextafterf(k.f_L0, 2.0f * k.f_L0 + 1.0f) - k.f_L0));
  k.f_eps_y = fmaxf(1e-15f, 4.0f * (nextafterf(k.f_L1, 2.0f * k.f_L1 + 1.0f) - k.f_L1));
  s->need_old = (c.problem == MCPM_PROBLEM_COUETTE || c.problem == MCPM_PROBLEM_WALL);
  s->need_x1 = (c.direction[0] == 1 || c.model == MCPM_MODEL_ESMC || c.problem == MCPM_PROBLEM_COUETTE);

  int dev = 0;
  int rc;
  if ((rc = cuda_check(s, cudaGetDevice(&dev), "cudaGetDevice"))) { delete s; return rc; }
  cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, dev);
  if ((rc = cuda_check(s, cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "stream"))) { delete s; return rc; }
  s->own_stream = s->stream;
  if ((rc = cuda_check(s, cudaStreamCreateWithFlags(&s->side, cudaStreamNonBlocking), "stream"))) { delete s; return rc; }
  cudaEventCreateWithFlags(&s->ev_fork, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&s->ev_join, cudaEventDisableTiming);
  if ((rc = cuda_check(s, cudaStreamCreateWithFlags(&s->side2, cudaStreamNonBlocking), "stream"))) { mcpm_session_destroy(s); return rc; }
  cudaEventCreateWithFlags(&s->ev_fork2, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&s->ev_net, cudaEventDisableTiming);
  if ((rc = cuda_check(s, cudaStreamCreateWithFlags(&s->h2d, cudaStreamNonBlocking), "stream"))) { mcpm_session_destroy(s); return rc; }
  if ((rc = cuda_check(s, cudaStreamCreateWithFlags(&s->d2h, cudaStreamNonBlocking), "stream"))) { mcpm_session_destroy(s); return rc; }
  cudaEventCreateWithFlags(&s->ev_in_free, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&s->ev_out_free, cudaEventDisableTiming);
  for (int f = 0; f < 5; ++f) {
    cudaEventCreateWithFlags(&s->ev_up[f], cudaEventDisableTiming);
    cudaEventCreateWithFlags(&s->ev_dn[f], cudaEventDisableTiming);
  }

  // tuning defaults (see mcpm_tune in the Python layer for the sweep)
  s->tune.bcap = (s->prec == MCPM_FP32) ? MCPM_UPD_BCAP : 3072;
  // cells up to a warp's staging capacity (bcap / 8) go to one warp each: the
  // split mcpm_autotune picked on every benchmark workload; it can still
  // choose another
  s->tune.wcap = s->tune.bcap / 8;
  s->tune.block = 256;

  const size_t cap = (size_t)s->cap, C = (size_t)s->C, rs = s->rsz;
  // FP32 sessions write slotted layouts (MCPM_SLOTTED=0 keeps the packed
  // layout and its scatter pass): room for every region's slack -- a
  // quarter of the count, at least 16, rounded to 8 -- besides the particles
  const char* sl_env = getenv("MCPM_SLOTTED");
  s->use_slotted = s->prec == MCPM_FP32 && !(sl_env && sl_env[0] == '0');
  // and, past the layout, spare slots for the cells whose regions overflow
  s->slots = s->use_slotted ? (int64_t)(2 * cap + cap / 4 + 24 * C + 64) : (int64_t)cap;
  const size_t slots = (size_t)s->slots;
  auto A = [&](void** p, size_t bytes) -> bool { return cudaMalloc(p, bytes ? bytes : 16) == cudaSuccess; };
  bool ok = true;
  auto alloc_set = [&](PBuf& P, size_t n) {
    if (s->need_x1) ok = ok && A(&P.x1, n * rs);
    ok = ok && A(&P.x2, n * rs) && A(&P.U1, n * rs) && A(&P.U2, n * rs) && A(&P.U3, n * rs) &&
         A((void**)&P.pid, n * 4);
    if (s->need_old) {
      if (s->need_x1) ok = ok && A(&P.x1o, n * rs);
      ok = ok && A(&P.x2o, n * rs);
    }
  };
  for (int b = 0; b < 2 && ok; ++b) alloc_set(s->P[b], slots);
  if (s->use_slotted) {
    alloc_set(s->ovf, cap);
    ok = ok && A((void**)&s->ovf_key, cap * 4) && A((void**)&s->ovf_n, 16) && A((void**)&s->doff, (C + 1) * 4) &&
         A((void**)&s->noff, (C + 1) * 4) && A((void**)&s->dcur, C * 4);
  }
  ok = ok && A((void**)&s->key, cap * 4) && A((void**)&s->cnt, C * 4) && A((void**)&s->cnt_next, C * 4) &&
       A((void**)&s->off, (C + 1) * 4) && A((void**)&s->cursor, C * 4) && A((void**)&s->list_small, C * 4) &&
       A((void**)&s->list_big, C * 4) && A((void**)&s->wl, WL_COUNT * 4) && A((void**)&s->work, WK_COUNT * 4) &&
       A((void**)&s->scan_blk, 8 * (C / 1024 + 2) * 4) &&
       A((void**)&s->cell, (size_t)CF_DEV_COUNT * C * 8) && A((void**)&s->pcell, (size_t)(PF_STRIDE + 2) * C * 4) && A((void**)&s->xi, 3 * cap * 8) &&
       A((void**)&s->inj, 3 * cap * 8) && A((void**)&s->stage, 5 * cap * 8) && A((void**)&s->stage_in, 5 * cap * 8) &&
       A((void**)&s->faces, ((size_t)k.N1 + 1 + 5000) * 8) && A((void**)&s->status, 16) &&
       A((void**)&s->dstep, 16) && A((void**)&s->bin_faces, ((size_t)k.N0 + k.N1 + 4) * 4);
  if (!ok) {
    s->err = "out of device memory";
    mcpm_session_destroy(s);
    return MCPM_ERR_CUDA;
  }
  {
    // FP32 binning face tables and windows (DevConsts f_face_x / f_face_y)
    std::vector<float> ft((size_t)k.N0 + k.N1 + 4);
    bin_face_table(ft.data(), k.N0, k.dx);
    bin_face_table(ft.data() + k.N0 + 2, k.N1, k.dy);
    if ((rc = cuda_check(s, cudaMemcpy(s->bin_faces, ft.data(), ft.size() * 4, cudaMemcpyHostToDevice), "face tables"))) {
      mcpm_session_destroy(s);
      return rc;
    }
    k.f_face_x = s->bin_faces;
    k.f_face_y = s->bin_faces + k.N0 + 2;
    k.f_bin_wx = bin_window(k.N0, k.dx);
    k.f_bin_wy = bin_window(k.N1, k.dy);
  }
  cudaMemsetAsync(s->cnt_next, 0, C * 4, s->stream);
  if (s->use_slotted) {
    cudaMemsetAsync(s->dcur, 0, C * 4, s->stream);
    cudaMemsetAsync(s->ovf_n, 0, 16, s->stream);
  }
  cudaMemsetAsync(s->cell, 0, (size_t)CF_DEV_COUNT * C * 8, s->stream);
  cudaMemsetAsync(s->pcell, 0, (size_t)(PF_STRIDE + 2) * C * 4, s->stream);
  cudaMemsetAsync(s->status, 0, 16, s->stream);
  cudaMemsetAsync(s->work, 0, WK_COUNT * 4, s->stream);
  cudaMemsetAsync(s->inj, 0, 3 * cap * 8, s->stream);
  cudaMemsetAsync(s->xi, 0, 3 * cap * 8, s->stream);

  if ((rc = cuda_check(s, update_set_smem_max(), "smem attribute"))) { mcpm_session_destroy(s); return rc; }
  if (c.long_range != MCPM_LR_NONE && !k.lr2d)
    if ((rc = cuda_check(s, pcr_set_smem(k.N1 + 1), "long-range smem"))) { mcpm_session_destroy(s); return rc; }
  s->tune.grid_mom = s->num_sms * moments_occupancy(*s);
  s->tune.grid_upd = s->num_sms * update_occupancy(*s);
  if (!k.lr2d && long_range_setup(*s)) { s->err = "long-range tables"; mcpm_session_destroy(s); return MCPM_ERR_CUDA; }
  if (k.lr2d && lr2d_setup(*s)) {
    if (s->err.empty()) s->err = "2-D long-range tables";
    int code = s->err.find("memory") != std::string::npos ? MCPM_ERR_CUDA : MCPM_ERR_ARG;
    mcpm_session_destroy(s);
    return code;
  }
  if ((rc = cuda_check(s, cudaStreamSynchronize(s->stream), "session init"))) { mcpm_session_destroy(s); return rc; }
  *out = s;
  return MCPM_OK;
}

int mcpm_session_destroy(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->own_stream && s->own_stream != s->stream) cudaStreamSynchronize(s->own_stream);
  cudaFree(s->samples);
  cudaFree(s->pw); cudaFree(s->pw_alt); cudaFree(s->cw); cudaFree(s->ar_flag); cudaFree(s->ar_ci); cudaFree(s->ar_h);
  cudaFree(s->ar_newid); cudaFree(s->ar_srank); cudaFree(s->ar_tiles); cudaFree(s->ar_tot);
  cudaFree(s->p_m);
  for (int b = 0; b < 2; ++b) {
    PBuf& P = s->P[b];
    cudaFree(P.x1); cudaFree(P.x2); cudaFree(P.U1); cudaFree(P.U2); cudaFree(P.U3); cudaFree(P.pid);
    cudaFree(P.x1o); cudaFree(P.x2o);
  }
  {
    PBuf& P = s->ovf;
    cudaFree(P.x1); cudaFree(P.x2); cudaFree(P.U1); cudaFree(P.U2); cudaFree(P.U3); cudaFree(P.pid);
    cudaFree(P.x1o); cudaFree(P.x2o);
  }
  cudaFree(s->ovf_key); cudaFree(s->ovf_n); cudaFree(s->doff); cudaFree(s->noff); cudaFree(s->dcur);
  cudaFree(s->key); cudaFree(s->cnt); cudaFree(s->cnt_next); cudaFree(s->off); cudaFree(s->cursor);
  cudaFree(s->list_small); cudaFree(s->list_big); cudaFree(s->wl); cudaFree(s->work); cudaFree(s->scan_blk); cudaFree(s->cell); cudaFree(s->pcell);
  cudaFree(s->xi); cudaFree(s->inj); cudaFree(s->stage); cudaFree(s->faces); cudaFree(s->lr_tab); cudaFree(s->status); cudaFree(s->dstep);
  cudaFree(s->bin_faces);
  for (uint4* t : s->rng_inj) cudaFree(t);
  lr2d_free(*s);
  cudaFree(s->sur_err);
  if (s->sur_err_h) cudaFreeHost(s->sur_err_h);
  if (s->ev_judge) cudaEventDestroy(s->ev_judge);
  if (s->graph) cudaGraphExecDestroy(s->graph);
  for (auto& r : s->prof_recs) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto e : s->prof_pool) cudaEventDestroy(e);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  if (s->side) { cudaStreamSynchronize(s->side); cudaStreamDestroy(s->side); }
  if (s->side2) { cudaStreamSynchronize(s->side2); cudaStreamDestroy(s->side2); }
  if (s->ev_fork2) cudaEventDestroy(s->ev_fork2);
  if (s->ev_net) cudaEventDestroy(s->ev_net);
  if (s->h2d) { cudaStreamSynchronize(s->h2d); cudaStreamDestroy(s->h2d); }
  if (s->d2h) { cudaStreamSynchronize(s->d2h); cudaStreamDestroy(s->d2h); }
  if (s->ev_fork) cudaEventDestroy(s->ev_fork);
  if (s->ev_join) cudaEventDestroy(s->ev_join);
  if (s->ev_in_free) cudaEventDestroy(s->ev_in_free);
  if (s->ev_out_free) cudaEventDestroy(s->ev_out_free);
  for (int f = 0; f < 5; ++f) {
    if (s->ev_up[f]) cudaEventDestroy(s->ev_up[f]);
    if (s->ev_dn[f]) cudaEventDestroy(s->ev_dn[f]);
  }
  cudaFree(s->stage_in);
  delete s;
  return MCPM_OK;
}

const char* mcpm_last_error(const mcpm_session* s) { return s ? s->err.c_str() : "no session"; }

int mcpm_sync(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  int rc = cuda_check(s, cudaStreamSynchronize(s->stream), "sync");
  if (!rc && s->d2h) rc = cuda_check(s, cudaStreamSynchronize(s->d2h), "sync (downloads)");
  if (!rc && s->h2d) rc = cuda_check(s, cudaStreamSynchronize(s->h2d), "sync (uploads)");
  if (!rc) rc = read_judge(s);
  return rc;
}

int mcpm_check_status(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  uint32_t st = 0;
  int rc = cuda_check(s, cudaMemcpyAsync(&st, s->status, 4, cudaMemcpyDeviceToHost, s->stream), "status");
  if (rc) return rc;
  if ((rc = cuda_check(s, cudaStreamSynchronize(s->stream), "status sync"))) return rc;
  if (st) {
    cudaMemsetAsync(s->status, 0, 4, s->stream);
    char buf[200];
    snprintf(buf, sizeof buf, "device status 0x%x:%s%s%s%s", st, (st & MCPM_ERR_OUT_OF_BOX) ? " particle out of box" : "",
             (st & MCPM_ERR_NAN) ? " NaN" : "", (st & MCPM_ERR_BC_LOOP) ? " wall re-flight did not converge" : "",
             (st & MCPM_ERR_ITER_LIMIT) ? " iteration limit" : "");
    s->err = buf;
  }
  return (int)st;
}

// binning + counting sort into cell order (the front of cell_update)
// A slotted layout left by the fused step packed into the other buffer:
// everything but the fused step works on packed layouts [0, N).
static int leave_slotted(mcpm_session* s) {
  if (!s->slotted) return MCPM_OK;
  int n = T_SCAN(launch_compact(*s));
  s->slotted = false;
  s->sorted = true;
  s->keys_current = false;
  return after_launch(s, n, "compact");
}

static int sort_by_cell(mcpm_session* s) {
  if (s->slotted) return leave_slotted(s);
  int n = 0;
  if (!s->keys_current) n += T_BIN(launch_bin(*s, s->step));
  n += T_SCAN(launch_scan(*s));
  n += T_SCAT(launch_scatter(*s));
  s->sorted = true;
  s->keys_current = false;
  return after_launch(s, n, "sort_by_cell");
}

// the upload's copies, conversions and binning, without waiting for them
static int upload_enqueue(mcpm_session* s, int64_t n, const double* x1, const double* x2, const double* U1,
                          const double* U2, const double* U3) {
  if (!s || n < 0 || n > s->cap || !x2 || !U1 || !U2 || !U3) return fail(s, MCPM_ERR_ARG, "upload: bad arguments");
  if (!x1 && s->need_x1) return fail(s, MCPM_ERR_ARG, "upload: x1 required for this configuration");
  s->N = n;
  const size_t cap = (size_t)s->cap, b = (size_t)n * 8;
  cudaStream_t st = s->stream;
  s->cur = 0;
  int k = 0;
  const double* src[5] = {x1, x2, U1, U2, U3};
  // each field is copied into the upload staging on the h2d stream (after
  // the previous upload's conversions have read it) and converted on the
  // session stream while the next one is copied; a pending download's
  // copies run meanwhile on the d2h stream
  cudaStreamWaitEvent(s->h2d, s->ev_in_free, 0);
  for (int f = 0; f < 5; ++f) {
    if (src[f]) cudaMemcpyAsync(s->stage_in + f * cap, src[f], b, cudaMemcpyHostToDevice, s->h2d);
    else cudaMemsetAsync(s->stage_in + f * cap, 0, b, s->h2d);
    cudaEventRecord(s->ev_up[f], s->h2d);
    cudaStreamWaitEvent(st, s->ev_up[f], 0);
    k += launch_convert_field(*s, f, n, st);
  }
  cudaEventRecord(s->ev_in_free, st);
  const PBuf& P = s->P[0];
  if (P.x1o && P.x1) cudaMemcpyAsync(P.x1o, P.x1, (size_t)n * s->rsz, cudaMemcpyDeviceToDevice, st);
  if (P.x2o) cudaMemcpyAsync(P.x2o, P.x2, (size_t)n * s->rsz, cudaMemcpyDeviceToDevice, st);
  int rc = after_launch(s, k, "upload");
  if (rc) return rc;
  s->step = 0;
  s->bc_calls = 0;
  s->omega_init = false;
  s->sorted = false;
  s->slotted = false;
  s->have_particles = true;
  // the cell keys at step 0 (this also checks that every particle is in
  // the box); the layout follows at the first cell_update or step, which
  // re-draws the keys if the caller sets another step number first
  rc = after_launch(s, T_BIN(launch_bin(*s, s->step)), "upload");
  s->keys_current = rc == MCPM_OK;
  return rc;
}

int mcpm_upload_particles(mcpm_session* s, int64_t n, const double* x1, const double* x2, const double* U1,
                          const double* U2, const double* U3) {
  const int rc = upload_enqueue(s, n, x1, x2, U1, U2, U3);
  if (rc) return rc;
  // the caller may reuse its arrays once this returns: wait for the copies
  // (not for the conversions, nor for a pending download)
  return cuda_check(s, cudaEventSynchronize(s->ev_up[4]), "upload copies");
}

int mcpm_upload_particles_async(mcpm_session* s, int64_t n, const double* x1, const double* x2, const double* U1,
                                const double* U2, const double* U3) {
  return upload_enqueue(s, n, x1, x2, U1, U2, U3);
}

int mcpm_set_old_positions(mcpm_session* s, const double* x1_old, const double* x2_old) {
  if (!s || !x2_old || !s->have_particles) return fail(s, MCPM_ERR_ARG, "set_old_positions: bad arguments");
  int rc;
  if (s->slotted && (rc = leave_slotted(s))) return rc;
  const PBuf& P = s->P[s->cur];
  if (!P.x2o) return MCPM_OK;  // the session keeps no old positions (nothing reads them)
  const size_t b = (size_t)s->N * 8;
  cudaStreamWaitEvent(s->stream, s->ev_in_free, 0);
  const double* src[2] = {x1_old, x2_old};
  void* dst[2] = {P.x1o, P.x2o};
  int k = 0;
  for (int f = 0; f < 2; ++f) {
    if (!src[f] || !dst[f]) continue;
    cudaMemcpyAsync(s->stage_in + (size_t)f * s->cap, src[f], b, cudaMemcpyHostToDevice, s->stream);
    k += launch_gather_field(*s, dst[f], s->stage_in + (size_t)f * s->cap);
  }
  cudaEventRecord(s->ev_in_free, s->stream);
  if ((rc = after_launch(s, k, "set_old_positions"))) return rc;
  return cuda_check(s, cudaStreamSynchronize(s->stream), "set_old_positions");
}

int mcpm_get_old_positions(mcpm_session* s, double* x1_old, double* x2_old) {
  if (!s || !x2_old || !s->have_particles) return fail(s, MCPM_ERR_ARG, "get_old_positions: bad arguments");
  const PBuf& P = s->P[s->cur];
  if (!P.x2o) return fail(s, MCPM_ERR_STATE, "get_old_positions: the session keeps no old positions");
  const size_t cap = (size_t)s->cap, b = (size_t)s->N * 8;
  cudaStreamWaitEvent(s->stream, s->ev_out_free, 0);
  double* dst[2] = {P.x1o ? x1_old : nullptr, x2_old};
  int k = 0;
  for (int f = 0; f < 2; ++f) {
    if (!dst[f]) continue;
    k += launch_convert_out_field(*s, 5 + f, s->N);
    cudaMemcpyAsync(dst[f], s->stage + (5 + f - 5) * cap, b, cudaMemcpyDeviceToHost, s->stream);
  }
  int rc = after_launch(s, k, "get_old_positions");
  if (rc) return rc;
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_old_positions");
}

// the download's conversions and copies, without waiting for them
static int download_enqueue(mcpm_session* s, int64_t n, double* x1, double* x2, double* U1, double* U2, double* U3) {
  if (!s || n != s->N || !x2 || !U1 || !U2 || !U3) return fail(s, MCPM_ERR_ARG, "download: bad arguments");
  const size_t cap = (size_t)s->cap, b = (size_t)n * 8;
  cudaStream_t st = s->stream;
  // a slotted layout is staged as it lies (and stays slotted for the next
  // step); each field is converted on the session stream, once the previous
  // download's copies have left the staging, and copied out on the d2h
  // stream while the next one is converted.  x1 is not tracked when it never
  // changes (no x streaming, no ESMC): the caller's array is left as it is,
  // like the reference's x1
  double* dsts[5] = {(x1 && s->need_x1) ? x1 : nullptr, x2, U1, U2, U3};
  cudaStreamWaitEvent(st, s->ev_out_free, 0);
  int k = 0;
  for (int f = 0; f < 5; ++f) {
    if (!dsts[f]) continue;
    k += launch_convert_out_field(*s, f, n);
    cudaEventRecord(s->ev_dn[f], st);
    cudaStreamWaitEvent(s->d2h, s->ev_dn[f], 0);
    cudaMemcpyAsync(dsts[f], s->stage + (size_t)f * cap, b, cudaMemcpyDeviceToHost, s->d2h);
  }
  cudaEventRecord(s->ev_out_free, s->d2h);
  return after_launch(s, k, "download");
}

int mcpm_download_particles(mcpm_session* s, int64_t n, double* x1, double* x2, double* U1, double* U2, double* U3) {
  const int rc = download_enqueue(s, n, x1, x2, U1, U2, U3);
  if (rc) return rc;
  return cuda_check(s, cudaEventSynchronize(s->ev_out_free), "download");
}

int mcpm_download_particles_async(mcpm_session* s, int64_t n, double* x1, double* x2, double* U1, double* U2,
                                  double* U3) {
  return download_enqueue(s, n, x1, x2, U1, U2, U3);
}

int mcpm_cell_update(mcpm_session* s) {
  if (!s || !s->have_particles) return fail(s, MCPM_ERR_STATE, "cell_update: no particles");
  int rc;
  if (s->needs_rebin) { s->sorted = false; s->needs_rebin = false; }  // cell_update always re-bins
  if (!s->sorted && (rc = sort_by_cell(s))) return rc;
  int n = 0;
  cudaMemsetAsync(s->work, 0, WK_COUNT * 4, s->stream);
  n += T_MOM(launch_moments(*s));
  n += T_SOLVE(launch_solve(*s, (s->cfg.model == MCPM_MODEL_FP_DENSE && s->step > 0) ? 1 : 0));
  n += T_LR(launch_node_density(*s));  // n_n (src/Main_Functions.cpp:2268-2364), 2-D screened Poisson only
  s->nodes_valid = s->lr2d != nullptr;
  // kernel smoothing (src/Main_Functions.cpp:2378-2427), for long_range 2
  if (s->cfg.long_range == MCPM_LR_DENSITY_EXPANSION) n += T_LR(launch_smoothing(*s));
  return after_launch(s, n, "cell_update");
}

int mcpm_random_generator(mcpm_session* s) {
  if (!s || !s->sorted) return fail(s, MCPM_ERR_STATE, "random_generator: call cell_update first");
  if (!is_fp_model(s->cfg.model)) return MCPM_OK;  // src/Fokker_Planck.cpp:22
  cudaMemsetAsync(s->work, 0, WK_COUNT * 4, s->stream);
  return after_launch(s, T_UPD(launch_update(*s, ST_RNG | ST_STORE_XI, 0)), "random_generator");
}

int mcpm_velocity_update(mcpm_session* s) {
  if (!s || !s->sorted) return fail(s, MCPM_ERR_STATE, "velocity_update: call cell_update first");
  if (int rc = read_judge(s)) return rc;  // a queued step's verdict picks the force
  int n = 0;
  uint32_t stages = 0;
  if (s->cfg.model == MCPM_MODEL_ESMC) n += T_ESMC(launch_esmc(*s));
  else if (s->cfg.model == MCPM_MODEL_DSMC_VHS) n += T_ESMC(launch_dsmc_vhs(*s));
  else if (is_fp_model(s->cfg.model)) stages |= ST_LOAD_XI | ST_FP;
  if (s->cfg.long_range != MCPM_LR_NONE) {
    n += long_range_force(s);
    stages |= ST_LR;
  }
  if (stages) {
    cudaMemsetAsync(s->work, 0, WK_COUNT * 4, s->stream);
    n += T_UPD(launch_update(*s, stages, 0));
  }
  return after_launch(s, n, "velocity_update");
}

static int position_stage(mcpm_session* s, uint32_t stage, int base, const char* what) {
  if (!s || !s->have_particles) return fail(s, MCPM_ERR_STATE, "no particles");
  int rc;
  if (!s->sorted && (rc = sort_by_cell(s))) return rc;  // group by the last binning
  cudaMemsetAsync(s->work, 0, WK_COUNT * 4, s->stream);
  rc = after_launch(s, T_UPD(launch_update(*s, stage, base)), what);
  // positions changed: the layout is still grouped by the binning of this
  // step (which DFP_extra_streaming needs), but it is stale for the next one
  s->keys_current = false;
  s->sorted = true;
  s->needs_rebin = true;
  return rc;
}

int mcpm_dfp_extra_streaming(mcpm_session* s) {
  if (s && s->cfg.model != MCPM_MODEL_FP_DENSE) return MCPM_OK;  // src/main.cpp:478
  return position_stage(s, ST_DFP, 0, "dfp_extra_streaming");
}
int mcpm_apply_bc(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  int base = s->bc_calls++;
  return position_stage(s, ST_BC1, base, "apply_bc");
}
int mcpm_store_old_positions(mcpm_session* s) {
  if (s && !s->need_old) return MCPM_OK;
  return position_stage(s, ST_OLD, 0, "store_old_positions");
}
int mcpm_stream_particles(mcpm_session* s) { return position_stage(s, ST_STREAM, 0, "stream_particles"); }

int mcpm_end_step(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  s->step++;
  s->bc_calls = 0;
  if (s->needs_rebin) { s->sorted = false; s->needs_rebin = false; }
  return MCPM_OK;
}

// the long-range force of a step: the attached network while it is in
// charge, else the plain path -- and on a judge step the plain path (whose
// kick is kept) followed by the network and the comparison of the two.
// branch: it runs beside the per-cell solve, the plain path on the cell
// densities the nodal deposit formed from the layout's counts
static int long_range_force(mcpm_session* s, bool branch) {
  const double* ncell = s->cell + (size_t)MCPM_CF_N * s->C;
  if (s->sur && s->sur_active && !s->sur_judge_now)
    return T_SUR(sur_forward_kick(*s, lr2d_node_density(*s), ncell));
  if (branch && s->sur && s->sur_judge_now && s->side2) {
    // a judge step in the branch: the network's forward on a stream of its
    // own beside the plain path (their inputs are the deposit's, their
    // outputs apart), the comparison once both are done
    int n = 0;
    cudaEventRecord(s->ev_fork2, s->stream);
    cudaStreamWaitEvent(s->side2, s->ev_fork2, 0);
    cudaStream_t branch_stream = s->stream;
    s->stream = s->side2;
    n += T_SUR(sur_judge_forward(*s, lr2d_node_density(*s), ncell));
    cudaEventRecord(s->ev_net, s->side2);
    s->stream = branch_stream;
    n += T_LR(launch_long_range_2d(*s, lr2d_count_density(*s)));
    cudaStreamWaitEvent(s->stream, s->ev_net, 0);
    return n + T_SUR(sur_judge_compare(*s));
  }
  int n = T_LR(branch ? launch_long_range_2d(*s, lr2d_count_density(*s)) : launch_long_range(*s));
  if (s->sur && s->sur_judge_now) n += T_SUR(sur_judge(*s, lr2d_node_density(*s), ncell));
  return n;
}

// one iteration of the loop body as fused kernels; returns the launches
static int step_once(mcpm_session* s, uint32_t stages) {
  const int m = s->cfg.model;
  int n = 0;
  if (s->needs_rebin) { s->sorted = false; s->needs_rebin = false; }
  if (s->slotted) {
    // the last particle pass wrote a slotted layout: its counts, work lists
    // and the next destination layout, then the repair of overflowed
    // regions (two launches that return at once when none overflowed)
    n += T_SCAN(launch_scan_slotted(*s));
    n += T_SCAT(launch_repair(*s));
    s->slotted = false;
  } else if (!s->sorted) {
    if (!s->keys_current) n += T_BIN(launch_bin(*s, s->step));
    n += T_SCAN(launch_scan(*s));
    n += T_SCAT(launch_scatter(*s));
  } else {
    cudaMemsetAsync(s->work, 0, WK_COUNT * 4, s->stream);
  }
  // the 2-D long-range force's branch -- the nodal deposit from the new
  // layout's counts and quadrants, then the network's inference or the
  // plain screened-Poisson path (on the judge steps both and the judge),
  // each writing the kick -- needs no moments: its cell densities are the
  // deposit's, formed from the counts as the per-cell solve forms them.  So
  // it runs on the side stream while the moment pass and the solves run here
  const bool net = s->sur && s->sur_active && !s->sur_judge_now;
  const bool branch = !s->prof && s->side && s->lr2d && s->cfg.long_range != MCPM_LR_NONE &&
                      (net || s->cfg.long_range == MCPM_LR_SCREENED_POISSON);
  if (branch) {
    cudaEventRecord(s->ev_fork, s->stream);
    cudaStreamWaitEvent(s->side, s->ev_fork, 0);
    cudaStream_t main_stream = s->stream;
    s->stream = s->side;
    n += launch_node_density(*s, true);
    n += long_range_force(s, true);
    s->stream = main_stream;
    cudaEventRecord(s->ev_join, s->side);
  }
  n += T_MOM(launch_moments(*s));
  n += T_SOLVE(launch_solve(*s, (m == MCPM_MODEL_FP_DENSE && s->step > 0) ? 1 : 0));
  if (!branch) n += T_LR(launch_node_density(*s));
  s->nodes_valid = s->lr2d != nullptr;
  if (m == MCPM_MODEL_ESMC) n += T_ESMC(launch_esmc(*s));
  else if (m == MCPM_MODEL_DSMC_VHS) n += T_ESMC(launch_dsmc_vhs(*s));
  if (branch) cudaStreamWaitEvent(s->stream, s->ev_join, 0);
  else if (s->cfg.long_range != MCPM_LR_NONE) n += long_range_force(s);
  const bool slot = s->use_slotted && (stages & ST_KEY);
  n += T_UPD(launch_update(*s, stages, 0, slot));
  k_step_advance<<<1, 1, 0, s->stream>>>(s->dstep);
  ++n;
  s->step++;
  const bool press = s->press;
  s->dstep_val = s->step;
  s->bc_calls = 0;
  s->sorted = false;
  if (slot) {
    // the new state sits in the other buffer, laid out by doff
    s->cur = 1 - s->cur;
    std::swap(s->off, s->doff);
    s->ovf_par ^= 1;
    s->slotted = true;
    s->keys_current = false;
  } else {
    s->keys_current = true;
  }
  // measure_pressure after the flight and the walls (src/main.cpp:490-492)
  if (press) n += launch_pressure(*s);
  return n;
}

// everything a captured step depends on besides device memory
static uint64_t graph_signature(const mcpm_session* s, uint32_t stages) {
  uint64_t h = 1469598103934665603ull;
  auto mix = [&](uint64_t v) { h = (h ^ v) * 1099511628211ull; };
  mix((uint64_t)(uintptr_t)s->stream);
  mix((uint64_t)s->cur);
  mix((uint64_t)(uintptr_t)s->off);
  mix((uint64_t)(uintptr_t)s->doff);
  mix((uint64_t)(uintptr_t)s->noff);
  mix((uint64_t)s->ovf_par);
  mix((uint64_t)s->slotted);
  mix(stages);
  mix((uint64_t)s->tune.wcap);
  mix((uint64_t)s->tune.bcap);
  mix((uint64_t)s->tune.grid_mom);
  mix((uint64_t)s->tune.grid_upd);
  mix((uint64_t)s->rng_mode);
  mix((uint64_t)(uintptr_t)s->sur);
  mix((uint64_t)s->sur_active);
  mix((uint64_t)s->N);  // the particle count changes with splits and deletions
  mix((uint64_t)s->press);
  mix((uint64_t)(uintptr_t)s->k.cell_w);
  mix((uint64_t)s->rng_inj_gen);
  return h;
}

// record two steady-state steps into s->graph; the host-side state is left
// as before the capture (nothing has run yet)
static int capture_pair(mcpm_session* s, uint32_t stages, uint64_t sig) {
  if (s->graph) { cudaGraphExecDestroy(s->graph); s->graph = nullptr; }
  int rc = after_launch(s, sync_dstep(*s), "step");
  if (rc) return rc;
  const int step0 = s->step, cur0 = s->cur, dval0 = s->dstep_val, par0 = s->ovf_par;
  const int64_t launches0 = s->launches;
  const bool keys0 = s->keys_current, sorted0 = s->sorted, slotted0 = s->slotted;
  int32_t *off0 = s->off, *doff0 = s->doff, *noff0 = s->noff;
  cudaGraph_t g = nullptr;
  if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    s->use_graphs = false;
    return MCPM_OK;
  }
  int n = step_once(s, stages);
  n += step_once(s, stages);
  cudaError_t e = cudaStreamEndCapture(s->stream, &g);
  s->step = step0; s->cur = cur0; s->dstep_val = dval0; s->launches = launches0; s->ovf_par = par0;
  s->keys_current = keys0; s->sorted = sorted0; s->needs_rebin = false; s->slotted = slotted0;
  s->off = off0; s->doff = doff0; s->noff = noff0;
  if (e == cudaSuccess && g) e = cudaGraphInstantiate(&s->graph, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    // a stream that cannot be captured: run the steps eagerly from now on
    cudaGetLastError();
    s->graph = nullptr;
    s->use_graphs = false;
    return MCPM_OK;
  }
  s->graph_sig = sig;
  s->graph_launches = n;
  return MCPM_OK;
}

// n_steps consecutive steps without a judge step: eager steps until the
// layout is in its steady state (binned by the previous step's update
// kernel, not yet reordered), then pairs of steps as one CUDA graph (the
// scatter ping-pongs the buffer pair, so two steps leave every pointer where
// it started; the step number the kernels read lives on the device and the
// graph advances it), then the odd step eagerly
static int run_steps(mcpm_session* s, int n_steps, uint32_t stages) {
  int it = 0, rc;
  // steady state: the last fused step left a slotted layout, or keys for
  // the scan and scatter
  auto steady = [&]() {
    return !s->needs_rebin && (s->use_slotted ? s->slotted : (s->keys_current && !s->sorted));
  };
  while (it < n_steps && (!steady() || n_steps - it < 2 || s->prof || !s->use_graphs)) {
    if ((rc = after_launch(s, step_once(s, stages), "step"))) return rc;
    ++it;
  }
  const int pairs = (n_steps - it) / 2;
  if (pairs > 0) {
    const uint64_t sig = graph_signature(s, stages);
    if (!s->graph || s->graph_sig != sig) {
      if ((rc = capture_pair(s, stages, sig))) return rc;
    }
    if (s->graph) {
      if ((rc = after_launch(s, sync_dstep(*s), "step"))) return rc;
      for (int p = 0; p < pairs; ++p)
        if ((rc = cuda_check(s, cudaGraphLaunch(s->graph, s->stream), "graph launch"))) return rc;
      s->launches += (int64_t)pairs * s->graph_launches;
      s->step += 2 * pairs;
      s->dstep_val = s->step;
      it += 2 * pairs;
      s->nodes_valid = s->lr2d != nullptr;
    }
  }
  for (; it < n_steps; ++it)
    if ((rc = after_launch(s, step_once(s, stages), "step"))) return rc;
  return MCPM_OK;
}

// the judge's verdict: relative L2 error of the network's kick against the
// plain path's on the step just run
// the judge step's error sums go to the host behind the step; the verdict
// is read when the next step (or a query) needs it, so that an end-to-end
// loop queues the next batch's transfers before the host waits
static int queue_judge(mcpm_session* s) {
  if (!s->ev_judge) {
    int rc = cuda_check(s, cudaEventCreateWithFlags(&s->ev_judge, cudaEventDisableTiming), "judge event");
    if (rc) return rc;
  }
  cudaMemcpyAsync(s->sur_err_h, s->sur_err, 16, cudaMemcpyDeviceToHost, s->stream);
  int rc = cuda_check(s, cudaEventRecord(s->ev_judge, s->stream), "judge");
  s->judge_pending = rc == MCPM_OK;
  return rc;
}

static int read_judge(mcpm_session* s) {
  if (!s->judge_pending) return MCPM_OK;
  s->judge_pending = false;
  int rc = cuda_check(s, cudaEventSynchronize(s->ev_judge), "judge");
  if (rc) return rc;
  const double se = s->sur_err_h[0], sp = s->sur_err_h[1];
  const double e = sp > 0.0 ? sqrt(se / sp) : (se > 0.0 ? INFINITY : 0.0);
  s->sur_last_err = e;
  ++s->sur_judged;
  s->sur_active = e <= s->sur_thr;
  if (!s->sur_active) ++s->sur_takeovers;
  return MCPM_OK;
}

// queues n_steps iterations; after a judge step of an attached learned
// force the host reads the verdict before it queues the next step
static int step_enqueue(mcpm_session* s, int32_t n_steps) {
  if (!s || !s->have_particles || n_steps < 0) return fail(s, MCPM_ERR_STATE, "step: no particles");
  const int m = s->cfg.model;
  if ((m == MCPM_MODEL_ESMC || m == MCPM_MODEL_DSMC_VHS) && !s->omega_init) {
    // src/main.cpp:236-269: cell_update at the current positions, then the majorant
    int rc = mcpm_cell_update(s);
    if (rc) return rc;
    if ((rc = mcpm_init_omega_max(s))) return rc;
  }
  if (s->step == 0) {
    // the loop of src/main.cpp starts at step 1 (:389)
    int rc = mcpm_set_step(s, 1);
    if (rc) return rc;
  }
  uint32_t stages = ST_BC1 | ST_OLD | ST_STREAM | ST_BC2 | ST_BC3 | ST_KEY;
  if (is_fp_model(m)) stages |= ST_RNG | ST_FP;
  if (m == MCPM_MODEL_FP_DENSE) stages |= ST_DFP;
  if (s->cfg.long_range != MCPM_LR_NONE) stages |= ST_LR;
  if (!s->need_old) stages &= ~ST_OLD;
  int it = 0, rc;
  while (it < n_steps) {
    if ((rc = read_judge(s))) return rc;  // the last judge step's verdict picks this step's force
    if (s->sur && (s->step - 1) % s->sur_every == 0) {
      // judge step: both paths, the plain kick applied, eagerly
      s->sur_judge_now = true;
      rc = after_launch(s, step_once(s, stages), "step");
      s->sur_judge_now = false;
      if (rc || (rc = queue_judge(s))) return rc;
      ++s->sur_plain_steps;
      ++it;
      continue;
    }
    int run = n_steps - it;
    if (s->sur) run = std::min(run, s->sur_every - (s->step - 1) % s->sur_every);
    if (s->sur) (s->sur_active ? s->sur_steps : s->sur_plain_steps) += run;
    if ((rc = run_steps(s, run, stages))) return rc;
    it += run;
  }
  return MCPM_OK;
}

int mcpm_step(mcpm_session* s, int32_t n_steps) {
  int rc = step_enqueue(s, n_steps);
  if (!rc) rc = read_judge(s);
  return rc ? rc : mcpm_check_status(s);
}

int mcpm_step_async(mcpm_session* s, int32_t n_steps) { return step_enqueue(s, n_steps); }

// ------------------------------------------------- learned Vlasov force
int mcpm_attach_surrogate(mcpm_session* s, mcpm_surrogate* m, int32_t judge_every, double threshold) {
  if (!s) return MCPM_ERR_ARG;
  if (int rc = read_judge(s)) return rc;
  if (!m) {
    s->sur = nullptr;
    s->sur_xin_ready = false;
    return MCPM_OK;
  }
  SurrogateNet* n = sur_net(m);
  if (!s->lr2d || s->prec != MCPM_FP32)
    return fail(s, MCPM_ERR_ARG, "attach_surrogate: needs an FP32 session with a 2-D Vlasov force");
  if (n->N0 != s->k.N0 || n->N1 != s->k.N1) return fail(s, MCPM_ERR_ARG, "attach_surrogate: grid size differs");
  if (judge_every < 1 || !(threshold > 0.0)) return fail(s, MCPM_ERR_ARG, "attach_surrogate: bad judge settings");
  if (!s->sur_err) {
    if (cudaMalloc((void**)&s->sur_err, 16) != cudaSuccess || cudaMallocHost((void**)&s->sur_err_h, 16) != cudaSuccess) {
      cudaGetLastError();
      return fail(s, MCPM_ERR_CUDA, "attach_surrogate: out of memory");
    }
  }
  s->sur = n;
  s->sur_xin_ready = false;  // the next nodal deposit writes this network's input
  s->sur_every = judge_every;
  s->sur_thr = threshold;
  s->sur_active = true;
  s->sur_last_err = -1.0;
  s->sur_judged = s->sur_takeovers = s->sur_steps = s->sur_plain_steps = 0;
  return MCPM_OK;
}

int mcpm_get_surrogate_stats(mcpm_session* s, mcpm_surrogate_stats* out) {
  if (!s || !out) return MCPM_ERR_ARG;
  if (int rc = read_judge(s)) return rc;
  out->last_error = s->sur_last_err;
  out->judged = s->sur_judged;
  out->takeovers = s->sur_takeovers;
  out->surrogate_steps = s->sur_steps;
  out->plain_steps = s->sur_plain_steps;
  out->active = (s->sur && s->sur_active) ? 1 : 0;
  return MCPM_OK;
}

int mcpm_eval_vlasov_2d(mcpm_session* s, int32_t method) {
  if (!s || (method != 0 && method != 1)) return MCPM_ERR_ARG;
  if (!s->lr2d || !s->nodes_valid) return fail(s, MCPM_ERR_STATE, "eval_vlasov_2d: needs a 2-D session after cell_update");
  if (method == 1 && !s->sur) return fail(s, MCPM_ERR_STATE, "eval_vlasov_2d: no network attached");
  const double* ncell = s->cell + (size_t)MCPM_CF_N * s->C;
  int n = method == 0 ? T_LR(launch_long_range(*s)) : T_SUR(sur_forward_kick(*s, lr2d_node_density(*s), ncell));
  return after_launch(s, n, "eval_vlasov_2d");
}

int mcpm_get_kick_2d(mcpm_session* s, float* out) {
  if (!s || !out) return MCPM_ERR_ARG;
  if (!s->lr2d || s->prec != MCPM_FP32) return fail(s, MCPM_ERR_STATE, "get_kick_2d: needs an FP32 2-D session");
  cudaMemcpy2DAsync(out, 16, s->pcell + PF_LA1, PF_STRIDE * 4, 16, s->C, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_kick_2d");
}

int mcpm_vlasov_snapshots(mcpm_session* s, int32_t n_snap, const double* fields, int32_t n_waves, uint64_t seed,
                          uint16_t* x, float* y) {
  if (!s || n_snap < 0 || n_waves < 0 || !fields || !x || !y) return MCPM_ERR_ARG;
  if (!s->lr2d) return fail(s, MCPM_ERR_STATE, "vlasov_snapshots: needs a 2-D long-range session");
  const size_t per = 1 + 4 * (size_t)n_waves;
  double* fd = nullptr;
  int rc = cuda_check(s, cudaMalloc((void**)&fd, (size_t)n_snap * per * 8 + 8), "vlasov_snapshots");
  if (rc) return rc;
  cudaMemcpyAsync(fd, fields, (size_t)n_snap * per * 8, cudaMemcpyHostToDevice, s->stream);
  int n = 0;
  for (int i = 0; i < n_snap; ++i)
    n += sur_snapshot(*s, fd + i * per, n_waves, seed, (uint32_t)i, lr2d_quadrants(*s), lr2d_node_density_mut(*s),
                      s->cell + (size_t)MCPM_CF_N * s->C, x + (size_t)i * s->C * MCPM_SUR_IN,
                      y + (size_t)i * s->C * MCPM_SUR_OUT);
  rc = after_launch(s, n, "vlasov_snapshots");
  cudaStreamSynchronize(s->stream);
  cudaFree(fd);
  s->nodes_valid = true;  // the nodal data now describe the last snapshot
  s->sorted = false;
  return rc ? rc : cuda_check(s, cudaGetLastError(), "vlasov_snapshots");
}

int mcpm_inject_normals(mcpm_session* s, int64_t n, const double* a, const double* b, const double* c) {
  if (!s || n != s->N || !a || !b || !c) return fail(s, MCPM_ERR_ARG, "inject_normals: bad arguments");
  const size_t cap = (size_t)s->cap;
  cudaMemcpyAsync(s->inj, a, n * 8, cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(s->inj + cap, b, n * 8, cudaMemcpyHostToDevice, s->stream);
  cudaMemcpyAsync(s->inj + 2 * cap, c, n * 8, cudaMemcpyHostToDevice, s->stream);
  s->rng_mode = MCPM_RNG_INJECTED;
  return cuda_check(s, cudaGetLastError(), "inject_normals");
}

int mcpm_inject_uniforms(mcpm_session* s, int32_t stream, int64_t n_rows, const double* u) {
  if (!s || stream < 0 || stream >= (int32_t)RNG_COUNT || n_rows < 0 || n_rows > 0xFFFFFFFFll)
    return fail(s, MCPM_ERR_ARG, "inject_uniforms: bad arguments");
  int rc = cuda_check(s, cudaStreamSynchronize(s->stream), "inject_uniforms");  // no kernel reads the old table
  if (rc) return rc;
  cudaFree(s->rng_inj[stream]);
  s->rng_inj[stream] = nullptr;
  s->k.rng_inj[stream] = nullptr;
  s->k.rng_inj_rows[stream] = 0;
  ++s->rng_inj_gen;
  if (n_rows == 0 || !u) return MCPM_OK;
  std::vector<uint4> w((size_t)n_rows);
  auto word = [](double v) -> uint32_t {
    if (!(v > 0.0)) return 0u;  // also NaN
    const double t = std::floor(v * 4294967296.0);
    return t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
  };
  for (int64_t r = 0; r < n_rows; ++r)
    w[r] = make_uint4(word(u[4 * r]), word(u[4 * r + 1]), word(u[4 * r + 2]), word(u[4 * r + 3]));
  if (cudaMalloc((void**)&s->rng_inj[stream], (size_t)n_rows * sizeof(uint4)) != cudaSuccess) {
    s->rng_inj[stream] = nullptr;
    cudaGetLastError();
    return fail(s, MCPM_ERR_CUDA, "inject_uniforms: out of device memory");
  }
  cudaMemcpy(s->rng_inj[stream], w.data(), (size_t)n_rows * sizeof(uint4), cudaMemcpyHostToDevice);
  s->k.rng_inj[stream] = s->rng_inj[stream];
  s->k.rng_inj_rows[stream] = (uint32_t)n_rows;
  return cuda_check(s, cudaGetLastError(), "inject_uniforms");
}

int mcpm_set_rng(mcpm_session* s, int32_t mode) {
  if (!s || (mode != MCPM_RNG_PHILOX && mode != MCPM_RNG_INJECTED)) return MCPM_ERR_ARG;
  s->rng_mode = mode;
  return MCPM_OK;
}

int mcpm_sample_cells(mcpm_session* s) {
  if (!s || !s->sorted) return fail(s, MCPM_ERR_STATE, "sample_cells: call cell_update first");
  if (!s->samples) {
    const size_t b = (size_t)MCPM_SF_COUNT * s->C * 8;
    if (cudaMalloc(&s->samples, b) != cudaSuccess) {
      s->samples = nullptr;
      return fail(s, MCPM_ERR_CUDA, "sample_cells: no device memory for the accumulators");
    }
    cudaMemsetAsync(s->samples, 0, b, s->stream);
  }
  return after_launch(s, launch_sample(*s), "sample_cells");
}

int mcpm_get_samples(mcpm_session* s, double* out) {
  if (!s || !out) return MCPM_ERR_ARG;
  const size_t b = (size_t)MCPM_SF_COUNT * s->C * 8;
  if (!s->samples) {
    memset(out, 0, b);
    return MCPM_OK;
  }
  cudaMemcpyAsync(out, s->samples, b, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_samples");
}

int mcpm_reset_samples(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  if (s->samples) cudaMemsetAsync(s->samples, 0, (size_t)MCPM_SF_COUNT * s->C * 8, s->stream);
  return MCPM_OK;
}

int mcpm_get_cells(mcpm_session* s, double* out) {
  if (!s || !out) return MCPM_ERR_ARG;
  cudaMemcpyAsync(out, s->cell, (size_t)MCPM_CF_COUNT * s->C * 8, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_cells");
}

int mcpm_get_node_density(mcpm_session* s, double* out) {
  if (!s || !out) return MCPM_ERR_ARG;
  if (!s->lr2d || s->cfg.long_range != MCPM_LR_SCREENED_POISSON || !s->nodes_valid)
    return fail(s, MCPM_ERR_STATE, "get_node_density: needs a 2-D screened-Poisson session after cell_update");
  cudaMemcpyAsync(out, lr2d_node_density(*s), (size_t)s->C * 4 * 8, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_node_density");
}

int mcpm_get_node_potential(mcpm_session* s, double* out) {
  if (!s || !out) return MCPM_ERR_ARG;
  if (!s->lr2d) return fail(s, MCPM_ERR_STATE, "get_node_potential: needs a 2-D long-range session");
  cudaMemcpyAsync(out, lr2d_potential(*s), (size_t)lr2d_num_nodes(*s) * 8, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_node_potential");
}

// ------------------------------------------------------------ pressure
// measure_pressure (src/Main_Functions.cpp:13-34) needs the positions before
// the flight: sessions without diffuse walls do not keep them until
// sampling is switched on, which adds the old-position arrays (both buffer
// sets and the overflow) and the p_m accumulators
int mcpm_set_pressure_sampling(mcpm_session* s, int32_t on) {
  if (!s) return MCPM_ERR_ARG;
  if (!on) {
    s->press = false;
    return MCPM_OK;
  }
  if (!s->p_m) {
    if (cudaMalloc((void**)&s->p_m, (size_t)s->C * 8) != cudaSuccess) {
      s->p_m = nullptr;
      cudaGetLastError();
      return fail(s, MCPM_ERR_CUDA, "pressure sampling: out of device memory");
    }
    cudaMemsetAsync(s->p_m, 0, (size_t)s->C * 8, s->stream);
  }
  if (!s->need_old) {
    const size_t n = (size_t)s->slots;
    for (int b = 0; b < 2; ++b)
      if (!s->P[b].x2o && cudaMalloc(&s->P[b].x2o, n * s->rsz) != cudaSuccess) {
        cudaGetLastError();
        return fail(s, MCPM_ERR_CUDA, "pressure sampling: out of device memory");
      }
    if (s->use_slotted && !s->ovf.x2o && cudaMalloc(&s->ovf.x2o, (size_t)s->cap * s->rsz) != cudaSuccess) {
      cudaGetLastError();
      return fail(s, MCPM_ERR_CUDA, "pressure sampling: out of device memory");
    }
    // the old positions start as the current ones
    if (s->have_particles) {
      if (s->slotted) {
        int rc = leave_slotted(s);
        if (rc) return rc;
      }
      cudaMemcpyAsync(s->P[s->cur].x2o, s->P[s->cur].x2, (size_t)s->N * s->rsz, cudaMemcpyDeviceToDevice, s->stream);
    }
    s->need_old = true;
  }
  s->press = true;
  return cuda_check(s, cudaStreamSynchronize(s->stream), "pressure sampling");
}

int mcpm_measure_pressure(mcpm_session* s) {
  if (!s || !s->have_particles) return fail(s, MCPM_ERR_STATE, "measure_pressure: no particles");
  if (!s->p_m) return fail(s, MCPM_ERR_STATE, "measure_pressure: switch pressure sampling on first");
  return after_launch(s, launch_pressure(*s), "measure_pressure");
}

int mcpm_get_pressure(mcpm_session* s, double* p_m) {
  if (!s || !p_m) return MCPM_ERR_ARG;
  if (!s->p_m) {
    memset(p_m, 0, (size_t)s->C * 8);
    return MCPM_OK;
  }
  cudaMemcpyAsync(p_m, s->p_m, (size_t)s->C * 8, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_pressure");
}

int mcpm_reset_pressure(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  if (s->p_m) cudaMemsetAsync(s->p_m, 0, (size_t)s->C * 8, s->stream);
  return MCPM_OK;
}

// ------------------------------------------------------------- output
int mcpm_write_post_processing(mcpm_session* s, int32_t step, double t_post, const char* dir,
                               const char* output_name, char* path, int32_t path_len) {
  if (!s || !dir || !output_name) return MCPM_ERR_ARG;
  const size_t C = (size_t)s->C;
  std::vector<double> cells((size_t)MCPM_CF_COUNT * C), samples, pm;
  std::vector<int32_t> cw;
  int rc = mcpm_get_cells(s, cells.data());
  if (rc) return rc;
  if (s->samples) {
    samples.resize((size_t)MCPM_SF_COUNT * C);
    if ((rc = mcpm_get_samples(s, samples.data()))) return rc;
  }
  if (s->p_m) {
    pm.resize(C);
    if ((rc = mcpm_get_pressure(s, pm.data()))) return rc;
  }
  if (s->cw) {
    cw.resize(C);
    cudaMemcpyAsync(cw.data(), s->cw, C * 4, cudaMemcpyDeviceToHost, s->stream);
    if ((rc = cuda_check(s, cudaStreamSynchronize(s->stream), "write_post_processing"))) return rc;
  }
  rc = mcpm_post_processing_write(&s->cfg, step, t_post, dir, output_name, cells.data(),
                                  samples.empty() ? nullptr : samples.data(), pm.empty() ? nullptr : pm.data(),
                                  cw.empty() ? nullptr : cw.data(), path, path_len);
  return rc ? fail(s, rc, "write_post_processing: cannot write the file") : MCPM_OK;
}

// ------------------------------------------------ interface problems
// the weights' arrays and the split / merge scratch, allocated on first use
static int weights_alloc(mcpm_session* s) {
  if (s->pw) return MCPM_OK;
  const size_t cap = (size_t)s->cap, C = (size_t)s->C;
  auto A = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes ? bytes : 16) == cudaSuccess; };
  const bool ok = A((void**)&s->pw, cap * 4) && A((void**)&s->pw_alt, cap * 4) && A((void**)&s->cw, C * 4) &&
                  A((void**)&s->ar_flag, cap) && A((void**)&s->ar_ci, 4 * C * 4) && A((void**)&s->ar_h, C * 8) &&
                  A((void**)&s->ar_newid, cap * 4) && A((void**)&s->ar_srank, cap * 4) &&
                  A((void**)&s->ar_tiles, 2 * ((size_t)addremove_tiles(s->cap) + 1) * 4) &&
                  A((void**)&s->ar_tot, 16);
  if (!ok) {
    cudaGetLastError();
    return fail(s, MCPM_ERR_CUDA, "weights: out of device memory");
  }
  // until the caller sets them, every particle and cell weighs 1
  std::vector<int32_t> one(cap > C ? cap : C, 1);
  cudaMemcpy(s->pw, one.data(), cap * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(s->cw, one.data(), C * 4, cudaMemcpyHostToDevice);
  s->k.cell_w = s->cw;
  return cuda_check(s, cudaGetLastError(), "weights");
}

int mcpm_set_particle_weights(mcpm_session* s, const int32_t* w) {
  if (!s || !w || !s->have_particles) return fail(s, MCPM_ERR_ARG, "set_particle_weights: no particles");
  int rc = weights_alloc(s);
  if (rc) return rc;
  cudaMemcpyAsync(s->pw, w, (size_t)s->N * 4, cudaMemcpyHostToDevice, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "set_particle_weights");
}

int mcpm_get_particle_weights(mcpm_session* s, int32_t* w) {
  if (!s || !w || !s->have_particles) return fail(s, MCPM_ERR_ARG, "get_particle_weights: no particles");
  int rc = weights_alloc(s);
  if (rc) return rc;
  cudaMemcpyAsync(w, s->pw, (size_t)s->N * 4, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_particle_weights");
}

int mcpm_set_cell_weights(mcpm_session* s, const int32_t* w) {
  if (!s || !w) return fail(s, MCPM_ERR_ARG, "set_cell_weights: bad arguments");
  int rc = weights_alloc(s);
  if (rc) return rc;
  cudaMemcpyAsync(s->cw, w, (size_t)s->C * 4, cudaMemcpyHostToDevice, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "set_cell_weights");
}

int mcpm_thermostat(mcpm_session* s, double Tc, double Th, double thermc, double thermh) {
  if (!s || !s->have_particles) return fail(s, MCPM_ERR_STATE, "thermostat: no particles");
  int rc;
  if (s->slotted && (rc = leave_slotted(s))) return rc;
  if (!s->sorted) return fail(s, MCPM_ERR_STATE, "thermostat: call cell_update first");
  return after_launch(s, launch_thermostat(*s, Tc, Th, thermc, thermh), "thermostat");
}

int mcpm_addremove_particles(mcpm_session* s, int32_t n_ratio, int64_t* n_out) {
  if (!s || !s->have_particles) return fail(s, MCPM_ERR_STATE, "addremove: no particles");
  if (n_ratio < 1) return fail(s, MCPM_ERR_ARG, "addremove: n_ratio must be >= 1");
  int rc = weights_alloc(s);
  if (rc) return rc;
  // the cells of the last binning (the reference's index[] of its last
  // cell_update), grouped
  if (s->slotted) {
    if ((rc = leave_slotted(s))) return rc;
  } else if (s->needs_rebin || !s->sorted) {
    s->needs_rebin = false;
    s->sorted = false;
    if ((rc = sort_by_cell(s))) return rc;
  }
  if ((rc = after_launch(s, launch_addremove_flags(*s, n_ratio, s->step), "addremove"))) return rc;
  unsigned long long tot[2] = {0, 0};
  cudaMemcpyAsync(tot, s->ar_tot, sizeof tot, cudaMemcpyDeviceToHost, s->stream);
  if ((rc = cuda_check(s, cudaStreamSynchronize(s->stream), "addremove counts"))) return rc;
  const int64_t n_split = (int64_t)tot[0], n_del = (int64_t)tot[1];
  if (n_split == 0 && n_del == 0) {
    // nothing split or deleted: the kept light particles take their cell's weight
    if ((rc = after_launch(s, launch_addremove_reweight(*s), "addremove"))) return rc;
    if (n_out) *n_out = s->N;
    return cuda_check(s, cudaStreamSynchronize(s->stream), "addremove");
  }
  const int64_t n_kept = s->N - n_del, n_new = (int64_t)(n_ratio - 1) * n_split;
  if (n_kept + n_new > s->cap) return fail(s, MCPM_ERR_CAPACITY, "addremove: the new particles exceed max_particles");
  if ((rc = after_launch(s, launch_addremove_move(*s, n_ratio, s->step, n_kept), "addremove"))) return rc;
  // the new state sits in the other buffer in the new id order
  s->cur = 1 - s->cur;
  s->N = n_kept + n_new;
  std::swap(s->pw, s->pw_alt);
  s->sorted = false;
  s->keys_current = false;
  s->needs_rebin = false;
  s->slotted = false;
  s->rng_mode = MCPM_RNG_PHILOX;  // injected normals were per old particle id
  if (n_out) *n_out = s->N;
  return cuda_check(s, cudaStreamSynchronize(s->stream), "addremove");
}

int mcpm_get_index(mcpm_session* s, int32_t* index) {
  if (!s || !index || !s->have_particles) return MCPM_ERR_ARG;
  int rc;
  if (s->needs_rebin || !s->sorted) {
    if (s->needs_rebin) { s->sorted = false; s->needs_rebin = false; }
    if ((rc = sort_by_cell(s))) return rc;
  }
  int32_t* tmp = (int32_t*)s->stage;
  cudaStreamWaitEvent(s->stream, s->ev_out_free, 0);  // a pending download's copies read the staging
  k_index<<<(int)((s->N + 255) / 256 > 4096 ? 4096 : (s->N + 255) / 256 + 1), 256, 0, s->stream>>>(s->off, s->C, s->P[s->cur].pid, tmp, s->N);
  if ((rc = after_launch(s, 1, "get_index"))) return rc;
  cudaMemcpyAsync(index, tmp, (size_t)s->N * 4, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_index");
}

int mcpm_get_normals(mcpm_session* s, double* a, double* b, double* c) {
  if (!s || !a || !b || !c) return MCPM_ERR_ARG;
  int rc0 = leave_slotted(s);
  if (rc0) return rc0;
  const size_t cap = (size_t)s->cap;
  cudaStreamWaitEvent(s->stream, s->ev_out_free, 0);  // a pending download's copies read the staging
  k_unpermute3<<<(int)((s->N + 255) / 256 > 4096 ? 4096 : (s->N + 255) / 256 + 1), 256, 0, s->stream>>>(s->xi, s->P[s->cur].pid, s->stage, s->N, s->cap);
  int rc = after_launch(s, 1, "get_normals");
  if (rc) return rc;
  cudaMemcpyAsync(a, s->stage, s->N * 8, cudaMemcpyDeviceToHost, s->stream);
  cudaMemcpyAsync(b, s->stage + cap, s->N * 8, cudaMemcpyDeviceToHost, s->stream);
  cudaMemcpyAsync(c, s->stage + 2 * cap, s->N * 8, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_normals");
}

int mcpm_get_layout(mcpm_session* s, int32_t* pid_by_slot, int32_t* off) {
  if (!s || !pid_by_slot || !off) return MCPM_ERR_ARG;
  if (!s->sorted) return fail(s, MCPM_ERR_STATE, "get_layout: layout not sorted; call cell_update first");
  cudaMemcpyAsync(pid_by_slot, s->P[s->cur].pid, (size_t)s->N * 4, cudaMemcpyDeviceToHost, s->stream);
  cudaMemcpyAsync(off, s->off, (size_t)(s->C + 1) * 4, cudaMemcpyDeviceToHost, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "get_layout");
}

int32_t mcpm_get_step(const mcpm_session* s) { return s ? s->step : -1; }
int mcpm_set_step(mcpm_session* s, int32_t step) {
  if (!s || step < 0) return MCPM_ERR_ARG;
  if (step != s->step && s->have_particles) {
    // the face jitter of the binning draws by step number: keys drawn at
    // another step are re-drawn by the next cell_update or step
    s->keys_current = false;
    if (s->slotted) {
      const int rc = leave_slotted(s);
      if (rc) return rc;
    }
    if (s->sorted) s->needs_rebin = true;
  }
  s->step = step;
  s->bc_calls = 0;
  return MCPM_OK;
}

int mcpm_set_cell_field(mcpm_session* s, int32_t f, const double* v) {
  if (!s || !v || f < 0 || f >= MCPM_CF_COUNT) return MCPM_ERR_ARG;
  cudaMemcpyAsync(s->cell + (size_t)f * s->C, v, (size_t)s->C * 8, cudaMemcpyHostToDevice, s->stream);
  return cuda_check(s, cudaStreamSynchronize(s->stream), "set_cell_field");
}

int mcpm_init_omega_max(mcpm_session* s) {
  if (!s) return MCPM_ERR_ARG;
  s->omega_init = true;
  return after_launch(s, launch_init_omega(*s), "init_omega_max");
}

int64_t mcpm_kernel_launches(const mcpm_session* s) { return s ? s->launches : -1; }

int mcpm_set_wcap(mcpm_session* s, int32_t wcap) {
  if (!s || wcap < 1 || wcap > s->tune.bcap / 8) return MCPM_ERR_ARG;
  s->tune.wcap = wcap;
  s->sorted = s->sorted && !s->have_particles;  // the work lists are rebuilt by the next scan
  if (s->have_particles) s->keys_current = false;
  return MCPM_OK;
}
int32_t mcpm_get_wcap(const mcpm_session* s) { return s ? s->tune.wcap : -1; }

// Autotuner: times `steps` fused steps for each candidate threads-per-cell
// split (cells up to wcap particles get a warp, larger ones a block) on the
// session's own particles, restoring the full state after every trial, and
// keeps the fastest.  The particle state is unchanged on return.
int mcpm_autotune(mcpm_session* s, int32_t steps, int32_t* chosen) {
  if (!s || !s->have_particles || steps < 1) return MCPM_ERR_STATE;
  int rc = leave_slotted(s);  // the trials start from a packed layout
  if (rc) return rc;
  const size_t rs = s->rsz, N = (size_t)s->N, C = (size_t)s->C;
  const PBuf& P = s->P[s->cur];
  void* arrs[7] = {P.x1, P.x2, P.U1, P.U2, P.U3, P.x1o, P.x2o};
  size_t bytes = 0;
  for (int i = 0; i < 7; ++i) if (arrs[i]) bytes += N * rs;
  bytes += N * 4 + (size_t)CF_DEV_COUNT * C * 8 + (size_t)PF_STRIDE * C * 4;
  char* save = nullptr;
  rc = cuda_check(s, cudaMalloc(&save, bytes), "autotune scratch");
  if (rc) return rc;
  cudaStream_t st = s->stream;
  auto copy_all = [&](bool to_save) {
    size_t o = 0;
    auto cp = [&](void* p, size_t b) {
      if (!p) return;
      if (to_save) cudaMemcpyAsync(save + o, p, b, cudaMemcpyDeviceToDevice, st);
      else cudaMemcpyAsync(p, save + o, b, cudaMemcpyDeviceToDevice, st);
      o += b;
    };
    for (int i = 0; i < 7; ++i) cp(arrs[i], N * rs);
    cp(P.pid, N * 4);
    cp(s->cell, (size_t)CF_DEV_COUNT * C * 8);
    cp(s->pcell, (size_t)PF_STRIDE * C * 4);
  };
  const int cur0 = s->cur, step0 = s->step;
  const bool sorted0 = s->sorted, keys0 = s->keys_current, rebin0 = s->needs_rebin, om0 = s->omega_init;
  const int64_t launches0 = s->launches;
  copy_all(true);
  // the fixed splits, and the largest cell a warp can stage (bcap / 8)
  const int cands[6] = {128, 256, 384, 512, 768, s->tune.bcap / 8};
  int best = s->tune.wcap;
  float best_ms = 1e30f;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int ci = 0; ci < 6 && rc == MCPM_OK; ++ci) {
    if (cands[ci] > s->tune.bcap / 8 || (ci == 5 && (cands[5] % 128) == 0)) continue;
    s->tune.wcap = cands[ci];
    s->cur = cur0; s->step = step0; s->keys_current = false; s->sorted = false; s->needs_rebin = false;
    s->slotted = false;
    s->omega_init = om0;
    rc = mcpm_step(s, 1);  // warm-up (and a re-scan with this split)
    if (rc) break;
    cudaEventRecord(e0, st);
    rc = mcpm_step(s, steps);
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) { best_ms = ms; best = cands[ci]; }
    // put the saved state back into the buffer set it came from
    s->cur = cur0;
    copy_all(false);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->cur = cur0; s->step = step0; s->sorted = sorted0; s->keys_current = keys0; s->needs_rebin = rebin0;
  s->slotted = false;
  s->omega_init = om0;
  s->tune.wcap = best;
  // the saved layout's work lists were built with the old split: rebuild
  if (s->sorted) { s->sorted = false; s->keys_current = false; }
  s->launches = launches0;
  cudaStreamSynchronize(st);
  cudaFree(save);
  if (chosen) *chosen = best;
  return rc;
}

int mcpm_set_stream(mcpm_session* s, void* stream) {
  if (!s) return MCPM_ERR_ARG;
  cudaStreamSynchronize(s->stream);
  s->stream = stream ? (cudaStream_t)stream : s->own_stream;
  return MCPM_OK;
}

int mcpm_profile(mcpm_session* s, int32_t enable) {
  if (!s) return MCPM_ERR_ARG;
  s->prof = enable != 0;
  return MCPM_OK;
}

int mcpm_profile_read(mcpm_session* s, double* ms, int64_t* launches, int32_t n) {
  if (!s || n < 0 || n > MCPM_K_COUNT) return MCPM_ERR_ARG;
  int rc = cuda_check(s, cudaStreamSynchronize(s->stream), "profile_read");
  if (rc) return rc;
  for (int i = 0; i < n; ++i) { if (ms) ms[i] = 0.0; if (launches) launches[i] = 0; }
  for (auto& r : s->prof_recs) {
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    if (r.cls < n) {
      if (ms) ms[r.cls] += t;
      if (launches) launches[r.cls] += r.n;
    }
    s->prof_pool.push_back(r.a);
    s->prof_pool.push_back(r.b);
  }
  s->prof_recs.clear();
  return MCPM_OK;
}

}  // extern "C"
