// mcpm_kernels.cu -- the particle-step kernels for sm_103a.
//
// Layout: particle state is SoA (x1, x2, U1, U2, U3, pid [, x1_old, x2_old])
// kept sorted by cell in HBM; a cell is the contiguous segment
// [off[c], off[c] + cnt[c]).  Per-cell data is SoA doubles [field][C].
//
// Per step (mcpm_step): scan (counts -> offsets + work lists) -> scatter
// (reorder into the new cell order) -> moments -> per-cell FP64 solves ->
// [long-range force] -> fused update (random_generator + Velocity_FP +
// kick + DFP_extra_streaming + BCs + free flight + re-binning).
//
// Cells are processed by persistent blocks fed from two prefix-sum work
// lists: cells with more than `wcap` particles are handled by a whole block,
// the rest by one warp each.  Compiled with --fmad=false: every multiply
// and add rounds separately, as in the reference (x86-64 without FMA); the
// FP32 kernels write their fused multiply-adds out (fmaf).
#include <cfloat>

#include <type_traits>
#include <utility>

#include "mcpm_device.cuh"
#include "mcpm_solve.cuh"

namespace mcpm {

#define FULL 0xffffffffu

template <typename real> struct PT {
  real *x1, *x2, *U1, *U2, *U3, *x1o, *x2o;
  int32_t* pid;
};
template <typename real> static PT<real> pt(const PBuf& b) {
  return {(real*)b.x1, (real*)b.x2, (real*)b.U1, (real*)b.U2, (real*)b.U3, (real*)b.x1o, (real*)b.x2o, b.pid};
}

// ======================================================= binning (a1)
// cell_update binning, src/Main_Functions.cpp:2231-2266, with the face
// jitter of :2238-2247 drawn from Philox.  Particles outside [0, Len] raise
// MCPM_ERR_OUT_OF_BOX (the reference exits); a particle on the far wall is
// binned into the last cell.

// floor((double)x / d) for a float x from its float estimate i = floor(x * (1/d)),
// which is at most one cell off: face[c] is the smallest float whose
// quotient reaches c (face[n + 1] = +inf)
__device__ __forceinline__ int face_fix(float x, int i, int n, const float* face) {
  const int c = i < 0 ? 0 : (i > n ? n : i);
  if (x < __ldg(face + c)) return c - 1;
  if (x >= __ldg(face + c + 1)) return c + 1;
  return c;
}

template <typename real>
__device__ __forceinline__ int bin_one(real x1, real x2, int pid, int step, const DevConsts& k, const KC<real>& kc,
                                       uint32_t& bad, int* jo = nullptr, int* ko = nullptr) {
  // FP64: r_floor(x / dx) as the reference.  FP32: the same cell, floor of
  // the double quotient of the float position: x * (1/dx) in float, and the
  // face tables where that quotient lies within rounding of an integer
  constexpr bool F32 = sizeof(real) == 4;
  int j = 0;
  int kk;
  if constexpr (F32) {
    if (k.dir0 == 1) {
      float tj;
      const float q = x1 * kc.idx;
      j = floor_to_int(q, &tj);
      const float fr = q - tj;
      if (fr < kc.wx || fr > 1.f - kc.wx) j = face_fix(x1, j, k.N0, kc.face_x);
      if (!(x1 >= 0.f && x1 <= kc.L0)) bad |= MCPM_ERR_OUT_OF_BOX;
    }
    float tk;
    const float q = x2 * kc.idy;
    kk = floor_to_int(q, &tk);
    const float fr = q - tk;
    if (fr < kc.wy || fr > 1.f - kc.wy) {
      kk = face_fix(x2, kk, k.N1, kc.face_y);
      // the face jitter, tested in double on the float position as the
      // reference tests its position (the band lies inside the window)
      if (kk > 0 && kk < k.N1 - 1) {
        const double xd = (double)x2;
        if (fabs(xd - k.dy * kk) < 1e-15 || fabs(xd - k.dy * (kk + 1)) < 1e-15) {
          uint4 r = rng_draw(k, (uint32_t)pid, (uint32_t)step, RNG_BIN, 0u);
          int sgn = (r.x >= 0x80000000u) ? 1 : -1;  // u01(r.x) > 0.5
          kk = (int)floor((xd + 1e-14 * sgn) / k.dy);
        }
      }
    }
  } else {
    const real dy = kc.dy;
    if (k.dir0 == 1) {
      j = (int)r_floor(x1 / kc.dx);
      if (!(x1 >= (real)0 && x1 <= kc.L0)) bad |= MCPM_ERR_OUT_OF_BOX;
    }
    const real tk = r_floor(x2 / dy);  // k as a real: dy * k needs no conversion
    kk = (int)tk;
    if (kk > 0 && kk < k.N1 - 1) {
      if (r_fabs(x2 - dy * tk) < (real)1e-15 || r_fabs(x2 - dy * (tk + (real)1)) < (real)1e-15) {
        uint4 r = rng_draw(k, (uint32_t)pid, (uint32_t)step, RNG_BIN, 0u);
        int sgn = (r.x >= 0x80000000u) ? 1 : -1;  // u01(r.x) > 0.5
        kk = (int)r_floor((x2 + (real)1e-14 * sgn) / dy);
      }
    }
  }
  if (!(x2 >= (real)0 && x2 <= kc.L1)) bad |= MCPM_ERR_OUT_OF_BOX;
  j = j < 0 ? 0 : (j > k.N0 - 1 ? k.N0 - 1 : j);
  kk = kk < 0 ? 0 : (kk > k.N1 - 1 ? k.N1 - 1 : kk);
  if (jo) *jo = j;
  if (ko) *ko = kk;
  return kk * k.N0 + j;
}

template <typename real>
__global__ void k_bin(PT<real> p, int64_t n, DevConsts k, int step, int32_t* key, int32_t* cnt_next,
                      uint32_t* status) {
  uint32_t bad = 0;
  const KC<real> kc = make_kc<real>(k);
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = i0 + threadIdx.x;
    bool act = i < n;
    int c = 0;
    if (act) {
      real x1 = p.x1 ? p.x1[i] : (real)0;
      c = bin_one<real>(x1, p.x2[i], p.pid[i], step, k, kc, bad);
      key[i] = c;
    }
    count_key(cnt_next, c, act);
  }
  raise_status(status, bad);
}

// ================================================ scan + work lists
// Counts of the new layout -> cnt, exclusive offsets, the two work lists
// (cells with <= wcap particles / more), max count, and -- for sessions
// with slotted layouts -- the region bases of the next destination layout;
// resets the accumulation counters and cursors for the next step.  Three
// passes over blocks of 1024 cells: block totals, scan of the totals,
// block-local scan + writes.
constexpr int SCAN_T = 1024;
constexpr int SCAN_Q = 4;       // scanned quantities: count, small, big, slots
constexpr int SCAN_STRIDE = 8;  // ints per block in the totals array

// region capacity of a cell of v particles in a slotted layout: a quarter
// (at least 16) of slack, rounded to whole 32-byte sectors of floats
__device__ __forceinline__ int slot_cap(int v) { return (v + max(16, v >> 2) + 7) & ~7; }

__device__ __forceinline__ void block_scan4(int (&v)[SCAN_Q], int (&t)[SCAN_Q], int (*sh)[32]) {
  // inclusive scan of four ints over a 1024-thread block; t = block totals
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) {
      const int a = __shfl_up_sync(FULL, v[q], d);
      if (lane >= d) v[q] += a;
    }
  }
  if (lane == 31) {
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) sh[q][warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
    int w[SCAN_Q];
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) w[q] = sh[q][lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
      for (int q = 0; q < SCAN_Q; ++q) {
        const int a = __shfl_up_sync(FULL, w[q], d);
        if (lane >= d) w[q] += a;
      }
    }
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) sh[q][lane] = w[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < SCAN_Q; ++q) {
    if (warp) v[q] += sh[q][warp - 1];
    t[q] = sh[q][31];
  }
}

__device__ __forceinline__ void scan_values(int (&v)[SCAN_Q], int c, int C, int count, int wcap) {
  v[0] = c < C ? count : 0;
  v[1] = (c < C && count <= wcap) ? 1 : 0;
  v[2] = (c < C && count > wcap) ? 1 : 0;
  v[3] = c < C ? slot_cap(count) : 0;
}

// pass 1: per-block totals (count, small cells, big cells, slots, max count)
__global__ void __launch_bounds__(SCAN_T) k_scan_blocks(const int32_t* counts, int32_t* blk, int C, int wcap) {
  __shared__ int sh[SCAN_Q][32];
  __shared__ int shm[32];
  const int c = blockIdx.x * SCAN_T + threadIdx.x;
  const int count = c < C ? counts[c] : 0;
  int v[SCAN_Q], t[SCAN_Q];
  scan_values(v, c, C, count, wcap);
  int mx = count;
#pragma unroll
  for (int d = 16; d >= 1; d >>= 1) mx = max(mx, __shfl_xor_sync(FULL, mx, d));
  if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = mx;
  block_scan4(v, t, sh);
  if (threadIdx.x == 0) {
    int m = shm[0];
    for (int w = 1; w < 32; ++w) m = max(m, shm[w]);
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) blk[SCAN_STRIDE * blockIdx.x + q] = t[q];
    blk[SCAN_STRIDE * blockIdx.x + SCAN_Q] = m;
  }
}

// overflow bookkeeping of slotted layouts: two overflow counters (the pass
// that wrote the layout and the next one alternate) and the cursor of the
// spare slots past the layout
enum { OVF_SPARE = 2, OVF_WORDS = 4 };

// pass 2: exclusive scan of the block totals (one block), list lengths; the
// overflow counter of the next slotted pass and the spare cursor start from
// zero
__global__ void __launch_bounds__(SCAN_T) k_scan_totals(int32_t* blk, int nblk, int32_t* wl, int32_t* work,
                                                        int32_t* ovf_n, int par) {
  __shared__ int sh[SCAN_Q][32];
  int carry[SCAN_Q] = {0, 0, 0, 0}, mx = 0;
  for (int base = 0; base < nblk; base += SCAN_T) {
    const int b = base + threadIdx.x;
    int v[SCAN_Q] = {0, 0, 0, 0}, e[SCAN_Q], t[SCAN_Q], m = 0;
    if (b < nblk) {
#pragma unroll
      for (int q = 0; q < SCAN_Q; ++q) v[q] = blk[SCAN_STRIDE * b + q];
      m = blk[SCAN_STRIDE * b + SCAN_Q];
    }
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) e[q] = v[q];
    block_scan4(v, t, sh);
    if (b < nblk) {  // exclusive bases in place of the totals
#pragma unroll
      for (int q = 0; q < SCAN_Q; ++q) blk[SCAN_STRIDE * b + q] = carry[q] + v[q] - e[q];
    }
#pragma unroll
    for (int d = 16; d >= 1; d >>= 1) m = max(m, __shfl_xor_sync(FULL, m, d));
    mx = max(mx, m);
#pragma unroll
    for (int q = 0; q < SCAN_Q; ++q) carry[q] += t[q];
    __syncthreads();
  }
  __shared__ int shm[32];
  if ((threadIdx.x & 31) == 0) shm[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x == 0) {
    int m = shm[0];
    for (int w = 1; w < 32; ++w) m = max(m, shm[w]);
    wl[WL_N] = carry[0]; wl[WL_NSMALL] = carry[1]; wl[WL_NBIG] = carry[2]; wl[WL_MAXCNT] = m;
    if (ovf_n) {
      ovf_n[par] = 0;
      ovf_n[OVF_SPARE] = 0;
    }
  }
  if (threadIdx.x < WK_COUNT) work[threadIdx.x] = 0;
}

// pass 3: block-local scan plus the block base; writes the layout.  off:
// packed offsets of the counts (null: the layout keeps its region bases);
// noff: the same packed offsets for the overflow repair; doff: region bases
// of the next slotted layout
struct ScanOut {
  int32_t *cnt_next, *cursor, *dcur;  // reset (dcur: may be null)
  const int32_t* src;                 // the counts: cnt_next or dcur
  int32_t *cnt, *off, *noff, *doff, *list_small, *list_big;
  const int32_t* blk;
  int C, wcap;
};
__global__ void __launch_bounds__(SCAN_T) k_scan_write(ScanOut a) {
  __shared__ int sh[SCAN_Q][32];
  const int c = blockIdx.x * SCAN_T + threadIdx.x;
  const int count = c < a.C ? a.src[c] : 0;
  int v[SCAN_Q], t[SCAN_Q];
  scan_values(v, c, a.C, count, a.wcap);
  const bool small = v[1], big = v[2];
  const int cap = v[3];
  block_scan4(v, t, sh);
  if (c < a.C) {
    const int32_t* bb = a.blk + SCAN_STRIDE * blockIdx.x;
    const int o = bb[0] + v[0] - count, po = bb[3] + v[3] - cap;
    a.cnt[c] = count;
    if (a.off) a.off[c] = o;
    if (a.noff) a.noff[c] = o;
    if (a.doff) a.doff[c] = po;
    if (small) a.list_small[bb[1] + v[1] - 1] = c;
    if (big) a.list_big[bb[2] + v[2] - 1] = c;
    a.cnt_next[c] = 0;
    a.cursor[c] = 0;
    if (a.dcur) a.dcur[c] = 0;
    if (c == a.C - 1) {
      if (a.off) a.off[a.C] = o + count;
      if (a.noff) a.noff[a.C] = o + count;
      if (a.doff) a.doff[a.C] = po + cap;
    }
  }
}

// ============================================================ scatter
// Reorders the particle arrays into cell order: slot = off[key] + rank,
// ranks handed out per cell by warp-aggregated atomics.
template <typename real>
__global__ void k_scatter(PT<real> src, PT<real> dst, const int32_t* key, const int32_t* off, int32_t* cursor,
                          int64_t n) {
  const int lane = threadIdx.x & 31;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = i0 + threadIdx.x;
    bool act = i < n;
    int c = act ? key[i] : -1;
    unsigned am = __ballot_sync(FULL, act);
    if (act) {
      // the particle's loads go out before the cursor atomic, so their
      // latency overlaps it
      const real x2 = src.x2[i], u1 = src.U1[i], u2 = src.U2[i], u3 = src.U3[i];
      const int32_t pid = src.pid[i];
      const real x1 = src.x1 ? src.x1[i] : (real)0;
      const real x1o = src.x1o ? src.x1o[i] : (real)0, x2o = src.x2o ? src.x2o[i] : (real)0;
      const int base = off[c];
      unsigned peers = __match_any_sync(am, c);
      int leader = __ffs(peers) - 1;
      int rank = __popc(peers & ((1u << lane) - 1u));
      int bse = 0;
      if (lane == leader) bse = atomicAdd(&cursor[c], __popc(peers));
      bse = __shfl_sync(peers, bse, leader);
      int64_t d = (int64_t)base + bse + rank;
      if (src.x1) dst.x1[d] = x1;
      dst.x2[d] = x2;
      dst.U1[d] = u1;
      dst.U2[d] = u2;
      dst.U3[d] = u3;
      dst.pid[d] = pid;
      if (src.x1o) dst.x1o[d] = x1o;
      if (src.x2o) dst.x2o[d] = x2o;
    }
  }
}

// ==================================================== slotted layouts
template <typename real>
__device__ __forceinline__ void copy_particle(const PT<real>& src, int64_t i, const PT<real>& dst, int64_t d) {
  if (src.x1) dst.x1[d] = src.x1[i];
  dst.x2[d] = src.x2[i];
  dst.U1[d] = src.U1[i];
  dst.U2[d] = src.U2[i];
  dst.U3[d] = src.U3[i];
  dst.pid[d] = src.pid[i];
  if (src.x1o) dst.x1o[d] = src.x1o[i];
  if (src.x2o) dst.x2o[d] = src.x2o[i];
}

// Packs a slotted layout into dst at the packed offsets noff: each cell's
// first min(total, capacity) particles from its region of src (bases off),
// the rest from the overflow arrays.
template <typename real>
__global__ void k_pack(PT<real> src, PT<real> dst, PT<real> ovf, const int32_t* ovf_key, const int32_t* ovf_n,
                       const int32_t* off, const int32_t* cnt, const int32_t* noff, int32_t* cursor, int C,
                       uint32_t* status) {
  const int n_ovf = *ovf_n;
  const int lane = threadIdx.x & 31;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t c = tid >> 5; c < C; c += nt >> 5) {
    const int s0 = off[c], m = min(cnt[c], off[c + 1] - s0), d0 = noff[c];
    for (int i = lane; i < m; i += 32) copy_particle(src, (int64_t)s0 + i, dst, (int64_t)d0 + i);
  }
  for (int64_t e = tid; e < n_ovf; e += nt) {
    const int c = ovf_key[e];
    const int d = noff[c] + (off[c + 1] - off[c]) + atomicAdd(&cursor[c], 1);
    // an overflow entry lies within its cell's packed range by construction
    // (its slot came from the cell's own counter); checked, not assumed
    if (d < noff[c] + cnt[c]) copy_particle(ovf, e, dst, (int64_t)d);
    else raise_status(status, MCPM_ERR_CAPACITY);
  }
}

// Repair of a slotted layout whose regions overflowed, in two launches that
// return at once when nothing did.  Every cell holding more particles than
// its region moves to the spare slots past the layout (from off[C] on): its
// region's particles here, the base of its new place in nbase (-1: the cell
// stays) and the slot its overflow entries start from in cursor.
template <typename real>
__global__ void k_relocate(PT<real> p, const int32_t* ovf_n, const int32_t* off, const int32_t* cnt, int32_t* nbase,
                           int32_t* cursor, int32_t* spare, int C) {
  if (*ovf_n == 0) return;
  const int lane = threadIdx.x & 31;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  const int end = off[C];
  for (int64_t c = tid >> 5; c < C; c += nt >> 5) {
    const int s0 = off[c], capc = off[c + 1] - s0, n = cnt[c];
    int nb = -1;
    if (n > capc) {
      if (lane == 0) nb = end + atomicAdd(spare, n);
      nb = __shfl_sync(FULL, nb, 0);
      for (int i = lane; i < capc; i += 32) copy_particle(p, (int64_t)s0 + i, p, (int64_t)nb + i);
      if (lane == 0) cursor[c] = capc;
    }
    if (lane == 0) nbase[c] = nb;
  }
}
// ... then the overflow entries after them, and the moved cells' bases
template <typename real>
__global__ void k_relocate_tail(PT<real> p, PT<real> ovf, const int32_t* ovf_key, const int32_t* ovf_n,
                                const int32_t* nbase, const int32_t* cnt, int32_t* cursor, int32_t* off, int C,
                                uint32_t* status) {
  const int n_ovf = *ovf_n;
  if (n_ovf == 0) return;
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  for (int64_t e = tid; e < n_ovf; e += nt) {
    const int c = ovf_key[e];
    // only cells that outgrew their regions have overflow entries, and they
    // were moved (nbase >= 0) with room for all cnt[c] particles; checked
    const int b = nbase[c], q = atomicAdd(&cursor[c], 1);
    if (b >= 0 && q < cnt[c]) copy_particle(ovf, e, p, (int64_t)b + q);
    else raise_status(status, MCPM_ERR_CAPACITY);
  }
  for (int64_t c = tid; c < C; c += nt)
    if (nbase[c] >= 0) off[c] = nbase[c];
}

// ================================================ cell access helpers
struct CellRef {
  const double* cell;
  int C;
  __device__ __forceinline__ double operator()(int f, int c) const { return cell[(size_t)f * C + c]; }
};

// persistent two-phase scheduler: block-sized cells first, then one warp per
// small cell.  fn_big(c) is called by the whole block, fn_small(c) by a warp.
template <typename FB, typename FS>
__device__ __forceinline__ void schedule_cells(const int32_t* list_big, const int32_t* list_small, const int32_t* wl,
                                               int32_t* work, int wk_big, int wk_small, FB fn_big, FS fn_small) {
  __shared__ int item;
  const int nbig = wl[WL_NBIG], nsmall = wl[WL_NSMALL];
  for (;;) {
    if (threadIdx.x == 0) item = atomicAdd(&work[wk_big], 1);
    __syncthreads();
    int it = item;
    __syncthreads();
    if (it >= nbig) break;
    fn_big(list_big[it]);
  }
  const int lane = threadIdx.x & 31;
  for (;;) {
    int it = 0;
    if (lane == 0) it = atomicAdd(&work[wk_small], 1);
    it = __shfl_sync(FULL, it, 0);
    if (it >= nsmall) break;
    fn_small(list_small[it]);
  }
}

// ============================================================ moments (a4)
// src/Main_Functions.cpp:2461-2593: mean velocity, then the central moments
// up to fifth order about it; T, n, gamma* per cell.
template <typename real> struct MomArgs {
  DevConsts k;
  double* cell;
  const int32_t *off, *cnt, *list_small, *list_big, *wl;
  int32_t* work;
  const real *U1, *U2, *U3;
};

// FP64 sessions (FP32 sessions take moments_cell_f32)
template <typename real, int TILE>
__device__ void moments_cell(int c, const MomArgs<real>& a, Acc<real>* red) {
  static_assert(sizeof(real) == 8, "the FP32 moment pass is moments_cell_f32");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = (TILE == 32) ? lane : threadIdx.x;
  const int s0 = a.off[c], n = a.cnt[c];
  const int C = a.k.C;
  Acc<real> u[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) u[q].zero();
  for (int i = t; i < n; i += TILE) {
    u[0].add(a.U1[s0 + i]);
    u[1].add(a.U2[s0 + i]);
    u[2].add(a.U3[s0 + i]);
  }
  tile_reduce<real, 3, TILE>(u, red);
  // cell mean velocity U_space (src/Main_Functions.cpp:2493-2500)
  real m0 = 0, m1 = 0, m2 = 0;
  if (n > 0) {
    const double weight = (double)n;
    m0 = u[0].get() / weight; m1 = u[1].get() / weight; m2 = u[2].get() / weight;
  }
  Acc<real> q[29];
#pragma unroll
  for (int j = 0; j < 29; ++j) q[j].zero();
  // the 29 products of src/Main_Functions.cpp:2502-2560 for particle i
  auto terms = [&](int i, real (&v)[29]) {
    real Mp1 = a.U1[s0 + i] - m0, Mp2 = a.U2[s0 + i] - m1, Mp3 = a.U3[s0 + i] - m2;
    real energy = Mp1 * Mp1 + Mp2 * Mp2 + Mp3 * Mp3;
    v[0] = Mp1; v[1] = Mp2; v[2] = Mp3;
    v[3] = Mp1 * Mp1; v[4] = Mp1 * Mp2; v[5] = Mp1 * Mp3;
    v[6] = Mp2 * Mp2; v[7] = Mp2 * Mp3; v[8] = Mp3 * Mp3;
    v[9] = Mp1 * Mp1 * Mp1; v[10] = Mp1 * Mp1 * Mp2; v[11] = Mp1 * Mp1 * Mp3;
    v[12] = Mp1 * Mp2 * Mp2; v[13] = Mp1 * Mp2 * Mp3; v[14] = Mp1 * Mp3 * Mp3;
    v[15] = Mp2 * Mp2 * Mp2; v[16] = Mp2 * Mp2 * Mp3; v[17] = Mp2 * Mp3 * Mp3;
    v[18] = Mp3 * Mp3 * Mp3;
    v[19] = Mp1 * Mp1 * energy; v[20] = Mp1 * Mp2 * energy; v[21] = Mp1 * Mp3 * energy;
    v[22] = Mp2 * Mp2 * energy; v[23] = Mp2 * Mp3 * energy; v[24] = Mp3 * Mp3 * energy;
    v[25] = Mp1 * energy * energy; v[26] = Mp2 * energy * energy; v[27] = Mp3 * energy * energy;
    v[28] = energy;
  };
  for (int i = t; i < n; i += TILE) {
    real v[29];
    terms(i, v);
#pragma unroll
    for (int j = 0; j < 29; ++j) q[j].add(v[j]);
  }
  // raw sums, one field per lane; the FP64 finalisation (divisions by the
  // weight, T, n, Y, gamma*) runs once per cell in k_solve
  Acc<real> tot = tile_reduce_lanes<real, 29, TILE>(q, red);
  if (TILE == 32 || warp == 0) {
    double* cl = a.cell;
    if (lane < 29) cl[(size_t)(CFI_RAW + lane) * C + c] = tot.get();
    else if (lane == 29) cl[(size_t)(MCPM_CF_U_SPACE + 0) * C + c] = (double)m0;
    else if (lane == 30) cl[(size_t)(MCPM_CF_U_SPACE + 1) * C + c] = (double)m1;
    else cl[(size_t)(MCPM_CF_U_SPACE + 2) * C + c] = (double)m2;
    if (lane == 0) cl[(size_t)MCPM_CF_NUM_INSIDE * C + c] = (double)n;
  }
}

// Sums of K floats over a tile of TILE threads (one warp or the block):
// per-lane running sums combined by an XOR butterfly (pairwise), every
// thread gets the totals.  red holds K * TILE / 32 floats.
template <int K, int TILE>
__device__ __forceinline__ void tile_sum_f32(float (&v)[K], float* red) {
#pragma unroll
  for (int q = 0; q < K; ++q)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(FULL, v[q], o);
  if constexpr (TILE > 32) {
    constexpr int W = TILE / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) {
#pragma unroll
      for (int q = 0; q < K; ++q) red[q * W + warp] = v[q];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < K; ++q) {
      float t = 0.f;
#pragma unroll
      for (int w = 0; w < W; ++w) t += red[q * W + w];
      v[q] = t;
    }
  }
}

// The FP32 moment pass without compensation: the cell mean from plain
// per-lane sums (butterfly), then one pass over the cell's velocities (from
// L1) with the 29 products in plain per-lane float sums -- P from the
// centred velocities, M3 = P c, M4 = P e, M5 = c e^2 -- and a reduce-scatter
// across the warp (recursive halving: 31 shuffles leave sum j on lane j),
// across the block's warps through shared memory for block-sized cells.
// Each lane sums n / TILE terms; the sums enter the FP64 finalisation as
// doubles.
template <int TILE>
__device__ void moments_cell_f32(int c, const MomArgs<float>& a, float* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int t = (TILE == 32) ? lane : threadIdx.x;
  const int s0 = a.off[c], n = a.cnt[c];
  const int C = a.k.C;
  float u[3] = {0.f, 0.f, 0.f};
  for (int i = t; i < n; i += TILE) {
    u[0] += a.U1[s0 + i];
    u[1] += a.U2[s0 + i];
    u[2] += a.U3[s0 + i];
  }
  tile_sum_f32<3, TILE>(u, red);
  float m0 = 0.f, m1 = 0.f, m2 = 0.f;
  if (n > 0) {
    const float w = (float)n;
    m0 = u[0] / w; m1 = u[1] / w; m2 = u[2] / w;
  }
  float v[32];
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = 0.f;
  for (int i = t; i < n; i += TILE) {
    const float c1 = a.U1[s0 + i] - m0, c2 = a.U2[s0 + i] - m1, c3 = a.U3[s0 + i] - m2;
    const float e = fmaf(c3, c3, fmaf(c2, c2, c1 * c1));
    const float p11 = c1 * c1, p12 = c1 * c2, p13 = c1 * c3, p22 = c2 * c2, p23 = c2 * c3, p33 = c3 * c3;
    const float e2 = e * e;
    v[0] += c1; v[1] += c2; v[2] += c3;
    v[3] += p11; v[4] += p12; v[5] += p13; v[6] += p22; v[7] += p23; v[8] += p33;
    v[9] = fmaf(p11, c1, v[9]); v[10] = fmaf(p11, c2, v[10]); v[11] = fmaf(p11, c3, v[11]);
    v[12] = fmaf(p12, c2, v[12]); v[13] = fmaf(p12, c3, v[13]); v[14] = fmaf(p13, c3, v[14]);
    v[15] = fmaf(p22, c2, v[15]); v[16] = fmaf(p22, c3, v[16]); v[17] = fmaf(p23, c3, v[17]);
    v[18] = fmaf(p33, c3, v[18]);
    v[19] = fmaf(p11, e, v[19]); v[20] = fmaf(p12, e, v[20]); v[21] = fmaf(p13, e, v[21]);
    v[22] = fmaf(p22, e, v[22]); v[23] = fmaf(p23, e, v[23]); v[24] = fmaf(p33, e, v[24]);
    v[25] = fmaf(c1, e2, v[25]); v[26] = fmaf(c2, e2, v[26]); v[27] = fmaf(c3, e2, v[27]);
    v[28] += e;
  }
  // reduce-scatter over the warp: after the level of width d a lane keeps
  // the half of its values whose index bit matches its lane bit
#pragma unroll
  for (int d = 16, W = 32; d >= 1; d >>= 1, W >>= 1) {
    const bool up = lane & d;
#pragma unroll
    for (int j = 0; j < W / 2; ++j) {
      const float send = up ? v[j] : v[W / 2 + j];
      const float keep = up ? v[W / 2 + j] : v[j];
      v[j] = keep + __shfl_xor_sync(FULL, send, d);
    }
  }
  float tot = v[0];  // sum number `lane`
  if constexpr (TILE > 32) {
    __syncthreads();
    red[warp * 32 + lane] = tot;
    __syncthreads();
    if (warp == 0) {
      tot = 0.f;
#pragma unroll
      for (int w = 0; w < TILE / 32; ++w) tot += red[w * 32 + lane];
    }
  }
  if (TILE == 32 || warp == 0) {
    double* cl = a.cell;
    if (lane < 29) cl[(size_t)(CFI_RAW + lane) * C + c] = (double)tot;
    else if (lane == 29) cl[(size_t)(MCPM_CF_U_SPACE + 0) * C + c] = (double)m0;
    else if (lane == 30) cl[(size_t)(MCPM_CF_U_SPACE + 1) * C + c] = (double)m1;
    else cl[(size_t)(MCPM_CF_U_SPACE + 2) * C + c] = (double)m2;
    if (lane == 0) cl[(size_t)MCPM_CF_NUM_INSIDE * C + c] = (double)n;
  }
}

// blocks of 256 threads resident per SM in the FP32 moment pass (5: 48
// registers hold the 29 plain sums without spilling; measured faster than 4,
// 6 spills)
#ifndef MCPM_MOM_MINB
#define MCPM_MOM_MINB 5
#endif
template <typename real>
__global__ void __launch_bounds__(256, sizeof(real) == 4 ? MCPM_MOM_MINB : 1) k_moments(MomArgs<real> a) {
  __shared__ Acc<real> red[29 * 8];
  if constexpr (sizeof(real) == 4) {
    float* rf = reinterpret_cast<float*>(red);
    schedule_cells(
        a.list_big, a.list_small, a.wl, a.work, WK_MOM_BIG, WK_MOM_SMALL,
        [&](int c) { moments_cell_f32<256>(c, a, rf); }, [&](int c) { moments_cell_f32<32>(c, a, rf); });
  } else {
    schedule_cells(
        a.list_big, a.list_small, a.wl, a.work, WK_MOM_BIG, WK_MOM_SMALL,
        [&](int c) { moments_cell<real, 256>(c, a, red); }, [&](int c) { moments_cell<real, 32>(c, a, red); });
  }
}

// ================================================== boundary conditions
template <typename real> struct PState {
  real x1, x2, x1o, x2o, u1, u2, u3;
};

// a particle's state into slot d of a set of arrays
__device__ __forceinline__ void store_state(const PT<float>& D, int64_t d, const PState<float>& s, int pid) {
  D.U1[d] = s.u1; D.U2[d] = s.u2; D.U3[d] = s.u3;
  if (D.x1) D.x1[d] = s.x1;
  D.x2[d] = s.x2;
  D.pid[d] = pid;
  if (D.x1o) D.x1o[d] = s.x1o;
  if (D.x2o) D.x2o[d] = s.x2o;
}

// BC_specular_reflection, src/Main_Functions.cpp:6399-6525
template <typename real>
__device__ __forceinline__ void bc_specular(PState<real>& s, const DevConsts& k, const KC<real>& kc, uint32_t& bad) {
  const real Tol1 = (real)1e-16, Tol2 = (real)-1e-16, L0 = kc.L0, L1 = kc.L1;
  int it = 0;
  for (;;) {
    if (k.dir0 == 1) {
      if (s.x1 - L0 > Tol2) { s.u1 = -s.u1; s.x1 = s.x1 - (real)2.0 * r_fabs(s.x1 - L0); }
      else if (s.x1 < Tol1) { s.u1 = -s.u1; s.x1 = s.x1 + (real)2.0 * r_fabs(s.x1); }
    }
    if (k.dir1 == 1) {
      if (s.x2 - L1 > Tol2) { s.u2 = -s.u2; s.x2 = s.x2 - (real)2.0 * r_fabs(s.x2 - L1); }
      else if (s.x2 < Tol1) { s.u2 = -s.u2; s.x2 = s.x2 + (real)2.0 * r_fabs(s.x2); }
    }
    bool done = true;
    if (k.dir0 == 1 && (s.x1 - L0 > (real)0 || s.x1 < (real)0)) done = false;
    if (k.dir1 == 1 && (s.x2 - L1 > (real)0 || s.x2 < (real)0)) done = false;
    if (done) break;
    if (++it > 64) { bad |= MCPM_ERR_BC_LOOP; break; }
  }
}

template <typename real>
__device__ __forceinline__ void bc_periodic(PState<real>& s, const DevConsts& k, const KC<real>& kc) {
  if (k.dir0 == 1) s.x1 = s.x1 - kc.L0 * r_floor(s.x1 / kc.L0);
  if (k.dir1 == 1) s.x2 = s.x2 - kc.L1 * r_floor(s.x2 / kc.L1);
}

// one diffuse re-emission draw: Rayleigh factor + two normals
template <typename real>
__device__ __forceinline__ void wall_draw(int pid, int step, int call, int it, const DevConsts& k, real& ray,
                                          real& z0, real& z1) {
  uint4 r = rng_draw(k, (uint32_t)pid, (uint32_t)step, RNG_BC, (uint32_t)((call << 8) | (it & 0xff)));
  if constexpr (sizeof(real) == 8) {
    ray = r_sqrt(-log(u01d(r.x)));
    double a = r_sqrt(-2.0 * log(u01d(r.y)));
    double sn, cs;
    sincos(kTwoPi * u01d(r.z), &sn, &cs);
    z0 = a * cs; z1 = a * sn;
  } else {
    ray = sqrtf(-logf(u01f(r.x)));
    float a = sqrtf(-2.0f * logf(u01f(r.y)));
    float sn, cs;
    sincospif(2.0f * u01f(r.z), &sn, &cs);
    z0 = a * cs; z1 = a * sn;
  }
}

// intersect_3D_x / _y, src/Main_Functions.cpp:2757-2806 (no motion in z)
template <typename real>
__device__ __forceinline__ real isect_x(real x, real xo, real yo, real xn, real yn) {
  real n0 = xn - xo, n1 = yn - yo, n2 = 0;
  real size = 0;
  size += n0 * n0; size += n1 * n1; size += n2 * n2;
  size = r_sqrt(size);
  n0 = n0 / size; n1 = n1 / size;
  if (r_fabs(n0) > (real)1e-16) return (n1 / n0) * (x - xo) + yo;
  return yn;
}
template <typename real>
__device__ __forceinline__ real isect_y(real y, real xo, real yo, real xn, real yn) {
  real n0 = xn - xo, n1 = yn - yo, n2 = 0;
  real size = 0;
  size += n0 * n0; size += n1 * n1; size += n2 * n2;
  size = r_sqrt(size);
  n0 = n0 / size; n1 = n1 / size;
  if (r_fabs(n1) > (real)1e-16) return (n0 / n1) * (y - yo) + xo;
  return xn;
}

// BC_thermal_wall_3D, src/Main_Functions.cpp:4917-5250, in 2-D
template <typename real>
__device__ void bc_thermal_wall(PState<real>& s, int call, int pid, int step, const DevConsts& k, const KC<real>& kc,
                                uint32_t& bad) {
  const real ex = kc.eps_x, ey = kc.eps_y, L0 = kc.L0, L1 = kc.L1, sg = kc.sigma, DT = kc.dt;
  const real mm = kc.m, kb = kc.kb;
  real dt = DT;
  int it = 0;
  const real Ue0 = r_fabs(s.x1 - s.x1o) / DT, Ue1 = r_fabs(s.x2 - s.x2o) / DT;
  for (;;) {
    real dt_remain, xw, yw, tU0, ray, z0, z1;
    if (it > 20) { bad |= MCPM_ERR_BC_LOOP; break; }
    if (dt < (real)1e-15) {
      if (s.x1 < ex) s.x1 = ex;
      else if (s.x1 > L0 - ex) s.x1 = L0 - ex;
      if (s.x2 < ey) s.x2 = ey;
      else if (s.x2 > L1 - ey) s.x2 = L1 - ey;
    }
    // a particle exactly on the x walls counts as having reached them (the
    // reference's > / < leave x == Len neither inside nor outside)
    int wall = -1;
    if (s.x1 - L0 >= (real)0) wall = 3;
    else if (s.x1 <= (real)0) wall = 2;
    else if (s.x2 > L1 - sg - ey) wall = 1;
    else if (s.x2 < sg + ey) wall = 0;
    if (wall >= 0) {
      const real Tw = kc.Tw[wall], Uw = kc.Uw[wall];
      if (wall >= 2) {  // x walls
        xw = (wall == 3) ? L0 - ex : ex;
        if (r_fabs(s.x1o - s.x1) > (real)1e-15) yw = isect_x<real>(xw, s.x1o, s.x2o, s.x1, s.x2);
        else yw = (real)0.5 * (s.x2o + s.x2);
        tU0 = (r_fabs(dt - DT) < (real)1e-15) ? Ue0 : s.u1;
        wall_draw<real>(pid, step, call, it, k, ray, z0, z1);
        real un = r_sqrt((real)2.0 * kb * Tw / (mm)) * ray;
        s.u1 = (wall == 3) ? -un : un;
        s.u2 = r_sqrt(kb * Tw / (mm)) * z0 + ((real)1.0 * Uw);
        s.u3 = r_sqrt(kb * Tw / (mm)) * z1;
        if (dt > (real)1e-15) {
          dt_remain = r_fabs((s.x1 - xw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          s.x1 = xw + dt_remain * s.u1;
          s.x2 = yw + dt_remain * s.u2;
          dt = dt - dt_remain;
          s.x1o = xw; s.x2o = yw;
        } else {
          s.x1 = xw;
        }
      } else {  // y walls at sigma and Len1 - sigma
        yw = (wall == 1) ? L1 - sg - ey : sg + ey;
        xw = isect_y<real>(yw, s.x1o, s.x2o, s.x1, s.x2);
        tU0 = (r_fabs(dt - DT) < (real)1e-15) ? Ue1 : s.u2;
        wall_draw<real>(pid, step, call, it, k, ray, z0, z1);
        s.u1 = r_sqrt(kb * Tw / (mm)) * z0 + ((real)1.0 * Uw);
        real un = r_sqrt((real)2.0 * kb * Tw / (mm)) * ray;
        s.u2 = (wall == 1) ? -un : un;
        s.u3 = r_sqrt(kb * Tw / (mm)) * z1;
        if (dt > (real)1e-15) {
          dt_remain = r_fabs((s.x2 - yw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          s.x1 = xw + dt_remain * s.u1;
          s.x2 = yw + dt_remain * s.u2;
          dt = dt - dt_remain;
          s.x1o = xw; s.x2o = yw;
        } else {
          s.x2 = yw;
        }
      }
    }
    if (s.x1 - L0 < (real)0 && s.x1 > (real)0 && s.x2 - L1 < (real)0 && s.x2 > (real)0) break;
    it++;
  }
}

// BC_wall, src/Main_Functions.cpp:4816-4914 (1-D: diffuse y = 0, specular y = Len1)
template <typename real>
__device__ void bc_wall(PState<real>& s, int call, int pid, int step, const DevConsts& k, const KC<real>& kc,
                        uint32_t& bad) {
  const real eps = kc.eps_y, L1 = kc.L1, DT = kc.dt, mm = kc.m, kb = kc.kb;
  const real Tw = kc.Tw[0], Uw = kc.Uw[0];
  real dt = DT;
  int it = 0;
  const real Ue1 = r_fabs(s.x2 - s.x2o) / DT;
  for (;;) {
    if (it > 20) { bad |= MCPM_ERR_BC_LOOP; break; }
    if (dt < (real)1e-15) {
      if (s.x2 < eps) s.x2 = eps;
      else if (s.x2 > L1 - eps) s.x2 = L1 - eps;
    } else if (s.x2 >= L1) {  // >= / <=: see bc_thermal_wall
      s.u2 = -s.u2;
      s.x2 = s.x2 - (real)2.0 * r_fabs(s.x2 - L1);
    } else if (s.x2 <= (real)0) {
      real yw = eps, ray, z0, z1;
      real tU0 = (r_fabs(dt - DT) < (real)1e-15) ? Ue1 : s.u2;
      wall_draw<real>(pid, step, call, it, k, ray, z0, z1);
      s.u1 = r_sqrt(kb * Tw / (mm)) * z0 + ((real)1.0 * Uw);
      s.u2 = r_sqrt((real)2.0 * kb * Tw / (mm)) * ray;
      s.u3 = r_sqrt(kb * Tw / mm) * z1;
      if (dt > (real)1e-15) {
        real dt_remain = r_fabs((s.x2 - yw) / tU0);
        dt_remain = dt < dt_remain ? dt : dt_remain;
        s.x2 = yw + dt_remain * s.u2;
        dt = dt - dt_remain;
        s.x2o = yw;
      } else {
        s.x2 = yw;
      }
    }
    if (s.x2 - L1 < (real)0 && s.x2 > (real)0) break;
    it++;
  }
}

// apply_BC, src/Main_Functions.cpp:1451-1492
template <typename real>
__device__ __forceinline__ void apply_bc(PState<real>& s, int call, int pid, int step, const DevConsts& k,
                                         const KC<real>& kc, uint32_t& bad) {
  switch (k.problem) {
    case MCPM_PROBLEM_CLOSED_BOX: bc_specular<real>(s, k, kc, bad); break;
    case MCPM_PROBLEM_COUETTE: bc_thermal_wall<real>(s, call, pid, step, k, kc, bad); break;
    case MCPM_PROBLEM_WALL: bc_wall<real>(s, call, pid, step, k, kc, bad); break;
    case MCPM_PROBLEM_PERIODIC: bc_periodic<real>(s, k, kc); break;
    default: break;
  }
}

// ====================================================== fused update
template <typename real> struct UpdArgs {
  DevConsts k;
  const double* cell;
  const float* pcell;
  const int32_t *off, *cnt, *list_small, *list_big, *wl;
  int32_t* work;
  PT<real> p;
  int32_t* key_out;
  int32_t* cnt_next;
  const double* inj;
  double* xi;
  int64_t cap;
  uint32_t* status;
  const int32_t* dstep;  // the step number (device copy: graph replays advance it)
  int rng_mode, bc_call_base;
  uint32_t stages;
  int wcap, bcap;
  const double* Vn;  // node potential of the 2-D Vlasov force (FP64 path)
  KC<real> kc;       // constants in the state's precision (read from the
                     // parameter bank, so they cost no registers)
  // slotted layouts (FP32 fused steps): the destination buffer, the region
  // bases of its layout and their slot counters, the overflow arrays and
  // their counter
  PT<real> d;
  const int32_t* doff;
  int32_t* dcur;
  PT<real> ovf;
  int32_t* ovf_key;
  int32_t* ovf_n;
};

template <typename real>
__device__ __forceinline__ void raw_normals_pid(const UpdArgs<real>& a, int step, int pid, real& z0, real& z1,
                                                real& z2) {
  if (a.rng_mode == MCPM_RNG_INJECTED) {
    z0 = (real)a.inj[pid]; z1 = (real)a.inj[a.cap + pid]; z2 = (real)a.inj[2 * a.cap + pid];
  } else {
    Normals3<real> z = normals3<real>(rng_draw(a.k, (uint32_t)pid, (uint32_t)step, RNG_FP, 0u));
    z0 = z.z0; z1 = z.z1; z2 = z.z2;
  }
}
template <typename real>
__device__ __forceinline__ void raw_normals(const UpdArgs<real>& a, int step, int64_t p, real& z0, real& z1,
                                            real& z2) {
  raw_normals_pid(a, step, a.p.pid[p], z0, z1, z2);
}

// Per-cell constants of the particle pass.  FP64: read from the double cell
// array, expressions as in the reference.  FP32: the packed float record.
template <typename real> struct CellK {
  real us0, us1, us2, A1, A2, A3, eq, lam, c[6], g[3], q[3];
  real al[6], be0, be1, gst, m3_0, m3_3, m3_5, m3_1, m3_6, m3_8, hq0, hq1, ph0, ph1, f2dt;
  // 2-D Vlasov kick: FP32 the packed coefficients (la1 lb1 la2 lb2), FP64
  // the four node potentials and the cell's corner / size (v, xn0 yn0 dxc dyc)
  real l2[4];
  double v[4], xn0, yn0, dxc, dyc;
};
template <typename real>
__device__ __forceinline__ void load_cellk(CellK<real>& K, int c, const UpdArgs<real>& a, uint32_t st) {
  if constexpr (sizeof(real) == 4) {
    float pf[PF_STRIDE];
    const float4* src = reinterpret_cast<const float4*>(a.pcell + (size_t)c * PF_STRIDE);
#pragma unroll
    for (int j = 0; j < PF_LA1 / 4; ++j) reinterpret_cast<float4*>(pf)[j] = __ldg(src + j);
    if ((st & ST_LR) && a.k.lr2d) {
      float4 l = __ldg(src + PF_LA1 / 4);
      K.l2[0] = l.x; K.l2[1] = l.y; K.l2[2] = l.z; K.l2[3] = l.w;
    }
    K.us0 = pf[PF_US0]; K.us1 = pf[PF_US1]; K.us2 = pf[PF_US2];
    K.A1 = pf[PF_A1]; K.A2 = pf[PF_A2]; K.A3 = pf[PF_A3]; K.eq = pf[PF_EQ]; K.lam = pf[PF_LAM];
#pragma unroll
    for (int j = 0; j < 6; ++j) { K.c[j] = pf[PF_C0 + j]; K.al[j] = pf[PF_AL0 + j]; }
#pragma unroll
    for (int j = 0; j < 3; ++j) { K.g[j] = pf[PF_G0 + j]; K.q[j] = pf[PF_Q0 + j]; }
    K.be0 = pf[PF_BE0]; K.be1 = pf[PF_BE1]; K.gst = pf[PF_GST];
    K.hq0 = pf[PF_HQ0]; K.hq1 = pf[PF_HQ1]; K.ph0 = pf[PF_PH0]; K.ph1 = pf[PF_PH1];
    K.f2dt = pf[PF_F2DT];
    K.m3_0 = K.m3_3 = K.m3_5 = K.m3_1 = K.m3_6 = K.m3_8 = 0.f;
  } else {
    const CellRef R{a.cell, a.k.C};
    K.us0 = R(MCPM_CF_U_SPACE + 0, c); K.us1 = R(MCPM_CF_U_SPACE + 1, c); K.us2 = R(MCPM_CF_U_SPACE + 2, c);
    K.A1 = R(CFI_A1, c); K.A2 = R(CFI_A2, c); K.A3 = R(CFI_A3, c); K.eq = R(CFI_3KT, c);
    K.lam = R(MCPM_CF_LAMBDA, c);
    for (int j = 0; j < 6; ++j) { K.c[j] = R(MCPM_CF_C + j, c); K.al[j] = R(MCPM_CF_ALPHA + j, c); }
    for (int j = 0; j < 3; ++j) { K.g[j] = R(MCPM_CF_GAMMA + j, c); K.q[j] = R(MCPM_CF_Q + j, c); }
    K.be0 = R(MCPM_CF_BETA + 0, c); K.be1 = R(MCPM_CF_BETA + 1, c); K.gst = R(MCPM_CF_GAMMA_ST, c);
    K.m3_0 = R(MCPM_CF_M3 + 0, c); K.m3_3 = R(MCPM_CF_M3 + 3, c); K.m3_5 = R(MCPM_CF_M3 + 5, c);
    K.m3_1 = R(MCPM_CF_M3 + 1, c); K.m3_6 = R(MCPM_CF_M3 + 6, c); K.m3_8 = R(MCPM_CF_M3 + 8, c);
    K.hq0 = K.hq1 = 0.0;
    K.ph0 = R(MCPM_CF_PHI + 0, c); K.ph1 = R(MCPM_CF_PHI + 1, c);
    if (a.k.model == MCPM_MODEL_FP_LINEAR) {
      // Velocity_FP_linear: M' <- A1 M' + A3 xi (src/Fokker_Planck.cpp:1262-1264)
      K.A2 = 0.0; K.lam = 0.0;
      for (int j = 0; j < 6; ++j) K.c[j] = 0.0;
      for (int j = 0; j < 3; ++j) K.g[j] = 0.0;
    }
    K.f2dt = (st & ST_LR) ? R(MCPM_CF_F2, c) * a.k.dt : 0.0;
    if ((st & ST_LR) && a.k.lr2d) {
      // cells[num].x_n[0], y_n[0], dx, dy as make_cells builds them (src/myIO.cpp:1456-1479)
      const int j = c % a.k.N0, kk = c / a.k.N0;
      double d0 = (double)j * a.k.dx, d1 = (double)(j + 1) * a.k.dx;
      double d2 = (double)kk * a.k.dy, d3 = (double)(kk + 1) * a.k.dy;
      K.dxc = d1 - d0; K.dyc = d3 - d2;
      K.xn0 = 0.5 * (d0 + d1) - K.dxc / 2.0;
      K.yn0 = 0.5 * (d2 + d3) - K.dyc / 2.0;
      const int id0 = kk * (a.k.N0 + 1) + j, id2 = id0 + a.k.N0 + 1;
      K.v[0] = a.Vn[id0]; K.v[1] = a.Vn[id0 + 1]; K.v[2] = a.Vn[id2]; K.v[3] = a.Vn[id2 + 1];
    }
  }
}

// sum / n and sqrt(sum / n) in the path's precision
template <typename real> __device__ __forceinline__ real cmean(const Acc<real>& s, int n) {
  if constexpr (sizeof(real) == 4) return s.getr() / (float)n;
  else return s.get() / (1.0 * n);
}
template <typename real> __device__ __forceinline__ real crms(const Acc<real>& s, int n) {
  if constexpr (sizeof(real) == 4) return sqrtf(s.getr() / (float)n);
  else return sqrt(s.get() / (1.0 * n));
}

// random_generator (src/Fokker_Planck.cpp:20-145) + Velocity_FP_parallel
// (:1065-1182) + long-range kick (src/Main_Functions.cpp:3937, :3578) +
// DFP_extra_streaming (src/Fokker_Planck.cpp:904-946) + apply_BC /
// store_old_positions / stream_particles (src/main.cpp:478-514) + the binning
// of the next cell_update, for one cell, by a tile of TILE threads.
// xs stages three values per particle in shared memory when the cell fits:
// the raw normals, then the new peculiar velocities M'.
// The FP64 path follows the reference's two-pass centring/normalisation of
// the normals.  Instantiated for FP64 sessions only (FP32 sessions run
// update_cell_f32 below); its float branches are not compiled into the
// library.
template <typename real, int TILE, uint32_t CST>
__device__ void update_cell(int c, const UpdArgs<real>& a, int step, real* xs, int xcap, Acc<real>* red) {
  constexpr bool F32 = sizeof(real) == 4;
  const int t = (TILE == 32) ? (threadIdx.x & 31) : threadIdx.x;
  const int64_t s0 = a.off[c];
  const int n = a.cnt[c];
  const DevConsts& k = a.k;
  const KC<real> kc = make_kc<real>(k);
  // stages known at compile time (CST) are folded by the compiler
  const uint32_t st = CST ? CST : a.stages;
  const bool rng = st & ST_RNG, fp = st & ST_FP, load_xi = st & ST_LOAD_XI, store_xi = st & ST_STORE_XI;
  const bool staged = rng && n <= xcap;
  CellK<real> K;
  load_cellk<real>(K, c, a, st);
  const real Us0 = K.us0, Us1 = K.us1, Us2 = K.us2;
  PT<real> P = a.p;
  real mean0 = 0, mean1 = 0, mean2 = 0, rms0 = 1, rms1 = 1, rms2 = 1;
  Acc<real> f1acc;
  f1acc.zero();
  // ---- pass A: draws, their per-cell sums, sum |M'|^2
  if (rng || fp) {
    constexpr int KA = F32 ? 7 : 4;
    Acc<real> sa[KA];
#pragma unroll
    for (int q = 0; q < KA; ++q) sa[q].zero();
    for (int i = t; i < n; i += TILE) {
      int64_t p = s0 + i;
      if (rng) {
        real z0, z1, z2;
        raw_normals(a, step, p, z0, z1, z2);
        if (staged) { xs[3 * i] = z0; xs[3 * i + 1] = z1; xs[3 * i + 2] = z2; }
        sa[0].add(z0); sa[1].add(z1); sa[2].add(z2);
        if constexpr (F32) { sa[4].add(z0 * z0); sa[5].add(z1 * z1); sa[6].add(z2 * z2); }
      }
      if (fp) {
        real m1 = P.U1[p] - Us0, m2 = P.U2[p] - Us1, m3 = P.U3[p] - Us2;
        sa[3].add(m1 * m1 + m2 * m2 + m3 * m3);
      }
    }
    tile_reduce<real, KA, TILE>(sa, red);
    f1acc = sa[3];
    if (rng) {
      mean0 = cmean(sa[0], n); mean1 = cmean(sa[1], n); mean2 = cmean(sa[2], n);
      if constexpr (F32) {
        const float rn = 1.0f / (float)n;
        rms0 = sqrtf(fmaxf(sa[4].getr() * rn - mean0 * mean0, 0.f));
        rms1 = sqrtf(fmaxf(sa[5].getr() * rn - mean1 * mean1, 0.f));
        rms2 = sqrtf(fmaxf(sa[6].getr() * rn - mean2 * mean2, 0.f));
      } else {
        // ---- pass B: per-cell RMS of the centred draws
        Acc<real> s3[3];
#pragma unroll
        for (int q = 0; q < 3; ++q) s3[q].zero();
        for (int i = t; i < n; i += TILE) {
          real z0, z1, z2;
          if (staged) { z0 = xs[3 * i]; z1 = xs[3 * i + 1]; z2 = xs[3 * i + 2]; }
          else raw_normals(a, step, s0 + i, z0, z1, z2);
          real d0 = z0 - mean0, d1 = z1 - mean1, d2 = z2 - mean2;
          s3[0].add(d0 * d0); s3[1].add(d1 * d1); s3[2].add(d2 * d2);
        }
        tile_reduce<real, 3, TILE>(s3, red);
        rms0 = crms(s3[0], n); rms1 = crms(s3[1], n); rms2 = crms(s3[2], n);
      }
    }
  }
  const real irms0 = (real)1 / rms0, irms1 = (real)1 / rms1, irms2 = (real)1 / rms2;
  // whitened normal of the i-th particle of the cell
  auto xiw = [&](int i, real& z0, real& z1, real& z2) {
    int64_t p = s0 + i;
    if (load_xi) {
      z0 = (real)a.xi[p]; z1 = (real)a.xi[a.cap + p]; z2 = (real)a.xi[2 * a.cap + p];
      return;
    }
    if (staged) { z0 = xs[3 * i]; z1 = xs[3 * i + 1]; z2 = xs[3 * i + 2]; }
    else raw_normals(a, step, p, z0, z1, z2);
    if (n > 1) {
      if constexpr (F32) {
        z0 = (z0 - mean0) * irms0; z1 = (z1 - mean1) * irms1; z2 = (z2 - mean2) * irms2;
      } else {
        z0 = (z0 - mean0) / rms0; z1 = (z1 - mean1) / rms1; z2 = (z2 - mean2) / rms2;
      }
    }
  };
  // the Ornstein-Uhlenbeck update of M' with the cubic drift
  auto mnew = [&](int i, real& m1, real& m2, real& m3) {
    int64_t p = s0 + i;
    m1 = P.U1[p] - Us0; m2 = P.U2[p] - Us1; m3 = P.U3[p] - Us2;
    if (n > 1) {
      real z0, z1, z2;
      xiw(i, z0, z1, z2);
      // the expressions of src/Fokker_Planck.cpp:1114-1130, evaluated left
      // to right; mad() fuses in the FP32 path only
      real energy = mad(m3, m3, mad(m2, m2, m1 * m1));
      real d0 = mad(K.c[2], m3, mad(K.c[1], m2, K.c[0] * m1));
      d0 = mad(K.g[0], energy - K.eq, d0);
      d0 = mad(K.lam, mad(m1, energy, -K.q[0]), d0);
      real d1 = mad(K.c[4], m3, mad(K.c[3], m2, K.c[1] * m1));
      d1 = mad(K.g[1], energy - K.eq, d1);
      d1 = mad(K.lam, mad(m2, energy, -K.q[1]), d1);
      real d2 = mad(K.c[5], m3, mad(K.c[4], m2, K.c[2] * m1));
      d2 = mad(K.g[2], energy - K.eq, d2);
      d2 = mad(K.lam, mad(m3, energy, -K.q[2]), d2);
      m1 = mad(K.A3, z0, mad(K.A2, d0, K.A1 * m1));
      m2 = mad(K.A3, z1, mad(K.A2, d1, K.A1 * m2));
      m3 = mad(K.A3, z2, mad(K.A2, d2, K.A1 * m3));
    } else {
      m1 = 0; m2 = 0; m3 = 0;
    }
  };
  uint32_t bad = 0;
  // ---- pass C (split mode): keep the whitened normals for velocity_update
  if (rng && store_xi) {
    for (int i = t; i < n; i += TILE) {
      real z0, z1, z2;
      xiw(i, z0, z1, z2);
      int64_t p = s0 + i;
      a.xi[p] = (double)z0; a.xi[a.cap + p] = (double)z1; a.xi[2 * a.cap + p] = (double)z2;
    }
  }
  // ---- pass C: M'_new, sum |M'_new|^2; M'_new replaces the staged normals
  Acc<real> f2acc;
  f2acc.zero();
  if (fp) {
    Acc<real> f2[1];
    f2[0].zero();
    for (int i = t; i < n; i += TILE) {
      real m1, m2, m3;
      mnew(i, m1, m2, m3);
      if (m2 != m2) bad |= MCPM_ERR_NAN;
      f2[0].add(m1 * m1 + m2 * m2 + m3 * m3);
      if (staged) { xs[3 * i] = m1; xs[3 * i + 1] = m2; xs[3 * i + 2] = m3; }
    }
    tile_reduce<real, 1, TILE>(f2, red);
    f2acc = f2[0];
  }
  const uint32_t pos_stages = ST_LR | ST_DFP | ST_BC1 | ST_OLD | ST_STREAM | ST_BC2 | ST_BC3 | ST_KEY;
  if (!(fp || (st & pos_stages))) {
    raise_status(a.status, bad);
    return;
  }
  // ---- pass D: final velocities, then the position pipeline
  real scale = (real)1;
  if (fp && n > 1) {
    if constexpr (F32) scale = sqrtf(fabsf(f1acc.getr() / f2acc.getr()));
    else scale = r_sqrt(r_fabs(f1acc.get() / f2acc.get()));
  }
  const real F2dt = (st & ST_LR) ? K.f2dt : (real)0;
  const real dtr = kc.dt;
  const int iters = (n + TILE - 1) / TILE;
  for (int r = 0; r < iters; ++r) {
    const int i = r * TILE + t;
    const bool act = i < n;
    int key = 0;
    if (act) {
      const int64_t p = s0 + i;
      PState<real> s;
      s.u1 = P.U1[p]; s.u2 = P.U2[p]; s.u3 = P.U3[p];
      s.x1 = P.x1 ? P.x1[p] : (real)0;
      s.x2 = P.x2[p];
      s.x1o = P.x1o ? P.x1o[p] : (real)0;
      s.x2o = P.x2o ? P.x2o[p] : (real)0;
      const int pid = P.pid[p];
      if (fp) {
        if (n > 1) {
          real m1, m2, m3;
          if (staged) { m1 = xs[3 * i]; m2 = xs[3 * i + 1]; m3 = xs[3 * i + 2]; }
          else mnew(i, m1, m2, m3);
          s.u1 = m1 * scale + Us0; s.u2 = m2 * scale + Us1; s.u3 = m3 * scale + Us2;
        } else {
          s.u1 = Us0; s.u2 = Us1; s.u3 = Us2;
        }
      }
      if (st & ST_LR) {
        if (k.lr2d) {
          if constexpr (F32) {
            // U -= grad(V) coef/m dt with the bilinear coordinates of the particle
            const float xi = s.x1 * kc.idx - (float)(c % k.N0), eta = s.x2 * kc.idy - (float)(c / k.N0);
            s.u1 = s.u1 - (K.l2[0] + K.l2[1] * eta);
            s.u2 = s.u2 - (K.l2[2] + K.l2[3] * xi);
          } else {
            // src/FEM.cpp:703-714 in its order of operations
            const double xi = (s.x1 - K.xn0) / K.dxc, eta = (s.x2 - K.yn0) / K.dyc;
            double F1 = 0.0, Fy = 0.0;
            F1 += (eta - 1.0) * K.v[0]; Fy += (xi - 1.0) * K.v[0];
            F1 += (1.0 - eta) * K.v[1]; Fy += (-xi) * K.v[1];
            F1 += (-eta) * K.v[2]; Fy += (-xi + 1) * K.v[2];
            F1 += eta * K.v[3]; Fy += xi * K.v[3];
            F1 = F1 / k.m * k.lr_coef / K.dxc;
            Fy = Fy / k.m * k.lr_coef / K.dyc;
            s.u1 = s.u1 - F1 * k.dt;
            s.u2 = s.u2 - Fy * k.dt;
          }
        } else {
          s.u2 = s.u2 + F2dt;
        }
      }
      if (st & ST_DFP) {
        real e = (s.u1 - Us0) * (s.u1 - Us0) + (s.u2 - Us1) * (s.u2 - Us1) + (s.u3 - Us2) * (s.u3 - Us2);
        if constexpr (!F32) {
          if (k.dir0 == 1) {
            s.x1 = s.x1 + dtr * ((s.u1 - Us0) * K.al[0] + (s.u2 - Us1) * K.al[1] + (s.u3 - Us2) * K.al[2] +
                                 K.be0 * (e - K.eq)) +
                   K.gst * ((s.u1 - Us1) * e - K.m3_0 - K.m3_3 - K.m3_5) * dtr;
            s.x1 = s.x1 - dtr * K.ph0;
          }
          if (k.dir1 == 1) {
            s.x2 = s.x2 + dtr * ((s.u1 - Us0) * K.al[3] + (s.u2 - Us1) * K.al[4] + (s.u3 - Us2) * K.al[5] +
                                 K.be1 * (e - K.eq)) +
                   K.gst * ((s.u2 - Us1) * e - K.m3_1 - K.m3_6 - K.m3_8) * dtr;
            s.x2 = s.x2 - dtr * K.ph1;
          }
        } else {
          if (k.dir0 == 1) {
            s.x1 = s.x1 + dtr * ((s.u1 - Us0) * K.al[0] + (s.u2 - Us1) * K.al[1] + (s.u3 - Us2) * K.al[2] +
                                 K.be0 * (e - K.eq)) +
                   K.gst * ((s.u1 - Us1) * e - K.hq0) * dtr;
            s.x1 = s.x1 - dtr * K.ph0;
          }
          if (k.dir1 == 1) {
            s.x2 = s.x2 + dtr * ((s.u1 - Us0) * K.al[3] + (s.u2 - Us1) * K.al[4] + (s.u3 - Us2) * K.al[5] +
                                 K.be1 * (e - K.eq)) +
                   K.gst * ((s.u2 - Us1) * e - K.hq1) * dtr;
            s.x2 = s.x2 - dtr * K.ph1;
          }
        }
      }
      if (st & ST_BC1) apply_bc<real>(s, a.bc_call_base + 0, pid, step, k, kc, bad);
      if (st & ST_OLD) { s.x1o = s.x1; s.x2o = s.x2; }
      if (st & ST_STREAM) {
        if (k.dir0 == 1) s.x1 = s.x1 + dtr * s.u1;
        if (k.dir1 == 1) s.x2 = s.x2 + dtr * s.u2;
      }
      if (st & ST_BC2) apply_bc<real>(s, a.bc_call_base + 1, pid, step, k, kc, bad);
      if (st & ST_BC3) apply_bc<real>(s, a.bc_call_base + 2, pid, step, k, kc, bad);
      P.U1[p] = s.u1; P.U2[p] = s.u2; P.U3[p] = s.u3;
      if (P.x1) P.x1[p] = s.x1;
      P.x2[p] = s.x2;
      if (P.x1o) P.x1o[p] = s.x1o;
      if (P.x2o) P.x2o[p] = s.x2o;
      if (st & ST_KEY) {
        key = bin_one<real>(s.x1, s.x2, pid, step + 1, k, kc, bad);
        a.key_out[p] = key;
      }
    }
    if (st & ST_KEY) count_key(a.cnt_next, key, act);
  }
  raise_status(a.status, bad);
}

// Launch shape of the FP32 particle pass: blocks of 256 threads resident
// per SM (the register budget: 5 blocks = 48 registers, measured fastest on
// GB300 against 3, 4 and 6 -- the pass is latency-bound, so warps in flight
// beat the few spills), and the unroll factor of its particle loops.
#ifndef MCPM_UPD_MINB
#define MCPM_UPD_MINB 5
#endif
#ifndef MCPM_UPD_MINB_SL
#define MCPM_UPD_MINB_SL 5
#endif
#ifndef MCPM_UPD_PF_C
#define MCPM_UPD_PF_C 1
#endif
#ifndef MCPM_UPD_PF_D
#define MCPM_UPD_PF_D 1
#endif
#ifndef MCPM_UPD_PF_A
#define MCPM_UPD_PF_A 1
#endif
#ifndef MCPM_UPD_UNROLL
#define MCPM_UPD_UNROLL 1
#endif
// 1: the record's constants of the velocity update held in registers for the
// particle loops (else read from the shared record at each use)
#ifndef MCPM_UPD_REGK
#define MCPM_UPD_REGK 0
#endif
#define MCPM_STR2(x) #x
#define MCPM_STR(x) MCPM_STR2(x)
#define UPD_UNROLL _Pragma(MCPM_STR(unroll MCPM_UPD_UNROLL))


// The FP32 particle pass: the stages of update_cell for float state, with
// plain FP32 per-lane sums of the whitening and energy terms combined
// pairwise (tile_sum_f32),
// fused multiply-adds throughout, and the packed per-cell record read into
// registers where each pass needs it.
template <int TILE, uint32_t CST, int PB, bool SL>
__device__ void update_cell_f32(int c, const UpdArgs<float>& a, int step, float* xs, int xcap, float* red,
                                float* R) {
  const int t = (TILE == 32) ? (threadIdx.x & 31) : threadIdx.x;
  const int64_t s0 = a.off[c];
  const int n = a.cnt[c];
  const DevConsts& k = a.k;
  const KC<float>& kc = a.kc;
  const uint32_t st = CST ? CST : a.stages;
  const bool rng = st & ST_RNG, fp = st & ST_FP, load_xi = st & ST_LOAD_XI, store_xi = st & ST_STORE_XI;
  const bool staged = rng && n <= xcap;
  // the cell's packed record in shared memory (R: PF_STRIDE floats of this
  // warp or block), read by broadcast where each pass needs a constant
  if (TILE == 32) __syncwarp();
  else __syncthreads();
  if (t < PF_STRIDE / 4)
    reinterpret_cast<float4*>(R)[t] = __ldg(reinterpret_cast<const float4*>(a.pcell + (size_t)c * PF_STRIDE) + t);
  if (TILE == 32) __syncwarp();
  else __syncthreads();
  const float Us0 = R[PF_US0], Us1 = R[PF_US1], Us2 = R[PF_US2];
  const PT<float>& P = a.p;  // pointers stay in the parameter bank
  float mean0 = 0.f, mean1 = 0.f, mean2 = 0.f, irms0 = 1.f, irms1 = 1.f, irms2 = 1.f, f1 = 0.f;
  // ---- pass A: draws and their per-cell sums.  sum |M'|^2 before the
  // update is the moment pass's energy sum (the same M' = U - U_space)
  f1 = R[PF_E2];
  if (rng) {
    float sa[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // z0 z1 z2 z0^2 z1^2 z2^2
#if MCPM_UPD_PF_A
    // the next particle's id is loaded while this one's draws are made
    int npid = t < n ? P.pid[s0 + t] : 0;
#endif
    UPD_UNROLL
    for (int i = t; i < n; i += TILE) {
      float z0, z1, z2;
#if MCPM_UPD_PF_A
      const int pid_i = npid;
      if (i + TILE < n) npid = P.pid[s0 + i + TILE];
      raw_normals_pid(a, step, pid_i, z0, z1, z2);
#else
      raw_normals(a, step, s0 + i, z0, z1, z2);
#endif
      if (staged) { xs[3 * i] = z0; xs[3 * i + 1] = z1; xs[3 * i + 2] = z2; }
      sa[0] += z0; sa[1] += z1; sa[2] += z2;
      sa[3] = fmaf(z0, z0, sa[3]); sa[4] = fmaf(z1, z1, sa[4]); sa[5] = fmaf(z2, z2, sa[5]);
    }
    tile_sum_f32<6, TILE>(sa, red);
    const float rn = 1.0f / (float)n;
    mean0 = sa[0] * rn; mean1 = sa[1] * rn; mean2 = sa[2] * rn;
    irms0 = 1.0f / sqrtf(fmaxf(fmaf(-mean0, mean0, sa[3] * rn), 0.f));
    irms1 = 1.0f / sqrtf(fmaxf(fmaf(-mean1, mean1, sa[4] * rn), 0.f));
    irms2 = 1.0f / sqrtf(fmaxf(fmaf(-mean2, mean2, sa[5] * rn), 0.f));
  }
  // whitened normal of the i-th particle of the cell
  auto xiw = [&](int i, float& z0, float& z1, float& z2) {
    const int64_t p = s0 + i;
    if (load_xi) {
      z0 = (float)a.xi[p]; z1 = (float)a.xi[a.cap + p]; z2 = (float)a.xi[2 * a.cap + p];
      return;
    }
    if (staged) { z0 = xs[3 * i]; z1 = xs[3 * i + 1]; z2 = xs[3 * i + 2]; }
    else raw_normals(a, step, p, z0, z1, z2);
    if (n > 1) { z0 = (z0 - mean0) * irms0; z1 = (z1 - mean1) * irms1; z2 = (z2 - mean2) * irms2; }
  };
  uint32_t bad = 0;
  // ---- pass C (split mode): keep the whitened normals for velocity_update
  if (rng && store_xi) {
    for (int i = t; i < n; i += TILE) {
      float z0, z1, z2;
      xiw(i, z0, z1, z2);
      const int64_t p = s0 + i;
      a.xi[p] = (double)z0; a.xi[a.cap + p] = (double)z1; a.xi[2 * a.cap + p] = (double)z2;
    }
  }
  // the Ornstein-Uhlenbeck update of M' with the cubic drift
  // (src/Fokker_Planck.cpp:1114-1130), constants from the shared record
#if MCPM_UPD_REGK
  const float kC0 = R[PF_C0], kC1 = R[PF_C0 + 1], kC2 = R[PF_C0 + 2], kC3 = R[PF_C0 + 3], kC4 = R[PF_C0 + 4],
              kC5 = R[PF_C0 + 5], kG0 = R[PF_G0], kG1 = R[PF_G1], kG2 = R[PF_G2], kQ0 = R[PF_Q0], kQ1 = R[PF_Q1],
              kQ2 = R[PF_Q2], kEQ = R[PF_EQ], kLAM = R[PF_LAM], kA1 = R[PF_A1], kA2 = R[PF_A2], kA3 = R[PF_A3];
#define RK(name, idx) name
#else
#define RK(name, idx) R[idx]
#endif
  auto mnew_u = [&](int i, float u1, float u2, float u3, float& m1, float& m2, float& m3) {
    m1 = u1 - Us0; m2 = u2 - Us1; m3 = u3 - Us2;
    if (n > 1) {
      float z0, z1, z2;
      xiw(i, z0, z1, z2);
      const float energy = fmaf(m3, m3, fmaf(m2, m2, m1 * m1));
      const float ee = energy - RK(kEQ, PF_EQ), lam = RK(kLAM, PF_LAM);
      float d0 = fmaf(RK(kC2, PF_C0 + 2), m3, fmaf(RK(kC1, PF_C0 + 1), m2, RK(kC0, PF_C0) * m1));
      d0 = fmaf(lam, fmaf(m1, energy, -RK(kQ0, PF_Q0)), fmaf(RK(kG0, PF_G0), ee, d0));
      float d1 = fmaf(RK(kC4, PF_C0 + 4), m3, fmaf(RK(kC3, PF_C0 + 3), m2, RK(kC1, PF_C0 + 1) * m1));
      d1 = fmaf(lam, fmaf(m2, energy, -RK(kQ1, PF_Q1)), fmaf(RK(kG1, PF_G1), ee, d1));
      float d2 = fmaf(RK(kC5, PF_C0 + 5), m3, fmaf(RK(kC4, PF_C0 + 4), m2, RK(kC2, PF_C0 + 2) * m1));
      d2 = fmaf(lam, fmaf(m3, energy, -RK(kQ2, PF_Q2)), fmaf(RK(kG2, PF_G2), ee, d2));
      const float A1 = RK(kA1, PF_A1), A2 = RK(kA2, PF_A2), A3 = RK(kA3, PF_A3);
#undef RK
      m1 = fmaf(A3, z0, fmaf(A2, d0, A1 * m1));
      m2 = fmaf(A3, z1, fmaf(A2, d1, A1 * m2));
      m3 = fmaf(A3, z2, fmaf(A2, d2, A1 * m3));
    } else {
      m1 = 0.f; m2 = 0.f; m3 = 0.f;
    }
  };
  auto mnew = [&](int i, float& m1, float& m2, float& m3) {
    const int64_t p = s0 + i;
    mnew_u(i, P.U1[p], P.U2[p], P.U3[p], m1, m2, m3);
  };
  // ---- pass C: M'_new, sum |M'_new|^2; M'_new replaces the staged normals
  float scale = 1.f;
  if (fp) {
    float f2[1] = {0.f};
#if MCPM_UPD_PF_C
    // the next particle's velocities are loaded while this one is computed
    float nu1 = 0.f, nu2 = 0.f, nu3 = 0.f;
    if (t < n) { nu1 = P.U1[s0 + t]; nu2 = P.U2[s0 + t]; nu3 = P.U3[s0 + t]; }
#endif
    UPD_UNROLL
    for (int i = t; i < n; i += TILE) {
      float m1, m2, m3;
#if MCPM_UPD_PF_C
      const float u1 = nu1, u2 = nu2, u3 = nu3;
      if (i + TILE < n) {
        const int64_t q = s0 + i + TILE;
        nu1 = P.U1[q]; nu2 = P.U2[q]; nu3 = P.U3[q];
      }
      mnew_u(i, u1, u2, u3, m1, m2, m3);
#else
      mnew(i, m1, m2, m3);
#endif
      if (m2 != m2) bad |= MCPM_ERR_NAN;
      f2[0] = fmaf(m3, m3, fmaf(m2, m2, fmaf(m1, m1, f2[0])));
      if (staged) { xs[3 * i] = m1; xs[3 * i + 1] = m2; xs[3 * i + 2] = m3; }
    }
    tile_sum_f32<1, TILE>(f2, red);
    if (n > 1) scale = sqrtf(fabsf(f1 / f2[0]));
  }
  const uint32_t pos_stages = ST_LR | ST_DFP | ST_BC1 | ST_OLD | ST_STREAM | ST_BC2 | ST_BC3 | ST_KEY;
  if (!(fp || (st & pos_stages))) {
    raise_status(a.status, bad);
    return;
  }
  // ---- pass D: final velocities, then the position pipeline
  const float dtr = kc.dt;
  const float fj = (float)(c % k.N0), fk = (float)(c / k.N0);
  const int iters = (n + TILE - 1) / TILE;
  // the next particle's positions and id are loaded while this one is moved
  // (measured 5% faster with the learned-force kick as well)
  constexpr bool PFD = MCPM_UPD_PF_D && CST != 0;
#if MCPM_UPD_REGK >= 2
  const float dLA1 = R[PF_LA1], dLB1 = R[PF_LB1], dLA2 = R[PF_LA2], dLB2 = R[PF_LB2], dF2DT = R[PF_F2DT];
  const float dEQ = R[PF_EQ], dGST = R[PF_GST], dBE0 = R[PF_BE0], dBE1 = R[PF_BE1], dHQ0 = R[PF_HQ0],
              dHQ1 = R[PF_HQ1], dPH0 = R[PF_PH0], dPH1 = R[PF_PH1];
  const float dAL[6] = {R[PF_AL0], R[PF_AL0 + 1], R[PF_AL0 + 2], R[PF_AL0 + 3], R[PF_AL0 + 4], R[PF_AL0 + 5]};
#define RD(name, idx) name
#define RDA(j) dAL[j]
#else
#define RD(name, idx) R[idx]
#define RDA(j) R[PF_AL0 + (j)]
#endif
  float nx1 = 0.f, nx2 = 0.f;
  int npid = 0;
  if (PFD && t < n) { nx1 = P.x1 ? P.x1[s0 + t] : 0.f; nx2 = P.x2[s0 + t]; npid = P.pid[s0 + t]; }
  UPD_UNROLL
  for (int r = 0; r < iters; ++r) {
    const int i = r * TILE + t;
    const bool act = i < n;
    int key = 0, pid = 0;
    PState<float> s;
    if constexpr (PFD) {
      s.x1 = nx1; s.x2 = nx2; pid = npid;
      if (i + TILE < n) {
        const int64_t q = s0 + i + TILE;
        nx1 = P.x1 ? P.x1[q] : 0.f; nx2 = P.x2[q]; npid = P.pid[q];
      }
    }
    if (act) {
      const int64_t p = s0 + i;
      if constexpr (!PFD) {
        s.x1 = P.x1 ? P.x1[p] : 0.f;
        s.x2 = P.x2[p];
        pid = P.pid[p];
      }
      s.x1o = P.x1o ? P.x1o[p] : 0.f;
      s.x2o = P.x2o ? P.x2o[p] : 0.f;
      if (fp) {
        if (n > 1) {
          float m1, m2, m3;
          if (staged) { m1 = xs[3 * i]; m2 = xs[3 * i + 1]; m3 = xs[3 * i + 2]; }
          else mnew(i, m1, m2, m3);
          s.u1 = fmaf(m1, scale, Us0); s.u2 = fmaf(m2, scale, Us1); s.u3 = fmaf(m3, scale, Us2);
        } else {
          s.u1 = Us0; s.u2 = Us1; s.u3 = Us2;
        }
      } else {
        s.u1 = P.U1[p]; s.u2 = P.U2[p]; s.u3 = P.U3[p];
      }
      if (st & ST_LR) {
        if (k.lr2d) {
          // U -= grad(V) coef/m dt with the bilinear coordinates of the particle
          const float xi = fmaf(s.x1, kc.idx, -fj), eta = fmaf(s.x2, kc.idy, -fk);
          s.u1 = s.u1 - fmaf(RD(dLB1, PF_LB1), eta, RD(dLA1, PF_LA1));
          s.u2 = s.u2 - fmaf(RD(dLB2, PF_LB2), xi, RD(dLA2, PF_LA2));
        } else {
          s.u2 = s.u2 + RD(dF2DT, PF_F2DT);
        }
      }
      if (st & ST_DFP) {
        // DFP_extra_streaming, src/Fokker_Planck.cpp:904-946 (the x1
        // heat-flux term uses U_space[1], as there)
        const float w1 = s.u1 - Us0, w2 = s.u2 - Us1, w3 = s.u3 - Us2;
        const float e = fmaf(w3, w3, fmaf(w2, w2, w1 * w1));
        const float ee = e - RD(dEQ, PF_EQ), gst = RD(dGST, PF_GST);
        if (k.dir0 == 1) {
          const float v = fmaf(RD(dBE0, PF_BE0), ee, fmaf(RDA(2), w3, fmaf(RDA(1), w2, RDA(0) * w1)));
          const float h = gst * fmaf(s.u1 - Us1, e, -RD(dHQ0, PF_HQ0));
          s.x1 = fmaf(h, dtr, fmaf(dtr, v, s.x1));
          s.x1 = fmaf(-dtr, RD(dPH0, PF_PH0), s.x1);
        }
        if (k.dir1 == 1) {
          const float v = fmaf(RD(dBE1, PF_BE1), ee, fmaf(RDA(5), w3, fmaf(RDA(4), w2, RDA(3) * w1)));
          const float h = gst * fmaf(w2, e, -RD(dHQ1, PF_HQ1));
          s.x2 = fmaf(h, dtr, fmaf(dtr, v, s.x2));
          s.x2 = fmaf(-dtr, RD(dPH1, PF_PH1), s.x2);
        }
      }
      // apply_BC: the box's wall type fixed at compile time where the
      // launch knows it (PB), else the run-time dispatch; true when the
      // call may have moved the particle
      auto bc = [&](int call) -> bool {
        if constexpr (PB == MCPM_PROBLEM_CLOSED_BOX) {
          // the first-pass tests of BC_specular_reflection: a particle that
          // triggers none of them is left as it is
          const bool r1 = k.dir0 == 1 && (s.x1 - kc.L0 > -1e-16f || s.x1 < 1e-16f);
          const bool r2 = k.dir1 == 1 && (s.x2 - kc.L1 > -1e-16f || s.x2 < 1e-16f);
          if (r1 || r2) bc_specular<float>(s, k, kc, bad);
          return r1 || r2;
        }
        else if constexpr (PB == MCPM_PROBLEM_PERIODIC) bc_periodic<float>(s, k, kc);
        else apply_bc<float>(s, a.bc_call_base + call, pid, step, k, kc, bad);
        return true;
      };
      if (st & ST_BC1) bc(0);
      if (st & ST_OLD) { s.x1o = s.x1; s.x2o = s.x2; }
      if (st & ST_STREAM) {
        if (k.dir0 == 1) s.x1 = fmaf(dtr, s.u1, s.x1);
        if (k.dir1 == 1) s.x2 = fmaf(dtr, s.u2, s.x2);
      }
      // the third call sees the second's position: between specular walls
      // it can only act where the second reflected the particle
      const bool moved = (st & ST_BC2) ? bc(1) : true;
      if ((st & ST_BC3) && (PB != MCPM_PROBLEM_CLOSED_BOX || moved)) bc(2);
      if constexpr (!SL) {
        P.U1[p] = s.u1; P.U2[p] = s.u2; P.U3[p] = s.u3;
        if (P.x1) P.x1[p] = s.x1;
        P.x2[p] = s.x2;
        if (P.x1o) P.x1o[p] = s.x1o;
        if (P.x2o) P.x2o[p] = s.x2o;
      }
      if (SL || (st & ST_KEY)) {
        key = bin_one<float>(s.x1, s.x2, pid, step + 1, k, kc, bad);
        if constexpr (!SL) a.key_out[p] = key;
      }
    }
    if constexpr (SL) {
      // the particle's slot in its new cell's region: one atomic per cell
      // and warp (the lanes bound for the same cell share it), the lane's
      // rank among them on top
      const int lane = threadIdx.x & 31;
      const unsigned am = __ballot_sync(FULL, act);
      if (act) {
        const unsigned peers = __match_any_sync(am, key);
        const int leader = __ffs(peers) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(&a.dcur[key], __popc(peers));
        base = __shfl_sync(peers, base, leader);
        const int slot = base + __popc(peers & ((1u << lane) - 1u));
        const int r0 = a.doff[key], capc = a.doff[key + 1] - r0;
        if (slot < capc) {
          store_state(a.d, (int64_t)r0 + slot, s, pid);
        } else {  // the region is full: to the overflow arrays
          const int64_t e = atomicAdd(a.ovf_n, 1);
          a.ovf_key[e] = key;
          store_state(a.ovf, e, s, pid);
        }
      }
    } else if (st & ST_KEY) {
      count_key(a.cnt_next, key, act);
    }
  }
#undef RD
#undef RDA
  raise_status(a.status, bad);
}

template <typename real, uint32_t CST, int PB = 0, bool SL = false>
__global__ void __launch_bounds__(256, sizeof(real) == 4 ? (CST ? (SL ? MCPM_UPD_MINB_SL : MCPM_UPD_MINB) : 3) : 1)
    k_update(UpdArgs<real> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ Acc<real> red[8 * 8];
  real* xs = reinterpret_cast<real*>(smem_raw);
  const int warp = threadIdx.x >> 5;
  const int step = *a.dstep;
  if constexpr (sizeof(real) == 4) {
    float* rf = reinterpret_cast<float*>(red);
    __shared__ __align__(16) float recs[8][PF_STRIDE];
    schedule_cells(
        a.list_big, a.list_small, a.wl, a.work, WK_UPD_BIG, WK_UPD_SMALL,
        [&](int c) { update_cell_f32<256, CST, PB, SL>(c, a, step, xs, a.bcap, rf, recs[0]); },
        [&](int c) {
          update_cell_f32<32, CST, PB, SL>(c, a, step, xs + (size_t)warp * 3 * (a.bcap / 8), a.bcap / 8, rf,
                                           recs[warp]);
        });
  } else {
    schedule_cells(
        a.list_big, a.list_small, a.wl, a.work, WK_UPD_BIG, WK_UPD_SMALL,
        [&](int c) { update_cell<real, 256, CST>(c, a, step, xs, a.bcap, red); },
        [&](int c) { update_cell<real, 32, CST>(c, a, step, xs + (size_t)warp * 3 * (a.bcap / 8), a.bcap / 8, red); });
  }
}

// the fused FP_dense step with specular or periodic walls and no long-range
// force: every stage fixed at compile time
constexpr uint32_t ST_FUSED_FP = ST_RNG | ST_FP | ST_DFP | ST_BC1 | ST_STREAM | ST_BC2 | ST_BC3 | ST_KEY;
// the fused step of the collision models (ESMC, DSMC): walls, flight and
// re-binning, with the old positions the diffuse walls and Couette flow
// keep (ST_FUSED_COLL_OLD) or without them
constexpr uint32_t ST_FUSED_COLL = ST_BC1 | ST_STREAM | ST_BC2 | ST_BC3 | ST_KEY;
constexpr uint32_t ST_FUSED_COLL_OLD = ST_FUSED_COLL | ST_OLD;

// ========================================================= host<->device
// one staged field into the state's precision (uploads: each field's
// conversion overlaps the copy of the next), and the particle ids
template <typename real>
__global__ void k_convert_field(real* dst, const double* src, int32_t* pid, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    dst[i] = (real)src[i];
    if (pid) pid[i] = (int32_t)i;
  }
}
// a staged field in particle-id order into the slots of a packed layout
template <typename real>
__global__ void k_gather_field(real* dst, const double* src, const int32_t* pid, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (real)src[pid[i]];
}
template <typename real>
__global__ void k_convert_out_field(PT<real> p, PT<real> ovf, const int32_t* ovf_n, const int32_t* off,
                                    const int32_t* dcur, int C, int f, double* dst, int64_t n) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  auto field = [&](const PT<real>& src) -> const real* {
    return f == 0 ? src.x1 : f == 1 ? src.x2 : f == 2 ? src.U1 : f == 3 ? src.U2 : f == 4 ? src.U3
                                                                        : f == 5 ? src.x1o : src.x2o;
  };
  const real* v = field(p);
  if (!dcur) {
    for (int64_t i = tid; i < n; i += nt) dst[p.pid[i]] = (double)v[i];
    return;
  }
  const int lane = threadIdx.x & 31;
  for (int64_t c = tid >> 5; c < C; c += nt >> 5) {
    const int s0 = off[c], m = min(dcur[c], off[c + 1] - s0);
    for (int i = lane; i < m; i += 32) dst[p.pid[s0 + i]] = (double)v[s0 + i];
  }
  const real* w = field(ovf);
  const int n_ovf = *ovf_n;
  for (int64_t e = tid; e < n_ovf; e += nt) dst[ovf.pid[e]] = (double)w[e];
}


// ============================================================ launchers
static inline int grid_for(int64_t n, int block, int max_blocks) {
  int64_t g = (n + block - 1) / block;
  if (g < 1) g = 1;
  if (g > max_blocks) g = max_blocks;
  return (int)g;
}

template <typename real> static int bin_impl(Session& s, int bin_step) {
  PT<real> p = pt<real>(s.P[s.cur]);
  // every key is recomputed: counts start from zero, whatever was pending
  cudaMemsetAsync(s.cnt_next, 0, (size_t)s.C * sizeof(int32_t), s.stream);
  k_bin<real><<<grid_for(s.N, 256, s.num_sms * 8), 256, 0, s.stream>>>(p, s.N, s.k, bin_step, s.key, s.cnt_next,
                                                                         s.status);
  return 1;
}
int launch_bin(Session& s, int bin_step) { return s.prec == MCPM_FP32 ? bin_impl<float>(s, bin_step) : bin_impl<double>(s, bin_step); }

static void scan_launch(Session& s, const int32_t* src, int32_t* off, int32_t* noff) {
  const int nblk = (s.C + SCAN_T - 1) / SCAN_T;
  k_scan_blocks<<<nblk, SCAN_T, 0, s.stream>>>(src, s.scan_blk, s.C, s.tune.wcap);
  k_scan_totals<<<1, SCAN_T, 0, s.stream>>>(s.scan_blk, nblk, s.wl, s.work, s.use_slotted ? s.ovf_n : nullptr,
                                            s.ovf_par);
  ScanOut o;
  o.cnt_next = s.cnt_next; o.cursor = s.cursor; o.dcur = s.dcur;
  o.src = src;
  o.cnt = s.cnt; o.off = off; o.noff = noff; o.doff = s.use_slotted ? s.doff : nullptr;
  o.list_small = s.list_small; o.list_big = s.list_big;
  o.blk = s.scan_blk; o.C = s.C; o.wcap = s.tune.wcap;
  k_scan_write<<<nblk, SCAN_T, 0, s.stream>>>(o);
}

int launch_scan(Session& s) {
  scan_launch(s, s.cnt_next, s.off, nullptr);
  return 3;
}

// the scan of a slotted layout: counts from the slot counters, the region
// bases stay (off), the packed offsets go to noff for the repair
int launch_scan_slotted(Session& s) {
  scan_launch(s, s.dcur, nullptr, s.noff);
  return 3;
}

template <typename real> static int repair_impl(Session& s, bool force) {
  PT<real> src = pt<real>(s.P[s.cur]), oth = pt<real>(s.P[1 - s.cur]), ov = pt<real>(s.ovf);
  const int32_t* ovn = s.ovf_n + (1 - s.ovf_par);  // the counter of the pass that made the layout
  const int g = s.num_sms * 4;
  if (force) {
    k_pack<real><<<g, 256, 0, s.stream>>>(src, oth, ov, s.ovf_key, ovn, s.off, s.cnt, s.noff, s.cursor, s.C,
                                          s.status);
    return 1;
  }
  k_relocate<real><<<g, 256, 0, s.stream>>>(src, ovn, s.off, s.cnt, s.noff, s.cursor, s.ovf_n + OVF_SPARE, s.C);
  k_relocate_tail<real><<<g, 256, 0, s.stream>>>(src, ov, s.ovf_key, ovn, s.noff, s.cnt, s.cursor, s.off, s.C,
                                                 s.status);
  return 2;
}
int launch_repair(Session& s) { return s.prec == MCPM_FP32 ? repair_impl<float>(s, false) : repair_impl<double>(s, false); }

// a slotted layout packed into the other buffer (host-side: the buffer and
// the offsets change places)
int launch_compact(Session& s) {
  int n = launch_scan_slotted(s);
  n += s.prec == MCPM_FP32 ? repair_impl<float>(s, true) : repair_impl<double>(s, true);
  s.cur = 1 - s.cur;
  std::swap(s.off, s.noff);
  return n;
}

template <typename real> static int scatter_impl(Session& s) {
  PT<real> src = pt<real>(s.P[s.cur]), dst = pt<real>(s.P[1 - s.cur]);
  k_scatter<real><<<grid_for(s.N, 256, s.num_sms * 8), 256, 0, s.stream>>>(src, dst, s.key, s.off, s.cursor, s.N);
  s.cur = 1 - s.cur;
  return 1;
}
int launch_scatter(Session& s) { return s.prec == MCPM_FP32 ? scatter_impl<float>(s) : scatter_impl<double>(s); }

template <typename real> static int moments_impl(Session& s) {
  PT<real> p = pt<real>(s.P[s.cur]);
  MomArgs<real> a{s.k, s.cell, s.off, s.cnt, s.list_small, s.list_big, s.wl, s.work, p.U1, p.U2, p.U3};
  k_moments<real><<<s.tune.grid_mom, 256, 0, s.stream>>>(a);
  return 1;
}
int launch_moments(Session& s) { return s.prec == MCPM_FP32 ? moments_impl<float>(s) : moments_impl<double>(s); }

// threads per block of the per-cell solves: MCPM_SOLVE_T, halved (down to
// 8) while the grid would have fewer blocks than SMs -- a small grid's cells
// then spread over the SMs' FP64 pipes instead of queueing on a few
int solve_block(const Session& s) {
  int t = MCPM_SOLVE_T;
  while (t > 8 && (s.C + t - 1) / t < s.num_sms) t >>= 1;
  return t;
}

int launch_solve(Session& s, int with_alpha) {
  // c_gamma_calculation and the Langevin constants (src/Main_Functions.cpp:2729)
  const int m = s.cfg.model;
  int fp = (m == MCPM_MODEL_FP_DENSE || m == MCPM_MODEL_FP_IDEAL_GAS || m == MCPM_MODEL_FP_LINEAR) ? 1 : 0;
  // the FP64 path reproduces the reference's solve exactly; the FP32 path
  // runs the leaner FP64 variant
  if (s.prec == MCPM_FP32) return launch_solve_fast(s, with_alpha, fp);
  const int bt = solve_block(s), nb = (s.C + bt - 1) / bt;
  k_solve<true><<<nb, bt, 0, s.stream>>>(s.k, s.cell, nullptr, with_alpha, fp, s.status);
  return 1;
}

// shared staging: bcap particles for the block path, bcap / 8 per warp for
// the warp path (cells above that capacity recompute instead of staging)
template <typename real> static size_t update_smem(const Session& s) {
  return 3 * sizeof(real) * (size_t)s.tune.bcap;
}

template <typename real> static int update_impl(Session& s, uint32_t stages, int bc_call_base, bool slotted) {
  const int n = sync_dstep(s);
  UpdArgs<real> a;
  a.k = s.k;
  a.cell = s.cell;
  a.pcell = s.pcell;
  a.off = s.off; a.cnt = s.cnt; a.list_small = s.list_small; a.list_big = s.list_big; a.wl = s.wl;
  a.work = s.work;
  a.p = pt<real>(s.P[s.cur]);
  a.key_out = s.key;
  a.cnt_next = s.cnt_next;
  a.inj = s.inj;
  a.xi = s.xi;
  a.cap = s.cap;
  a.status = s.status;
  a.dstep = s.dstep;
  a.rng_mode = s.rng_mode;
  a.bc_call_base = bc_call_base;
  a.stages = stages;
  a.wcap = s.tune.wcap;
  a.bcap = s.tune.bcap;
  a.Vn = lr2d_potential(s);
  a.kc = make_kc<real>(s.k);
  a.d = pt<real>(s.P[1 - s.cur]);
  a.doff = s.doff;
  a.dcur = s.dcur;
  a.ovf = pt<real>(s.ovf);
  a.ovf_key = s.ovf_key;
  a.ovf_n = s.ovf_n ? s.ovf_n + s.ovf_par : nullptr;
  size_t sm = update_smem<real>(s);
  const dim3 g(s.tune.grid_upd), b(256);
  const bool spec = s.k.problem == MCPM_PROBLEM_CLOSED_BOX, per = s.k.problem == MCPM_PROBLEM_PERIODIC;
  constexpr int SPEC = MCPM_PROBLEM_CLOSED_BOX, PER = MCPM_PROBLEM_PERIODIC;
  constexpr uint32_t F = ST_FUSED_FP, FL = ST_FUSED_FP | ST_LR;
  if constexpr (sizeof(real) == 4) {
    if (slotted) {
      // the pass writes the slotted layout of the other buffer
      if (stages == F) {
        if (spec) k_update<real, F, SPEC, true><<<g, b, sm, s.stream>>>(a);
        else if (per) k_update<real, F, PER, true><<<g, b, sm, s.stream>>>(a);
        else k_update<real, F, 0, true><<<g, b, sm, s.stream>>>(a);
      } else if (stages == FL) {
        if (spec) k_update<real, FL, SPEC, true><<<g, b, sm, s.stream>>>(a);
        else if (per) k_update<real, FL, PER, true><<<g, b, sm, s.stream>>>(a);
        else k_update<real, FL, 0, true><<<g, b, sm, s.stream>>>(a);
      } else if (stages == ST_FUSED_COLL_OLD) {
        k_update<real, ST_FUSED_COLL_OLD, 0, true><<<g, b, sm, s.stream>>>(a);
      } else if (stages == ST_FUSED_COLL) {
        k_update<real, ST_FUSED_COLL, 0, true><<<g, b, sm, s.stream>>>(a);
      } else {
        k_update<real, 0u, 0, true><<<g, b, sm, s.stream>>>(a);
      }
      return n + 1;
    }
    if (stages == F) {
      if (spec) k_update<real, F, SPEC><<<g, b, sm, s.stream>>>(a);
      else if (per) k_update<real, F, PER><<<g, b, sm, s.stream>>>(a);
      else k_update<real, F><<<g, b, sm, s.stream>>>(a);
      return n + 1;
    }
    if (stages == FL) {
      if (spec) k_update<real, FL, SPEC><<<g, b, sm, s.stream>>>(a);
      else if (per) k_update<real, FL, PER><<<g, b, sm, s.stream>>>(a);
      else k_update<real, FL><<<g, b, sm, s.stream>>>(a);
      return n + 1;
    }
  }
  if (stages == F) k_update<real, F><<<g, b, sm, s.stream>>>(a);
  else if (stages == FL) k_update<real, FL><<<g, b, sm, s.stream>>>(a);
  else k_update<real, 0u><<<g, b, sm, s.stream>>>(a);
  return n + 1;
}
int launch_update(Session& s, uint32_t stages, int bc_call_base, bool slotted) {
  return s.prec == MCPM_FP32 ? update_impl<float>(s, stages, bc_call_base, slotted)
                             : update_impl<double>(s, stages, bc_call_base, false);
}

template <typename real> static int conv_field_impl(Session& s, int f, int64_t n, cudaStream_t st) {
  const PBuf& b = s.P[s.cur];
  void* dsts[5] = {b.x1, b.x2, b.U1, b.U2, b.U3};
  if (!dsts[f]) return 0;
  k_convert_field<real><<<grid_for(n, 256, s.num_sms * 8), 256, 0, st>>>(
      (real*)dsts[f], s.stage_in + (size_t)f * s.cap, f == 2 ? b.pid : nullptr, n);
  return 1;
}
int launch_convert_field(Session& s, int field, int64_t n, cudaStream_t st) {
  return s.prec == MCPM_FP32 ? conv_field_impl<float>(s, field, n, st) : conv_field_impl<double>(s, field, n, st);
}
int launch_gather_field(Session& s, void* dst, const double* src) {
  const PBuf& b = s.P[s.cur];
  if (s.prec == MCPM_FP32)
    k_gather_field<float><<<grid_for(s.N, 256, s.num_sms * 8), 256, 0, s.stream>>>((float*)dst, src, b.pid, s.N);
  else
    k_gather_field<double><<<grid_for(s.N, 256, s.num_sms * 8), 256, 0, s.stream>>>((double*)dst, src, b.pid, s.N);
  return 1;
}
template <typename real> static int conv_out_field_impl(Session& s, int f, int64_t n) {
  const bool sl = s.slotted;
  k_convert_out_field<real><<<s.num_sms * 8, 256, 0, s.stream>>>(
      pt<real>(s.P[s.cur]), pt<real>(s.ovf), sl ? s.ovf_n + (1 - s.ovf_par) : nullptr, s.off, sl ? s.dcur : nullptr,
      s.C, f, s.stage + (size_t)(f < 5 ? f : f - 5) * s.cap, n);  // old positions: the first two slices
  return 1;
}
int launch_convert_out_field(Session& s, int field, int64_t n) {
  return s.prec == MCPM_FP32 ? conv_out_field_impl<float>(s, field, n) : conv_out_field_impl<double>(s, field, n);
}
// the dynamic shared memory the update kernel needs, for the session setup
size_t update_smem_bytes(const Session& s) {
  return s.prec == MCPM_FP32 ? update_smem<float>(s) : update_smem<double>(s);
}
cudaError_t update_set_smem_max() {
  int dev = 0, mx = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&mx, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  mx -= 4096;  // leave room for the static reduction scratch and cell records
  constexpr uint32_t F = ST_FUSED_FP, FL = ST_FUSED_FP | ST_LR;
  constexpr int SPEC = MCPM_PROBLEM_CLOSED_BOX, PER = MCPM_PROBLEM_PERIODIC;
  const void* fns[] = {
      (const void*)k_update<float, 0u>,          (const void*)k_update<double, 0u>,
      (const void*)k_update<float, F>,           (const void*)k_update<double, F>,
      (const void*)k_update<float, FL>,          (const void*)k_update<double, FL>,
      (const void*)k_update<float, F, SPEC>,     (const void*)k_update<float, F, PER>,
      (const void*)k_update<float, FL, SPEC>,    (const void*)k_update<float, FL, PER>,
      (const void*)k_update<float, F, 0, true>,  (const void*)k_update<float, F, SPEC, true>,
      (const void*)k_update<float, F, PER, true>, (const void*)k_update<float, FL, 0, true>,
      (const void*)k_update<float, FL, SPEC, true>, (const void*)k_update<float, FL, PER, true>,
      (const void*)k_update<float, 0u, 0, true>,  (const void*)k_update<float, ST_FUSED_COLL_OLD, 0, true>,
      (const void*)k_update<float, ST_FUSED_COLL, 0, true>};
  cudaError_t e = cudaSuccess;
  for (const void* f : fns)
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  return e;
}
int update_occupancy(const Session& s) {
  int nb = 0;
  size_t sm = update_smem_bytes(s);
  // the fused step's kernel sets the persistent grid (the split-mode
  // variant, with every stage decided at run time, holds fewer blocks)
  if (s.prec == MCPM_FP32 && s.use_slotted)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_update<float, ST_FUSED_FP, 0, true>, 256, sm);
  else if (s.prec == MCPM_FP32)
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_update<float, ST_FUSED_FP>, 256, sm);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_update<double, 0u>, 256, sm);
  return nb < 1 ? 1 : nb;
}
int moments_occupancy(const Session& s) {
  int nb = 0;
  if (s.prec == MCPM_FP32) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_moments<float>, 256, 0);
  else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_moments<double>, 256, 0);
  return nb < 1 ? 1 : nb;
}

}  // namespace mcpm
