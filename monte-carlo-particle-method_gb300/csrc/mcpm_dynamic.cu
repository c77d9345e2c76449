// mcpm_dynamic.cu -- the interface problems' per-cell thermostat and the
// particle split / merge that changes N (the reference's problem `inverted`).
//
//   thermostat                    src/Main_Functions.cpp:1674-1869 (its live
//                                 branch: the cells within thermc of y = 0 and
//                                 within thermh of y = Len rescaled to Tc / Th)
//   inverted_addremove_particles  src/Main_Functions.cpp:1206-1450
//
// Both work on the packed, cell-sorted layout of the last cell_update (the
// reference's cells[].indices_inside).  The split / merge writes the new
// state into the other buffer in the new particle-id order -- the survivors
// in their old id order, then the copies of each split particle -- and
// leaves the layout to the next binning, as the reference leaves its new
// arrays to the next cell_update.  Per-particle weights (the reference's
// n_ratio[]) live in particle-id order, per-cell weights in cell order.
#include <cfloat>

#include "mcpm_device.cuh"

namespace mcpm {

#define FULL 0xffffffffu

template <typename real> struct DynP {
  real *x1, *x2, *U1, *U2, *U3, *x1o, *x2o;
  int32_t* pid;
};
template <typename real> static DynP<real> ptd(const PBuf& b) {
  return {(real*)b.x1, (real*)b.x2, (real*)b.U1, (real*)b.U2, (real*)b.U3, (real*)b.x1o, (real*)b.x2o, b.pid};
}

// the y coordinate of cell c's centre as make_cells forms it
// (src/myIO.cpp:1458-1467): 0.5 (k dy + (k + 1) dy)
__device__ __forceinline__ double cell_center_y(int c, const DevConsts& k) {
  const int kk = c / k.N0;
  return 0.5 * ((double)kk * k.dy + (double)(kk + 1) * k.dy);
}

// ------------------------------------------------------------ thermostat
// One warp per cell num < N[1] (the reference's loop bound): a cell whose
// centre lies below thermc takes temperature Tc, above Len[1] - thermh Th,
// by U <- lamb (U - U_space) + U_space with lamb = sqrt(T_target / T), for
// cells with T > 0 (src/Main_Functions.cpp:1780-1855).
template <typename real>
__global__ void k_thermostat(DevConsts k, const double* cell, const int32_t* off, const int32_t* cnt, DynP<real> p,
                             double Tc, double Th, double thermc, double thermh) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int ncell = min(k.N1, k.C);
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < ncell; c += warps) {
    const double yc = cell_center_y(c, k);
    double target;
    if (yc < thermc) target = Tc;
    else if (yc > k.L1 - thermh) target = Th;
    else continue;
    const double T = cell[(size_t)MCPM_CF_T * k.C + c];
    if (!(T > 0.0)) continue;
    const double lamb = sqrt(target / T);
    const double us0 = cell[(size_t)(MCPM_CF_U_SPACE + 0) * k.C + c];
    const double us1 = cell[(size_t)(MCPM_CF_U_SPACE + 1) * k.C + c];
    const double us2 = cell[(size_t)(MCPM_CF_U_SPACE + 2) * k.C + c];
    const int s0 = off[c], n = cnt[c];
    for (int i = lane; i < n; i += 32) {
      const int q = s0 + i;
      p.U1[q] = (real)(lamb * ((double)p.U1[q] - us0) + us0);
      p.U2[q] = (real)(lamb * ((double)p.U2[q] - us1) + us1);
      p.U3[q] = (real)(lamb * ((double)p.U3[q] - us2) + us2);
    }
  }
}

// --------------------------------------------------- split / merge: flags
// Per particle of cell c (weight w, cell weight cw): w > cw -> split (flag
// 1); w < cw -> deleted with probability 1 - 1/n_ratio (flag -1) or kept
// with the cell's weight (flag 2); else kept (flag 0)
// (src/Main_Functions.cpp:1258-1284).  Per cell: the split particles
// (numb_new), the kept ones (numb_rem), the kept weight (weight) and the
// largest kept particle id (the reference's mean loop keeps the last one);
// totals of split and deleted particles.
enum { ARC_NEW = 0, ARC_REM = 1, ARC_W = 2, ARC_LAST = 3, ARC_COUNT = 4 };

__global__ void k_ar_flags(DevConsts k, const int32_t* off, const int32_t* cnt, const int32_t* pid,
                           const int32_t* pw, const int32_t* cw, int8_t* flag, int32_t* ci,
                           unsigned long long* tot, double ratio, int step) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int C = k.C;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < C; c += warps) {
    const int s0 = off[c], n = cnt[c], cwc = cw[c];
    int nn = 0, nr = 0, wt = 0, nd = 0, last = -1;
    for (int i = lane; i < n; i += 32) {
      const int q = pid[s0 + i];
      const int w = pw[q];
      int8_t f;
      if (w > cwc) {
        f = 1; ++nn; wt += w;
      } else if (w < cwc) {
        const uint4 r = rng_draw(k, (uint32_t)q, (uint32_t)step, RNG_ADDREM_DEL, 0u);
        if (u01d(r.x) < ratio) { f = -1; ++nd; }
        else { f = 2; ++nr; wt += cwc; }
      } else {
        f = 0; ++nr; wt += w;
      }
      flag[q] = f;
      if (f != -1) last = max(last, q);
    }
    nn = __reduce_add_sync(FULL, nn);
    nr = __reduce_add_sync(FULL, nr);
    wt = __reduce_add_sync(FULL, wt);
    nd = __reduce_add_sync(FULL, nd);
    last = __reduce_max_sync(FULL, last);
    if (lane == 0) {
      ci[(size_t)ARC_NEW * C + c] = nn;
      ci[(size_t)ARC_REM * C + c] = nr;
      ci[(size_t)ARC_W * C + c] = wt;
      ci[(size_t)ARC_LAST * C + c] = last;
      if (nn) atomicAdd(&tot[0], (unsigned long long)nn);
      if (nd) atomicAdd(&tot[1], (unsigned long long)nd);
    }
  }
}

// ----------------------------------------------- split / merge: the width
// The velocity spread of the copies, per cell (src/Main_Functions.cpp:
// 1298-1327): the reference's mean loop assigns rather than adds, so its
// "mean" is the last kept particle's weighted velocity over the cell's kept
// weight -- kept as it is; sig = sqrt(sum over kept of |U - mean|^2 w /
// weight); h = 1.06 sig (numb_rem + n_ratio)^(-1/5) (:1346).
template <typename real>
__global__ void k_ar_width(DevConsts k, const int32_t* off, const int32_t* cnt, DynP<real> p, const int32_t* pw,
                           const int32_t* cw, const int8_t* flag, const int32_t* ci, double* h, int g) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  const int C = k.C;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < C; c += warps) {
    const int last = ci[(size_t)ARC_LAST * C + c];
    if (ci[(size_t)ARC_NEW * C + c] == 0 || last < 0) {
      if (lane == 0) h[c] = 0.0;
      continue;
    }
    const int s0 = off[c], n = cnt[c], cwc = cw[c];
    const double weight = 1.0 * ci[(size_t)ARC_W * C + c];
    // the last kept particle's velocity and weight
    double l1 = 0.0, l2 = 0.0, l3 = 0.0, lw = 0.0;
    for (int i = lane; i < n; i += 32) {
      const int q = p.pid[s0 + i];
      if (q == last) {
        l1 = (double)p.U1[s0 + i]; l2 = (double)p.U2[s0 + i]; l3 = (double)p.U3[s0 + i];
        lw = (double)(flag[q] == 2 ? cwc : pw[q]);
      }
    }
    const unsigned who = __ballot_sync(FULL, lw != 0.0);
    const int src = who ? __ffs(who) - 1 : 0;
    l1 = __shfl_sync(FULL, l1, src); l2 = __shfl_sync(FULL, l2, src); l3 = __shfl_sync(FULL, l3, src);
    lw = __shfl_sync(FULL, lw, src);
    const double m1 = l1 * lw / weight, m2 = l2 * lw / weight, m3 = l3 * lw / weight;
    double sg = 0.0;
    for (int i = lane; i < n; i += 32) {
      const int q = p.pid[s0 + i];
      const int8_t f = flag[q];
      if (f == -1) continue;
      const double d1 = (double)p.U1[s0 + i] - m1, d2 = (double)p.U2[s0 + i] - m2, d3 = (double)p.U3[s0 + i] - m3;
      const double energy = d1 * d1 + d2 * d2 + d3 * d3;
      sg = sg + energy * (double)(f == 2 ? cwc : pw[q]);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sg += __shfl_xor_sync(FULL, sg, o);
    if (lane == 0) {
      const double sig = sqrt(sg / weight);
      h[c] = 1.06 * sig * pow(1.0 * (ci[(size_t)ARC_REM * C + c] + g), -1.0 / 5.0);
    }
  }
}

// ------------------------------------------------ split / merge: the ranks
// Exclusive scans over particle ids of the kept flags (-> new id of a kept
// particle) and of the split flags (-> rank of a split particle), in tiles
// of AR_TILE ids: tile totals, a scan of the totals, the tile-local scans.
constexpr int AR_T = 256, AR_PER = 8, AR_TILE = AR_T * AR_PER;

__global__ void __launch_bounds__(AR_T) k_ar_scan_tiles(const int8_t* flag, int64_t n, int32_t* tiles, int ntiles) {
  __shared__ int sk[AR_T / 32], ss[AR_T / 32];
  const int64_t base = (int64_t)blockIdx.x * AR_TILE;
  int kk = 0, sp = 0;
  for (int u = 0; u < AR_PER; ++u) {
    const int64_t i = base + (int64_t)u * AR_T + threadIdx.x;
    if (i < n) { const int8_t f = flag[i]; kk += f != -1; sp += f == 1; }
  }
  kk = __reduce_add_sync(FULL, kk);
  sp = __reduce_add_sync(FULL, sp);
  if ((threadIdx.x & 31) == 0) { sk[threadIdx.x >> 5] = kk; ss[threadIdx.x >> 5] = sp; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0, b = 0;
    for (int w = 0; w < AR_T / 32; ++w) { a += sk[w]; b += ss[w]; }
    tiles[blockIdx.x] = a;
    tiles[ntiles + blockIdx.x] = b;
  }
}

// exclusive scan of the tile totals in place, one block
__global__ void __launch_bounds__(1024) k_ar_scan_top(int32_t* tiles, int ntiles) {
  __shared__ int part[2][1024];
  const int per = (ntiles + 1023) / 1024, t = threadIdx.x;
  const int lo = min(ntiles, t * per), hi = min(ntiles, lo + per);
  int a = 0, b = 0;
  for (int i = lo; i < hi; ++i) { a += tiles[i]; b += tiles[ntiles + i]; }
  part[0][t] = a;
  part[1][t] = b;
  __syncthreads();
  if (t == 0) {
    int x = 0, y = 0;
    for (int i = 0; i < 1024; ++i) {
      const int p0 = part[0][i], p1 = part[1][i];
      part[0][i] = x; part[1][i] = y;
      x += p0; y += p1;
    }
  }
  __syncthreads();
  a = part[0][t];
  b = part[1][t];
  for (int i = lo; i < hi; ++i) {
    const int p0 = tiles[i], p1 = tiles[ntiles + i];
    tiles[i] = a; tiles[ntiles + i] = b;
    a += p0; b += p1;
  }
}

__global__ void __launch_bounds__(AR_T) k_ar_scan_apply(const int8_t* flag, int64_t n, const int32_t* tiles,
                                                        int ntiles, int32_t* newid, int32_t* srank) {
  __shared__ int wk[AR_T / 32], ws[AR_T / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int bk = tiles[blockIdx.x], bs = tiles[ntiles + blockIdx.x];
  const int64_t base = (int64_t)blockIdx.x * AR_TILE;
  for (int u = 0; u < AR_PER; ++u) {
    const int64_t i = base + (int64_t)u * AR_T + threadIdx.x;
    const int8_t f = i < n ? flag[i] : (int8_t)-1;
    const unsigned mk = __ballot_sync(FULL, f != -1), ms = __ballot_sync(FULL, f == 1);
    const unsigned below = (1u << lane) - 1u;
    if (lane == 0) { wk[warp] = __popc(mk); ws[warp] = __popc(ms); }
    __syncthreads();
    int ok = 0, os = 0, tk = 0, ts = 0;
    for (int w = 0; w < AR_T / 32; ++w) {
      if (w < warp) { ok += wk[w]; os += ws[w]; }
      tk += wk[w]; ts += ws[w];
    }
    if (i < n) {
      newid[i] = bk + ok + __popc(mk & below);
      srank[i] = bs + os + __popc(ms & below);
    }
    bk += tk;
    bs += ts;
    __syncthreads();
  }
}

// ------------------------------------------------ split / merge: the move
// One warp per cell of the packed layout: every kept particle to its new id
// in the other buffer, and for a split particle its n_ratio - 1 copies at
// n_kept + rank (n_ratio - 1) + j, velocities U + h z with z standard normals
// (Philox, keyed by the parent's id, the step and j; the reference draws
// them from std::mt19937), positions copied (src/Main_Functions.cpp:
// 1341-1358, 1376-1398).  New weights: the cell's weight, as the reference
// resets every particle's n_ratio to its cell's (:1436-1443).
template <typename real>
__global__ void k_ar_move(DevConsts k, const int32_t* off, const int32_t* cnt, DynP<real> s, DynP<real> d,
                          const int8_t* flag, const int32_t* newid, const int32_t* srank, const double* h,
                          const int32_t* cw, int32_t* pw_new, int64_t n_kept, int g, int step) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < k.C; c += warps) {
    const int s0 = off[c], n = cnt[c], cwc = cw[c];
    const double hc = h[c];
    for (int i = lane; i < n; i += 32) {
      const int q = s.pid[s0 + i];
      const int8_t f = flag[q];
      if (f == -1) continue;
      const int sl = s0 + i;
      const int64_t e = newid[q];
      const real x1 = s.x1 ? s.x1[sl] : (real)0, x2 = s.x2[sl];
      const real u1 = s.U1[sl], u2 = s.U2[sl], u3 = s.U3[sl];
      if (d.x1) d.x1[e] = x1;
      d.x2[e] = x2;
      d.U1[e] = u1; d.U2[e] = u2; d.U3[e] = u3;
      if (d.x1o) d.x1o[e] = s.x1o[sl];
      if (d.x2o) d.x2o[e] = s.x2o[sl];
      d.pid[e] = (int32_t)e;
      pw_new[e] = cwc;
      if (f != 1) continue;
      for (int j = 0; j < g - 1; ++j) {
        const int64_t e2 = n_kept + (int64_t)srank[q] * (g - 1) + j;
        const Normals3<double> z = normals3<double>(rng_draw(k, (uint32_t)q, (uint32_t)step, RNG_ADDREM_NEW,
                                                           (uint32_t)j));
        if (d.x1) d.x1[e2] = x1;
        d.x2[e2] = x2;
        d.U1[e2] = (real)((double)u1 + hc * z.z0);
        d.U2[e2] = (real)((double)u2 + hc * z.z1);
        d.U3[e2] = (real)((double)u3 + hc * z.z2);
        if (d.x1o) d.x1o[e2] = s.x1o[sl];
        if (d.x2o) d.x2o[e2] = s.x2o[sl];
        d.pid[e2] = (int32_t)e2;
        pw_new[e2] = cwc;
      }
    }
  }
}

// nothing was split or deleted: the kept light particles take their cell's
// weight in place (src/Main_Functions.cpp:1275-1279)
__global__ void k_ar_reweight(DevConsts k, const int32_t* off, const int32_t* cnt, const int32_t* pid,
                              const int8_t* flag, const int32_t* cw, int32_t* pw) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < k.C; c += warps) {
    const int s0 = off[c], n = cnt[c];
    for (int i = lane; i < n; i += 32) {
      const int q = pid[s0 + i];
      if (flag[q] == 2) pw[q] = cw[c];
    }
  }
}

// ------------------------------------------------------- measure_pressure
// src/Main_Functions.cpp:13-34: every particle whose cell row changed over
// the step (floor(x2_old / dy) -> floor(x2 / dy)) adds Fn m |U2| to p_m of
// each row index it crossed, num1 <= num < num2 (the reference indexes
// cells by the row number, as in its 1-D boxes).  The state may be packed
// (n particles in [0, n)) or slotted (each cell's region, then the overflow
// entries).
template <typename real>
__global__ void k_pressure(DevConsts k, DynP<real> p, DynP<real> ovf, const int32_t* ovf_n, const int32_t* off,
                           const int32_t* dcur, int64_t n, double coef, double* p_m) {
  const int64_t tid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x, nt = (int64_t)gridDim.x * blockDim.x;
  auto one = [&](real x2, real x2o, real u2) {
    const int numO = (int)floor((double)x2o / k.dy), numN = (int)floor((double)x2 / k.dy);
    int lo = -1, hi = -1;
    if (numN > numO) { lo = numO; hi = numN; }
    else if (numN < numO) { lo = numN; hi = numO; }
    for (int num = lo; num < hi; ++num)
      if (num >= 0 && num < k.C) atomicAdd(&p_m[num], coef * fabs((double)u2));
  };
  if (!dcur) {
    for (int64_t i = tid; i < n; i += nt) one(p.x2[i], p.x2o[i], p.U2[i]);
    return;
  }
  const int lane = threadIdx.x & 31;
  for (int64_t c = tid >> 5; c < k.C; c += nt >> 5) {
    const int s0 = off[c], m = min(dcur[c], off[c + 1] - s0);
    for (int i = lane; i < m; i += 32) one(p.x2[s0 + i], p.x2o[s0 + i], p.U2[s0 + i]);
  }
  const int n_ovf = *ovf_n;
  for (int64_t e = tid; e < n_ovf; e += nt) one(ovf.x2[e], ovf.x2o[e], ovf.U2[e]);
}

static int warp_grid(const Session& s, int cells) {
  const int blocks = (cells + 7) / 8;  // 8 warps of 256 threads
  return blocks < 1 ? 1 : (blocks > s.num_sms * 16 ? s.num_sms * 16 : blocks);
}

template <typename real> static int thermostat_impl(Session& s, double Tc, double Th, double thermc, double thermh) {
  k_thermostat<real><<<warp_grid(s, s.k.N1 < s.C ? s.k.N1 : s.C), 256, 0, s.stream>>>(
      s.k, s.cell, s.off, s.cnt, ptd<real>(s.P[s.cur]), Tc, Th, thermc, thermh);
  return 1;
}
int launch_thermostat(Session& s, double Tc, double Th, double thermc, double thermh) {
  return s.prec == MCPM_FP32 ? thermostat_impl<float>(s, Tc, Th, thermc, thermh)
                             : thermostat_impl<double>(s, Tc, Th, thermc, thermh);
}

int launch_addremove_flags(Session& s, int g, int step) {
  cudaMemsetAsync(s.ar_tot, 0, 2 * sizeof(unsigned long long), s.stream);
  const double ratio = 1.0 - 1.0 / (g * 1.0);  // src/Main_Functions.cpp:1256
  k_ar_flags<<<warp_grid(s, s.C), 256, 0, s.stream>>>(s.k, s.off, s.cnt, s.P[s.cur].pid, s.pw, s.cw, s.ar_flag,
                                                      s.ar_ci, s.ar_tot, ratio, step);
  return 1;
}

template <typename real> static int addremove_move_impl(Session& s, int g, int step, int64_t n_kept) {
  int n = 0;
  k_ar_width<real><<<warp_grid(s, s.C), 256, 0, s.stream>>>(s.k, s.off, s.cnt, ptd<real>(s.P[s.cur]), s.pw, s.cw,
                                                            s.ar_flag, s.ar_ci, s.ar_h, g);
  ++n;
  const int ntiles = (int)((s.N + AR_TILE - 1) / AR_TILE);
  k_ar_scan_tiles<<<ntiles > 0 ? ntiles : 1, AR_T, 0, s.stream>>>(s.ar_flag, s.N, s.ar_tiles, ntiles);
  k_ar_scan_top<<<1, 1024, 0, s.stream>>>(s.ar_tiles, ntiles);
  k_ar_scan_apply<<<ntiles > 0 ? ntiles : 1, AR_T, 0, s.stream>>>(s.ar_flag, s.N, s.ar_tiles, ntiles, s.ar_newid,
                                                                   s.ar_srank);
  n += 3;
  k_ar_move<real><<<warp_grid(s, s.C), 256, 0, s.stream>>>(s.k, s.off, s.cnt, ptd<real>(s.P[s.cur]),
                                                           ptd<real>(s.P[1 - s.cur]), s.ar_flag, s.ar_newid,
                                                           s.ar_srank, s.ar_h, s.cw, s.pw_alt, n_kept, g, step);
  return n + 1;
}
int launch_addremove_move(Session& s, int g, int step, int64_t n_kept) {
  return s.prec == MCPM_FP32 ? addremove_move_impl<float>(s, g, step, n_kept)
                             : addremove_move_impl<double>(s, g, step, n_kept);
}

int launch_addremove_reweight(Session& s) {
  k_ar_reweight<<<warp_grid(s, s.C), 256, 0, s.stream>>>(s.k, s.off, s.cnt, s.P[s.cur].pid, s.ar_flag, s.cw, s.pw);
  return 1;
}

int addremove_tiles(int64_t n) { return (int)((n + AR_TILE - 1) / AR_TILE); }

template <typename real> static int pressure_impl(Session& s) {
  const bool sl = s.slotted;
  k_pressure<real><<<s.num_sms * 8, 256, 0, s.stream>>>(
      s.k, ptd<real>(s.P[s.cur]), ptd<real>(s.ovf), sl ? s.ovf_n + (1 - s.ovf_par) : nullptr, s.off,
      sl ? s.dcur : nullptr, s.N, s.k.Fn * s.k.m, s.p_m);
  return 1;
}
int launch_pressure(Session& s) { return s.prec == MCPM_FP32 ? pressure_impl<float>(s) : pressure_impl<double>(s); }

}  // namespace mcpm
