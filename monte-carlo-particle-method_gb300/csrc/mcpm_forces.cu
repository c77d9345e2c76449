// mcpm_forces.cu -- ESMC collisions and the 1-D Vlasov long-range force.
#include <algorithm>
#include <cstring>
#include <type_traits>
#include <vector>

#include "mcpm_device.cuh"

namespace mcpm {

#define FULL 0xffffffffu

template <typename real> struct PT2 {
  real *x1, *x2, *U1, *U2, *U3;
};

// ================================================================ ESMC
// Collision_ESMC_new3, src/collisions.cpp:583-720, restated per cell:
// cell I runs m_I = floor(omega_max N_I / 2 + u) candidates (the reference's
// slot sampling without replacement gives every cell exactly its m_I).
// Cells whose partner neighbourhoods overlap are never processed together
// (colour classes of stride 2R+1, R = ceil(sigma/dx)); inside a cell a warp
// holds 32 consecutive candidates and applies the longest prefix whose
// particle pairs are disjoint, so the result equals processing the
// candidates one after another in order.  The candidates past the prefix
// move down the warp to the next round (their draws, directions, partners
// and cell lookups depend on positions only, which collisions do not
// change); only the lanes that empty draw new ones.

// slots of the collision cell a warp's conflict table covers; larger cells
// test their candidates pairwise over the warp
constexpr int ESMC_TAB = 256;
// FP32 blocks of 4 warps resident per SM: 12 (40 registers) holds a whole
// colour class of a 256 x 256 box at once -- one wave of cells instead of
// a full wave and a partial one; measured 0.85 -> 0.45 ms of collisions per
// step at 6.5M particles (8 blocks 0.49, 16 blocks 0.55 ms)
#ifndef MCPM_ESMC_MINB
#define MCPM_ESMC_MINB 12
#endif

// Whether a lower lane's valid candidate shares a particle with this lane's
// (si: a slot of the collision cell [o, o + n); sj: the partner, in the cell
// or a neighbour).  Slots of the collision cell go through the warp's table
// (each valid lane marks its slots with its lane by atomicMin; a slot whose
// mark is below the lane was claimed by a lower lane); partners outside the
// cell can only meet other such partners: __match_any_sync.  tab holds
// ESMC_TAB entries of 32 on entry and on return.
__device__ __forceinline__ bool esmc_conflict(int* tab, int o, int n, bool valid, int si, int sj) {
  const int lane = threadIdx.x & 31;
  const unsigned lower = (1u << lane) - 1u;
  bool conflict = false;
  if (n <= ESMC_TAB) {
    const bool jin = valid && sj >= o && sj < o + n;
    if (valid) atomicMin(&tab[si - o], lane);
    if (jin) atomicMin(&tab[sj - o], lane);
    __syncwarp();
    if (valid) conflict = tab[si - o] < lane || (jin && tab[sj - o] < lane);
    const unsigned mj = __match_any_sync(FULL, (valid && !jin) ? sj : -1 - lane);
    if (valid && !jin && (mj & lower)) conflict = true;
    __syncwarp();
    if (valid) tab[si - o] = 32;
    if (jin) tab[sj - o] = 32;
    __syncwarp();
  } else {
    for (int l = 0; l < 31; ++l) {
      const int oi = __shfl_sync(FULL, si, l), oj = __shfl_sync(FULL, sj, l);
      const int ov = __shfl_sync(FULL, (int)valid, l);
      if (l < lane && ov && valid && (oi == si || oi == sj || oj == si || oj == sj)) conflict = true;
    }
  }
  return conflict;
}

template <typename real>
__global__ void __launch_bounds__(128, sizeof(real) == 4 ? MCPM_ESMC_MINB : 1)
    k_esmc(DevConsts k, double* cell, const float* yn, const int32_t* off, const int32_t* cnt, PT2<real> p,
           const int32_t* dstep, int cx, int cy, int Sx, int Sy, uint32_t* status) {
  __shared__ int tabs[4][ESMC_TAB];
  const int lane = threadIdx.x & 31;
  int* tab = tabs[threadIdx.x >> 5];
  for (int e = lane; e < ESMC_TAB; e += 32) tab[e] = 32;
  __syncwarp();
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nA = (k.N0 - cx + Sx - 1) / Sx, nB = (k.N1 - cy + Sy - 1) / Sy;
  if (gw >= nA * nB) return;
  const int I = (cy + Sy * (gw / nA)) * k.N0 + (cx + Sx * (gw % nA));
  const int C = k.C;
  const int step = *dstep;
  const int NI = cnt[I];
  const int oI = off[I];
  const double om_max = cell[(size_t)MCPM_CF_OMEGA_MAX * C + I];
  const double mreal = r_floor(0.5 * om_max * (1.0 * NI) + u01d(rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_ESMC_M, 0u).x));
  // a non-finite or absurd majorant would make the candidate loop unbounded
  const double mcap = 64.0 * NI + 4096.0;
  int mI = 0;
  if (mreal >= 0.0 && mreal <= mcap) mI = (int)mreal;
  else if (lane == 0) raise_status(status, MCPM_ERR_ITER_LIMIT);
  // FP32 sessions run the candidate arithmetic in float (uniforms from the
  // top 23 bits, the acceptance test as dummy > u om_max); FP64 sessions
  // keep the reference's double arithmetic
  constexpr bool F32 = sizeof(real) == 4;
  typedef typename std::conditional<F32, float, double>::type cr;  // Y and n_J as the test uses them
  double omega = 0.0;
  float omega_f = 0.f;
  const float om_max_f = (float)om_max;
  const float coef_f = (float)(4.0 * 3.14159265358979323846 * k.sigma * k.sigma * k.dt);
  const real pi = (real)3.14159265358979323846;
  const real sg = (real)k.sigma;
  if (NI > 0) {
    int base = 0;
    // this lane's candidate (number base + lane): its slots, direction and
    // the Y and n_J of its test; `have` once it holds them
    bool have = false, valid = false;
    int si = -1, sj = -1;
    real d0 = 0, d1 = 0, d2 = 0;
    cr Ymid = 0, nJ = 0;
    while (base < mI) {
      const int kc = base + lane;
      if (!have) {
        valid = false;
        si = -1;
        sj = -1;
        d0 = d1 = d2 = 0;
        Ymid = nJ = 0;
        if (kc < mI) {
          uint4 r = rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_ESMC, (uint32_t)kc);
          si = oI + pick(r.x, NI);
          const real uy = F32 ? (real)u01f(r.y) : (real)u01d(r.y), uz = F32 ? (real)u01f(r.z) : (real)u01d(r.z);
          real theta = (real)2.0 * pi * uy;
          real cph = (real)2.0 * uz - (real)1.0;
          real sph = r_sqrt((real)1.0 - cph * cph);
          real sn, cs;
          r_sincos(theta, &sn, &cs);
          d0 = cs * sph; d1 = sn * sph; d2 = cph;
          real xi1 = p.x1[si], xi2 = p.x2[si];
          real xx = xi1 + sg * d0, yy = xi2 + sg * d1;
          int i0 = (int)r_floor(xx / (real)k.dx), i1 = (int)r_floor(yy / (real)k.dy);
          if (i0 >= 0 && i0 < k.N0 && i1 >= 0 && i1 < k.N1) {
            int J = i1 * k.N0 + i0;
            // n_J is loaded beside the partner cell's count and offset
            // (FP32 sessions: the solve's float copy, no conversion here)
            cr nJc;
            if constexpr (F32) nJc = yn[C + J];
            else nJc = cell[(size_t)MCPM_CF_N * C + J];
            int NJ = cnt[J];
            if (NJ > 0) {
              sj = off[J] + pick(r.w, NJ);
              if (sj != si) {
                real xm0 = (xi1 + p.x1[sj]) / (real)2.0, xm1 = (xi2 + p.x2[sj]) / (real)2.0;
                int m0 = (int)r_floor(xm0 / (real)k.dx), m1 = (int)r_floor(xm1 / (real)k.dy);
                m0 = m0 < 0 ? 0 : (m0 > k.N0 - 1 ? k.N0 - 1 : m0);
                m1 = m1 < 0 ? 0 : (m1 > k.N1 - 1 ? k.N1 - 1 : m1);
                if constexpr (F32) Ymid = yn[m1 * k.N0 + m0];
                else Ymid = cell[(size_t)CFI_Y * C + m1 * k.N0 + m0];
                nJ = nJc;
                valid = true;
              }
            }
          }
        }
      }
      // longest prefix of candidates with pairwise disjoint particles
      const bool conflict = esmc_conflict(tab, oI, NI, valid, si, sj);
      unsigned cm = __ballot_sync(FULL, conflict);
      int take = cm ? (__ffs(cm) - 1) : 32;
      if (take > mI - base) take = mI - base;
      if (lane < take && valid) {
        real g0 = p.U1[si] - p.U1[sj], g1 = p.U2[si] - p.U2[sj], g2 = p.U3[si] - p.U3[sj];
        real gd = g0 * d0 + g1 * d1 + g2 * d2;
        bool accept;
        if constexpr (F32) {
          const float dummy = coef_f * (float)gd * Ymid * nJ;
          omega_f = fmaxf(omega_f, dummy);
          const float u = u01f(rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_ESMC_ACC, (uint32_t)kc).x);
          accept = dummy > u * om_max_f;
        } else {
          double dummy = 4.0 * 3.14159265358979323846 * k.sigma * k.sigma * (double)gd * Ymid * nJ * k.dt;
          if (dummy - omega > 0.0) omega = dummy;
          double u = u01d(rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_ESMC_ACC, (uint32_t)kc).x);
          accept = dummy / om_max > u;
        }
        if (accept) {
          p.U1[si] = p.U1[si] - gd * d0; p.U2[si] = p.U2[si] - gd * d1; p.U3[si] = p.U3[si] - gd * d2;
          p.U1[sj] = p.U1[sj] + gd * d0; p.U2[sj] = p.U2[sj] + gd * d1; p.U3[sj] = p.U3[sj] + gd * d2;
        }
      }
      __syncwarp();
      // the candidates past the prefix move down by `take` lanes
      const int src = (lane + take) & 31;
      have = lane + take < 32;
      valid = __shfl_sync(FULL, valid, src);
      si = __shfl_sync(FULL, si, src);
      sj = __shfl_sync(FULL, sj, src);
      d0 = __shfl_sync(FULL, d0, src);
      d1 = __shfl_sync(FULL, d1, src);
      d2 = __shfl_sync(FULL, d2, src);
      Ymid = __shfl_sync(FULL, Ymid, src);
      nJ = __shfl_sync(FULL, nJ, src);
      base += take;
    }
  }
  if constexpr (F32) {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) omega_f = fmaxf(omega_f, __shfl_xor_sync(FULL, omega_f, m));
    omega = (double)omega_f;
  } else {
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) omega = fmax(omega, __shfl_xor_sync(FULL, omega, m));
  }
  if (lane == 0) cell[(size_t)MCPM_CF_OMEGA_MAX * C + I] = omega > om_max ? omega : om_max;
}

template <typename real> static int esmc_impl(Session& s) {
  int n = sync_dstep(s);
  const PBuf& b = s.P[s.cur];
  PT2<real> p{(real*)b.x1, (real*)b.x2, (real*)b.U1, (real*)b.U2, (real*)b.U3};
  int Rx = (int)ceil(s.k.sigma / s.k.dx), Ry = (int)ceil(s.k.sigma / s.k.dy);
  if (Rx < 1) Rx = 1;
  if (Ry < 1) Ry = 1;
  int Sx = (s.k.N0 > 1) ? 2 * Rx + 1 : 1, Sy = 2 * Ry + 1;
  for (int cy = 0; cy < Sy; ++cy)
    for (int cx = 0; cx < Sx; ++cx) {
      int nA = (s.k.N0 - cx + Sx - 1) / Sx, nB = (s.k.N1 - cy + Sy - 1) / Sy;
      int warps = nA * nB;
      if (warps <= 0) continue;
      int blocks = (warps * 32 + 127) / 128;
      k_esmc<real><<<blocks, 128, 0, s.stream>>>(s.k, s.cell,
                                                 s.prec == MCPM_FP32 ? s.pcell + (size_t)PF_STRIDE * s.C : nullptr,
                                                 s.off, s.cnt, p, s.dstep, cx, cy, Sx, Sy, s.status);
      ++n;
    }
  return n;
}
int launch_esmc(Session& s) { return s.prec == MCPM_FP32 ? esmc_impl<float>(s) : esmc_impl<double>(s); }

// ============================================================ DSMC VHS
// Collision_DSMC_VHS, src/collisions.cpp:2063-2141: Bird's no-time-counter
// scheme inside each cell, one warp per cell (pairs never leave their cell,
// so all cells run in one launch).  Cell I with N_I > 1 runs
// m_I = floor(pi sigma^2 N_I n_I crm_I dt / 2 + u) candidates: two distinct
// particles of the cell chosen uniformly (the reference redraws the second
// until it differs, the same distribution), sigma_T = |g|^(2 - 2 visp)
// crref^(2 visp - 1), accepted when sigma_T / crm_I > u, then an isotropic
// post-collision relative velocity of the same magnitude (cos theta =
// 2 a1 - 1, phi = 2 pi a2) about the pair's centre of mass.  As in the ESMC
// kernel a warp draws 32 candidates and applies the longest prefix with
// disjoint pairs, which equals processing them one after another (both
// particles of a pair lie in the cell: the warp's slot table of the ESMC
// kernel finds every conflict).  The majorant then becomes
// max(1.1 max sigma_T, 0.9 crm_I) (:2135).
// FP32 blocks of 4 warps declared resident per SM: 8 (measured 0.116 ms of
// collisions per step on the 6.5M-particle box against 0.128 ms unbounded
// and 0.126 ms at 12 blocks, whose 40 registers spill)
#ifndef MCPM_DSMC_MINB
#define MCPM_DSMC_MINB 8
#endif
template <typename real>
__global__ void __launch_bounds__(128, sizeof(real) == 4 ? MCPM_DSMC_MINB : 1)
    k_dsmc_vhs(DevConsts k, double* cell, const int32_t* off, const int32_t* cnt, PT2<real> p, const int32_t* dstep,
               uint32_t* status) {
  __shared__ int tabs[4][ESMC_TAB];
  const int lane = threadIdx.x & 31;
  int* tab = tabs[threadIdx.x >> 5];
  for (int e = lane; e < ESMC_TAB; e += 32) tab[e] = 32;
  __syncwarp();
  const int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (I >= k.C) return;
  const int NI = cnt[I];
  if (NI < 2) return;  // warp-uniform
  const int C = k.C;
  const int step = *dstep;
  const double crm = cell[(size_t)MCPM_CF_OMEGA_MAX * C + I];
  const double nI = cell[(size_t)MCPM_CF_N * C + I];
  const double pi = 3.14159265358979323846;
  const double Mc = pi * k.sigma * k.sigma * ((double)NI * nI) * crm * k.dt / 2.0;
  const double mreal = r_floor(Mc + u01d(rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_DSMC_M, 0u).x));
  // a non-finite or absurd majorant would make the candidate loop unbounded
  const double mcap = 64.0 * NI + 4096.0;
  int mI = 0;
  if (mreal >= 0.0 && mreal <= mcap) mI = (int)mreal;
  else if (lane == 0) raise_status(status, MCPM_ERR_ITER_LIMIT);
  constexpr bool F32 = sizeof(real) == 4;
  const real e = (real)k.vhs_e, cr = (real)k.vhs_cr, crm_r = (real)crm, half = (real)0.5;
  const int o = off[I];
  real seen = 0;
  int base = 0;
  while (base < mI) {
    const int kc = base + lane;
    const bool valid = kc < mI;
    int si = -1, sj = -1;
    uint4 r = make_uint4(0u, 0u, 0u, 0u);
    if (valid) {
      r = rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_DSMC, (uint32_t)kc);
      const int a = pick(r.x, NI);
      int b = pick(r.y, NI - 1);
      b += (b >= a) ? 1 : 0;
      si = o + a;
      sj = o + b;
    }
    // longest prefix of candidates with pairwise disjoint particles
    const bool conflict = esmc_conflict(tab, o, NI, valid, si, sj);
    const unsigned cm = __ballot_sync(FULL, conflict);
    int take = cm ? (__ffs(cm) - 1) : 32;
    if (take > mI - base) take = mI - base;
    if (lane < take) {
      const real u1i = p.U1[si], u2i = p.U2[si], u3i = p.U3[si];
      const real u1j = p.U1[sj], u2j = p.U2[sj], u3j = p.U3[sj];
      const real Vr = r_sqrt((u1i - u1j) * (u1i - u1j) + (u2i - u2j) * (u2i - u2j) + (u3i - u3j) * (u3i - u3j));
      const real sigmat = r_pow(Vr, e) * cr;
      if (sigmat - seen > (real)0) seen = sigmat;
      const real uacc = F32 ? (real)u01f(r.z) : (real)u01d(r.z);
      if (sigmat / crm_r > uacc) {
        const uint32_t w2 = rng_draw(k, (uint32_t)I, (uint32_t)step, RNG_DSMC_ACC, (uint32_t)kc).x;
        const real a1 = F32 ? (real)u01f(r.w) : (real)u01d(r.w);
        const real a2 = F32 ? (real)u01f(w2) : (real)u01d(w2);
        const real theta = r_acos((real)2.0 * a1 - (real)1.0);
        const real ph = (real)2.0 * (real)pi * a2;
        real st, ct, sp, cp;
        r_sincos(theta, &st, &ct);
        r_sincos(ph, &sp, &cp);
        const real v0 = Vr * ct, v1 = Vr * st * cp, v2 = Vr * st * sp;
        const real c0 = half * (u1i + u1j), c1 = half * (u2i + u2j), c2 = half * (u3i + u3j);
        p.U1[si] = c0 + half * v0; p.U2[si] = c1 + half * v1; p.U3[si] = c2 + half * v2;
        p.U1[sj] = c0 - half * v0; p.U2[sj] = c1 - half * v1; p.U3[sj] = c2 - half * v2;
      }
    }
    __syncwarp();
    base += take;
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    const real t = __shfl_xor_sync(FULL, seen, m);
    seen = t > seen ? t : seen;
  }
  if (lane == 0) {
    const double a = 1.1 * (double)seen, b = 0.9 * crm;
    cell[(size_t)MCPM_CF_OMEGA_MAX * C + I] = a < b ? b : a;  // std::max(a, b)
  }
}

template <typename real> static int dsmc_impl(Session& s) {
  int n = sync_dstep(s);
  const PBuf& b = s.P[s.cur];
  PT2<real> p{(real*)b.x1, (real*)b.x2, (real*)b.U1, (real*)b.U2, (real*)b.U3};
  const int blocks = (int)(((int64_t)s.C * 32 + 127) / 128);
  k_dsmc_vhs<real><<<blocks, 128, 0, s.stream>>>(s.k, s.cell, s.off, s.cnt, p, s.dstep, s.status);
  return n + 1;
}
int launch_dsmc_vhs(Session& s) { return s.prec == MCPM_FP32 ? dsmc_impl<float>(s) : dsmc_impl<double>(s); }

// ============================================================== sampling
// cell_poly_velocity, src/Main_Functions.cpp:1918-1968: per cell the particle
// count and the raw sums of U, U U, U1^m U2^n U3^(3-m-n) (m = 0..3,
// n = 0..3-m) and U U |U|^2, added to the session's accumulators.  One warp
// per cell; the state is widened to double and summed per lane, the warp
// reduces and lane 0 adds to the [MCPM_SF_COUNT][C] accumulators.
template <typename real>
__global__ void __launch_bounds__(128) k_sample(int C, double* smp, const int32_t* off, const int32_t* cnt,
                                                const real* U1, const real* U2, const real* U3) {
  constexpr int NS = MCPM_SF_COUNT - 1;
  const int lane = threadIdx.x & 31;
  const int num = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (num >= C) return;
  const int n = cnt[num];
  if (n == 0) return;  // warp-uniform: nothing to add
  const int64_t o = off[num];
  double a[NS];
#pragma unroll
  for (int j = 0; j < NS; ++j) a[j] = 0.0;
  for (int i = lane; i < n; i += 32) {
    const double u1 = (double)U1[o + i], u2 = (double)U2[o + i], u3 = (double)U3[o + i];
    a[0] += u1; a[1] += u2; a[2] += u3;
    a[3] += u1 * u1; a[4] += u1 * u2; a[5] += u1 * u3;
    a[6] += u2 * u2; a[7] += u2 * u3; a[8] += u3 * u3;
    const double p1[4] = {1.0, u1, u1 * u1, u1 * u1 * u1};
    const double p2[4] = {1.0, u2, u2 * u2, u2 * u2 * u2};
    const double p3[4] = {1.0, u3, u3 * u3, u3 * u3 * u3};
    int id = 9;
#pragma unroll
    for (int m = 0; m < 4; ++m)
#pragma unroll
      for (int q = 0; q < 4 - m; ++q) a[id++] += p1[m] * p2[q] * p3[3 - m - q];
    const double e = u1 * u1 + u2 * u2 + u3 * u3;
    a[19] += u1 * u1 * e; a[20] += u1 * u2 * e; a[21] += u1 * u3 * e;
    a[22] += u2 * u2 * e; a[23] += u2 * u3 * e; a[24] += u3 * u3 * e;
  }
#pragma unroll
  for (int j = 0; j < NS; ++j)
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) a[j] += __shfl_xor_sync(FULL, a[j], m);
  if (lane == 0) {
    smp[(size_t)MCPM_SF_WEIGHT * C + num] += (double)n;
#pragma unroll
    for (int j = 0; j < NS; ++j) smp[(size_t)(1 + j) * C + num] += a[j];
  }
}

int launch_sample(Session& s) {
  const PBuf& b = s.P[s.cur];
  const int blocks = (int)(((int64_t)s.C * 32 + 127) / 128);
  if (s.prec == MCPM_FP32)
    k_sample<float><<<blocks, 128, 0, s.stream>>>(s.C, s.samples, s.off, s.cnt, (const float*)b.U1,
                                                  (const float*)b.U2, (const float*)b.U3);
  else
    k_sample<double><<<blocks, 128, 0, s.stream>>>(s.C, s.samples, s.off, s.cnt, (const double*)b.U1,
                                                   (const double*)b.U2, (const double*)b.U3);
  return 1;
}

// ESMC majorant initialisation, src/main.cpp:250-269
__global__ void k_init_omega(DevConsts k, double* cell, double Ygas) {
  const int C = k.C;
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  const double pi = acos(-1.0);
  double thermal = sqrt(k.kb * cell[(size_t)MCPM_CF_T * C + c] / k.m);
  double crm = 10.0 * (thermal);
  double om = 4.0 * pi * k.sigma * k.sigma * crm * cell[(size_t)MCPM_CF_N * C + c] * k.dt;
  if (k.model == MCPM_MODEL_ESMC) om = om * Ygas;
  // DSMC_VHS keeps cells[].crm, its majorant relative speed, in this field
  cell[(size_t)MCPM_CF_OMEGA_MAX * C + c] = (k.model == MCPM_MODEL_DSMC_VHS) ? crm : om;
}
int launch_init_omega(Session& s) {
  double nb = s.k.n * s.k.b;
  double Ygas = 1.0 + 0.625 * s.k.n * s.k.b + 0.2869 * (nb * nb) + 0.115 * pow(nb, 3.0);
  k_init_omega<<<(s.C + 127) / 128, 128, 0, s.stream>>>(s.k, s.cell, Ygas);
  return 1;
}

// ======================================================= 1-D Vlasov force
// Quadrature points of the face integrals are built once per session on the
// host: for point q, the offset r cos(phi) and the weight w.  Both 1-D
// routines integrate over r (GL 50) x phi (GL 50, [0, pi]).

// Gauss-Legendre nodes/weights on [-1,1] (Newton on P_n); the 50-point table
// is rounded to 8 decimals because the reference's literals are
// (src/Main_Functions.cpp:3327-3346, :3649-3667).
static void gl_nodes(int n, double* xs, double* ws) {
  for (int i = 0; i < n; ++i) {
    double x = cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5)), dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int kk = 2; kk <= n; ++kk) { double p2 = ((2.0 * kk - 1.0) * x * p1 - (kk - 1.0) * p0) / kk; p0 = p1; p1 = p2; }
      dp = n * (x * p1 - p0) / (x * x - 1.0);
      double d = p1 / dp;
      x -= d;
      if (fabs(d) < 1e-17) break;
    }
    double p0 = 1.0, p1 = x;
    for (int kk = 2; kk <= n; ++kk) { double p2 = ((2.0 * kk - 1.0) * x * p1 - (kk - 1.0) * p0) / kk; p0 = p1; p1 = p2; }
    dp = n * (x * p1 - p0) / (x * x - 1.0);
    xs[n - 1 - i] = x;
    ws[n - 1 - i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  for (int i = 0; i < n / 2; ++i) {
    double xa = 0.5 * (xs[n - 1 - i] - xs[i]), wa = 0.5 * (ws[n - 1 - i] + ws[i]);
    xs[i] = -xa; xs[n - 1 - i] = xa; ws[i] = wa; ws[n - 1 - i] = wa;
  }
  if (n == 50)
    for (int i = 0; i < n; ++i) { xs[i] = nearbyint(xs[i] * 1e8) / 1e8; ws[i] = nearbyint(ws[i] * 1e8) / 1e8; }
}

// mode 1: vlasov_taking_the_integral (src/Main_Functions.cpp:3641-3796),
//   r in [eqdist, 3 eqdist], weight (sigma/r)^6 r^2 2 pi dr sin(phi) dphi
// mode 3: poisson_solver wall values (:3399-3431),
//   r in [0, 3 eqdist], weight exp(-bst r)/2 r dr sin(phi) dphi
static void build_quad(const Session& s, int mode, std::vector<double>& off, std::vector<double>& w) {
  double xi[50], wi[50], rr[50], dr[50], ph[50], dph[50];
  gl_nodes(50, xi, wi);
  const double pi = acos(-1.0);
  double b = 3.0 * s.cfg.eqdist, a = (mode == 1) ? 1.0 * s.cfg.eqdist : 0.0 * s.cfg.eqdist, c = 0.0, d = pi;
  for (int i = 0; i < 50; ++i) { rr[i] = (b - a) / 2.0 * xi[i] + (a + b) / 2.0; dr[i] = wi[i] * (b - a) / 2.0; }
  for (int i = 0; i < 50; ++i) { ph[i] = (d - c) / 2.0 * xi[i] + (c + d) / 2.0; dph[i] = wi[i] * (d - c) / 2.0; }
  off.resize(2500);
  w.resize(2500);
  for (int i = 0; i < 50; ++i) {
    double radial;
    if (mode == 1) radial = -(-pow(s.cfg.sigma / rr[i], 6.0)) * rr[i] * rr[i] * (2.0 * pi) * dr[i];
    else radial = exp(-s.cfg.bst * rr[i]) / (2.0) * rr[i] * dr[i];
    for (int ii = 0; ii < 50; ++ii) {
      off[i * 50 + ii] = rr[i] * cos(ph[ii]);
      w[i * 50 + ii] = (mode == 1 ? -radial : radial) * sin(ph[ii]) * dph[ii];
    }
  }
}

// ---- per-session tables (device), laid out in Session::lr_tab:
//  direct:  int dmin, dmax; double W[dmax - dmin + 1]; exceptions (fc, q, da, dg, w)
//  screened Poisson: int idx0[2500], idxN[2500]; double w[2500];
//                    double alpha[L][nf], gamma[L][nf], dfin[nf]
struct LRTab {
  int mode, nf, levels;
  int dmin, dmax;
  int n_exc;
  const double* W;       // stencil weights, dmax - dmin + 1
  const int* exc_i;      // [n_exc][4]: face, cell of the point, cell the stencil assumes
  const double* exc_w;   // [n_exc] the point's weight
  const int* idx0;       // GF wall points: cell of each point for face 0 / face N1
  const int* idxN;
  const double* wq;      // GF point weights
  const double* pa;      // PCR coefficients [levels][nf]
  const double* pg;
  const double* dfin;    // final diagonal
  double corr;           // the analytic r < sigma part's factor (formed on the host, as the reference forms it)
};

// One block: the whole 1-D long-range force.  direct (long_range 1,
// vlasov_taking_the_integral): V_f = sum_D W[D] n[clamp(f + D)] with the
// stencil verified against the reference's per-point cell lookup at session
// set-up, plus any points where that lookup is not translation invariant.
// screened Poisson (long_range 3, poisson_solver): wall values by the
// per-point quadrature, the constant tridiagonal matrix solved by parallel
// cyclic reduction with precomputed coefficients, minus the analytic r < sigma
// part.  Then F2 = -(V_{f+1} - V_f)/dy / m * coef per cell.
__global__ void __launch_bounds__(1024) k_long_range_1d(DevConsts k, double* cell, float* pcell, LRTab t,
                                                        double coef) {
  extern __shared__ double sh[];
  const int nf = t.nf, N1 = k.N1, C = k.C;
  const double* n = cell + (size_t)MCPM_CF_N * C;
  double* V = sh;            // [nf]
  double* r2 = sh + nf;      // [nf] (PCR ping-pong)
  auto ncl = [&](int c) -> double { return n[c < 0 ? 0 : (c > N1 - 1 ? N1 - 1 : c)]; };
  if (t.mode == MCPM_LR_DIRECT) {
    for (int fc = threadIdx.x; fc < nf; fc += blockDim.x) {
      double v = 0.0;
      for (int d = t.dmin; d <= t.dmax; ++d) v += t.W[d - t.dmin] * ncl(fc + d);
      V[fc] = v;
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int e = 0; e < t.n_exc; ++e) {
        const int* x = t.exc_i + 4 * e;
        V[x[0]] += t.exc_w[e] * (ncl(x[1]) - ncl(x[2]));
      }
    __syncthreads();
  } else {
    // wall values at face 0 and face N1: every thread sums its share of
    // both walls' 2,500 points (independent gathers), the warps' partial
    // sums are added in a fixed order
    __shared__ double wpart[2][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    double a0 = 0.0, aN = 0.0;
    for (int q = threadIdx.x; q < 2500; q += blockDim.x) {
      const double w = t.wq[q];
      a0 += w * n[t.idx0[q]];
      aN += w * n[t.idxN[q]];
    }
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) {
      a0 += __shfl_xor_sync(FULL, a0, m);
      aN += __shfl_xor_sync(FULL, aN, m);
    }
    if (lane == 0) { wpart[0][warp] = a0; wpart[1][warp] = aN; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double s0 = 0.0, sN = 0.0;
      for (int w = 0; w < nw; ++w) { s0 += wpart[0][w]; sN += wpart[1][w]; }
      V[0] = s0;
      V[nf - 1] = sN;
    }
    __syncthreads();
    const double dy2 = k.dy * k.dy;
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      if (i == 0 || i == nf - 1) r2[i] = V[i];
      else r2[i] = ((n[i] + n[i - 1]) / 2.0) * dy2;
    }
    __syncthreads();
    double* src = r2;
    double* dst = V;
    // the first face of this thread: its coefficients are loaded one level
    // ahead, so that their latency overlaps the level before
    const int i0 = threadIdx.x;
    double an = 0.0, gn = 0.0;
    if (i0 < nf && t.levels > 0) { an = t.pa[i0]; gn = t.pg[i0]; }
    for (int lv = 0, s = 1; lv < t.levels; ++lv, s <<= 1) {
      const double* pa = t.pa + (size_t)lv * nf;
      const double* pg = t.pg + (size_t)lv * nf;
      const double a_i0 = an, g_i0 = gn;
      if (i0 < nf && lv + 1 < t.levels) { an = pa[nf + i0]; gn = pg[nf + i0]; }
      for (int i = i0; i < nf; i += blockDim.x) {
        const double ai = i == i0 ? a_i0 : pa[i], gi = i == i0 ? g_i0 : pg[i];
        double v = src[i];
        if (i - s >= 0) v += ai * src[i - s];
        if (i + s < nf) v += gi * src[i + s];
        dst[i] = v;
      }
      __syncthreads();
      double* tmp = src; src = dst; dst = tmp;
    }
    const double corr = t.corr;
    for (int i = threadIdx.x; i < nf; i += blockDim.x) {
      double nj = i == 0 ? n[0] : (i == N1 ? n[N1 - 1] : (n[i] + n[i - 1]) / 2.0);
      dst[i] = src[i] / t.dfin[i] - nj * corr;
    }
    __syncthreads();
    if (dst != V)
      for (int i = threadIdx.x; i < nf; i += blockDim.x) V[i] = dst[i];
    __syncthreads();
  }
  for (int num = threadIdx.x; num < N1; num += blockDim.x) {
    double F2 = -(V[num + 1] - V[num]) / k.dy;
    F2 = F2 / k.m * coef;
    for (int j = 0; j < k.N0; ++j) {
      cell[(size_t)MCPM_CF_F2 * C + num * k.N0 + j] = F2;
      if (pcell) pcell[(size_t)(num * k.N0 + j) * PF_STRIDE + PF_F2DT] = (float)(F2 * k.dt);
    }
  }
}

// ============================================ density expansion (long_range 2)
// The kernel smoothing of cell_update (src/Main_Functions.cpp:2378-2427): at
// the centre of every cell, a Gaussian of width h = dy/2 cut at r_cut = 2 dy
// over the particles of rows k-2..k+2 of its column (a row past a wall takes
// the wall row's particles shifted by whole cells) gives n_smooth and the
// derivative sums dn2 and dn3.  velocity_update's density-expansion force
// (:1632-1653) is then dummyF = dn2 4 pi (sigma 2^(1/6))^3 phi / m 2, applied
// as U2 -= dummyF dt except in cell 0 and cell N[1]-1 (the reference compares
// the linear cell index with N[1]-1, kept as it is); F2 holds -dummyF, and
// the particle pass's kick adds F2 dt.  One warp per cell: each lane sums its
// share of the ~5 cells' particles, the warp reduces in double.
template <typename real>
__global__ void __launch_bounds__(128) k_smoothing(DevConsts k, double* cell, float* pcell, const int32_t* off,
                                                   const int32_t* cnt, const real* x2) {
  const int lane = threadIdx.x & 31;
  const int num = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (num >= k.C) return;
  const int C = k.C;
  const int j = num % k.N0, kr = num / k.N0;
  const double dy = k.dy;
  const double r1 = 0.5 * ((double)kr * dy + (double)(kr + 1) * dy);  // cell_center[1], src/myIO.cpp:1466
  const double r_cut = 2.0 * dy, h = r_cut / 4.0;
  const int search = (int)floor(r_cut / dy);
  // per-term factors, in the order the reference forms them
  const real a_n = (real)(k.Fn / k.de_s2p / h), a_w = (real)(1.0 / k.de_s2p / h), ih2 = (real)(-1.0 / h / h);
  const real ih2p = (real)(1.0 / h / h), s2h2 = (real)k.de_s2h2, mb = (real)k.Fn, h_r = (real)h;
  const real r1_r = (real)r1, rc_r = (real)r_cut;
  real ns = 0, d2 = 0, d3 = 0;
  for (int kk = kr - search; kk <= kr + search; ++kk) {
    const int kkk = kk < 0 ? 0 : (kk > k.N1 - 1 ? k.N1 - 1 : kk);
    const int num2 = kkk * k.N0 + j;
    const int64_t o = off[num2];
    const int n2 = cnt[num2];
    const real shift = (real)((double)(kk - kkk) * dy);
    for (int i = lane; i < n2; i += 32) {
      const real r2 = x2[o + i] + shift;
      const real r1r2 = r2 - r1_r;
      const real rr = r2 > r1_r ? r1r2 : -r1r2;
      if (rr < rc_r) {
        const real e = r_exp(-rr * rr / h_r / h_r / (real)2.0);
        ns += a_n * e;
        const real W = a_w * e;
        d2 += mb * W * r1r2 * ih2;
        d3 += mb * W * s2h2 * ((real)3.0 * r1r2 - ih2p * r1r2 * r1r2 * r1r2);
      }
    }
  }
  double dns = (double)ns, dd2 = (double)d2, dd3 = (double)d3;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    dns += __shfl_xor_sync(FULL, dns, m);
    dd2 += __shfl_xor_sync(FULL, dd2, m);
    dd3 += __shfl_xor_sync(FULL, dd3, m);
  }
  if (lane == 0) {
    cell[(size_t)MCPM_CF_N_SMOOTH * C + num] = dns;
    cell[(size_t)MCPM_CF_DN2 * C + num] = dd2;
    cell[(size_t)MCPM_CF_DN3 * C + num] = dd3;
    const double pi = 3.14159265358979323846;
    const double dummyF = dd2 * 4.0 * pi * k.de_p * k.phi / k.m * 2.0;
    const double F2 = (num != 0 && num != k.N1 - 1) ? -dummyF : 0.0;
    cell[(size_t)MCPM_CF_F2 * C + num] = F2;
    if (pcell) pcell[(size_t)num * PF_STRIDE + PF_F2DT] = (float)(F2 * k.dt);
  }
}

int launch_smoothing(Session& s) {
  const PBuf& b = s.P[s.cur];
  const int blocks = (int)(((int64_t)s.C * 32 + 127) / 128);
  if (s.prec == MCPM_FP32)
    k_smoothing<float><<<blocks, 128, 0, s.stream>>>(s.k, s.cell, s.pcell, s.off, s.cnt, (const float*)b.x2);
  else
    k_smoothing<double><<<blocks, 128, 0, s.stream>>>(s.k, s.cell, nullptr, s.off, s.cnt, (const double*)b.x2);
  return 1;
}

int launch_long_range(Session& s) {
  const int mode = s.cfg.long_range;
  if (mode == MCPM_LR_DENSITY_EXPANSION) return launch_smoothing(s);
  if (mode != MCPM_LR_DIRECT && mode != MCPM_LR_SCREENED_POISSON) return 0;
  if (s.k.lr2d) return launch_long_range_2d(s);
  const LRTab* t = reinterpret_cast<const LRTab*>(s.lr_host);
  const double coef = mode == MCPM_LR_DIRECT ? s.cfg.phi : s.cfg.ast;
  k_long_range_1d<<<1, 1024, 2 * t->nf * sizeof(double), s.stream>>>(
      s.k, s.cell, s.prec == MCPM_FP32 ? s.pcell : nullptr, *t, coef);
  return 1;
}

// host-side tables for the session (called at creation): see LRTab
int long_range_setup(Session& s) {
  const int mode = s.cfg.long_range;
  if (mode != MCPM_LR_DIRECT && mode != MCPM_LR_SCREENED_POISSON) return 0;
  std::vector<double> off, w;
  build_quad(s, mode, off, w);
  const int N1 = s.k.N1, nf = N1 + 1;
  const double dy = s.k.dy;
  LRTab t{};
  t.mode = mode;
  t.nf = nf;
  std::vector<char> blob;
  auto put = [&](const void* p, size_t b) -> size_t {
    size_t o = (blob.size() + 15) & ~size_t(15);
    blob.resize(o + b);
    memcpy(blob.data() + o, p, b);
    return o;
  };
  size_t oW = 0, oEi = 0, oEw = 0, oI0 = 0, oIN = 0, oWq = 0, oPa = 0, oPg = 0, oDf = 0;
  if (mode == MCPM_LR_DIRECT) {
    // the reference's cell of point q seen from face fc (src/Main_Functions.cpp:3772-3773)
    auto cellof = [&](int fc, int q) { return (int)floor((fc * dy + off[q]) / dy); };
    std::vector<int> dgen(2500);
    int dmin = 1 << 30, dmax = -(1 << 30);
    const int fref = nf / 2;
    for (int q = 0; q < 2500; ++q) {
      dgen[q] = cellof(fref, q) - fref;
      dmin = std::min(dmin, dgen[q]);
      dmax = std::max(dmax, dgen[q]);
    }
    std::vector<double> W(dmax - dmin + 1, 0.0);
    for (int q = 0; q < 2500; ++q) W[dgen[q] - dmin] += w[q];
    std::vector<int> exi;
    std::vector<double> exw;
    for (int fc = 0; fc < nf; ++fc)
      for (int q = 0; q < 2500; ++q) {
        int c = cellof(fc, q);
        if (c - fc != dgen[q]) {
          exi.push_back(fc); exi.push_back(c); exi.push_back(fc + dgen[q]); exi.push_back(q);
          exw.push_back(w[q]);
        }
      }
    t.dmin = dmin;
    t.dmax = dmax;
    t.n_exc = (int)exw.size();
    oW = put(W.data(), W.size() * 8);
    if (!exw.empty()) {
      oEi = put(exi.data(), exi.size() * 4);
      oEw = put(exw.data(), exw.size() * 8);
    }
  } else {
    std::vector<int> i0(2500), iN(2500);
    for (int q = 0; q < 2500; ++q) {
      int c0 = (int)floor((0 * dy + off[q]) / dy), cN = (int)floor((N1 * dy + off[q]) / dy);
      i0[q] = c0 < 0 ? 0 : (c0 > N1 - 1 ? N1 - 1 : c0);
      iN[q] = cN < 0 ? 0 : (cN > N1 - 1 ? N1 - 1 : cN);
    }
    oI0 = put(i0.data(), 2500 * 4);
    oIN = put(iN.data(), 2500 * 4);
    oWq = put(w.data(), 2500 * 8);
    // PCR of the constant matrix (src/Main_Functions.cpp:3375-3466):
    // row 0 and row nf-1 are the Dirichlet rows, interior rows -1, 2+(dy b)^2, -1
    std::vector<double> l(nf), d(nf), u(nf);
    const double ad = 2.0 + (dy * s.cfg.bst) * (dy * s.cfg.bst);
    for (int i = 0; i < nf; ++i) {
      if (i == 0 || i == nf - 1) { l[i] = 0.0; d[i] = 1.0; u[i] = 0.0; }
      else { l[i] = -1.0; d[i] = ad; u[i] = -1.0; }
    }
    int levels = 0;
    while ((1 << levels) < nf) ++levels;
    std::vector<double> pa((size_t)levels * nf), pg((size_t)levels * nf);
    for (int lv = 0, st = 1; lv < levels; ++lv, st <<= 1) {
      std::vector<double> nl(nf), nd(nf), nu(nf);
      for (int i = 0; i < nf; ++i) {
        double al = 0.0, ga = 0.0, dd = d[i], lo = 0.0, uo = 0.0;
        if (i - st >= 0) { al = -l[i] / d[i - st]; lo = al * l[i - st]; dd += al * u[i - st]; }
        if (i + st < nf) { ga = -u[i] / d[i + st]; uo = ga * u[i + st]; dd += ga * l[i + st]; }
        pa[(size_t)lv * nf + i] = al;
        pg[(size_t)lv * nf + i] = ga;
        nl[i] = lo; nd[i] = dd; nu[i] = uo;
      }
      l.swap(nl); d.swap(nd); u.swap(nu);
    }
    t.levels = levels;
    {
      const double sg = s.cfg.sigma, b = s.cfg.bst;
      double corr = 1.0 - (sg * b + 1.0) * exp(-b * sg);
      t.corr = corr / b / b;
    }
    oPa = put(pa.data(), pa.size() * 8);
    oPg = put(pg.data(), pg.size() * 8);
    oDf = put(d.data(), nf * 8);
  }
  if (cudaMalloc(&s.lr_tab, blob.size() + 16) != cudaSuccess) return 1;
  cudaMemcpy(s.lr_tab, blob.data(), blob.size(), cudaMemcpyHostToDevice);
  char* base = (char*)s.lr_tab;
  if (mode == MCPM_LR_DIRECT) {
    t.W = (const double*)(base + oW);
    t.exc_i = t.n_exc ? (const int*)(base + oEi) : nullptr;
    t.exc_w = t.n_exc ? (const double*)(base + oEw) : nullptr;
  } else {
    t.idx0 = (const int*)(base + oI0);
    t.idxN = (const int*)(base + oIN);
    t.wq = (const double*)(base + oWq);
    t.pa = (const double*)(base + oPa);
    t.pg = (const double*)(base + oPg);
    t.dfin = (const double*)(base + oDf);
  }
  static_assert(sizeof(LRTab) <= sizeof(s.lr_host), "LRTab fits the session's slot");
  memcpy(s.lr_host, &t, sizeof(LRTab));
  return 0;
}

cudaError_t pcr_set_smem(int nf) {
  return cudaFuncSetAttribute(k_long_range_1d, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * nf * (int)sizeof(double));
}

}  // namespace mcpm
