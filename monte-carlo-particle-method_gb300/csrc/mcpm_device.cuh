// mcpm_device.cuh -- device helpers shared by the particle-step kernels:
// counter-based Philox draws, the reference's scalar laws (Y(n), mu(T)),
// compensated FP32 accumulation and warp / block reductions.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/mcpm.h"
#include "mcpm_internal.h"

namespace mcpm {

// ------------------------------------------------------------------ Philox
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 10 rounds of two
// 32x32->64 multiplies, key bumped by the Weyl constants between rounds.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}
__device__ __forceinline__ uint4 philox(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
  return philox(make_uint4(c0, c1, c2, c3), make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
}

// Philox4x32-10 with the round keys given (rk[2r], rk[2r + 1]: the key
// after r bumps), so that no key arithmetic runs per draw
__device__ __forceinline__ uint4 philox_rk(uint4 c, const uint32_t (&rk)[20]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
    uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ rk[2 * r], lo1, hi0 ^ c.w ^ rk[2 * r + 1], lo0);
  }
  return c;
}

// an injected draw: row (key + counter) mod rows of the caller's table (a
// call out of line, so that the Philox path keeps its registers)
static __device__ __noinline__ uint4 rng_injected(const uint4* inj, uint32_t rows, uint32_t key, uint32_t ctr) {
  return inj[((uint64_t)key + ctr) % rows];
}
// the four words of a draw: the stream's injected row when the caller
// injected uniforms for it, else Philox keyed by the seed with counter
// (key, step, stream, counter)
__device__ __forceinline__ uint4 rng_draw(const DevConsts& k, uint32_t key, uint32_t step, uint32_t stream,
                                          uint32_t ctr) {
  const uint4* inj = k.rng_inj[stream];
  if (__builtin_expect(inj != nullptr, 0)) return rng_injected(inj, k.rng_inj_rows[stream], key, ctr);
  return philox_rk(make_uint4(key, step, stream, ctr), k.rk);
}

__device__ __forceinline__ double u01d(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }
// uniform in (0,1) from the top 23 bits, built in the mantissa of a float in
// [1,2) (no integer-to-float conversion): k 2^-23 + 2^-24, k = x >> 9
__device__ __forceinline__ float u01f(uint32_t x) {
  return __uint_as_float(0x3F800000u | (x >> 9)) - 0.99999994039535522461f;
}
__device__ __forceinline__ int pick(uint32_t r, int n) { return (int)(((uint64_t)r * (uint64_t)n) >> 32); }

constexpr double kTwoPi = 6.283185307179586476925286766559;

template <typename real> struct Normals3 { real z0, z1, z2; };

// three standard normals (Box-Muller on the four Philox words)
template <typename real> __device__ __forceinline__ Normals3<real> normals3(uint4 r);
template <> __device__ __forceinline__ Normals3<double> normals3<double>(uint4 r) {
  double a = sqrt(-2.0 * log(u01d(r.x)));
  double b = sqrt(-2.0 * log(u01d(r.z)));
  double s1, c1;
  sincos(kTwoPi * u01d(r.y), &s1, &c1);
  return {a * c1, a * s1, b * cos(kTwoPi * u01d(r.w))};
}
// FP32 path: the hardware approximations of log and sin/cos (a few ulp,
// about 1e-6 absolute on [0, 2 pi)) -- ample for Monte Carlo draws
template <> __device__ __forceinline__ Normals3<float> normals3<float>(uint4 r) {
  // the approximate log of u just below 1 may come out slightly positive
  const float a = sqrtf(fmaxf(-2.0f * __logf(u01f(r.x)), 0.0f));
  const float b = sqrtf(fmaxf(-2.0f * __logf(u01f(r.z)), 0.0f));
  float s1, c1;
  __sincosf(6.28318530717958647692f * u01f(r.y), &s1, &c1);
  return {a * c1, a * s1, b * __cosf(6.28318530717958647692f * u01f(r.w))};
}

// a*b + c: one rounding (FMA) in the FP32 path, two roundings in the FP64
// path, which reproduces the reference's arithmetic
template <typename real> __device__ __forceinline__ real mad(real a, real b, real c);
template <> __device__ __forceinline__ float mad<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double mad<double>(double a, double b, double c) { return a * b + c; }

// ------------------------------------------- math in the path's precision
// Explicit float/double overloads, so that a float argument never goes
// through a double routine (GB300's FP64 rate is 1/64 of FP32).
__device__ __forceinline__ float r_floor(float x) { return floorf(x); }
__device__ __forceinline__ double r_floor(double x) { return ::floor(x); }
__device__ __forceinline__ float r_fabs(float x) { return fabsf(x); }
__device__ __forceinline__ double r_fabs(double x) { return ::fabs(x); }
__device__ __forceinline__ float r_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double r_sqrt(double x) { return ::sqrt(x); }
__device__ __forceinline__ float r_log(float x) { return __logf(x); }
__device__ __forceinline__ double r_log(double x) { return ::log(x); }
__device__ __forceinline__ void r_sincos(float x, float* s, float* c) { __sincosf(x, s, c); }
__device__ __forceinline__ void r_sincos(double x, double* s, double* c) { ::sincos(x, s, c); }
__device__ __forceinline__ float r_pow(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double r_pow(double x, double y) { return ::pow(x, y); }
__device__ __forceinline__ float r_acos(float x) { return acosf(x); }
__device__ __forceinline__ float r_exp(float x) { return expf(x); }
__device__ __forceinline__ double r_exp(double x) { return ::exp(x); }
__device__ __forceinline__ double r_acos(double x) { return ::acos(x); }

// ------------------------------------------------ constants in real type
// The FP32 kernels read float copies prepared on the host, so that no
// double->float conversion (an FP64-pipe instruction) runs per particle.
template <typename real> struct KC {
  real dx, dy, L0, L1, dt, sigma, m, kb, Tw[4], Uw[4];
  real idx, idy;  // 1/dx, 1/dy (FP32 binning)
  real eps_x, eps_y;  // diffuse-wall offsets
  const float *face_x, *face_y;  // FP32 binning face tables (DevConsts)
  float wx, wy;
};
template <typename real> __host__ __device__ __forceinline__ KC<real> make_kc(const DevConsts& k) {
  KC<real> c;
  if constexpr (sizeof(real) == 4) {
    c.dx = k.f_dx; c.dy = k.f_dy; c.L0 = k.f_L0; c.L1 = k.f_L1; c.dt = k.f_dt;
    c.sigma = k.f_sigma; c.m = k.f_m; c.kb = k.f_kb;
    for (int i = 0; i < 4; ++i) { c.Tw[i] = k.f_Tw[i]; c.Uw[i] = k.f_Uw[i]; }
    c.idx = k.f_idx; c.idy = k.f_idy; c.eps_x = k.f_eps_x; c.eps_y = k.f_eps_y;
    c.face_x = k.f_face_x; c.face_y = k.f_face_y; c.wx = k.f_bin_wx; c.wy = k.f_bin_wy;
  } else {
    c.dx = k.dx; c.dy = k.dy; c.L0 = k.L0; c.L1 = k.L1; c.dt = k.dt;
    c.sigma = k.sigma; c.m = k.m; c.kb = k.kb;
    for (int i = 0; i < 4; ++i) { c.Tw[i] = k.Tw[i]; c.Uw[i] = k.Uw[i]; }
    c.idx = 1.0 / k.dx; c.idy = 1.0 / k.dy; c.eps_x = k.eps_x; c.eps_y = k.eps_y;
    c.face_x = nullptr; c.face_y = nullptr; c.wx = 0.f; c.wy = 0.f;
  }
  return c;
}

// --------------------------------------------------------------- laws
// increase_collision_rate, src/Main_Functions.cpp:1906-1915
__device__ __forceinline__ double ycoll(double n, double b) {
  double nb = n * b;
  return 1.0 + 0.625 * n * b + 0.2869 * (nb * nb) + 0.115 * pow(nb, 3.0);
}
// scale_mu, src/Main_Functions.cpp:1970-1973 (pow(x, 0.5) == sqrt(x) exactly)
__device__ __forceinline__ double scale_mu(double T, const DevConsts& k) {
  double r = T / k.T0;
  return k.mu * (k.visp == 0.5 ? sqrt(r) : pow(r, k.visp));
}

// ---------------------------------------------------- compensated sums
// Knuth TwoSum: s + e == a + b exactly (needs separate rounding: the kernels
// are compiled with --fmad=false).
struct CSum {
  float hi, lo;
};
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void cadd(CSum& acc, float x) {
  float s, e;
  two_sum(acc.hi, x, s, e);
  acc.hi = s;
  acc.lo += e;
}
__device__ __forceinline__ CSum ccombine(CSum a, CSum b) {
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  e += a.lo + b.lo;
  CSum r;
  r.hi = s + e;
  r.lo = e - (r.hi - s);
  return r;
}
__device__ __forceinline__ double cvalue(CSum a) { return (double)a.hi + (double)a.lo; }

// accumulator abstraction: double sums in FP64 mode, compensated float in FP32
// (the float form serves only code written for both precisions; the FP32
// sessions' kernels sum in plain float runs combined pairwise)
template <typename real> struct Acc;
template <> struct Acc<double> {
  double v;
  __device__ __forceinline__ void zero() { v = 0.0; }
  __device__ __forceinline__ void add(double x) { v += x; }
  __device__ __forceinline__ double get() const { return v; }
  __device__ __forceinline__ double getr() const { return v; }
  __device__ __forceinline__ void shfl_xor(int m) { v += __shfl_xor_sync(0xffffffffu, v, m); }
  __device__ __forceinline__ void merge(const Acc& o) { v += o.v; }
  __device__ __forceinline__ Acc xor_fetch(int m) const {
    Acc o;
    o.v = __shfl_xor_sync(0xffffffffu, v, m);
    return o;
  }
};
template <> struct Acc<float> {
  CSum c;
  __device__ __forceinline__ void zero() { c.hi = 0.f; c.lo = 0.f; }
  __device__ __forceinline__ void add(float x) { cadd(c, x); }
  __device__ __forceinline__ double get() const { return cvalue(c); }
  // the value in float (no FP64 instruction)
  __device__ __forceinline__ float getr() const { return c.hi + c.lo; }
  __device__ __forceinline__ void shfl_xor(int m) {
    CSum o;
    o.hi = __shfl_xor_sync(0xffffffffu, c.hi, m);
    o.lo = __shfl_xor_sync(0xffffffffu, c.lo, m);
    c = ccombine(c, o);
  }
  __device__ __forceinline__ void merge(const Acc& o) { c = ccombine(c, o.c); }
  __device__ __forceinline__ Acc xor_fetch(int m) const {
    Acc o;
    o.c.hi = __shfl_xor_sync(0xffffffffu, c.hi, m);
    o.c.lo = __shfl_xor_sync(0xffffffffu, c.lo, m);
    return o;
  }
};

// Warp reduction of K <= 32 accumulators by recursive halving: at each
// butterfly stage a lane keeps half of its fields and ships the other half to
// its partner, so a warp does 31 combines instead of 5K.  On return every
// lane holds the warp total of one field, *field.
template <typename real, int K>
__device__ __forceinline__ Acc<real> warp_reduce_halving(Acc<real> (&a)[K], int* field) {
  static_assert(K <= 32, "one accumulator per lane");
  constexpr int P = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
  const int lane = threadIdx.x & 31;
  Acc<real> v[P];
#pragma unroll
  for (int q = 0; q < P; ++q) {
    if (q < K) v[q] = a[q];
    else v[q].zero();
  }
  int base = 0;
#pragma unroll
  for (int F = P, m = 16; m >= 1; m >>= 1) {
    if (F > 1) {
      const bool up = (lane & m) != 0;
      const int h = F / 2;
#pragma unroll
      for (int j = 0; j < P / 2; ++j) {
        if (j < h) {
          Acc<real> keep = up ? v[j + h] : v[j];
          Acc<real> send = up ? v[j] : v[j + h];
          keep.merge(send.xor_fetch(m));  // the partner ships its copy of my field
          v[j] = keep;
        }
      }
      if (up) base += h;
      F = h;
    } else {
      v[0].shfl_xor(m);
    }
  }
  *field = base;
  return v[0];
}

// Reduce K <= 32 accumulators over a tile; returns to lane l (of warp 0
// when TILE > 32) the total of accumulator l, so that K results can be
// written by K lanes at once.
template <typename real, int K, int TILE>
__device__ __forceinline__ Acc<real> tile_reduce_lanes(Acc<real> (&a)[K], Acc<real>* smem) {
  static_assert(K > 16 && K <= 32, "one accumulator per lane");
  const int lane = threadIdx.x & 31;
  int f;
  Acc<real> r = warp_reduce_halving<real, K>(a, &f);
  // for K > 16 every lane holds a distinct field f == lane
  if constexpr (TILE > 32) {
    constexpr int W = TILE / 32;
    const int warp = threadIdx.x >> 5;
    __syncthreads();
    if (lane < K) smem[lane * W + warp] = r;
    __syncthreads();
    if (warp == 0 && lane < K) {
      Acc<real> t = smem[lane * W];
      for (int w = 1; w < W; ++w) t.merge(smem[lane * W + w]);
      r = t;
    }
  }
  return r;
}

// lane that holds field q after warp_reduce_halving with P fields
template <int P> __device__ __forceinline__ int halving_lane(int q) {
  int l = 0, m = 16;
#pragma unroll
  for (int h = P / 2; h >= 1; h >>= 1, m >>= 1)
    if (q & h) l |= m;
  return l;
}

// Reduce K accumulators over a tile of TILE threads (32 = one warp, or a
// whole block); every thread of the tile gets all K totals.  smem must hold
// K * (TILE/32) Acc entries when TILE > 32.
template <typename real, int K, int TILE>
__device__ __forceinline__ void tile_reduce(Acc<real> (&a)[K], Acc<real>* smem) {
  constexpr int P = K <= 1 ? 1 : K <= 2 ? 2 : K <= 4 ? 4 : K <= 8 ? 8 : K <= 16 ? 16 : 32;
  int f;
  Acc<real> r = warp_reduce_halving<real, K>(a, &f);
  if constexpr (TILE == 32) {
#pragma unroll
    for (int q = 0; q < K; ++q) {
      Acc<real> t;
      // fetch field q from the lane that holds it
      if constexpr (sizeof(real) == 8) {
        t.v = __shfl_sync(0xffffffffu, r.v, halving_lane<P>(q));
      } else {
        t.c.hi = __shfl_sync(0xffffffffu, r.c.hi, halving_lane<P>(q));
        t.c.lo = __shfl_sync(0xffffffffu, r.c.lo, halving_lane<P>(q));
      }
      a[q] = t;
    }
  } else {
    // one partial per warp and field; warp 0 merges (lane q takes field q)
    // and leaves the totals in smem[q * W] for every thread to read
    constexpr int W = TILE / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __syncthreads();
    if ((lane & (32 / P - 1)) == 0 && f < K) smem[f * W + warp] = r;
    __syncthreads();
    if (warp == 0 && lane < K) {
      Acc<real> t = smem[lane * W];
      for (int w = 1; w < W; ++w) t.merge(smem[lane * W + w]);
      smem[lane * W] = t;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < K; ++q) a[q] = smem[q * W];
  }
}


// floor(t) for -1 < t < 2^23 without a float-to-int conversion instruction:
// adding 2^23 with rounding toward -inf leaves floor(t) in the mantissa.
// Values outside that range come out below 0 or at or above 2^23 and are
// clamped by the caller.  Returns the integer; *tf gets floor(t) as a float.
__device__ __forceinline__ int floor_to_int(float t, float* tf) {
  const float f = __fadd_rd(t, 8388608.0f);
  *tf = f - 8388608.0f;
  return __float_as_int(f) - 0x4B000000;
}

__device__ __forceinline__ void raise_status(uint32_t* status, uint32_t bits) {
  if (bits) atomicOr(status, bits);
}

// warp-aggregated atomic increment of a per-cell counter
__device__ __forceinline__ void count_key(int32_t* cnt, int key, bool active) {
  unsigned am = __ballot_sync(0xffffffffu, active);
  if (!active) return;
  unsigned peers = __match_any_sync(am, key);
  int leader = __ffs(peers) - 1;
  if ((int)(threadIdx.x & 31) == leader) atomicAdd(&cnt[key], __popc(peers));
}

// volume of cell c exactly as make_cells builds it, src/myIO.cpp:1456-1465
__device__ __forceinline__ double cell_volume(int c, const DevConsts& k) {
  int j = c % k.N0, kk = c / k.N0;
  double d0 = (double)j * k.dx, d1 = (double)(j + 1) * k.dx;
  double d2 = (double)kk * k.dy, d3 = (double)(kk + 1) * k.dy;
  double d4 = 0.0 * k.dz, d5 = 1.0 * k.dz;
  return (d1 - d0) * (d3 - d2) * (d5 - d4);
}

}  // namespace mcpm
