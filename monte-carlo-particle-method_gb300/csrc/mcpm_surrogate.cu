// mcpm_surrogate.cu -- learned Vlasov force of a 2-D box (no counterpart in
// the reference, whose only learned model is the off-path hybrid NN/GPR).
//
// A 4-layer convolutional operator on the N1 x N0 cell grid maps the
// densities the plain node-grid force consumes to the node-potential
// differences the particle kick reads:
//
//   input  x[c][16] (bf16): v_k = 10 (b n_n[c][k] - 0.25), k = 0..3 (the
//          four corner nodal densities of cell_update, src/Main_Functions.cpp:
//          2268-2364), v_4 = 10 (b n[c] - 0.25) (cell density), each split
//          into hi = bf16(v) in channels 0..4 and lo = bf16(v - hi) in
//          channels 6..10; channel 5 = 1 (inside mask: the zero padding
//          marks the walls); channels 11..15 zero;
//   conv3x3 16->64, ReLU, conv3x3 64->64, ReLU, conv3x3 64->64, ReLU,
//   conv3x3 64->16 (outputs 0..3 used), zero padding, no stride;
//   output y[c][4] (fp32) x out_scale = (V1-V0, V3-V2, V2-V0, V3-V1), the
//          differences of the corner potentials of cell c (corner 0 lower
//          left, 1 lower right, 2 upper left, 3 upper right), from which the
//          kick coefficients of the FP32 particle pass follow
//          (src/FEM.cpp:567-578): U1 -= g1 (d0 + (d1 - d0) eta),
//          U2 -= g2 (d2 + (d3 - d2) xi), g = coef / m / dx dt.
//
// Every convolution is an implicit GEMM on the tensor cores: rows are 128
// consecutive cells, columns the output channels, and the reduction runs
// over the nine taps x input channels; each tap's shifted 128-cell input
// tile and weight tile are staged by cp.async into swizzled shared memory
// (zero fill outside the grid), fed by ldmatrix to mma.m16n8k16 (bf16 in,
// fp32 accumulate).  The same kernel computes the data gradient of the
// backward pass (weights transposed and flipped, times the ReLU mask), and a
// second kernel the weight gradient (the reduction over cells, ldmatrix
// .trans operands).  Every forward layer of inference runs on the
// fifth-generation tensor cores (tcgen05, mcpm_surrogate_tc.cu).
//
// Parameters: one fp32 array (layout SP_OFF_* below, [co][tap][ci] with
// tap = 3 (dy + 1) + (dx + 1)), trained by Adam on fp32 master weights; the
// kernels read a bf16 copy.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mcpm_device.cuh"
#include "mcpm_surrogate.h"

namespace mcpm {
namespace sur {

typedef __nv_bfloat16 bf16;

// ----------------------------------------------------------- primitives
__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
  const int sz = valid ? 16 : 0;  // 0: fill the 16 bytes with zeros, read nothing
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(sz) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x4_t(uint32_t (&r)[4], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
               : "r"(addr));
}
__device__ __forceinline__ void ldsm_x2_t(uint32_t (&r)[2], uint32_t addr) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x2.trans.shared.b16 {%0,%1}, [%2];\n"
               : "=r"(r[0]), "=r"(r[1])
               : "r"(addr));
}
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// byte offset of 16-byte chunk ch of row `row` in a tile whose rows hold CH
// chunks, XOR-swizzled so that the eight rows an ldmatrix phase reads fall
// in eight different bank groups
template <int CH> __device__ __forceinline__ int swz(int row, int ch) {
  static_assert(CH == 8 || CH == 2, "rows of 128 or 32 bytes");
  if constexpr (CH == 8) return row * 128 + ((ch ^ (row & 7)) << 4);
  else return row * 32 + ((ch ^ ((row >> 2) & 1)) << 4);
}

constexpr int TM = 128;  // cells per tile (GEMM rows)
constexpr int NT = 256;  // threads per block (8 warps)

// epilogues of the convolution kernel
enum { EPI_RELU = 0, EPI_OUT = 1, EPI_MASK = 2, EPI_KICK = 3 };

struct ConvArgs {
  const bf16* x;      // [P][CIN]
  const bf16* w;      // [COUT][9][CIN]
  const float* bias;  // [COUT] (EPI_RELU, EPI_OUT, EPI_KICK)
  void* out;          // bf16 [P][COUT] (EPI_RELU, EPI_MASK), float [P][4] (EPI_OUT)
  const bf16* mask;   // [P][COUT] activations whose sign gates the gradient (EPI_MASK)
  float* pcell;       // packed per-cell record (EPI_KICK)
  int N0, N1, C, P;   // grid, cells per image, cells in the batch
  float g1, g2, oscale;
};

template <int CIN, int COUT> constexpr int conv_smem() { return 3 * (TM * CIN * 2 + COUT * CIN * 2); }

// out = epilogue(sum_{tap, ci} x[p + off(tap)][ci] w[co][tap][ci])
template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(NT) k_conv(ConvArgs a) {
  constexpr int CH = CIN / 8;
  constexpr int A_BYTES = TM * CIN * 2, STAGE = A_BYTES + COUT * CIN * 2;
  constexpr int WN = COUT >= 64 ? 2 : 1, WM = 8 / WN, WTM = TM / WM, WTN = COUT / WN;
  constexpr int MI = WTM / 16, NI = WTN / 8;
  static_assert(NI % 2 == 0 && MI >= 1, "warp tile");
  constexpr int A_PER = (TM * CH + NT - 1) / NT;
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp % WM, wn = warp / WM;
  const int p0 = blockIdx.x * TM;
  const int N0 = a.N0, N1 = a.N1;

  int ay[A_PER], ax[A_PER], ab[A_PER];
  bool aok[A_PER];
#pragma unroll
  for (int j = 0; j < A_PER; ++j) {
    const int e = tid + NT * j, row = e / CH, p = p0 + row;
    aok[j] = e < TM * CH && p < a.P;
    const int pp = aok[j] ? p : 0;
    const int b = pp / a.C, c = pp - b * a.C;
    ay[j] = c / N0;
    ax[j] = c - ay[j] * N0;
    ab[j] = b * a.C;
  }
  auto load = [&](int tap, int st) {
    unsigned char* As = smem + st * STAGE;
    unsigned char* Bs = As + A_BYTES;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
#pragma unroll
    for (int j = 0; j < A_PER; ++j) {
      const int e = tid + NT * j;
      if (e < TM * CH) {
        const int row = e / CH, ch = e % CH;
        const int yy = ay[j] + dy, xx = ax[j] + dx;
        const bool v = aok[j] && yy >= 0 && yy < N1 && xx >= 0 && xx < N0;
        const bf16* src = v ? a.x + ((size_t)(ab[j] + yy * N0 + xx) * CIN + ch * 8) : a.x;
        cp_async16(smem_u32(As + swz<CH>(row, ch)), src, v);
      }
    }
    for (int e = tid; e < COUT * CH; e += NT) {
      const int row = e / CH, ch = e % CH;
      cp_async16(smem_u32(Bs + swz<CH>(row, ch)), a.w + ((size_t)(row * 9 + tap) * CIN + ch * 8), true);
    }
  };

  float acc[MI][NI][4];
#pragma unroll
  for (int i = 0; i < MI; ++i)
#pragma unroll
    for (int j = 0; j < NI; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) acc[i][j][q] = 0.f;

  load(0, 0);
  cp_async_commit();
  load(1, 1);
  cp_async_commit();
  for (int tap = 0; tap < 9; ++tap) {
    cp_async_wait<1>();
    __syncthreads();
    if (tap + 2 < 9) load(tap + 2, (tap + 2) % 3);
    cp_async_commit();
    const unsigned char* As = smem + (tap % 3) * STAGE;
    const unsigned char* Bs = As + A_BYTES;
#pragma unroll
    for (int kk = 0; kk < CIN / 16; ++kk) {
      uint32_t af[MI][4], bfr[NI][2];
#pragma unroll
      for (int mi = 0; mi < MI; ++mi)
        ldsm_x4(af[mi], smem_u32(As + swz<CH>(wm * WTM + mi * 16 + (lane & 15), kk * 2 + (lane >> 4))));
#pragma unroll
      for (int ni = 0; ni < NI; ni += 2) {
        uint32_t r[4];
        ldsm_x4(r, smem_u32(Bs + swz<CH>(wn * WTN + ni * 8 + (lane & 7) + ((lane >> 4) << 3),
                                         kk * 2 + ((lane >> 3) & 1))));
        bfr[ni][0] = r[0]; bfr[ni][1] = r[1]; bfr[ni + 1][0] = r[2]; bfr[ni + 1][1] = r[3];
      }
#pragma unroll
      for (int mi = 0; mi < MI; ++mi)
#pragma unroll
        for (int ni = 0; ni < NI; ++ni) mma16816(acc[mi][ni], af[mi], bfr[ni][0], bfr[ni][1]);
    }
  }
  cp_async_wait<0>();

#pragma unroll
  for (int mi = 0; mi < MI; ++mi)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int p = p0 + wm * WTM + mi * 16 + (lane >> 2) + h * 8;
#pragma unroll
      for (int ni = 0; ni < NI; ++ni) {
        const int col = wn * WTN + ni * 8 + 2 * (lane & 3);
        float v0 = acc[mi][ni][2 * h], v1 = acc[mi][ni][2 * h + 1];
        if constexpr (EPI == EPI_RELU) {
          v0 = fmaxf(v0 + a.bias[col], 0.f);
          v1 = fmaxf(v1 + a.bias[col + 1], 0.f);
          if (p < a.P)
            *reinterpret_cast<__nv_bfloat162*>(static_cast<bf16*>(a.out) + (size_t)p * COUT + col) =
                __floats2bfloat162_rn(v0, v1);
        } else if constexpr (EPI == EPI_MASK) {
          if (p < a.P) {
            const __nv_bfloat162 m = *reinterpret_cast<const __nv_bfloat162*>(a.mask + (size_t)p * COUT + col);
            v0 = __bfloat162float(m.x) > 0.f ? v0 : 0.f;
            v1 = __bfloat162float(m.y) > 0.f ? v1 : 0.f;
            *reinterpret_cast<__nv_bfloat162*>(static_cast<bf16*>(a.out) + (size_t)p * COUT + col) =
                __floats2bfloat162_rn(v0, v1);
          }
        } else if constexpr (EPI == EPI_OUT) {
          if (col < 4 && p < a.P) {
            float* o = static_cast<float*>(a.out) + (size_t)p * 4 + col;
            o[0] = v0 + a.bias[col];
            o[1] = v1 + a.bias[col + 1];
          }
        } else {  // EPI_KICK: lanes 4q hold outputs 0, 1 of a cell, lanes 4q + 1 outputs 2, 3
          if (ni == 0 && wn == 0) {
            const float w2 = __shfl_down_sync(0xffffffffu, v0, 1), w3 = __shfl_down_sync(0xffffffffu, v1, 1);
            if ((lane & 3) == 0 && p < a.P) {
              const float d0 = (v0 + a.bias[0]) * a.oscale, d1 = (v1 + a.bias[1]) * a.oscale;
              const float d2 = (w2 + a.bias[2]) * a.oscale, d3 = (w3 + a.bias[3]) * a.oscale;
              *reinterpret_cast<float4*>(a.pcell + (size_t)p * PF_STRIDE + PF_LA1) =
                  make_float4(d0 * a.g1, (d1 - d0) * a.g1, d2 * a.g2, (d3 - d2) * a.g2);
            }
          }
        }
      }
    }
}

struct WgArgs {
  const bf16* x;   // [P][CIN] layer input
  const bf16* dz;  // [P][COUT] gradient of the layer's pre-activation
  float* part;     // [gridDim.x][9][COUT][CIN]
  int N0, N1, C, P, ntiles;
};

template <int CIN, int COUT> constexpr int wgrad_smem() { return 2 * (TM * CIN * 2 + TM * COUT * 2); }

// part[g][tap][co][ci] = sum over the tiles of block g of dz[p][co] x[p + off(tap)][ci]
template <int CIN, int COUT>
__global__ void __launch_bounds__(NT) k_wgrad(WgArgs a) {
  constexpr int CHI = CIN / 8, CHO = COUT / 8;
  constexpr int X_BYTES = TM * CIN * 2, STAGE = X_BYTES + TM * COUT * 2;
  constexpr int WM = COUT / 16, WN = 8 / WM, WTN = CIN / WN, NI = WTN / 8;
  static_assert(WM * WN == 8 && NI >= 1, "warp tile");
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp % WM, wn = warp / WM;
  const int tap = blockIdx.y, dy = tap / 3 - 1, dx = tap % 3 - 1;
  const int N0 = a.N0, N1 = a.N1;

  auto load = [&](int t, int st) {
    unsigned char* Xs = smem + st * STAGE;
    unsigned char* Ds = Xs + X_BYTES;
    const int p0 = t * TM;
    for (int e = tid; e < TM * CHI; e += NT) {
      const int row = e / CHI, ch = e % CHI, p = p0 + row;
      bool v = p < a.P;
      const int pp = v ? p : 0;
      const int b = pp / a.C, c = pp - b * a.C, y = c / N0, x = c - y * N0;
      const int yy = y + dy, xx = x + dx;
      v = v && yy >= 0 && yy < N1 && xx >= 0 && xx < N0;
      const bf16* src = v ? a.x + ((size_t)(b * a.C + yy * N0 + xx) * CIN + ch * 8) : a.x;
      cp_async16(smem_u32(Xs + swz<CHI>(row, ch)), src, v);
    }
    for (int e = tid; e < TM * CHO; e += NT) {
      const int row = e / CHO, ch = e % CHO, p = p0 + row;
      const bool v = p < a.P;
      cp_async16(smem_u32(Ds + swz<CHO>(row, ch)), v ? a.dz + ((size_t)p * COUT + ch * 8) : a.dz, v);
    }
  };

  float acc[NI][4];
#pragma unroll
  for (int j = 0; j < NI; ++j)
#pragma unroll
    for (int q = 0; q < 4; ++q) acc[j][q] = 0.f;

  int t = blockIdx.x, it = 0;
  if (t < a.ntiles) load(t, 0);
  cp_async_commit();
  for (; t < a.ntiles; t += gridDim.x, ++it) {
    if (t + (int)gridDim.x < a.ntiles) load(t + gridDim.x, (it + 1) & 1);
    cp_async_commit();
    cp_async_wait<1>();
    __syncthreads();
    const unsigned char* Xs = smem + (it & 1) * STAGE;
    const unsigned char* Ds = Xs + X_BYTES;
#pragma unroll
    for (int kk = 0; kk < TM / 16; ++kk) {
      uint32_t af[4];
      ldsm_x4_t(af, smem_u32(Ds + swz<CHO>(kk * 16 + (lane & 7) + ((lane >> 4) << 3), wm * 2 + ((lane >> 3) & 1))));
      if constexpr (NI == 1) {
        uint32_t r[2];
        ldsm_x2_t(r, smem_u32(Xs + swz<CHI>(kk * 16 + (lane & 7) + (((lane >> 3) & 1) << 3), wn * (WTN / 8))));
        mma16816(acc[0], af, r[0], r[1]);
      } else {
#pragma unroll
        for (int ni = 0; ni < NI; ni += 2) {
          uint32_t r[4];
          ldsm_x4_t(r, smem_u32(Xs + swz<CHI>(kk * 16 + (lane & 7) + (((lane >> 3) & 1) << 3),
                                               (wn * WTN + ni * 8) / 8 + (lane >> 4))));
          mma16816(acc[ni], af, r[0], r[1]);
          mma16816(acc[ni + 1], af, r[2], r[3]);
        }
      }
    }
    __syncthreads();
  }
  cp_async_wait<0>();
  float* out = a.part + ((size_t)blockIdx.x * 9 + tap) * COUT * CIN;
#pragma unroll
  for (int ni = 0; ni < NI; ++ni)
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int co = wm * 16 + (lane >> 2) + h * 8;
      const int ci = wn * WTN + ni * 8 + 2 * (lane & 3);
      out[(size_t)co * CIN + ci] = acc[ni][2 * h];
      out[(size_t)co * CIN + ci + 1] = acc[ni][2 * h + 1];
    }
}

// grad[(co 9 + tap) CIN + ci] = sum_g part[g][tap][co][ci] (fixed order)
__global__ void k_wgrad_reduce(const float* part, int G, int cin, int cout, float* grad) {
  const int n = 9 * cout * cin;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int tap = e / (cout * cin), r = e - tap * cout * cin, co = r / cin, ci = r - co * cin;
    float s = 0.f;
    for (int g = 0; g < G; ++g) s += part[(size_t)g * n + e];
    grad[((size_t)co * 9 + tap) * cin + ci] = s;
  }
}

// per-block column sums of dz[P][cout] -> part[block][cout]
__global__ void k_bias_part(const bf16* dz, int P, int cout, float* part) {
  __shared__ float red[NT];
  const int rows = NT / cout, co = threadIdx.x % cout, r0 = threadIdx.x / cout;
  float s = 0.f;
  for (int p = blockIdx.x * rows + r0; p < P; p += gridDim.x * rows) s += __bfloat162float(dz[(size_t)p * cout + co]);
  red[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x < cout) {
    float t = 0.f;
    for (int r = 0; r < rows; ++r) t += red[r * cout + threadIdx.x];
    part[(size_t)blockIdx.x * cout + threadIdx.x] = t;
  }
}
__global__ void k_bias_reduce(const float* part, int G, int cout, float* grad) {
  const int co = threadIdx.x;
  if (co >= cout) return;
  float s = 0.f;
  for (int g = 0; g < G; ++g) s += part[(size_t)g * cout + co];
  grad[co] = s;
}

// loss = mean over cells and outputs of (y - ts t)^2; dz4 = its gradient
// (bf16, 16 channels, 4..15 zero); per-block sums of (y - ts t)^2, (ts t)^2
__global__ void k_loss(const float* y, const float* t, float ts, int P, bf16* dz4, double* part) {
  __shared__ double r0[NT], r1[NT];
  const float g = 2.0f / (4.0f * (float)P);
  double se = 0.0, st = 0.0;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const float4 yy = *reinterpret_cast<const float4*>(y + (size_t)p * 4);
    const float4 tt = *reinterpret_cast<const float4*>(t + (size_t)p * 4);
    const float e0 = yy.x - ts * tt.x, e1 = yy.y - ts * tt.y, e2 = yy.z - ts * tt.z, e3 = yy.w - ts * tt.w;
    se += (double)e0 * e0 + (double)e1 * e1 + (double)e2 * e2 + (double)e3 * e3;
    st += (double)(ts * tt.x) * (ts * tt.x) + (double)(ts * tt.y) * (ts * tt.y) + (double)(ts * tt.z) * (ts * tt.z) +
          (double)(ts * tt.w) * (ts * tt.w);
    __nv_bfloat162 q[8];
    q[0] = __floats2bfloat162_rn(g * e0, g * e1);
    q[1] = __floats2bfloat162_rn(g * e2, g * e3);
    for (int i = 2; i < 8; ++i) q[i] = __floats2bfloat162_rn(0.f, 0.f);
    uint4* o = reinterpret_cast<uint4*>(dz4 + (size_t)p * 16);
    o[0] = *reinterpret_cast<uint4*>(&q[0]);
    o[1] = *reinterpret_cast<uint4*>(&q[4]);
  }
  r0[threadIdx.x] = se;
  r1[threadIdx.x] = st;
  __syncthreads();
  for (int s = NT / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) { r0[threadIdx.x] += r0[threadIdx.x + s]; r1[threadIdx.x] += r1[threadIdx.x + s]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = r0[0]; part[2 * blockIdx.x + 1] = r1[0]; }
}
// the G block partials (a, b) summed by one warp in a fixed order: lane l
// takes partials l, l + 32, ..., then an XOR butterfly (deterministic; one
// chain of G dependent FP64 adds was the judge step's slowest launch)
__global__ void k_pair_reduce(const double* part, int G, double* out) {
  if (blockIdx.x != 0) return;
  const int lane = threadIdx.x & 31;
  double a = 0.0, b = 0.0;
  if (threadIdx.x < 32)
    for (int g = lane; g < G; g += 32) { a += part[2 * g]; b += part[2 * g + 1]; }
  if (threadIdx.x >= 32) return;
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, m);
    b += __shfl_xor_sync(0xffffffffu, b, m);
  }
  if (lane == 0) {
    out[0] = a;
    out[1] = b;
  }
}

// Adam on the fp32 master parameters, then their bf16 copy
__global__ void k_adam(float* p, float* m, float* v, const float* g, bf16* w, int n, float lr, float b1, float b2,
                       float eps, float bc1, float bc2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi, vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    w[i] = __float2bfloat16_rn(pi);
  }
}
__global__ void k_to_bf16(const float* p, bf16* w, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) w[i] = __float2bfloat16_rn(p[i]);
}
// weights of the data gradient: F[ci][8 - tap][co] = W[co][tap][ci]
__global__ void k_flip(const bf16* W, int cout, int cin, bf16* F) {
  const int n = cout * 9 * cin;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int co = e / (9 * cin), r = e - co * 9 * cin, tap = r / cin, ci = r - tap * cin;
    F[((size_t)ci * 9 + (8 - tap)) * cout + co] = W[e];
  }
}

// ---------------------------------------------------- session-side kernels
// network input of every cell from the nodal densities and cell densities:
// each value v = 10 (b n - 0.25) as a bf16 pair hi = bf16(v), lo = bf16(v -
// hi) (channels 0..4 and 6..10), so the input keeps ~16 significant bits --
// the kick follows from density differences between neighbouring nodes,
// a few percent of the density, below a single bf16's resolution
__global__ void k_input(const double* nnd, const double* n, double b, int C, bf16* x) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    __align__(16) bf16 q[16];
    const double* nn = nnd + (size_t)c * 4;
#pragma unroll
    for (int k = 0; k < 4; ++k) sur_hi_lo(10.0 * (b * nn[k] - 0.25), q[k], q[6 + k]);
    sur_hi_lo(10.0 * (b * n[c] - 0.25), q[4], q[10]);
    q[5] = __float2bfloat16_rn(1.0f);
#pragma unroll
    for (int k = 11; k < 16; ++k) q[k] = __float2bfloat16_rn(0.0f);
    uint4* o = reinterpret_cast<uint4*>(x + (size_t)c * 16);
    o[0] = *reinterpret_cast<uint4*>(&q[0]);
    o[1] = *reinterpret_cast<uint4*>(&q[8]);
  }
}
// training target: the corner-potential differences of every cell
__global__ void k_target(const double* V, int N0, int C, float* y) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    const int j = c % N0, kk = c / N0;
    const int id0 = kk * (N0 + 1) + j, id2 = id0 + N0 + 1;
    const double v0 = V[id0], v1 = V[id0 + 1], v2 = V[id2], v3 = V[id2 + 1];
    *reinterpret_cast<float4*>(y + (size_t)c * 4) =
        make_float4((float)(v1 - v0), (float)(v3 - v2), (float)(v2 - v0), (float)(v3 - v1));
  }
}
// judge: per-block sums of |kick_surrogate - kick_plain|^2 and |kick_plain|^2
// over the four kick coefficients of every cell
__global__ void k_judge(const float* y, float oscale, float g1, float g2, const float* pcell, int C, double* part) {
  __shared__ double r0[NT], r1[NT];
  double se = 0.0, sp = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
    const float4 yy = *reinterpret_cast<const float4*>(y + (size_t)c * 4);
    const float d0 = yy.x * oscale, d1 = yy.y * oscale, d2 = yy.z * oscale, d3 = yy.w * oscale;
    const float s[4] = {d0 * g1, (d1 - d0) * g1, d2 * g2, (d3 - d2) * g2};
    const float4 pp = *reinterpret_cast<const float4*>(pcell + (size_t)c * PF_STRIDE + PF_LA1);
    const float q[4] = {pp.x, pp.y, pp.z, pp.w};
    for (int i = 0; i < 4; ++i) {
      se += (double)(s[i] - q[i]) * (s[i] - q[i]);
      sp += (double)q[i] * q[i];
    }
  }
  r0[threadIdx.x] = se;
  r1[threadIdx.x] = sp;
  __syncthreads();
  for (int st = NT / 2; st > 0; st >>= 1) {
    if (threadIdx.x < st) { r0[threadIdx.x] += r0[threadIdx.x + st]; r1[threadIdx.x] += r1[threadIdx.x + st]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { part[2 * blockIdx.x] = r0[0]; part[2 * blockIdx.x + 1] = r1[0]; }
}

// training snapshots: quadrant counts of a smooth packing-fraction field
// nb(x, y) = nbar + sum_k a_k sin(2 pi (kx x / L0 + ky y / L1) + phi_k),
// clipped to [0.05, 0.45], sampled at the quadrant centres; each quadrant
// holds round(lambda + sqrt(lambda) z) particles, lambda = nb / b vol / 4 / Fn
// (the normal limit of the count fluctuations of a free-streaming gas)
__global__ void k_snap_counts(const double* fld, int K, DevConsts k, uint64_t seed, uint32_t snap, int32_t* qc) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 4 * k.C; e += gridDim.x * blockDim.x) {
    const int c = e >> 2, q = e & 3;
    const int j = c % k.N0, kk = c / k.N0;
    const double x = ((double)j + 0.25 + 0.5 * (q & 1)) * k.dx, y = ((double)kk + 0.25 + 0.5 * (q >> 1)) * k.dy;
    double nb = fld[0];
    for (int w = 0; w < K; ++w) {
      const double* f = fld + 1 + 4 * w;
      nb += f[0] * sin(kTwoPi * (f[1] * x / k.L0 + f[2] * y / k.L1) + f[3]);
    }
    nb = fmin(fmax(nb, 0.05), 0.45);
    const double lam = nb / k.b * cell_volume(c, k) * 0.25 / k.Fn;
    const Normals3<double> z = normals3<double>(philox(seed, snap, (uint32_t)e, 0x53555247u, 0u));
    qc[e] = (int32_t)fmax(0.0, rint(lam + sqrt(lam) * z.z0));
  }
}
__global__ void k_cell_density(const int32_t* qc, DevConsts k, double* n) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < k.C; c += gridDim.x * blockDim.x) {
    const int cnt = qc[4 * c] + qc[4 * c + 1] + qc[4 * c + 2] + qc[4 * c + 3];
    n[c] = k.Fn * (double)cnt / cell_volume(c, k);
  }
}

}  // namespace sur

// ================================================================ host side
using namespace sur;

static int gblocks(long n, int bs, int cap) { return (int)std::max(1L, std::min((n + bs - 1) / bs, (long)cap)); }


static constexpr int WG_G = 64;     // blocks per tap of the weight-gradient kernels
static constexpr int RED_G = 256;   // blocks of the loss / judge reductions

static bool set_smem_attrs() {
  static bool done = false, ok = true;
  if (done) return ok;
  done = true;
  auto set = [&](const void* f, int bytes) {
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess) ok = false;
  };
  set((const void*)k_conv<16, 64, EPI_RELU>, conv_smem<16, 64>());
  set((const void*)k_conv<64, 64, EPI_RELU>, conv_smem<64, 64>());
  set((const void*)k_conv<64, 16, EPI_OUT>, conv_smem<64, 16>());
  set((const void*)k_conv<64, 16, EPI_KICK>, conv_smem<64, 16>());
  set((const void*)k_conv<16, 64, EPI_MASK>, conv_smem<16, 64>());
  set((const void*)k_conv<64, 64, EPI_MASK>, conv_smem<64, 64>());
  set((const void*)k_wgrad<16, 64>, wgrad_smem<16, 64>());
  set((const void*)k_wgrad<64, 64>, wgrad_smem<64, 64>());
  set((const void*)k_wgrad<64, 16>, wgrad_smem<64, 16>());
  return ok;
}

template <int CIN, int COUT, int EPI> static void conv(const SurrogateNet& n, ConvArgs a, cudaStream_t st) {
  const int tiles = (a.P + TM - 1) / TM;
  k_conv<CIN, COUT, EPI><<<tiles, NT, conv_smem<CIN, COUT>(), st>>>(a);
}

static ConvArgs cargs(const SurrogateNet& n, int P) {
  ConvArgs a{};
  a.N0 = n.N0; a.N1 = n.N1; a.C = n.C; a.P = P;
  return a;
}

// forward of a batch: x -> a1 -> a2 -> a3 -> y (fp32 [P][4]) or, with
// pcell, the kick coefficients; returns the launches
static int forward(SurrogateNet& n, const bf16* x, int B, float* y, float* pcell, float g1, float g2,
                   cudaStream_t st, bool allow_tc, uint32_t* status) {
  const int P = B * n.C;
  int launches = 0;
  // the inference path (allow_tc): every layer on tcgen05 (the per-tap
  // mma.sync kernels if a tensor map is refused); the training path: the
  // per-tap kernels the backward pass mirrors
  bool infer = allow_tc && n.tc;
  auto refused = [&]() {
    n.tc = false;
    n.err = "tensor map rejected; the tcgen05 path is off for this network";
  };
  ConvArgs a = cargs(n, P);
  a.x = x; a.w = n.w16 + SP_OFF_W1; a.bias = n.p32 + SP_OFF_B1; a.out = n.a1;
  int r1 = infer ? tc_conv16_relu(x, n.w16 + SP_OFF_W1, n.p32 + SP_OFF_B1, n.a1, n.N0, n.N1, P, n.num_sms, status, st)
                 : 0;
  if (r1 > 0) {
    launches += r1;
    n.tc_launches += r1;
  } else {
    if (infer) refused();
    infer = false;
    conv<16, 64, EPI_RELU>(n, a, st);
    ++launches;
  }
  for (int l = 0; l < 2; ++l) {
    const bf16* in = l == 0 ? n.a1 : n.a2;
    bf16* out = l == 0 ? n.a2 : n.a3;
    const int wo = l == 0 ? SP_OFF_W2 : SP_OFF_W3, bo = l == 0 ? SP_OFF_B2 : SP_OFF_B3;
    if (infer) {
      const int r = tc_conv64_relu(in, n.w16 + wo, n.p32 + bo, out, n.N0, n.N1, P, n.num_sms, status, st);
      if (r > 0) {
        launches += r;
        n.tc_launches += r;
        continue;
      }
      // the TMA descriptor was refused: this network stays on mma.sync
      refused();
      infer = false;
    }
    a = cargs(n, P);
    a.x = in; a.w = n.w16 + wo; a.bias = n.p32 + bo; a.out = out;
    conv<64, 64, EPI_RELU>(n, a, st);
    ++launches;
  }
  a = cargs(n, P);
  a.x = n.a3; a.w = n.w16 + SP_OFF_W4; a.bias = n.p32 + SP_OFF_B4;
  if (infer) {
    const int r = tc_conv_out(n.a3, n.w16 + SP_OFF_W4, n.p32 + SP_OFF_B4, y, pcell, g1, g2, (float)n.oscale, n.N0,
                              n.N1, P, n.num_sms, status, st);
    if (r > 0) {
      n.tc_launches += r;
      return launches + r;
    }
    refused();
  }
  if (pcell) {
    a.pcell = pcell; a.g1 = g1; a.g2 = g2; a.oscale = (float)n.oscale;
    conv<64, 16, EPI_KICK>(n, a, st);
  } else {
    a.out = y;
    conv<64, 16, EPI_OUT>(n, a, st);
  }
  return launches + 1;
}

template <int CIN, int COUT>
static void wgrad(SurrogateNet& n, const bf16* x, const bf16* dz, int P, float* grad_w, float* grad_b, cudaStream_t st) {
  WgArgs a{x, dz, n.part, n.N0, n.N1, n.C, P, (P + TM - 1) / TM};
  const int G = std::min(WG_G, a.ntiles);
  k_wgrad<CIN, COUT><<<dim3(G, 9), NT, wgrad_smem<CIN, COUT>(), st>>>(a);
  k_wgrad_reduce<<<gblocks(9L * CIN * COUT, 256, 1024), 256, 0, st>>>(n.part, G, CIN, COUT, grad_w);
  const int Gb = std::min(WG_G * 4, (P + 15) / 16);
  k_bias_part<<<Gb, NT, 0, st>>>(dz, P, COUT, n.partb);
  k_bias_reduce<<<1, 64, 0, st>>>(n.partb, Gb, COUT, grad_b);
}

// loss and gradients of all parameters for one batch: the forward and the
// data gradients on tcgen05 when the network's tensor path is on (the
// per-tap mma.sync kernels otherwise), the weight gradients on mma.sync
static void backward(SurrogateNet& n, const bf16* x, const float* t, int B, float ts, cudaStream_t st) {
  const int P = B * n.C;
  forward(n, x, B, n.y, nullptr, 0.f, 0.f, st, true, n.status);
  // dz_out = conv^T(dz_in) gated by the forward activation: tcgen05, else mma.sync
  auto dgrad = [&](int cin, const bf16* dz_in, const bf16* wf, const bf16* act, bf16* dz_out) {
    if (n.tc) {
      const int r = tc_conv_mask(cin, dz_in, wf, act, dz_out, n.N0, n.N1, P, n.num_sms, n.status, st);
      if (r > 0) {
        n.tc_launches += r;
        return;
      }
      n.tc = false;
      n.err = "tensor map rejected; the tcgen05 path is off for this network";
    }
    ConvArgs a = cargs(n, P);
    a.x = dz_in; a.w = wf; a.mask = act; a.out = dz_out;
    if (cin == 16) conv<16, 64, EPI_MASK>(n, a, st);
    else conv<64, 64, EPI_MASK>(n, a, st);
  };
  const int Gl = gblocks(P, NT, RED_G);
  k_loss<<<Gl, NT, 0, st>>>(n.y, t, ts, P, n.dz4, n.lpart);
  k_pair_reduce<<<1, 32, 0, st>>>(n.lpart, Gl, n.loss);
  // layer 4: dz4 -> dW4, db4; dz3 = (dz4 * W4^T) masked by a3
  wgrad<64, 16>(n, n.a3, n.dz4, P, n.grad + SP_OFF_W4, n.grad + SP_OFF_B4, st);
  dgrad(16, n.dz4, n.f16 + SF_OFF_F4, n.a3, n.dzA);
  // layer 3
  wgrad<64, 64>(n, n.a2, n.dzA, P, n.grad + SP_OFF_W3, n.grad + SP_OFF_B3, st);
  dgrad(64, n.dzA, n.f16 + SF_OFF_F3, n.a2, n.dzB);
  // layer 2
  wgrad<64, 64>(n, n.a1, n.dzB, P, n.grad + SP_OFF_W2, n.grad + SP_OFF_B2, st);
  dgrad(64, n.dzB, n.f16 + SF_OFF_F2, n.a1, n.dzA);
  // layer 1
  wgrad<16, 64>(n, x, n.dzA, P, n.grad + SP_OFF_W1, n.grad + SP_OFF_B1, st);
}

static void refresh_weights(SurrogateNet& n, cudaStream_t st, bool from_p32) {
  if (from_p32) k_to_bf16<<<gblocks(SP_NPARAM, 256, 512), 256, 0, st>>>(n.p32, n.w16, SP_NPARAM);
  k_flip<<<gblocks(16L * 9 * 64, 256, 512), 256, 0, st>>>(n.w16 + SP_OFF_W4, 16, 64, n.f16 + SF_OFF_F4);
  k_flip<<<gblocks(64L * 9 * 64, 256, 512), 256, 0, st>>>(n.w16 + SP_OFF_W3, 64, 64, n.f16 + SF_OFF_F3);
  k_flip<<<gblocks(64L * 9 * 64, 256, 512), 256, 0, st>>>(n.w16 + SP_OFF_W2, 64, 64, n.f16 + SF_OFF_F2);
}

// ------------------------------------------------ session-side launchers
// the network input of the session's cells: already written by the nodal
// deposit when it ran with the network attached, else packed here
static int sur_input(Session& s, const double* nnd, const double* ncell) {
  if (s.sur_xin_ready) return 0;
  k_input<<<gblocks(s.C, 256, s.num_sms * 8), 256, 0, s.stream>>>(nnd, ncell, s.k.b, s.C, s.sur->xin);
  return 1;
}

int sur_forward_kick(Session& s, const double* nnd, const double* ncell) {
  SurrogateNet& n = *s.sur;
  const double g1 = s.k.lr_coef / s.k.m / s.k.dx * s.k.dt, g2 = s.k.lr_coef / s.k.m / s.k.dy * s.k.dt;
  const int in = sur_input(s, nnd, ncell);
  return in + forward(n, n.xin, 1, nullptr, s.pcell, (float)g1, (float)g2, s.stream, true, s.status);
}

int sur_judge_forward(Session& s, const double* nnd, const double* ncell) {
  SurrogateNet& n = *s.sur;
  const int launches = sur_input(s, nnd, ncell);
  return launches + forward(n, n.xin, 1, n.y, nullptr, 0.f, 0.f, s.stream, true, s.status);
}

int sur_judge_compare(Session& s) {
  SurrogateNet& n = *s.sur;
  const double g1 = s.k.lr_coef / s.k.m / s.k.dx * s.k.dt, g2 = s.k.lr_coef / s.k.m / s.k.dy * s.k.dt;
  const int Gj = gblocks(s.C, NT, RED_G);
  k_judge<<<Gj, NT, 0, s.stream>>>(n.y, (float)n.oscale, (float)g1, (float)g2, s.pcell, s.C, n.lpart);
  k_pair_reduce<<<1, 32, 0, s.stream>>>(n.lpart, Gj, s.sur_err);
  return 2;
}

int sur_judge(Session& s, const double* nnd, const double* ncell) {
  const int launches = sur_judge_forward(s, nnd, ncell);
  return launches + sur_judge_compare(s);
}

int sur_snapshot(Session& s, const double* fld_dev, int K, uint64_t seed, uint32_t snap, int32_t* qc, double* nnd,
                 double* ncell, uint16_t* x, float* y) {
  const int cap = s.num_sms * 16;
  k_snap_counts<<<gblocks(4L * s.C, 256, cap), 256, 0, s.stream>>>(fld_dev, K, s.k, seed, snap, qc);
  k_cell_density<<<gblocks(s.C, 256, cap), 256, 0, s.stream>>>(qc, s.k, ncell);
  int launches = 2 + launch_node_density_from(s, qc);
  launches += launch_long_range_2d(s);
  k_input<<<gblocks(s.C, 256, cap), 256, 0, s.stream>>>(nnd, ncell, s.k.b, s.C, reinterpret_cast<bf16*>(x));
  k_target<<<gblocks(s.C, 256, cap), 256, 0, s.stream>>>(lr2d_potential(s), s.k.N0, s.C, y);
  return launches + 2;
}

}  // namespace mcpm

// ================================================================ C-ABI
using namespace mcpm;

struct mcpm_surrogate : public SurrogateNet {};

static int sfail(mcpm_surrogate* m, int code, const char* msg) {
  if (m) m->err = msg;
  return code;
}
static int scheck(mcpm_surrogate* m, cudaError_t e, const char* where) {
  if (e == cudaSuccess) return MCPM_OK;
  char buf[256];
  snprintf(buf, sizeof buf, "%s: %s", where, cudaGetErrorString(e));
  m->err = buf;
  return MCPM_ERR_CUDA;
}

namespace mcpm {
SurrogateNet* sur_net(mcpm_surrogate* m) { return m; }
}

// the device status word of the standalone calls (a bounded wait that ran out)
static int status_check(mcpm_surrogate* m) {
  uint32_t st = 0;
  cudaMemcpy(&st, m->status, 4, cudaMemcpyDeviceToHost);
  if (!st) return MCPM_OK;
  cudaMemset(m->status, 0, 4);
  m->err = "device status: a bounded wait of the tensor-core convolution ran out";
  return (int)st;
}

extern "C" {

int mcpm_surrogate_create(int32_t n0, int32_t n1, int32_t max_batch, mcpm_surrogate** out) {
  if (!out || n0 < 1 || n1 < 1 || max_batch < 1) return MCPM_ERR_ARG;
  *out = nullptr;
  const int64_t C = (int64_t)n0 * n1, P = C * max_batch;
  if (P > ((int64_t)1 << 30)) return MCPM_ERR_CAPACITY;
  mcpm_surrogate* m = new (std::nothrow) mcpm_surrogate();
  if (!m) return MCPM_ERR_CAPACITY;
  m->N0 = n0; m->N1 = n1; m->C = (int)C; m->maxB = max_batch; m->Pmax = P;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, dev);
  bool ok = set_smem_attrs();
  m->tc_ok = m->tc = tc_setup() == 0;
  auto A = [&](void** p, size_t bytes) { return ok && (ok = cudaMalloc(p, bytes) == cudaSuccess); };
  const size_t np = SP_NPARAM;
  A((void**)&m->p32, np * 4); A((void**)&m->m, np * 4); A((void**)&m->v, np * 4); A((void**)&m->grad, np * 4);
  A((void**)&m->w16, np * 2); A((void**)&m->f16, (size_t)SF_N * 2);
  A((void**)&m->xin, (size_t)P * 16 * 2);
  A((void**)&m->a1, (size_t)P * 64 * 2); A((void**)&m->a2, (size_t)P * 64 * 2); A((void**)&m->a3, (size_t)P * 64 * 2);
  A((void**)&m->dzA, (size_t)P * 64 * 2); A((void**)&m->dzB, (size_t)P * 64 * 2); A((void**)&m->dz4, (size_t)P * 16 * 2);
  A((void**)&m->y, (size_t)P * 4 * 4);
  A((void**)&m->part, (size_t)WG_G * 9 * 64 * 64 * 4); A((void**)&m->partb, (size_t)WG_G * 4 * 64 * 4);
  A((void**)&m->lpart, (size_t)RED_G * 2 * 8); A((void**)&m->loss, 2 * 8); A((void**)&m->status, 16);
  if (ok) ok = cudaMallocHost((void**)&m->loss_h, 2 * 8) == cudaSuccess;
  if (ok) ok = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) == cudaSuccess;
  if (ok) {
    cudaMemset(m->p32, 0, np * 4); cudaMemset(m->m, 0, np * 4); cudaMemset(m->v, 0, np * 4);
    cudaMemset(m->grad, 0, np * 4); cudaMemset(m->w16, 0, np * 2); cudaMemset(m->f16, 0, (size_t)SF_N * 2);
    cudaMemset(m->status, 0, 16);
    ok = cudaDeviceSynchronize() == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    mcpm_surrogate_destroy(m);
    return MCPM_ERR_CUDA;
  }
  *out = m;
  return MCPM_OK;
}

int mcpm_surrogate_destroy(mcpm_surrogate* m) {
  if (!m) return MCPM_OK;
  if (m->stream) cudaStreamSynchronize(m->stream);
  cudaFree(m->p32); cudaFree(m->m); cudaFree(m->v); cudaFree(m->grad); cudaFree(m->w16); cudaFree(m->f16);
  cudaFree(m->xin); cudaFree(m->a1); cudaFree(m->a2); cudaFree(m->a3); cudaFree(m->dzA); cudaFree(m->dzB);
  cudaFree(m->dz4); cudaFree(m->y); cudaFree(m->part); cudaFree(m->partb); cudaFree(m->lpart); cudaFree(m->loss);
  cudaFree(m->status);
  if (m->loss_h) cudaFreeHost(m->loss_h);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return MCPM_OK;
}

const char* mcpm_surrogate_last_error(const mcpm_surrogate* m) { return m ? m->err.c_str() : "null surrogate"; }

int mcpm_surrogate_set_params(mcpm_surrogate* m, const float* params, int64_t n, double out_scale) {
  if (!m || !params || n != SP_NPARAM || !(out_scale > 0.0)) return sfail(m, MCPM_ERR_ARG, "set_params: bad arguments");
  m->oscale = out_scale;
  cudaMemcpyAsync(m->p32, params, (size_t)n * 4, cudaMemcpyHostToDevice, m->stream);
  cudaMemsetAsync(m->m, 0, (size_t)n * 4, m->stream);
  cudaMemsetAsync(m->v, 0, (size_t)n * 4, m->stream);
  refresh_weights(*m, m->stream, true);
  return scheck(m, cudaStreamSynchronize(m->stream), "set_params");
}

int mcpm_surrogate_get_params(mcpm_surrogate* m, float* params, int64_t n) {
  if (!m || !params || n != SP_NPARAM) return sfail(m, MCPM_ERR_ARG, "get_params: bad arguments");
  cudaMemcpyAsync(params, m->p32, (size_t)n * 4, cudaMemcpyDeviceToHost, m->stream);
  return scheck(m, cudaStreamSynchronize(m->stream), "get_params");
}

int mcpm_surrogate_set_tensor_path(mcpm_surrogate* m, int32_t tcgen05) {
  if (!m) return MCPM_ERR_ARG;
  m->tc = tcgen05 != 0 && m->tc_ok;
  return MCPM_OK;
}

int mcpm_surrogate_launches(const mcpm_surrogate* m, int64_t* tcgen05_launches, int32_t* tcgen05_on) {
  if (!m) return MCPM_ERR_ARG;
  if (tcgen05_launches) *tcgen05_launches = m->tc_launches;
  if (tcgen05_on) *tcgen05_on = m->tc ? 1 : 0;
  return MCPM_OK;
}

int mcpm_surrogate_forward(mcpm_surrogate* m, const uint16_t* x, int32_t batch, float* y) {
  if (!m || !x || !y || batch < 1 || batch > m->maxB) return sfail(m, MCPM_ERR_ARG, "forward: bad arguments");
  forward(*m, reinterpret_cast<const bf16*>(x), batch, y, nullptr, 0.f, 0.f, m->stream, true, m->status);
  if (cudaError_t e = cudaGetLastError()) return scheck(m, e, "forward");
  int rc = scheck(m, cudaStreamSynchronize(m->stream), "forward");
  return rc ? rc : status_check(m);
}

int mcpm_surrogate_gradients(mcpm_surrogate* m, const uint16_t* x, const float* target, int32_t batch,
                             double target_scale, float* grad, double* loss) {
  if (!m || !x || !target || batch < 1 || batch > m->maxB) return sfail(m, MCPM_ERR_ARG, "gradients: bad arguments");
  backward(*m, reinterpret_cast<const bf16*>(x), target, batch, (float)target_scale, m->stream);
  if (cudaError_t e = cudaGetLastError()) return scheck(m, e, "gradients");
  if (grad) cudaMemcpyAsync(grad, m->grad, (size_t)SP_NPARAM * 4, cudaMemcpyDeviceToHost, m->stream);
  if (loss) cudaMemcpyAsync(loss, m->loss, 16, cudaMemcpyDeviceToHost, m->stream);
  return scheck(m, cudaStreamSynchronize(m->stream), "gradients");
}

int mcpm_surrogate_train_step(mcpm_surrogate* m, const uint16_t* x, const float* target, int32_t batch,
                              double target_scale, double lr, int32_t t, double* loss) {
  if (!m || !x || !target || batch < 1 || batch > m->maxB || t < 1 || !(lr > 0.0))
    return sfail(m, MCPM_ERR_ARG, "train_step: bad arguments");
  backward(*m, reinterpret_cast<const bf16*>(x), target, batch, (float)target_scale, m->stream);
  const double b1 = 0.9, b2 = 0.999;
  k_adam<<<gblocks(SP_NPARAM, 256, 1024), 256, 0, m->stream>>>(m->p32, m->m, m->v, m->grad, m->w16, SP_NPARAM,
                                                               (float)lr, (float)b1, (float)b2, 1e-8f,
                                                               (float)(1.0 - pow(b1, t)), (float)(1.0 - pow(b2, t)));
  refresh_weights(*m, m->stream, false);
  if (cudaError_t e = cudaGetLastError()) return scheck(m, e, "train_step");
  if (loss) {
    cudaMemcpyAsync(m->loss_h, m->loss, 16, cudaMemcpyDeviceToHost, m->stream);
    int rc = scheck(m, cudaStreamSynchronize(m->stream), "train_step");
    loss[0] = m->loss_h[0];
    loss[1] = m->loss_h[1];
    return rc;
  }
  return MCPM_OK;
}

int mcpm_surrogate_sync(mcpm_surrogate* m) {
  if (!m) return MCPM_ERR_ARG;
  return scheck(m, cudaStreamSynchronize(m->stream), "sync");
}

}  // extern "C"
