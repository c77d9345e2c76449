// mcpm_surrogate_tc.cu -- the 3x3 convolutions of the learned Vlasov force's
// inference on the fifth-generation tensor cores (tcgen05): the 16 -> 64
// input layer, the two 64 -> 64 layers and the 64 -> 16 output layer.
//
// Implicit GEMM per output tile of 128 consecutive cells of one grid row
// (M = 128) and all COUT output channels (N = COUT), reduced over 9 taps x
// CIN input channels (K = 9 CIN):
//   * the activations are an NHWC bf16 tensor [B][N1][N0][CIN]; the tile of
//     tap (dy, dx) is one TMA box {CIN ch, 128 cells, 1, 1} at (0, x0 + dx,
//     y + dy, b) -- boxes reaching past the grid are zero-filled by the TMA
//     unit, which is the convolution's zero padding;
//   * the 9 weight tiles [COUT co][CIN ci] stay in shared memory for the
//     life of the persistent block;
//   * both operands land with the swizzle that the K-major UMMA
//     shared-memory descriptor reads (rows of 2 CIN bytes: the 128-byte
//     swizzle for CIN = 64, the 32-byte one for CIN = 16); each tap issues
//     CIN / 16 tcgen05.mma of K = 16 into an fp32 accumulator of COUT TMEM
//     columns;
//   * two accumulators alternate so that the epilogue of one tile (TMEM ->
//     registers, + bias, then ReLU to bf16, or the output layer's kick
//     coefficients into the packed cell record, or its four outputs)
//     overlaps the MMAs of the next.
// Warp roles (6 warps): warp 0 issues the TMA loads, warp 1 allocates TMEM
// and issues the MMAs, warps 2-5 drain the accumulators (warp w reads TMEM
// lanes 32 (w % 4) .. 32 (w % 4) + 31).  Every mbarrier wait is bounded
// (1 s by the global timer): a wait that runs out raises
// MCPM_ERR_ITER_LIMIT in the status word, every role stops, the block waits
// (bounded) for its own copies and MMAs in flight, frees its TMEM and exits.
#include <cuda.h>
#include <cuda_bf16.h>

#include <cstdint>
#include <cstring>

#include "../../include/mcpm.h"
#include "mcpm_internal.h"
#include "mcpm_surrogate.h"

namespace mcpm {
namespace tc {

constexpr int TM = 128, NTHREADS = 192, MAXSTAGE = 16;
constexpr uint64_t WAIT_NS = 1000000000ull;    // bound of every wait
// epilogues: bias + ReLU to bf16 activations; the output layer's kick
// coefficients into the packed cell record; its four outputs as fp32
// (inference); and, for training, the data gradient of a layer input: the
// accumulator gated by the sign of the layer's forward activation
enum { TEPI_RELU = 0, TEPI_KICK = 1, TEPI_OUT = 2, TEPI_MASK = 3 };

// the shape of one layer: rows of RB = 2 CIN bytes
template <int CIN, int COUT> struct Cfg {
  static_assert(CIN == 16 || CIN == 64, "input rows of 32 or 128 bytes");
  static_assert(COUT % 16 == 0 && COUT >= 16 && COUT <= 256, "UMMA N for M = 128");
  static constexpr int RB = 2 * CIN;
  // a stage holds one grid row of the tile with its left and right halo
  // cells (TM + 2 rows of RB bytes), and the MMAs read its three column
  // shifts at one-row offsets: a tile takes three boxes, one per grid row.
  // Stages in flight (three tiles of the input layer's 4 KB boxes, two of
  // the 17 KB ones) and persistent blocks per SM: the narrow layers' MMAs
  // are short, so several blocks per SM overlap their load latencies
  // (shared memory and TMEM allow it: 3 x 65 KB and 3 x 128 columns,
  // 2 x 88 KB and 2 x 32 columns; the 64 -> 64 layer 1 x 176 KB)
  static constexpr int NSTAGE = CIN == 16 ? 9 : (COUT == 16 ? 4 : 6);
  static constexpr int CTAS_PER_SM = CIN == 16 ? 3 : (COUT == 16 ? 2 : 1);
  static_assert(NSTAGE <= MAXSTAGE, "barrier slots");
  static constexpr int BOX_ROWS = TM + 2;              // cells per activation box
  static constexpr int A_BYTES = BOX_ROWS * RB;        // one activation box
  static constexpr int A_STRIDE = (A_BYTES + 1023) / 1024 * 1024;  // stages on swizzle-pattern boundaries
  static constexpr int B_BYTES = COUT * RB;            // one tap of the weights
  static constexpr int SMEM_B = 0;                     // 9 weight taps
  static constexpr int SMEM_A = SMEM_B + 9 * B_BYTES;  // NSTAGE activation stages
  static constexpr int SMEM_BAR = SMEM_A + NSTAGE * A_STRIDE;
  static constexpr int SMEM_BYTES = SMEM_BAR + 512 + 1024;  // barriers + alignment slack
  static_assert(SMEM_BYTES <= 227 * 1024, "shared memory per block");
  static constexpr uint32_t TMEM_COLS = 2 * COUT < 32 ? 32u : (uint32_t)(2 * COUT);  // two accumulators
  static constexpr int KSTEPS = CIN / 16;
  // descriptor layout type: SWIZZLE_128B (2) or SWIZZLE_32B (6); the stride
  // between 8-row groups is 8 rows
  static constexpr uint64_t LAYOUT = CIN == 64 ? 2 : 6;
  static constexpr uint32_t SBO = 8 * RB;
  static_assert(SMEM_A % 1024 == 0 && A_STRIDE % 1024 == 0 && B_BYTES % 256 == 0, "swizzle atoms aligned");
  static_assert(CIN == 16 || B_BYTES % 1024 == 0, "128-byte swizzle atoms aligned");
};

struct Bars {
  uint64_t full[MAXSTAGE], empty[MAXSTAGE], acc_full[2], acc_empty[2], wbar, done;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t n) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(n) : "memory");
}
__device__ __forceinline__ void bar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool bar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// waits for the phase of the given parity to complete; false if the block
// is aborting or the wait ran out (which starts the abort)
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity, volatile int* abort, uint32_t* status,
                                         bool heed_abort = true) {
  if (bar_try(b, parity)) return true;
  const uint64_t t0 = gtimer();
  while (true) {
    if (bar_try(b, parity)) return true;
    if (heed_abort && *abort) return false;
    if (gtimer() - t0 > WAIT_NS) {
      *abort = 1;
      atomicOr(status, (uint32_t)MCPM_ERR_ITER_LIMIT);
      return false;
    }
  }
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(su32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(su32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          su32(dst)),
      "l"((uint64_t)map), "r"(c0), "r"(c1), "r"(su32(bar))
      : "memory");
}
// K-major operand: rows of 2 CIN bytes swizzled at that width, 8-row
// groups SBO bytes apart (stride byte offset), descriptor version 1
// (an operand may start a whole number of rows into a stage: the swizzle
// follows the shared-memory address, so the one-row shifts of a box read
// with the matrix base offset left at 0 -- measured: bit-identical to the
// mma.sync path, while the base offset set to the row gives garbage)
template <int CIN, int COUT> __device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)1 << 16;                               // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(Cfg<CIN, COUT>::SBO >> 4) << 32;      // stride byte offset
  d |= (uint64_t)1 << 46;                               // version
  d |= Cfg<CIN, COUT>::LAYOUT << 61;                    // swizzle mode
  return d;
}
// kind::f16 instruction descriptor: fp32 accumulator, bf16 A and B, both
// K-major, N = COUT, M = 128
template <int COUT> __device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t acc) {
  constexpr uint32_t IDESC =
      (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(COUT >> 3) << 17) | ((uint32_t)(TM >> 4) << 24);
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
          d_tmem),
      "l"(a), "l"(b), "r"(IDESC), "r"(acc)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

struct Args {
  const float* bias;        // [COUT]
  void* out;                // bf16 [P][COUT] (TEPI_RELU, TEPI_MASK), fp32 [P][4] (TEPI_OUT)
  const __nv_bfloat16* mask;  // [P][COUT] forward activations gating the gradient (TEPI_MASK)
  float* pcell;             // packed per-cell record (TEPI_KICK)
  uint32_t* status;
  int N0, N1, rows, tiles_per_row, ntiles;  // rows = B N1
  float g1, g2, oscale;                     // TEPI_KICK
};

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(NTHREADS, 1)
    k_conv_tc(const __grid_constant__ CUtensorMap tmx, const __grid_constant__ CUtensorMap tmw, Args a) {
  using L = Cfg<CIN, COUT>;
  constexpr int A_BYTES = L::A_BYTES, B_BYTES = L::B_BYTES, SMEM_A = L::SMEM_A, SMEM_B = L::SMEM_B,
                SMEM_BAR = L::SMEM_BAR;
  constexpr uint32_t TMEM_COLS = L::TMEM_COLS;
  constexpr int NSTAGE = L::NSTAGE;
  static_assert(sizeof(Bars) <= 512, "barrier block");
  static_assert((EPI == TEPI_RELU || EPI == TEPI_MASK) ? COUT == 64 : COUT == 16, "epilogue shapes");
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  Bars* bars = reinterpret_cast<Bars*>(smem + SMEM_BAR);
  volatile int* abort = &bars->abort;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int s = 0; s < NSTAGE; ++s) { bar_init(&bars->full[s], 1); bar_init(&bars->empty[s], 1); }
    for (int b = 0; b < 2; ++b) { bar_init(&bars->acc_full[b], 1); bar_init(&bars->acc_empty[b], 4); }
    bar_init(&bars->wbar, 1);
    bar_init(&bars->done, 1);
    bars->abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&bars->tmem_base)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = bars->tmem_base;
  // programmatic dependent launch: the next layer's blocks may start their
  // set-up (barriers, TMEM, weights) while this layer finishes; each block
  // reads the previous kernel's output only after griddepcontrol.wait (a
  // kernel launched without the attribute passes it at once)
  if (threadIdx.x == 0) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");

  if (warp == 0) {
    if (lane == 0) {
      // producer: the weights once, then one activation box per tap
      asm volatile("prefetch.tensormap [%0];" ::"l"((uint64_t)&tmx) : "memory");
      bar_expect_tx(&bars->wbar, 9 * B_BYTES);
      for (int t = 0; t < 9; ++t) tma_load_2d(smem + SMEM_B + t * B_BYTES, &tmw, t * CIN, 0, &bars->wbar);
      asm volatile("griddepcontrol.wait;" ::: "memory");  // the activations are the previous kernel's output
      int last_par[NSTAGE];
      for (int s = 0; s < NSTAGE; ++s) last_par[s] = -1;
      uint32_t i = 0;
      bool ok = true;
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x) {
        const int row = tile / a.tiles_per_row, x0 = (tile - row * a.tiles_per_row) * TM;
        const int b = row / a.N1, y = row - b * a.N1;
        for (int dy = 0; dy < 3; ++dy, ++i) {
          const int s = i % NSTAGE;
          const uint32_t ph = (i / NSTAGE) & 1;
          if (!(ok = bar_wait(&bars->empty[s], ph ^ 1, abort, a.status))) break;
          bar_expect_tx(&bars->full[s], A_BYTES);
          // cells x0-1 .. x0+128 of grid row y+dy-1 (outside the grid: zeros)
          tma_load_4d(smem + SMEM_A + s * L::A_STRIDE, &tmx, 0, x0 - 1, y + dy - 1, b, &bars->full[s]);
          last_par[s] = (int)ph;
        }
      }
      // our own copies in flight land before the block exits
      bar_wait(&bars->wbar, 0, abort, a.status, false);
      for (int s = 0; s < NSTAGE; ++s)
        if (last_par[s] >= 0) bar_wait(&bars->full[s], (uint32_t)last_par[s], abort, a.status, false);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMA issuer
      bool ok = bar_wait(&bars->wbar, 0, abort, a.status);
      fence_after();
      uint32_t i = 0, j = 0;
      const uint32_t sa = su32(smem + SMEM_A), sb = su32(smem + SMEM_B);
      for (int tile = blockIdx.x; tile < a.ntiles && ok; tile += gridDim.x, ++j) {
        const uint32_t buf = j & 1, aph = (j >> 1) & 1;
        if (!(ok = bar_wait(&bars->acc_empty[buf], aph ^ 1, abort, a.status))) break;
        fence_after();
        const uint32_t d = tmem + buf * COUT;
        for (int dy = 0; dy < 3; ++dy, ++i) {
          const int s = i % NSTAGE;
          if (!(ok = bar_wait(&bars->full[s], (i / NSTAGE) & 1, abort, a.status))) break;
          fence_after();
          // taps 3 dy + dx: the box's rows dx .. dx + 127 (the cells x0+dx-1 ..)
#pragma unroll
          for (int dx = 0; dx < 3; ++dx) {
            const int tap = 3 * dy + dx;
#pragma unroll
            for (int kk = 0; kk < L::KSTEPS; ++kk)
              mma_bf16<COUT>(d, sdesc<CIN, COUT>(sa + s * L::A_STRIDE + dx * L::RB + kk * 32),
                             sdesc<CIN, COUT>(sb + tap * B_BYTES + kk * 32), (tap | kk) != 0 ? 1u : 0u);
          }
          mma_commit(&bars->empty[s]);  // the stage is free once these MMAs have read it
        }
        if (!ok) break;
        mma_commit(&bars->acc_full[buf]);
      }
      // every MMA issued here has completed before the block exits
      mma_commit(&bars->done);
      bar_wait(&bars->done, 0, abort, a.status, false);
    }
  } else {
    // epilogue: warp w drains TMEM lanes 32 (w % 4) .. + 31 = tile rows
    const int q = warp & 3;
    uint32_t j = 0;
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the outputs may be what the previous kernel reads
    for (int tile = blockIdx.x; tile < a.ntiles; tile += gridDim.x, ++j) {
      const uint32_t buf = j & 1, aph = (j >> 1) & 1;
      if (!bar_wait(&bars->acc_full[buf], aph, abort, a.status)) break;
      __syncwarp();
      fence_after();
      constexpr int NC = COUT / 16;
      uint32_t r[NC][16];
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + buf * COUT;
#pragma unroll
      for (int c = 0; c < NC; ++c) tmem_ld16(taddr + c * 16, r[c]);
      tmem_wait_ld();
      fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(&bars->acc_empty[buf]);
      const int row = tile / a.tiles_per_row, x0 = (tile - row * a.tiles_per_row) * TM;
      const int x = x0 + 32 * q + lane;
      if (x < a.N0) {
        const size_t p = (size_t)row * a.N0 + x;
        if constexpr (EPI == TEPI_MASK) {
          uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(a.out) + p * COUT);
          const uint4* mk = reinterpret_cast<const uint4*>(a.mask + p * COUT);
#pragma unroll
          for (int c = 0; c < NC; ++c) {
#pragma unroll
            for (int hq = 0; hq < 2; ++hq) {
              const uint4 m4 = mk[2 * c + hq];
              const __nv_bfloat162* m2 = reinterpret_cast<const __nv_bfloat162*>(&m4);
              __nv_bfloat162 h[4];
#pragma unroll
              for (int e = 0; e < 4; ++e) {
                const int k = 8 * hq + 2 * e;
                const float v0 = __bfloat162float(m2[e].x) > 0.f ? __uint_as_float(r[c][k]) : 0.f;
                const float v1 = __bfloat162float(m2[e].y) > 0.f ? __uint_as_float(r[c][k + 1]) : 0.f;
                h[e] = __floats2bfloat162_rn(v0, v1);
              }
              o[2 * c + hq] = *reinterpret_cast<uint4*>(&h[0]);
            }
          }
        } else if constexpr (EPI == TEPI_RELU) {
          uint4* o = reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(a.out) + p * COUT);
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            __nv_bfloat162 h[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) {
              const float v0 = fmaxf(__uint_as_float(r[c][2 * e]) + a.bias[c * 16 + 2 * e], 0.f);
              const float v1 = fmaxf(__uint_as_float(r[c][2 * e + 1]) + a.bias[c * 16 + 2 * e + 1], 0.f);
              h[e] = __floats2bfloat162_rn(v0, v1);
            }
            o[2 * c] = *reinterpret_cast<uint4*>(&h[0]);
            o[2 * c + 1] = *reinterpret_cast<uint4*>(&h[4]);
          }
        } else {
          // outputs 0..3: the differences of the cell's corner potentials
          const float o0 = __uint_as_float(r[0][0]) + a.bias[0], o1 = __uint_as_float(r[0][1]) + a.bias[1];
          const float o2 = __uint_as_float(r[0][2]) + a.bias[2], o3 = __uint_as_float(r[0][3]) + a.bias[3];
          if constexpr (EPI == TEPI_KICK) {
            const float d0 = o0 * a.oscale, d1 = o1 * a.oscale, d2 = o2 * a.oscale, d3 = o3 * a.oscale;
            *reinterpret_cast<float4*>(a.pcell + p * PF_STRIDE + PF_LA1) =
                make_float4(d0 * a.g1, (d1 - d0) * a.g1, d2 * a.g2, (d3 - d2) * a.g2);
          } else {
            *reinterpret_cast<float4*>(static_cast<float*>(a.out) + p * 4) = make_float4(o0, o1, o2, o3);
          }
        }
      }
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  if (warp == 1)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
}

typedef CUresult (*EncodeTiled)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiled g_encode = nullptr;

}  // namespace tc

namespace tc {
template <int CIN, int COUT, int EPI> static int set_smem() {
  return cudaFuncSetAttribute(k_conv_tc<CIN, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              Cfg<CIN, COUT>::SMEM_BYTES) == cudaSuccess
             ? 0
             : 1;
}

// the activation map [B][N1][N0][CIN] read as boxes {CIN, 130, 1, 1} (a
// grid row of the tile with its halo cells), and the
// weights [COUT][9 CIN] as boxes {CIN, COUT} (one tap), both swizzled as the
// UMMA descriptors read them
template <int CIN, int COUT>
static bool maps(const void* x, const void* w, int N0, int N1, int B, CUtensorMap& mx, CUtensorMap& mw) {
  const CUtensorMapSwizzle sw = CIN == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_32B;
  const cuuint64_t rb = 2 * CIN;
  cuuint64_t dims[4] = {(cuuint64_t)CIN, (cuuint64_t)N0, (cuuint64_t)N1, (cuuint64_t)B};
  cuuint64_t strides[3] = {rb, (cuuint64_t)N0 * rb, (cuuint64_t)N0 * N1 * rb};
  cuuint32_t box[4] = {(cuuint32_t)CIN, (cuuint32_t)Cfg<CIN, COUT>::BOX_ROWS, 1, 1}, es[4] = {1, 1, 1, 1};
  if (g_encode(&mx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(x), dims, strides, box, es,
               CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
    return false;
  cuuint64_t wd[2] = {(cuuint64_t)(9 * CIN), (cuuint64_t)COUT};
  cuuint64_t ws[1] = {(cuuint64_t)(9 * CIN * 2)};
  cuuint32_t wb[2] = {(cuuint32_t)CIN, (cuuint32_t)COUT}, we[2] = {1, 1};
  return g_encode(&mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(w), wd, ws, wb, we,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// one layer over P cells (whole grid rows of N0 cells); returns the launches,
// -1 if a tensor map was refused
template <int CIN, int COUT, int EPI>
static int launch(const __nv_bfloat16* x, const __nv_bfloat16* w, Args a, int P, int num_sms, cudaStream_t st) {
  if (!g_encode || P <= 0) return 0;
  const int rows = P / a.N0, B = rows / a.N1;
  CUtensorMap mx, mw;
  if (!maps<CIN, COUT>(x, w, a.N0, a.N1, B, mx, mw)) return -1;
  a.rows = rows;
  a.tiles_per_row = (a.N0 + TM - 1) / TM;
  a.ntiles = rows * a.tiles_per_row;
  const int slots = num_sms * Cfg<CIN, COUT>::CTAS_PER_SM;
  const int grid = a.ntiles < slots ? a.ntiles : slots;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(NTHREADS);
  cfg.dynamicSmemBytes = Cfg<CIN, COUT>::SMEM_BYTES;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (cudaLaunchKernelEx(&cfg, k_conv_tc<CIN, COUT, EPI>, mx, mw, a) != cudaSuccess) {
    cudaGetLastError();
    return -1;
  }
  return 1;
}
}  // namespace tc

int tc_setup() {
  using namespace tc;
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      cudaGetLastError();
      return 1;
    }
    g_encode = (EncodeTiled)fn;
  }
  if (set_smem<64, 64, TEPI_RELU>() | set_smem<16, 64, TEPI_RELU>() | set_smem<64, 16, TEPI_KICK>() |
      set_smem<64, 16, TEPI_OUT>() | set_smem<64, 64, TEPI_MASK>() | set_smem<16, 64, TEPI_MASK>()) {
    cudaGetLastError();
    return 1;
  }
  return 0;
}

static tc::Args base_args(const float* bias, int N0, int N1, uint32_t* status) {
  tc::Args a;
  std::memset(&a, 0, sizeof a);
  a.bias = bias;
  a.status = status;
  a.N0 = N0;
  a.N1 = N1;
  return a;
}

int tc_conv64_relu(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* out, int N0,
                   int N1, int P, int num_sms, uint32_t* status, cudaStream_t st) {
  tc::Args a = base_args(bias, N0, N1, status);
  a.out = out;
  return tc::launch<64, 64, tc::TEPI_RELU>(x, w, a, P, num_sms, st);
}

int tc_conv16_relu(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* out, int N0,
                   int N1, int P, int num_sms, uint32_t* status, cudaStream_t st) {
  tc::Args a = base_args(bias, N0, N1, status);
  a.out = out;
  return tc::launch<16, 64, tc::TEPI_RELU>(x, w, a, P, num_sms, st);
}

int tc_conv_mask(int cin, const __nv_bfloat16* x, const __nv_bfloat16* w, const __nv_bfloat16* mask,
                 __nv_bfloat16* out, int N0, int N1, int P, int num_sms, uint32_t* status, cudaStream_t st) {
  tc::Args a = base_args(nullptr, N0, N1, status);
  a.out = out;
  a.mask = mask;
  if (cin == 16) return tc::launch<16, 64, tc::TEPI_MASK>(x, w, a, P, num_sms, st);
  if (cin == 64) return tc::launch<64, 64, tc::TEPI_MASK>(x, w, a, P, num_sms, st);
  return -1;
}

int tc_conv_out(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, float* y, float* pcell, float g1,
                float g2, float oscale, int N0, int N1, int P, int num_sms, uint32_t* status, cudaStream_t st) {
  tc::Args a = base_args(bias, N0, N1, status);
  if (pcell) {
    a.pcell = pcell;
    a.g1 = g1;
    a.g2 = g2;
    a.oscale = oscale;
    return tc::launch<64, 16, tc::TEPI_KICK>(x, w, a, P, num_sms, st);
  }
  a.out = y;
  return tc::launch<64, 16, tc::TEPI_OUT>(x, w, a, P, num_sms, st);
}

}  // namespace mcpm
