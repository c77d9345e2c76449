// mcpm_lr2d.cu -- the Vlasov force of a 2-D box on the node grid.
//
// Reference: compute_Vlasov_2D (src/FEM.cpp:613-726, long_range 1) and
// compute_SP_2D (src/FEM.cpp:249-610, long_range 3), reached from
// velocity_update (src/Main_Functions.cpp:1618-1663), with the nodal
// deposit n_n of cell_update (src/Main_Functions.cpp:2268-2364).
//
// Node (i, j), 0 <= i <= N0, 0 <= j <= N1, has id j (N0 + 1) + i and sits at
// the corner of the cells around it; its coordinates are the ones make_cells
// gives the cell corners (src/myIO.cpp:1456-1479), which are separable:
// xx_i depends on the column only, yy_j on the row only.
//
// Both paths integrate the cell density n(x) over a sphere around a point by
// a GL(q)^3 product rule in (r, phi, theta), looking up the cell of each
// point with the box edges clamped.  Seen from any node the point with
// offset (r cos phi sin theta, r sin phi sin theta) lands in the cell at a
// fixed offset (dj, dk) from the node, except for points whose offset lies
// within rounding distance of a cell face; so the integral is a fixed stencil
// of per-offset weight sums, W[dk][dj], applied to the clamped densities.
// The set-up checks every point whose offset is that close to a face against
// each row and column the exact way the reference computes it, and records
// per node the points whose cell differs (corrections the node kernels add).
//
// direct (long_range 1): V(node) = sum W n over GL(100)^3, r in [sigma,
//   3 sigma], weight (sigma/r)^6 r^2 dr dphi sin(theta) dtheta.
// screened Poisson (long_range 3): bilinear FEM of -lap V + bst^2 V = n_n on
//   the node grid with Dirichlet rows on the walls holding the Green's-
//   function potential (GL(50)^3, r in [0, 3 sigma], weight exp(-bst r)/(4 pi)
//   r dr ...).  The interior operator is K (x) M + M (x) K + bst^2 vol M (x) M
//   of the 1-D unit stiffness K = tridiag(-1, 2, -1) and mass
//   M = tridiag(1/6, 2/3, 1/6) -- the reference assembles exactly these
//   element matrices (src/FEM.cpp:50-106) -- so it is diagonalised by the
//   discrete sine transform: U = S_y ((S_y B S_x) / mu) S_x with the
//   orthonormal DST-I matrices S and mu_qp = kx_p my_q + mx_p ky_q +
//   bst^2 vol mx_p my_q.  The reference solves the same system with PARDISO.
//   The operator's condition number is about 2 (mu lies in [~3.3, ~5.5] for
//   bst ~ 2.3 and unit cells), so the transforms run in FP32 and the solution
//   is accumulated in FP64 by iterative refinement: U += solve32(b - L U),
//   with the residual of the 9-point operator taken in FP64; each pass gains
//   ~6 digits.
//   Then the analytic near-field part is subtracted (src/FEM.cpp:491-546).
// The kick (src/FEM.cpp:567-578, :703-714): U -= grad_bilinear(V) coef / m dt
// with coef = phi (direct) or ast (screened Poisson), applied by the particle
// pass (update kernel) from the node values (FP64) or from per-cell
// coefficients packed here (FP32).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "mcpm_device.cuh"
#include "mcpm_surrogate.h"

namespace mcpm {

#define FULL 0xffffffffu

struct LR2D {
  int mode;                 // MCPM_LR_DIRECT or MCPM_LR_SCREENED_POISSON
  int N0, N1, nn, nx, ny;   // cells per row / column, nodes, interior nodes per row / column
  int R0lo, R0hi, R1lo, R1hi;  // stencil offsets dj in [R0lo, R0hi], dk in [R1lo, R1hi]
  int sw;                   // stencil width R0hi - R0lo + 1
  int n_exc;
  double* W = nullptr;      // stencil [R1hi - R1lo + 1][sw]
  int* exc_off = nullptr;   // [nn + 1] per-node range of correction points
  int* exc_i = nullptr;     // [n_exc][4]: dj, dk the point's cell, dj, dk the stencil's
  double* exc_w = nullptr;  // [n_exc]
  double* V = nullptr;      // [nn] node potential
  double* nnd = nullptr;    // [C][4] nodal densities n_n
  double* ncell = nullptr;  // [C] cell densities from the layout's counts (the per-cell solve's values)
  double* vol = nullptr;    // [C] cell volumes, cell_volume() formed once at set-up
  int32_t* qc = nullptr;    // [C][4] particles per cell quadrant
  float *Sx = nullptr, *Sy = nullptr, *mu = nullptr, *Bf = nullptr, *Tf = nullptr;  // FP32 transforms
  double *B = nullptr, *U = nullptr;  // FP64 right-hand side and solution (interior, rows y)
  double lambda2vol;                  // bst^2 vol, the mass coefficient of the operator
  double near1, near2;                // the near-field constants of src/FEM.cpp:491-496
  int iters;                          // refinement passes
  float *qtx = nullptr, *qty = nullptr;  // [N0], [N1] cell-centre thresholds (smallest float >= centre)
  int* wall = nullptr;      // [n_wall] ids of the wall nodes
  int n_wall;
  size_t smem;              // dynamic shared memory of the node kernels
};

// ------------------------------------------------------------ geometry --
// the corner coordinate of column i (row j) as make_cells builds the cells
// (cells[num].x_n, src/myIO.cpp:1472-1479), from the cell left of / right of it
__host__ __device__ inline double node_coord(int i, int N, double d) {
  const int c = i < N ? i : N - 1;
  double d0 = (double)c * d, d1 = (double)(c + 1) * d;
  double dc = d1 - d0, cen = 0.5 * (d0 + d1);
  return i < N ? cen - dc / 2.0 : cen + dc / 2.0;
}
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ------------------------------------------------------------- kernels --
// quadrant counts of cell_update's nodal deposit: particle on the left of
// the cell centre and below it -> 0, right/below 1, left/above 2, right/above 3
template <typename real>
__global__ void k_quadrants(DevConsts k, const int32_t* off, const int32_t* cnt, const real* x1, const real* x2,
                            int32_t* qc) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < k.C; c += warps) {
    const int j = c % k.N0, kk = c / k.N0;
    const double cx = 0.5 * ((double)j * k.dx + (double)(j + 1) * k.dx);
    const double cy = 0.5 * ((double)kk * k.dy + (double)(kk + 1) * k.dy);
    // x < cx in exact arithmetic, compared in the state's precision: for
    // float x, x < cx  <=>  x < the smallest float >= cx
    real tx, ty;
    if constexpr (sizeof(real) == 4) {
      float fx = (float)cx, fy = (float)cy;
      tx = (double)fx >= cx ? fx : nextafterf(fx, INFINITY);
      ty = (double)fy >= cy ? fy : nextafterf(fy, INFINITY);
    } else {
      tx = cx; ty = cy;
    }
    const int64_t s0 = off[c];
    const int n = cnt[c];
    int q[4] = {0, 0, 0, 0};
    for (int i = lane; i - lane < n; i += 32) {
      int quad = -1;
      if (i < n) quad = (x1[s0 + i] < tx ? 0 : 1) + (x2[s0 + i] < ty ? 0 : 2);
#pragma unroll
      for (int t = 0; t < 4; ++t) q[t] += __popc(__ballot_sync(FULL, quad == t));
    }
    if (lane < 4) qc[(size_t)c * 4 + lane] = q[lane];
  }
}

// The FP32 sessions' quadrant counts: the same comparison against the
// cell-centre thresholds (the smallest float at or above each centre),
// four particles per lane in flight and the counts summed by warp
// reductions.
__global__ void k_quadrants_f32(DevConsts k, const int32_t* off, const int32_t* cnt, const float* x1, const float* x2,
                                const float* qtx, const float* qty, int32_t* qc) {
  const int lane = threadIdx.x & 31;
  const int warps = (gridDim.x * blockDim.x) >> 5;
  for (int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < k.C; c += warps) {
    const float tx = qtx[c % k.N0], ty = qty[c / k.N0];
    const int64_t s0 = off[c];
    const int n = cnt[c];
    int q1 = 0, q2 = 0, q3 = 0, m = 0;
    for (int i = lane; i < n; i += 128) {
      float a[4], b[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool in = i + 32 * u < n;
        a[u] = in ? x1[s0 + i + 32 * u] : 0.f;
        b[u] = in ? x2[s0 + i + 32 * u] : 0.f;
        if (in) {
          const int q = (a[u] < tx ? 0 : 1) + (b[u] < ty ? 0 : 2);
          q1 += q == 1; q2 += q == 2; q3 += q == 3;
          ++m;
        }
      }
    }
    q1 = __reduce_add_sync(0xffffffffu, q1);
    q2 = __reduce_add_sync(0xffffffffu, q2);
    q3 = __reduce_add_sync(0xffffffffu, q3);
    m = __reduce_add_sync(0xffffffffu, m);
    if (lane == 0) *reinterpret_cast<int4*>(qc + (size_t)c * 4) = make_int4(m - q1 - q2 - q3, q1, q2, q3);
  }
}

// n_n[c][slot]: the particles nearest to the slot's node, counted over every
// cell sharing the node, each adding Fn/volume(c); wall nodes doubled per
// wall (src/Main_Functions.cpp:2268-2364).  exact: the sum of equal terms in
// sequence, as the reference accumulates it.
__global__ void k_cell_volumes(DevConsts k, double* vol) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < k.C; c += gridDim.x * blockDim.x) vol[c] = cell_volume(c, k);
}

__global__ void k_node_density(DevConsts k, const double* vol, const int32_t* qc, double* nnd, int exact,
                               __nv_bfloat16* xin = nullptr, const int32_t* ccnt = nullptr,
                               double* ncell = nullptr) {
  // the network's first layer (launched as a programmatic dependent) may
  // begin its set-up; it reads the input after this grid completes
  if (threadIdx.x == 0) asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
  const int N0 = k.N0, N1 = k.N1;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 4 * k.C; e += gridDim.x * blockDim.x) {
    const int c = e >> 2, slot = e & 3;
    const int j = c % N0, kk = c / N0;
    const int ni = j + (slot & 1), nj = kk + (slot >> 1);  // the node
    int count = 0;
    // the cells around node (ni, nj) and the quadrant of each that is nearest to it
    if (ni < N0 && nj < N1) count += qc[(size_t)(nj * N0 + ni) * 4 + 0];
    if (ni > 0 && nj < N1) count += qc[(size_t)(nj * N0 + ni - 1) * 4 + 1];
    if (ni < N0 && nj > 0) count += qc[(size_t)((nj - 1) * N0 + ni) * 4 + 2];
    if (ni > 0 && nj > 0) count += qc[(size_t)((nj - 1) * N0 + ni - 1) * 4 + 3];
    const double v = k.Fn / vol[c];
    double acc = 0.0;
    if (exact) {
      for (int t = 0; t < count; ++t) acc += v;
    } else {
      acc = (double)count * v;
    }
    if (kk == 0 && slot < 2) acc = acc * 2.0;
    if (kk == N1 - 1 && slot >= 2) acc = acc * 2.0;
    if (j == 0 && (slot & 1) == 0) acc = acc * 2.0;
    if (j == N0 - 1 && (slot & 1) == 1) acc = acc * 2.0;
    nnd[e] = acc;
    // the cell density n = Fn N / V as the moment finalisation forms it,
    // from the cell's count (so that the deposit and what reads it need no
    // moment pass)
    double ncv = 0.0;
    if ((xin || ncell) && slot == 0) {
      ncv = (k.cell_w ? k.cell_w[c] : 1) * k.Fn * (double)ccnt[c] / vol[c];
      if (ncell) ncell[c] = ncv;
    }
    if (xin) {
      // the learned force's input for this cell: the nodal density of the
      // slot as a bf16 pair in channels slot and 6 + slot; slot 0 adds the
      // cell density (4, 10), the inside mask (5) and the zero channels
      __nv_bfloat16* xc = xin + (size_t)c * 16;
      sur_hi_lo(10.0 * (k.b * acc - 0.25), xc[slot], xc[6 + slot]);
      if (slot == 0) {
        sur_hi_lo(10.0 * (k.b * ncv - 0.25), xc[4], xc[10]);
        xc[5] = __float2bfloat16_rn(1.0f);
        for (int q = 11; q < 16; ++q) xc[q] = __float2bfloat16_rn(0.0f);
      }
    }
  }
}

// the sphere integral at node (i, j): the stencil on the clamped cell
// densities plus the node's correction points
__device__ __forceinline__ double node_integral(const LR2D& t, const double* W, const double* n, int i, int j,
                                                int node) {
  double v = 0.0;
  const int N0 = t.N0, N1 = t.N1;
  for (int dk = t.R1lo; dk <= t.R1hi; ++dk) {
    const double* n_row = n + (size_t)clampi(j + dk, 0, N1 - 1) * N0;
    const double* w_row = W + (size_t)(dk - t.R1lo) * t.sw - t.R0lo;
    for (int dj = t.R0lo; dj <= t.R0hi; ++dj) v += w_row[dj] * n_row[clampi(i + dj, 0, N0 - 1)];
  }
  for (int e = t.exc_off[node]; e < t.exc_off[node + 1]; ++e) {
    const int* x = t.exc_i + 4 * e;
    double na = n[(size_t)clampi(j + x[1], 0, N1 - 1) * N0 + clampi(i + x[0], 0, N0 - 1)];
    double nc = n[(size_t)clampi(j + x[3], 0, N1 - 1) * N0 + clampi(i + x[2], 0, N0 - 1)];
    v += t.exc_w[e] * (na - nc);
  }
  return v;
}

// direct path: every node; screened Poisson: the wall nodes (their
// Green's-function values, stored in V until the finish kernel)
__global__ void k_node_potential(LR2D t, const double* n, int walls_only) {
  extern __shared__ double Ws[];
  const int nw = (t.R1hi - t.R1lo + 1) * t.sw;
  for (int q = threadIdx.x; q < nw; q += blockDim.x) Ws[q] = t.W[q];
  __syncthreads();
  const int total = walls_only ? t.n_wall : t.nn;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
    const int node = walls_only ? t.wall[e] : e;
    const int i = node % (t.N0 + 1), j = node / (t.N0 + 1);
    t.V[node] = node_integral(t, Ws, n, i, j, node);
  }
}

// element matrices of compute_SP_2D (src/FEM.cpp:50-106)
__constant__ double c_dudv[4][4] = {{2.0 / 3.0, -1.0 / 6.0, -1.0 / 6.0, -1.0 / 3.0},
                                    {-1.0 / 6.0, 2.0 / 3.0, -1.0 / 3.0, -1.0 / 6.0},
                                    {-1.0 / 6.0, -1.0 / 3.0, 2.0 / 3.0, -1.0 / 6.0},
                                    {-1.0 / 3.0, -1.0 / 6.0, -1.0 / 6.0, 2.0 / 3.0}};
__constant__ double c_uv[4][4] = {{1.0 / 9.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0},
                                  {1.0 / 18.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 18.0},
                                  {1.0 / 18.0, 1.0 / 36.0, 1.0 / 9.0, 1.0 / 18.0},
                                  {1.0 / 36.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 9.0}};

// right-hand side of the interior rows: the load vector sum_cells (uv n_n)
// vol in cell order (src/FEM.cpp:276-300), minus the columns of the wall
// nodes times their Dirichlet values (the wall rows are identities)
__global__ void k_sp_rhs(LR2D t, DevConsts k) {
  const int nx = t.nx, ny = t.ny, N0 = t.N0;
  const double lambda2 = k.bst * k.bst;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nx * ny; e += gridDim.x * blockDim.x) {
    const int i = e % nx + 1, j = e / nx + 1;  // interior node
    double b = 0.0, elim = 0.0;
    // cells (i-1, j-1), (i, j-1), (i-1, j), (i, j): the node is their corner 3, 2, 1, 0
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int ci = i - 1 + (q & 1), cj = j - 1 + (q >> 1), slot = 3 - q;
      const int c = cj * N0 + ci;
      const double vol = t.vol[c];
      const double* nn = t.nnd + (size_t)c * 4;
      double v = 0.0;
      for (int l = 0; l < 4; ++l) v += nn[l] * c_uv[slot][l];
      b += v * vol;
      for (int l = 0; l < 4; ++l) {
        const int gi = ci + (l & 1), gj = cj + (l >> 1);
        if (gi == 0 || gi == N0 || gj == 0 || gj == t.N1) {
          const double a = c_dudv[slot][l] + lambda2 * c_uv[slot][l] * vol;
          elim += a * t.V[gj * (N0 + 1) + gi];
        }
      }
    }
    t.B[e] = b - elim;
  }
}

// C[M][N] = A[M][K] B[K][N] (row-major, FP32): 32 x 32 outputs per block of
// 256 threads, 2 x 2 per thread, K staged through shared memory in slices of
// 32.  Epilogue: mode 0 store, 1 store divided elementwise by D, 2 U = acc
// (FP64), 3 U += acc (FP64).
__global__ void __launch_bounds__(256) k_sgemm(int M, int N, int K, const float* A, const float* B, float* C,
                                               const float* D, double* U, int mode) {
  __shared__ float As[32][33], Bs[32][33];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  for (int k0 = 0; k0 < K; k0 += 32) {
    for (int e = threadIdx.x; e < 32 * 32; e += 256) {
      const int r = e >> 5, q = e & 31;
      As[r][q] = (r0 + r < M && k0 + q < K) ? A[(size_t)(r0 + r) * K + k0 + q] : 0.f;
      Bs[r][q] = (k0 + r < K && c0 + q < N) ? B[(size_t)(k0 + r) * N + c0 + q] : 0.f;
    }
    __syncthreads();
#pragma unroll 8
    for (int q = 0; q < 32; ++q) {
      const float a0 = As[2 * ty][q], a1 = As[2 * ty + 1][q];
      const float b0 = Bs[q][2 * tx], b1 = Bs[q][2 * tx + 1];
      acc[0][0] = fmaf(a0, b0, acc[0][0]); acc[0][1] = fmaf(a0, b1, acc[0][1]);
      acc[1][0] = fmaf(a1, b0, acc[1][0]); acc[1][1] = fmaf(a1, b1, acc[1][1]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int row = r0 + 2 * ty + i, col = c0 + 2 * tx + j;
      if (row >= M || col >= N) continue;
      const size_t o = (size_t)row * N + col;
      if (mode == 0) C[o] = acc[i][j];
      else if (mode == 1) C[o] = acc[i][j] / D[o];
      else if (mode == 2) U[o] = (double)acc[i][j];
      else U[o] += (double)acc[i][j];
    }
}

// The same product for K <= SGEMM_KMAX: the block's 32 rows of A and 32
// columns of B over the whole of K are staged into shared memory at once
// (one round of independent loads instead of one round trip per 32-wide
// slice, which bounds these small transforms), then each output sums over
// k = 0 .. K-1 in the same order as k_sgemm (the same results bit for bit).
constexpr int SGEMM_KMAX = 256;
constexpr size_t sgemm_fullk_smem(int K) { return (size_t)(32 * (K + 1) + K * 33) * sizeof(float); }
__global__ void __launch_bounds__(256) k_sgemm_fullk(int M, int N, int K, const float* A, const float* B, float* C,
                                                     const float* D, double* U, int mode) {
  extern __shared__ float sg[];
  float* As = sg;                    // [32][K + 1]
  float* Bs = sg + 32 * (K + 1);     // [K][33]
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int e = threadIdx.x; e < 32 * K; e += 256) {
    const int r = e / K, q = e - r * K;
    As[r * (K + 1) + q] = r0 + r < M ? A[(size_t)(r0 + r) * K + q] : 0.f;
  }
  for (int e = threadIdx.x; e < K * 32; e += 256) {
    const int q = e >> 5, c = e & 31;
    Bs[q * 33 + c] = c0 + c < N ? B[(size_t)q * N + c0 + c] : 0.f;
  }
  __syncthreads();
  float acc[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
  const float* a0p = As + (2 * ty) * (K + 1);
  const float* a1p = a0p + (K + 1);
#pragma unroll 8
  for (int q = 0; q < K; ++q) {
    const float a0 = a0p[q], a1 = a1p[q];
    const float b0 = Bs[q * 33 + 2 * tx], b1 = Bs[q * 33 + 2 * tx + 1];
    acc[0][0] = fmaf(a0, b0, acc[0][0]); acc[0][1] = fmaf(a0, b1, acc[0][1]);
    acc[1][0] = fmaf(a1, b0, acc[1][0]); acc[1][1] = fmaf(a1, b1, acc[1][1]);
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int row = r0 + 2 * ty + i, col = c0 + 2 * tx + j;
      if (row >= M || col >= N) continue;
      const size_t o = (size_t)row * N + col;
      if (mode == 0) C[o] = acc[i][j];
      else if (mode == 1) C[o] = acc[i][j] / D[o];
      else if (mode == 2) U[o] = (double)acc[i][j];
      else U[o] += (double)acc[i][j];
    }
}

// C = A B on the session's stream: the whole-K kernel where K allows
static void sgemm(dim3 g, int M, int N, int K, const float* A, const float* B, float* C, const float* D, double* U,
                  int mode, cudaStream_t st) {
  if (K <= SGEMM_KMAX) k_sgemm_fullk<<<g, 256, sgemm_fullk_smem(K), st>>>(M, N, K, A, B, C, D, U, mode);
  else k_sgemm<<<g, 256, 0, st>>>(M, N, K, A, B, C, D, U, mode);
}

// the right-hand side in FP32 for the first pass
__global__ void k_to_f32(const double* a, float* b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) b[i] = (float)a[i];
}

// residual b - L U of the interior rows in FP64 (the wall columns are in b):
// L = K (x) M + M (x) K + c M (x) M on the 3 x 3 neighbourhood, with the 1-D
// unit stiffness K (2, -1) and mass M (2/3, 1/6)
__global__ void k_sp_residual(LR2D t) {
  const int nx = t.nx, ny = t.ny;
  const double c = t.lambda2vol;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nx * ny; e += gridDim.x * blockDim.x) {
    const int p = e % nx, q = e / nx;
    double lu = 0.0;
#pragma unroll
    for (int dq = -1; dq <= 1; ++dq) {
      const int qq = q + dq;
      if (qq < 0 || qq >= ny) continue;
      const double ky = dq == 0 ? 2.0 : -1.0, my = dq == 0 ? 2.0 / 3.0 : 1.0 / 6.0;
#pragma unroll
      for (int dp = -1; dp <= 1; ++dp) {
        const int pp = p + dp;
        if (pp < 0 || pp >= nx) continue;
        const double kx = dp == 0 ? 2.0 : -1.0, mx = dp == 0 ? 2.0 / 3.0 : 1.0 / 6.0;
        lu += (kx * my + mx * ky + c * mx * my) * t.U[(size_t)qq * nx + pp];
      }
    }
    t.Bf[e] = (float)(t.B[e] - lu);
  }
}

// node potential of the screened-Poisson path: the solved interior values
// or the wall values, minus the analytic near-field part
// (src/FEM.cpp:491-546; the corner and edge index rules restated)
__global__ void k_sp_finish(LR2D t, double dummy, double dummy2) {
  const int N0 = t.N0, N1 = t.N1;
  for (int id = blockIdx.x * blockDim.x + threadIdx.x; id < t.nn; id += gridDim.x * blockDim.x) {
    const int i = id % (N0 + 1), j = id / (N0 + 1);
    double x = (i > 0 && i < N0 && j > 0 && j < N1) ? t.U[(size_t)(j - 1) * t.nx + (i - 1)] : t.V[id];
    int ii = i, jj = j, kq = 0;
    int ipm[4] = {0, -1, 0, 0}, jpm[4] = {0, 0, 0, -1}, kpm[4] = {1, 0, 2, 0};
    if (i == N0) { ii = i - 1; jj = j; kq = 1; kpm[0] = kq; }
    if (j == N1) { ii = i; jj = j - 1; kq = 2; kpm[2] = kq; }
    if (i == N0 && j == N1) { ii = i - 1; jj = j - 1; kq = 3; kpm[0] = kq; kpm[2] = kq; }
    if (i == 0) { ipm[1] = 0; jpm[1] = 0; kpm[1] = 0; }
    if (j == 0) { ipm[3] = 0; jpm[3] = 0; kpm[3] = 0; }
    int num = jj * N0 + ii;
    const double d2 = t.nnd[(size_t)num * 4 + kq] * dummy;
    double d3 = -4.0 * t.nnd[(size_t)num * 4 + kq] * dummy2;
#pragma unroll
    for (int ll = 0; ll < 4; ++ll) {
      num = (jj + jpm[ll]) * N0 + ii + ipm[ll];
      d3 += t.nnd[(size_t)num * 4 + kpm[ll]] * dummy2;
    }
    t.V[id] = x + -(d2 + d3);
  }
}

// FP32 path: the kick per cell as U1 -= LA1 + LB1 eta, U2 -= LA2 + LB2 xi,
// the node differences taken in FP64
__global__ void k_lr2d_pack(DevConsts k, const double* V, float* pcell) {
  const int N0 = k.N0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < k.C; c += gridDim.x * blockDim.x) {
    const int j = c % N0, kk = c / N0;
    const int id0 = kk * (N0 + 1) + j, id2 = id0 + N0 + 1;
    const double v0 = V[id0], v1 = V[id0 + 1], v2 = V[id2], v3 = V[id2 + 1];
    const double g1 = k.lr_coef / k.m / k.dx * k.dt, g2 = k.lr_coef / k.m / k.dy * k.dt;
    const double cross = (v0 - v1) - (v2 - v3);
    float* pf = pcell + (size_t)c * PF_STRIDE;
    pf[PF_LA1] = (float)((v1 - v0) * g1);
    pf[PF_LB1] = (float)(cross * g1);
    pf[PF_LA2] = (float)((v2 - v0) * g2);
    pf[PF_LB2] = (float)(cross * g2);
  }
}

// ------------------------------------------------------------ set-up --
static void gl_table(int n, double* xs, double* ws) {
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
  if (n == 50)  // the 8-decimal table of compute_SP_2D (src/FEM.cpp:333-351)
    for (int i = 0; i < n; ++i) { xs[i] = nearbyint(xs[i] * 1e8) / 1e8; ws[i] = nearbyint(ws[i] * 1e8) / 1e8; }
}

struct Stencil {
  int R0lo, R0hi, R1lo, R1hi;
  std::vector<double> W;
  std::vector<int> exc_off, exc_i;
  std::vector<double> exc_w;
};

// the per-offset weights of the sphere rule and the per-node corrections
// (see the file comment).  kind 1: compute_Vlasov_2D, kind 3: the
// Green's-function wall values of compute_SP_2D.
static bool build_stencil(const Session& s, int kind, Stencil& st, std::string& err) {
  const DevConsts& k = s.k;
  const int N0 = k.N0, N1 = k.N1;
  const int nq = kind == 1 ? 100 : 50;
  const double pi = acos(-1.0);
  std::vector<double> xi(nq), wi(nq), rr(nq), dr(nq), ph(nq), dph(nq), th(nq), dth(nq), cph(nq), sph(nq), sth(nq);
  gl_table(nq, xi.data(), wi.data());
  const double a = kind == 1 ? 1.0 * k.sigma : 0.0, b = 3.0 * k.sigma;
  const double cc = 0.0, dd = 2 * pi, ee = 0.0, ff = pi;
  for (int i = 0; i < nq; ++i) {
    rr[i] = (b - a) / 2.0 * xi[i] + (a + b) / 2.0; dr[i] = wi[i] * (b - a) / 2.0;
    ph[i] = (dd - cc) / 2.0 * xi[i] + (cc + dd) / 2.0; dph[i] = wi[i] * (dd - cc) / 2.0;
    th[i] = (ff - ee) / 2.0 * xi[i] + (ff + ee) / 2.0; dth[i] = wi[i] * (ff - ee) / 2.0;
    cph[i] = cos(ph[i]); sph[i] = sin(ph[i]); sth[i] = sin(th[i]);
  }
  const size_t Q = (size_t)nq * nq * nq;
  std::vector<double> ox(Q), oy(Q), w(Q);
  for (int i = 0; i < nq; ++i) {
    const double radial = kind == 1 ? pow(k.sigma / rr[i], 6.0) * rr[i] * rr[i] * dr[i]
                                    : exp(-k.bst * rr[i]) / (4.0 * pi) * rr[i] * dr[i];
    for (int ii = 0; ii < nq; ++ii)
      for (int iii = 0; iii < nq; ++iii) {
        const size_t q = ((size_t)i * nq + ii) * nq + iii;
        ox[q] = rr[i] * cph[ii] * sth[iii];
        oy[q] = rr[i] * sph[ii] * sth[iii];
        w[q] = radial * dph[ii] * sth[iii] * dth[iii];
      }
  }
  // node coordinates of every column / row
  std::vector<double> xc(N0 + 1), yc(N1 + 1);
  for (int i = 0; i <= N0; ++i) xc[i] = node_coord(i, N0, k.dx);
  for (int j = 0; j <= N1; ++j) yc[j] = node_coord(j, N1, k.dy);
  // the offsets a node sees, and the points close enough to a face that
  // the rounding of the node coordinate may move them
  const double mx = 1e-13 * (N0 + 4) + 1e-12, my = 1e-13 * (N1 + 4) + 1e-12;
  std::vector<int> djc(Q), dkc(Q);
  std::vector<size_t> unsafe;
  st.R0lo = st.R1lo = 1 << 30;
  st.R0hi = st.R1hi = -(1 << 30);
  for (size_t q = 0; q < Q; ++q) {
    const double tx = ox[q] / k.dx, ty = oy[q] / k.dy;
    const double fx = floor(tx), fy = floor(ty);
    djc[q] = (int)fx; dkc[q] = (int)fy;
    if (std::min(tx - fx, fx + 1.0 - tx) < mx || std::min(ty - fy, fy + 1.0 - ty) < my) unsafe.push_back(q);
    st.R0lo = std::min(st.R0lo, djc[q]); st.R0hi = std::max(st.R0hi, djc[q]);
    st.R1lo = std::min(st.R1lo, dkc[q]); st.R1hi = std::max(st.R1hi, dkc[q]);
  }
  // corrections: for an unsafe point the reference's own lookup per column
  // and row (src/FEM.cpp:177-178, :225-226)
  struct Ent { int node, dja, dka, djc, dkc; double w; };
  std::vector<Ent> ents;
  for (size_t q : unsafe) {
    std::vector<int> dja(N0 + 1), dka(N1 + 1);
    bool any = false;
    for (int i = 0; i <= N0; ++i) {
      dja[i] = (int)floor((xc[i] + ox[q]) / k.dx) - i;
      any |= dja[i] != djc[q];
    }
    for (int j = 0; j <= N1; ++j) {
      dka[j] = (int)floor((yc[j] + oy[q]) / k.dy) - j;
      any |= dka[j] != dkc[q];
    }
    if (!any) continue;
    for (int j = 0; j <= N1; ++j)
      for (int i = 0; i <= N0; ++i) {
        if (dja[i] == djc[q] && dka[j] == dkc[q]) continue;
        if (kind == 3 && i > 0 && i < N0 && j > 0 && j < N1) continue;  // wall nodes only
        ents.push_back({j * (N0 + 1) + i, dja[i], dka[j], djc[q], dkc[q], w[q]});
        if (ents.size() > (size_t)4 << 20) { err = "too many face-coincident quadrature points"; return false; }
      }
  }
  std::stable_sort(ents.begin(), ents.end(), [](const Ent& x, const Ent& y) { return x.node < y.node; });
  const int nn = (N0 + 1) * (N1 + 1);
  st.exc_off.assign(nn + 1, 0);
  for (const Ent& e : ents) st.exc_off[e.node + 1]++;
  for (int i = 0; i < nn; ++i) st.exc_off[i + 1] += st.exc_off[i];
  for (const Ent& e : ents) {
    st.exc_i.insert(st.exc_i.end(), {e.dja, e.dka, e.djc, e.dkc});
    st.exc_w.push_back(e.w);
  }
  const int sw = st.R0hi - st.R0lo + 1, sh = st.R1hi - st.R1lo + 1;
  if ((size_t)sw * sh > 20000) { err = "Vlasov stencil too wide for the cell size"; return false; }
  st.W.assign((size_t)sw * sh, 0.0);
  for (size_t q = 0; q < Q; ++q) st.W[(size_t)(dkc[q] - st.R1lo) * sw + (djc[q] - st.R0lo)] += w[q];
  return true;
}

// orthonormal DST-I matrix of order n: S[a][p] = sqrt(2/(n+1)) sin(pi (a+1)(p+1)/(n+1))
static void dst_matrix(int n, std::vector<double>& S, std::vector<double>& lamK, std::vector<double>& lamM) {
  S.resize((size_t)n * n);
  lamK.resize(n);
  lamM.resize(n);
  const double pi = acos(-1.0), sc = sqrt(2.0 / (n + 1));
  const long period = 2L * (n + 1);
  for (int a = 0; a < n; ++a)
    for (int p = 0; p < n; ++p) {
      long m = ((long)(a + 1) * (p + 1)) % period;  // reduce the angle exactly
      S[(size_t)a * n + p] = sc * sin(pi * (double)m / (double)(n + 1));
    }
  for (int p = 0; p < n; ++p) {
    const double cth = cos(pi * (p + 1) / (double)(n + 1));
    lamK[p] = 2.0 - 2.0 * cth;
    lamM[p] = 2.0 / 3.0 + cth / 3.0;
  }
}

int lr2d_setup(Session& s) {
  const int mode = s.cfg.long_range;
  if (!(s.k.lr2d)) return 0;
  LR2D* t = new (std::nothrow) LR2D();
  if (!t) return 1;
  s.lr2d = t;
  const DevConsts& k = s.k;
  t->mode = mode;
  t->N0 = k.N0; t->N1 = k.N1;
  t->nn = (k.N0 + 1) * (k.N1 + 1);
  t->nx = k.N0 - 1; t->ny = k.N1 - 1;
  Stencil st;
  if (!build_stencil(s, mode == MCPM_LR_DIRECT ? 1 : 3, st, s.err)) return 1;
  t->R0lo = st.R0lo; t->R0hi = st.R0hi; t->R1lo = st.R1lo; t->R1hi = st.R1hi;
  t->sw = st.R0hi - st.R0lo + 1;
  t->n_exc = (int)st.exc_w.size();
  t->smem = st.W.size() * sizeof(double);
  auto A = [&](void** p, size_t bytes) { return cudaMalloc(p, bytes ? bytes : 16) == cudaSuccess; };
  auto H = [&](void* d, const void* h, size_t bytes) {
    return bytes == 0 || cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  bool ok = A((void**)&t->W, t->smem) && H(t->W, st.W.data(), t->smem) &&
            A((void**)&t->exc_off, st.exc_off.size() * 4) && H(t->exc_off, st.exc_off.data(), st.exc_off.size() * 4) &&
            A((void**)&t->exc_i, st.exc_i.size() * 4) && H(t->exc_i, st.exc_i.data(), st.exc_i.size() * 4) &&
            A((void**)&t->exc_w, st.exc_w.size() * 8) && H(t->exc_w, st.exc_w.data(), st.exc_w.size() * 8) &&
            A((void**)&t->V, (size_t)t->nn * 8) && A((void**)&t->nnd, (size_t)k.C * 4 * 8) &&
            A((void**)&t->ncell, (size_t)k.C * 8) && A((void**)&t->vol, (size_t)k.C * 8) &&
            A((void**)&t->qc, (size_t)k.C * 4 * 4);
  if (ok && s.prec == MCPM_FP32) {
    // the FP32 quadrant pass compares positions with thresholds: x < the
    // centre of the column / row in exact arithmetic <=> x < the smallest
    // float at or above it (the comparison k_quadrants makes)
    std::vector<float> tx(k.N0), ty(k.N1);
    for (int j = 0; j < k.N0; ++j) {
      const double cx = 0.5 * ((double)j * k.dx + (double)(j + 1) * k.dx);
      const float f = (float)cx;
      tx[j] = (double)f >= cx ? f : nextafterf(f, INFINITY);
    }
    for (int j = 0; j < k.N1; ++j) {
      const double cy = 0.5 * ((double)j * k.dy + (double)(j + 1) * k.dy);
      const float f = (float)cy;
      ty[j] = (double)f >= cy ? f : nextafterf(f, INFINITY);
    }
    ok = A((void**)&t->qtx, tx.size() * 4) &&
         H(t->qtx, tx.data(), tx.size() * 4) && A((void**)&t->qty, ty.size() * 4) && H(t->qty, ty.data(), ty.size() * 4);
  }
  if (ok && mode == MCPM_LR_SCREENED_POISSON) {
    std::vector<double> Sx, Sy, kx, mx, ky, my;
    dst_matrix(t->nx, Sx, kx, mx);
    dst_matrix(t->ny, Sy, ky, my);
    const double c = k.bst * k.bst * (k.dx * k.dy * k.dz);
    std::vector<float> mu((size_t)t->nx * t->ny), Sxf(Sx.begin(), Sx.end()), Syf(Sy.begin(), Sy.end());
    for (int q = 0; q < t->ny; ++q)
      for (int p = 0; p < t->nx; ++p)
        mu[(size_t)q * t->nx + p] = (float)(kx[p] * my[q] + mx[p] * ky[q] + c * mx[p] * my[q]);
    t->lambda2vol = c;
    {
      const double b = k.bst, sg = k.sigma;
      double d1 = 1.0 - (sg * b + 1.0) * exp(-b * sg);
      t->near1 = d1 / b / b;
      double d2 = (-1.0 / 6.0 * pow(b, 3) * pow(sg, 3) - 1.0 / 2.0 * pow(b, 2) * pow(sg, 2) - b * sg + exp(b * sg) - 1) *
                  exp(-b * sg) / pow(b, 4);
      t->near2 = d2 / pow(k.dx, 2);
    }
    t->iters = s.prec == MCPM_FP64 ? 3 : 2;
    std::vector<int> wall;
    for (int j = 0; j <= k.N1; ++j)
      for (int i = 0; i <= k.N0; ++i)
        if (i == 0 || i == k.N0 || j == 0 || j == k.N1) wall.push_back(j * (k.N0 + 1) + i);
    t->n_wall = (int)wall.size();
    const size_t nxy = (size_t)t->nx * t->ny;  // T: the transforms' scratch
    ok = A((void**)&t->Sx, Sxf.size() * 4) && H(t->Sx, Sxf.data(), Sxf.size() * 4) &&
         A((void**)&t->Sy, Syf.size() * 4) && H(t->Sy, Syf.data(), Syf.size() * 4) &&
         A((void**)&t->mu, nxy * 4) && H(t->mu, mu.data(), nxy * 4) && A((void**)&t->B, nxy * 8) &&
         A((void**)&t->U, nxy * 8) && A((void**)&t->Bf, nxy * 4) && A((void**)&t->Tf, nxy * 4) &&
         A((void**)&t->wall, wall.size() * 4) &&
         H(t->wall, wall.data(), wall.size() * 4);
  }
  if (!ok) { s.err = "2-D long-range tables: out of device memory"; return 1; }
  if (t->smem > 48 * 1024 &&
      cudaFuncSetAttribute(k_node_potential, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)t->smem) != cudaSuccess) {
    s.err = "2-D long-range stencil: shared memory";
    return 1;
  }
  if (cudaFuncSetAttribute(k_sgemm_fullk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)sgemm_fullk_smem(SGEMM_KMAX)) != cudaSuccess) {
    s.err = "2-D long-range transforms: shared memory";
    return 1;
  }
  cudaMemset(t->V, 0, (size_t)t->nn * 8);
  cudaMemset(t->nnd, 0, (size_t)k.C * 4 * 8);
  // on the default stream, finished before any session stream reads them
  k_cell_volumes<<<std::max(1, std::min((k.C + 255) / 256, s.num_sms * 8)), 256>>>(k, t->vol);
  if (cudaStreamSynchronize(0) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
    s.err = "2-D long-range tables: cell volumes";
    return 1;
  }
  return 0;
}

void lr2d_free(Session& s) {
  LR2D* t = s.lr2d;
  if (!t) return;
  cudaFree(t->W); cudaFree(t->exc_off); cudaFree(t->exc_i); cudaFree(t->exc_w); cudaFree(t->V); cudaFree(t->nnd); cudaFree(t->ncell); cudaFree(t->vol);
  cudaFree(t->qc); cudaFree(t->Sx); cudaFree(t->Sy); cudaFree(t->mu); cudaFree(t->B); cudaFree(t->U); cudaFree(t->Bf); cudaFree(t->Tf);
  cudaFree(t->wall); cudaFree(t->qtx); cudaFree(t->qty);
  delete t;
  s.lr2d = nullptr;
}

const double* lr2d_potential(const Session& s) { return s.lr2d ? s.lr2d->V : nullptr; }
const double* lr2d_node_density(const Session& s) { return s.lr2d ? s.lr2d->nnd : nullptr; }
int lr2d_num_nodes(const Session& s) { return s.lr2d ? s.lr2d->nn : 0; }

// ------------------------------------------------------------ launches --
static int blocks_for(long n, int bs, int cap) { return (int)std::max(1L, std::min((n + bs - 1) / bs, (long)cap)); }

int32_t* lr2d_quadrants(Session& s) { return s.lr2d ? s.lr2d->qc : nullptr; }
double* lr2d_node_density_mut(Session& s) { return s.lr2d ? s.lr2d->nnd : nullptr; }

// nodal densities from given quadrant counts (training snapshots)
int launch_node_density_from(Session& s, const int32_t* qc) {
  LR2D* t = s.lr2d;
  if (!t) return 0;
  k_node_density<<<blocks_for(4L * s.C, 256, s.num_sms * 16), 256, 0, s.stream>>>(s.k, t->vol, qc, t->nnd, 0);
  return 1;
}

int launch_node_density(Session& s, bool count_density) {
  LR2D* t = s.lr2d;
  // the screened-Poisson force and the learned force read them
  if (!t || (t->mode != MCPM_LR_SCREENED_POISSON && !s.sur)) return 0;
  // with the network attached the deposit also writes the network's input
  __nv_bfloat16* xin = s.sur ? s.sur->xin : nullptr;
  s.sur_xin_ready = xin != nullptr;
  const int g = blocks_for((long)s.C * 32, 256, s.num_sms * 16);
  if (s.prec == MCPM_FP32) {
    const PBuf& P = s.P[s.cur];
    k_quadrants_f32<<<g, 256, 0, s.stream>>>(s.k, s.off, s.cnt, (const float*)P.x1, (const float*)P.x2, t->qtx,
                                             t->qty, t->qc);
  } else {
    const PBuf& P = s.P[s.cur];
    k_quadrants<double><<<g, 256, 0, s.stream>>>(s.k, s.off, s.cnt, (const double*)P.x1, (const double*)P.x2, t->qc);
  }
  k_node_density<<<blocks_for(4L * s.C, 256, s.num_sms * 16), 256, 0, s.stream>>>(
      s.k, t->vol, t->qc, t->nnd, s.prec == MCPM_FP64, xin, s.cnt, count_density ? t->ncell : nullptr);
  return 2;
}

const double* lr2d_count_density(const Session& s) { return s.lr2d ? s.lr2d->ncell : nullptr; }

int launch_long_range_2d(Session& s, const double* n) {
  LR2D* t = s.lr2d;
  if (!t) return 0;
  if (!n) n = s.cell + (size_t)MCPM_CF_N * s.C;
  int launches = 0;
  const int cap = s.num_sms * 16;
  if (t->mode == MCPM_LR_DIRECT) {
    k_node_potential<<<blocks_for(t->nn, 128, cap), 128, t->smem, s.stream>>>(*t, n, 0);
    launches = 1;
  } else {
    k_node_potential<<<blocks_for(t->n_wall, 128, cap), 128, t->smem, s.stream>>>(*t, n, 1);
    k_sp_rhs<<<blocks_for((long)t->nx * t->ny, 256, cap), 256, 0, s.stream>>>(*t, s.k);
    const int nx = t->nx, ny = t->ny;
    dim3 g((nx + 31) / 32, (ny + 31) / 32);
    const int nxy = nx * ny;
    k_to_f32<<<blocks_for(nxy, 256, cap), 256, 0, s.stream>>>(t->B, t->Bf, nxy);
    launches = 3;
    for (int it = 0; it < t->iters; ++it) {
      if (it > 0) {
        k_sp_residual<<<blocks_for(nxy, 256, cap), 256, 0, s.stream>>>(*t);
        ++launches;
      }
      // delta = S_y ((S_y r S_x) / mu) S_x  (rows y, columns x); U (+)= delta
      sgemm(g, ny, nx, ny, t->Sy, t->Bf, t->Tf, nullptr, nullptr, 0, s.stream);
      sgemm(g, ny, nx, nx, t->Tf, t->Sx, t->Bf, t->mu, nullptr, 1, s.stream);
      sgemm(g, ny, nx, ny, t->Sy, t->Bf, t->Tf, nullptr, nullptr, 0, s.stream);
      sgemm(g, ny, nx, nx, t->Tf, t->Sx, nullptr, nullptr, t->U, it == 0 ? 2 : 3, s.stream);
      launches += 4;
    }
    k_sp_finish<<<blocks_for(t->nn, 256, cap), 256, 0, s.stream>>>(*t, t->near1, t->near2);
    ++launches;
  }
  if (s.prec == MCPM_FP32) {
    k_lr2d_pack<<<blocks_for(s.C, 256, cap), 256, 0, s.stream>>>(s.k, t->V, s.pcell);
    ++launches;
  }
  return launches;
}

}  // namespace mcpm
