// mcpm_noalloc.cu -- an allocation-free entry point for the 1-D
// screened-Poisson Vlasov force.
//
// Some callers cannot allocate device memory themselves: code running inside
// a host framework whose allocator owns the GPU (and forbids cudaMalloc
// behind its back), code that must not allocate between CUDA-graph replays,
// or plugins handed only the device buffers they read and write.  For them
// mcpm_poisson_force_1d_noalloc computes what poisson_solver computes
// (src/Main_Functions.cpp:3285-3581) -- the per-cell force of the
// screened-Poisson face potential with Green's-function wall values, minus
// the analytic r < sigma part -- from a device array of cell densities into a
// device array of forces, using no memory but a fixed scratch array that the
// library reserves when it is loaded.
//
// The scratch is the file-scope __device__ array below, of fixed size
// (MCPM_NOALLOC_MAX_CELLS + 1 = 7000 face values plus the 2 x 2500-entry
// quadrature table, 96 KB).  Every GPU that loads the library holds it until the
// process exits.  All calls on a device share it and it keeps the last call's
// contents; each call rewrites every entry it reads before reading it (the
// quadrature table by a kernel of its own, so no host buffer is involved).
// Calls whose work overlaps on the same GPU (two streams, or two host
// threads) race on it; calls on different GPUs use different copies.
#include <cmath>
#include <cstring>

#include "mcpm_device.cuh"

namespace mcpm {
namespace {

constexpr int kQuad = 2500;  // GL(50) x GL(50)
constexpr int kFaces = MCPM_NOALLOC_MAX_CELLS + 1;
constexpr int kMaxDevices = 64;

__device__ __align__(256) double g_scratch[kFaces + 2 * kQuad];

// device address of g_scratch per device (host code cannot use the symbol)
double* g_scratch_ptr[kMaxDevices] = {nullptr};

#define FULL 0xffffffffu

// Gauss-Legendre nodes / weights on [-1, 1]; the 50-point table rounded to
// 8 decimals, as the reference's literals are (src/Main_Functions.cpp:3327-3346)
void gl50(double* xs, double* ws) {
  const int n = 50;
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
  for (int i = 0; i < n; ++i) { xs[i] = nearbyint(xs[i] * 1e8) / 1e8; ws[i] = nearbyint(ws[i] * 1e8) / 1e8; }
}

struct Params {
  int N1;
  double dy, sigma, bst, ast, m;
};

// GL(50) radial points r_i in [0, 3 eqdist] and polar angles phi_i in
// [0, pi] with their interval weights (poisson_solver :3362-3397), formed on
// the host per call and passed by value
struct QuadNodes {
  double rr[50], dr[50], ph[50], dph[50];
  double bst;
};

// the wall-integral quadrature table into the scratch: points r cos(phi)
// and weights exp(-bst r) / 2 r dr sin(phi) dphi
__global__ void k_noalloc_table(QuadNodes q, double* scratch) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < kQuad; t += gridDim.x * blockDim.x) {
    const int i = t / 50, ii = t % 50;
    const double radial = exp(-q.bst * q.rr[i]) / (2.0) * q.rr[i] * q.dr[i];
    scratch[kFaces + t] = q.rr[i] * cos(q.ph[ii]);
    scratch[kFaces + kQuad + t] = radial * sin(q.ph[ii]) * q.dph[ii];
  }
}

// density of cell num with the reference's edge clamping
__device__ __forceinline__ double nclamp(const double* n, int num, int N1) {
  return n[num > -1 && num < N1 ? num : (num < 0 ? 0 : N1 - 1)];
}

// the wall values V(0), V(L) by quadrature (poisson_solver :3399-3431):
// warp w integrates face w == 0 ? 0 : N1
__global__ void k_noalloc_walls(Params p, const double* ncell, double* scratch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int fc = w == 0 ? 0 : p.N1;
  const double* qoff = scratch + kFaces;
  const double* qw = scratch + kFaces + kQuad;
  double acc = 0.0;
  for (int q = lane; q < kQuad; q += 32) {
    double y = fc * p.dy + qoff[q];
    int num = (int)floor(y / p.dy);
    acc += qw[q] * nclamp(ncell, num, p.N1);
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(FULL, acc, m);
  if (lane == 0) scratch[fc] = acc;
}

// the tridiagonal system (:3375-3470) by parallel cyclic reduction in shared
// memory, minus the analytic r < sigma part (:3539-3558), then the force
// per cell (:3568-3577).  One block of 1024 threads.
__global__ void __launch_bounds__(1024) k_noalloc_pcr_force(Params p, const double* ncell, double* scratch,
                                                            double* F2) {
  extern __shared__ double sh[];
  const int nf = p.N1 + 1;
  double *l = sh, *d = sh + nf, *u = sh + 2 * nf, *r = sh + 3 * nf;
  const double a_diag = 2.0 + (p.dy * p.bst) * (p.dy * p.bst);
  const double dy2 = p.dy * p.dy;
  auto nj = [&](int i) -> double {
    if (i == 0) return ncell[0];
    if (i == p.N1) return ncell[p.N1 - 1];
    return (ncell[i] + ncell[i - 1]) / 2.0;
  };
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    if (i == 0) { l[i] = 0.0; d[i] = 1.0; u[i] = 0.0; r[i] = scratch[0]; }
    else if (i == nf - 1) { l[i] = 0.0; d[i] = 1.0; u[i] = 0.0; r[i] = scratch[nf - 1]; }
    else { l[i] = -1.0; d[i] = a_diag; u[i] = -1.0; r[i] = nj(i) * dy2; }
  }
  __syncthreads();
  for (int s = 1; s < nf; s <<= 1) {
    double nl[8], nd[8], nu[8], nr[8];
    int q = 0;
    for (int i = threadIdx.x; i < nf; i += blockDim.x, ++q) {
      double li = l[i], ui = u[i], ri = r[i];
      double lo = 0.0, uo = 0.0, ro = 0.0, dd = d[i];
      if (i - s >= 0) { double al = -li / d[i - s]; lo = al * l[i - s]; dd += al * u[i - s]; ro += al * r[i - s]; }
      if (i + s < nf) { double ga = -ui / d[i + s]; uo = ga * u[i + s]; dd += ga * l[i + s]; ro += ga * r[i + s]; }
      nl[q] = lo; nd[q] = dd; nu[q] = uo; nr[q] = ri + ro;
    }
    __syncthreads();
    q = 0;
    for (int i = threadIdx.x; i < nf; i += blockDim.x, ++q) { l[i] = nl[q]; d[i] = nd[q]; u[i] = nu[q]; r[i] = nr[q]; }
    __syncthreads();
  }
  double corr = 1.0 - (p.sigma * p.bst + 1.0) * exp(-p.bst * p.sigma);
  corr = corr / p.bst / p.bst;
  for (int i = threadIdx.x; i < nf; i += blockDim.x) scratch[i] = r[i] / d[i] - nj(i) * corr;
  __syncthreads();
  for (int num = threadIdx.x; num < p.N1; num += blockDim.x) {
    double f = -(scratch[num + 1] - scratch[num]) / p.dy;
    F2[num] = f / p.m * p.ast;
  }
}

}  // namespace
}  // namespace mcpm

using namespace mcpm;

extern "C" int mcpm_poisson_force_1d_noalloc(const double* n_cell, int32_t n_cells, const mcpm_config* cfg,
                                             double* F2, void* stream) {
  if (!cfg || !n_cell || !F2) return MCPM_ERR_ARG;
  if (n_cells < 1 || n_cells > MCPM_NOALLOC_MAX_CELLS) return MCPM_ERR_CAPACITY;
  if (!(cfg->length[1] > 0 && cfg->bst > 0 && cfg->m > 0 && cfg->eqdist > 0)) return MCPM_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return MCPM_ERR_CUDA;
  cudaStream_t st = (cudaStream_t)stream;
  // once per device, with that device current: the scratch array's device address
  if (!g_scratch_ptr[dev]) {
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) return MCPM_ERR_CUDA;
    if (cudaFuncSetAttribute(k_noalloc_pcr_force, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             4 * kFaces * (int)sizeof(double)) != cudaSuccess)
      return MCPM_ERR_CUDA;
    g_scratch_ptr[dev] = (double*)ptr;
  }
  double* scratch = g_scratch_ptr[dev];
  // the quadrature nodes of the wall integrals, r in [0, 3 eqdist] and phi
  // in [0, pi] (:3362-3397); the table itself is formed on the GPU
  QuadNodes qn;
  double xi[50], wi[50];
  gl50(xi, wi);
  const double pi = acos(-1.0);
  const double bb = 3.0 * cfg->eqdist, aa = 0.0 * cfg->eqdist, cc = 0.0, dd = pi;
  for (int i = 0; i < 50; ++i) { qn.rr[i] = (bb - aa) / 2.0 * xi[i] + (aa + bb) / 2.0; qn.dr[i] = wi[i] * (bb - aa) / 2.0; }
  for (int i = 0; i < 50; ++i) { qn.ph[i] = (dd - cc) / 2.0 * xi[i] + (cc + dd) / 2.0; qn.dph[i] = wi[i] * (dd - cc) / 2.0; }
  qn.bst = cfg->bst;
  k_noalloc_table<<<10, 256, 0, st>>>(qn, scratch);
  Params p;
  p.N1 = n_cells;
  p.dy = cfg->length[1] / n_cells;
  p.sigma = cfg->sigma;
  p.bst = cfg->bst;
  p.ast = cfg->ast;
  p.m = cfg->m;
  k_noalloc_walls<<<1, 64, 0, st>>>(p, n_cell, scratch);
  k_noalloc_pcr_force<<<1, 1024, 4 * (n_cells + 1) * sizeof(double), st>>>(p, n_cell, scratch, F2);
  if (cudaGetLastError() != cudaSuccess) return MCPM_ERR_CUDA;
  return MCPM_OK;
}
