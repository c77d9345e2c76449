// mcpm_forces.cu -- ESMC collisions and the 1-D Vlasov long-range force.
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
// draws 32 candidates at once and applies the longest prefix whose particle
// pairs are disjoint, so the result equals processing the candidates one
// after another in order.
template <typename real>
__global__ void __launch_bounds__(128) k_esmc(DevConsts k, double* cell, const int32_t* off, const int32_t* cnt,
                                              PT2<real> p, int step, int cx, int cy, int Sx, int Sy,
                                              uint32_t* status) {
  const int lane = threadIdx.x & 31;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nA = (k.N0 - cx + Sx - 1) / Sx, nB = (k.N1 - cy + Sy - 1) / Sy;
  if (gw >= nA * nB) return;
  const int I = (cy + Sy * (gw / nA)) * k.N0 + (cx + Sx * (gw % nA));
  const int C = k.C;
  const int NI = cnt[I];
  const double om_max = cell[(size_t)MCPM_CF_OMEGA_MAX * C + I];
  const double mreal = r_floor(0.5 * om_max * (1.0 * NI) + u01d(philox(k.seed, (uint32_t)I, (uint32_t)step, RNG_ESMC_M, 0u).x));
  // a non-finite or absurd majorant would make the candidate loop unbounded
  const double mcap = 64.0 * NI + 4096.0;
  int mI = 0;
  if (mreal >= 0.0 && mreal <= mcap) mI = (int)mreal;
  else if (lane == 0) raise_status(status, MCPM_ERR_ITER_LIMIT);
  double omega = 0.0;
  const real pi = (real)3.14159265358979323846;
  const real sg = (real)k.sigma;
  if (NI > 0) {
    int base = 0;
    while (base < mI) {
      const int kc = base + lane;
      bool valid = false;
      int64_t si = -1, sj = -1;
      real d0 = 0, d1 = 0, d2 = 0;
      double Ymid = 0.0, nJ = 0.0;
      if (kc < mI) {
        uint4 r = philox(k.seed, (uint32_t)I, (uint32_t)step, RNG_ESMC, (uint32_t)kc);
        si = (int64_t)off[I] + pick(r.x, NI);
        real theta = (real)2.0 * pi * (real)u01d(r.y);
        real cph = (real)2.0 * (real)u01d(r.z) - (real)1.0;
        real sph = r_sqrt((real)1.0 - cph * cph);
        real sn, cs;
        r_sincos(theta, &sn, &cs);
        d0 = cs * sph; d1 = sn * sph; d2 = cph;
        real xi1 = p.x1[si], xi2 = p.x2[si];
        real xx = xi1 + sg * d0, yy = xi2 + sg * d1;
        int i0 = (int)r_floor(xx / (real)k.dx), i1 = (int)r_floor(yy / (real)k.dy);
        if (i0 >= 0 && i0 < k.N0 && i1 >= 0 && i1 < k.N1) {
          int J = i1 * k.N0 + i0;
          int NJ = cnt[J];
          if (NJ > 0) {
            sj = (int64_t)off[J] + pick(r.w, NJ);
            if (sj != si) {
              real xm0 = (xi1 + p.x1[sj]) / (real)2.0, xm1 = (xi2 + p.x2[sj]) / (real)2.0;
              int m0 = (int)r_floor(xm0 / (real)k.dx), m1 = (int)r_floor(xm1 / (real)k.dy);
              m0 = m0 < 0 ? 0 : (m0 > k.N0 - 1 ? k.N0 - 1 : m0);
              m1 = m1 < 0 ? 0 : (m1 > k.N1 - 1 ? k.N1 - 1 : m1);
              Ymid = cell[(size_t)CFI_Y * C + m1 * k.N0 + m0];
              nJ = cell[(size_t)MCPM_CF_N * C + J];
              valid = true;
            }
          }
        }
      }
      // longest prefix of candidates with pairwise disjoint particles
      bool conflict = false;
      for (int l = 0; l < 31; ++l) {
        int64_t oi = __shfl_sync(FULL, si, l), oj = __shfl_sync(FULL, sj, l);
        int ov = __shfl_sync(FULL, (int)valid, l);
        if (l < lane && ov && valid && (oi == si || oi == sj || oj == si || oj == sj)) conflict = true;
      }
      unsigned cm = __ballot_sync(FULL, conflict);
      int take = cm ? (__ffs(cm) - 1) : 32;
      if (take > mI - base) take = mI - base;
      if (lane < take && valid) {
        real g0 = p.U1[si] - p.U1[sj], g1 = p.U2[si] - p.U2[sj], g2 = p.U3[si] - p.U3[sj];
        real gd = g0 * d0 + g1 * d1 + g2 * d2;
        double dummy = 4.0 * 3.14159265358979323846 * k.sigma * k.sigma * (double)gd * Ymid * nJ * k.dt;
        if (dummy - omega > 0.0) omega = dummy;
        double u = u01d(philox(k.seed, (uint32_t)I, (uint32_t)step, RNG_ESMC_ACC, (uint32_t)kc).x);
        if (dummy / om_max > u) {
          p.U1[si] = p.U1[si] - gd * d0; p.U2[si] = p.U2[si] - gd * d1; p.U3[si] = p.U3[si] - gd * d2;
          p.U1[sj] = p.U1[sj] + gd * d0; p.U2[sj] = p.U2[sj] + gd * d1; p.U3[sj] = p.U3[sj] + gd * d2;
        }
      }
      __syncwarp();
      base += take;
    }
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) omega = fmax(omega, __shfl_xor_sync(FULL, omega, m));
  if (lane == 0) cell[(size_t)MCPM_CF_OMEGA_MAX * C + I] = omega > om_max ? omega : om_max;
}

template <typename real> static int esmc_impl(Session& s) {
  const PBuf& b = s.P[s.cur];
  PT2<real> p{(real*)b.x1, (real*)b.x2, (real*)b.U1, (real*)b.U2, (real*)b.U3};
  int Rx = (int)ceil(s.k.sigma / s.k.dx), Ry = (int)ceil(s.k.sigma / s.k.dy);
  if (Rx < 1) Rx = 1;
  if (Ry < 1) Ry = 1;
  int Sx = (s.k.N0 > 1) ? 2 * Rx + 1 : 1, Sy = 2 * Ry + 1;
  int n = 0;
  for (int cy = 0; cy < Sy; ++cy)
    for (int cx = 0; cx < Sx; ++cx) {
      int nA = (s.k.N0 - cx + Sx - 1) / Sx, nB = (s.k.N1 - cy + Sy - 1) / Sy;
      int warps = nA * nB;
      if (warps <= 0) continue;
      int blocks = (warps * 32 + 127) / 128;
      k_esmc<real><<<blocks, 128, 0, s.stream>>>(s.k, s.cell, s.off, s.cnt, p, s.step, cx, cy, Sx, Sy, s.status);
      ++n;
    }
  return n;
}
int launch_esmc(Session& s) { return s.prec == MCPM_FP32 ? esmc_impl<float>(s) : esmc_impl<double>(s); }

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
  cell[(size_t)MCPM_CF_OMEGA_MAX * C + c] = om;
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

// face potential by direct quadrature: one warp per face
__global__ void k_face_quad(DevConsts k, const double* cell, const double* qoff, const double* qw, double* V,
                            int nfaces, int face0, int face_stride) {
  const int lane = threadIdx.x & 31;
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (wid >= nfaces) return;
  const int fc = face0 + wid * face_stride;
  const int C = k.C;
  double acc = 0.0;
  for (int q = lane; q < 2500; q += 32) {
    double y = fc * k.dy + qoff[q];
    int num = (int)floor(y / k.dy);
    int nc = num > -1 && num < k.N1 ? num : (num < 0 ? 0 : k.N1 - 1);
    acc += qw[q] * cell[(size_t)MCPM_CF_N * C + nc];
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(FULL, acc, m);
  if (lane == 0) V[fc] = acc;
}

// F2 per cell from the face potential, src/Main_Functions.cpp:3924-3938 / :3568-3577
__global__ void k_face_force(DevConsts k, double* cell, float* pcell, const double* V, double coef) {
  const int C = k.C;
  int num = blockIdx.x * blockDim.x + threadIdx.x;
  if (num >= k.N1) return;
  double F2 = -(V[num + 1] - V[num]) / k.dy;
  F2 = F2 / k.m * coef;
  for (int j = 0; j < k.N0; ++j) {
    cell[(size_t)MCPM_CF_F2 * C + num * k.N0 + j] = F2;
    if (pcell) pcell[(size_t)(num * k.N0 + j) * PF_STRIDE + PF_F2DT] = (float)(F2 * k.dt);
  }
}

// poisson_solver's tridiagonal system (src/Main_Functions.cpp:3375-3470)
// solved by parallel cyclic reduction in one block; afterwards the analytic
// r < sigma part is subtracted (:3539-3558).  V[0], V[nf-1] hold the wall
// values on entry.
__global__ void k_poisson_pcr(DevConsts k, const double* cell, double* V, int nf) {
  extern __shared__ double sh[];
  double *l = sh, *d = sh + nf, *u = sh + 2 * nf, *r = sh + 3 * nf;
  const int C = k.C;
  const double a_diag = 2.0 + (k.dy * k.bst) * (k.dy * k.bst);
  const double dy2 = k.dy * k.dy;
  auto nj = [&](int i) -> double {
    if (i == 0) return cell[(size_t)MCPM_CF_N * C + 0];
    if (i == k.N1) return cell[(size_t)MCPM_CF_N * C + (k.N1 - 1)];
    return (cell[(size_t)MCPM_CF_N * C + i] + cell[(size_t)MCPM_CF_N * C + i - 1]) / 2.0;
  };
  for (int i = threadIdx.x; i < nf; i += blockDim.x) {
    if (i == 0) { l[i] = 0.0; d[i] = 1.0; u[i] = 0.0; r[i] = V[0]; }
    else if (i == nf - 1) { l[i] = 0.0; d[i] = 1.0; u[i] = 0.0; r[i] = V[nf - 1]; }
    else { l[i] = -1.0; d[i] = a_diag; u[i] = -1.0; r[i] = nj(i) * dy2; }
  }
  __syncthreads();
  for (int s = 1; s < nf; s <<= 1) {
    // each thread updates its equations into registers, then writes back
    double nl[8], nd[8], nu[8], nr[8];
    int cntq = 0;
    for (int i = threadIdx.x; i < nf; i += blockDim.x, ++cntq) {
      double al = 0.0, ga = 0.0;
      double li = l[i], di = d[i], ui = u[i], ri = r[i];
      double lo = 0.0, uo = 0.0, ro = 0.0, dd = di;
      if (i - s >= 0) { al = -li / d[i - s]; lo = al * l[i - s]; dd += al * u[i - s]; ro += al * r[i - s]; }
      if (i + s < nf) { ga = -ui / d[i + s]; uo = ga * u[i + s]; dd += ga * l[i + s]; ro += ga * r[i + s]; }
      nl[cntq] = lo; nd[cntq] = dd; nu[cntq] = uo; nr[cntq] = ri + ro;
    }
    __syncthreads();
    cntq = 0;
    for (int i = threadIdx.x; i < nf; i += blockDim.x, ++cntq) { l[i] = nl[cntq]; d[i] = nd[cntq]; u[i] = nu[cntq]; r[i] = nr[cntq]; }
    __syncthreads();
  }
  double dummy = 1.0 - (k.sigma * k.bst + 1.0) * exp(-k.bst * k.sigma);
  dummy = dummy / k.bst / k.bst;
  for (int i = threadIdx.x; i < nf; i += blockDim.x) V[i] = r[i] / d[i] - nj(i) * dummy;
}

int launch_long_range(Session& s) {
  const int mode = s.cfg.long_range;
  if (mode != MCPM_LR_DIRECT && mode != MCPM_LR_SCREENED_POISSON) return 0;
  const int nf = s.k.N1 + 1;
  double* V = s.faces;
  double* qoff = s.faces + nf;          // 2500
  double* qw = s.faces + nf + 2500;     // 2500
  int n = 0;
  if (mode == MCPM_LR_DIRECT) {
    k_face_quad<<<(nf * 32 + 127) / 128, 128, 0, s.stream>>>(s.k, s.cell, qoff, qw, V, nf, 0, 1);
    ++n;
    k_face_force<<<(s.k.N1 + 127) / 128, 128, 0, s.stream>>>(s.k, s.cell, s.prec == MCPM_FP32 ? s.pcell : nullptr, V, s.cfg.phi);
    ++n;
  } else {
    // the two wall values, then the PCR solve
    k_face_quad<<<1, 64, 0, s.stream>>>(s.k, s.cell, qoff, qw, V, 2, 0, nf - 1);
    ++n;
    k_poisson_pcr<<<1, 1024, 4 * nf * sizeof(double), s.stream>>>(s.k, s.cell, V, nf);
    ++n;
    k_face_force<<<(s.k.N1 + 127) / 128, 128, 0, s.stream>>>(s.k, s.cell, s.prec == MCPM_FP32 ? s.pcell : nullptr, V, s.cfg.ast);
    ++n;
  }
  return n;
}

// host-side table upload for the session (called at creation)
int long_range_setup(Session& s) {
  const int mode = s.cfg.long_range;
  if (mode != MCPM_LR_DIRECT && mode != MCPM_LR_SCREENED_POISSON) return 0;
  std::vector<double> off, w;
  build_quad(s, mode, off, w);
  const int nf = s.k.N1 + 1;
  cudaMemcpy(s.faces + nf, off.data(), 2500 * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(s.faces + nf + 2500, w.data(), 2500 * sizeof(double), cudaMemcpyHostToDevice);
  return 0;
}

cudaError_t pcr_set_smem(int nf) {
  return cudaFuncSetAttribute(k_poisson_pcr, cudaFuncAttributeMaxDynamicSharedMemorySize, 4 * nf * (int)sizeof(double));
}

}  // namespace mcpm
