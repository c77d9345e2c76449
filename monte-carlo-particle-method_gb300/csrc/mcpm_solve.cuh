// mcpm_solve.cuh -- the per-cell FP64 solves of cell_update (moment
// finalisation, Lambda, alpha/beta, c/gamma, the Velocity_FP_parallel
// constants and the FP32 sessions' packed record), shared by two
// translation units: mcpm_kernels.cu instantiates the exact variant
// (compiled with --fmad=false: every multiply and add rounds separately,
// as in the reference) and mcpm_solve_fast.cu the FP32 sessions' variant
// (compiled with --fmad=true, so that its multiply-adds contract into FP64
// fused multiply-adds: the kernel is bound by GB300's FP64 pipe).
#pragma once

#include "mcpm_device.cuh"

namespace mcpm {

// ===================================================== per-cell solves
// Gauss_Jordan, src/Math_Func.cpp:165-232, restated exactly: scaled partial
// pivoting over the full row, reciprocal-then-multiply factor, full-row
// updates, back substitution.
// maxx_magnittude (src/Math_Func.cpp:107-119): first index of the largest
// |a_i|.  For non-NaN doubles |x| orders like the integer value of its bits
// with the sign cleared, so the comparisons run on the integer pipe; NaN
// entries never win a comparison, and a NaN a[0] makes every comparison
// false (index 0), as in the reference.
__device__ __forceinline__ unsigned long long absbits(double x) {
  return (unsigned long long)__double_as_longlong(x) & 0x7FFFFFFFFFFFFFFFull;
}
__device__ __forceinline__ int gj_maxmag(const double* a, int n) {
  const unsigned long long INF = 0x7FF0000000000000ull;
  unsigned long long b = absbits(a[0]);
  if (b > INF) return 0;
  int l = 0;
  for (int i = 0; i < n; ++i) {
    unsigned long long v = absbits(a[i]);
    if (v <= INF && b < v) { b = v; l = i; }
  }
  return l;
}
template <int n>
__device__ void gauss_jordan(double* A, double* R, double* x) {
  double z[n];
  for (int i = 0; i < n - 1; ++i) {
    for (int ii = 0; ii < n; ++ii) z[ii] = 0.0;
    int k = 0;
    for (int j = i; j < n; ++j) {
      const double* row = &A[j * n];
      int bb = gj_maxmag(row, n);
      z[k] = fabs(row[i]) / fabs(row[bb]);
      k++;
    }
    k = gj_maxmag(z, n);
    k = i + k;
    if (i != k && k < n) {
      for (int j = 0; j < n; ++j) { double b = A[i * n + j]; A[i * n + j] = A[k * n + j]; A[k * n + j] = b; }
      double c = R[i]; R[i] = R[k]; R[k] = c;
    }
    const double rinv = 1.0 / A[i * n + i];
    for (int j = i + 1; j < n; ++j) {
      double F = rinv * A[j * n + i];
      for (int kk = 0; kk < n; ++kk) A[j * n + kk] = A[j * n + kk] - F * A[i * n + kk];
      R[j] = R[j] - F * R[i];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double a = 0;
    for (int j = i + 1; j < n; ++j) a = a + A[i * n + j] * x[j];
    x[i] = (R[i] - a) / (A[i * n + i]);
  }
}

// Gauss-Jordan for the FP32 path's per-cell solve (still FP64): partial
// pivoting on |A[j][i]|, reciprocal of the pivot, FMA elimination of the
// columns right of the pivot only.  Same precision class as the reference's
// solve at about a third of its FP64 instruction count.
template <int n>
__device__ void gauss_jordan_fast(double* A, double* R, double* x) {
  const unsigned long long INF = 0x7FF0000000000000ull;
  double rinv[n];
  for (int i = 0; i < n; ++i) {
    int k = i;
    unsigned long long b = absbits(A[i * n + i]);
    for (int j = i + 1; j < n; ++j) {
      unsigned long long v = absbits(A[j * n + i]);
      if (v <= INF && v > b) { b = v; k = j; }
    }
    if (k != i) {
      for (int j = i; j < n; ++j) { double t = A[i * n + j]; A[i * n + j] = A[k * n + j]; A[k * n + j] = t; }
      double t = R[i]; R[i] = R[k]; R[k] = t;
    }
    const double r = 1.0 / A[i * n + i];
    rinv[i] = r;
    for (int j = i + 1; j < n; ++j) {
      const double F = r * A[j * n + i];
      for (int kk = i + 1; kk < n; ++kk) A[j * n + kk] = fma(-F, A[i * n + kk], A[j * n + kk]);
      R[j] = fma(-F, R[i], R[j]);
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double a = R[i];
    for (int j = i + 1; j < n; ++j) a = fma(-A[i * n + j], x[j], a);
    x[i] = a * rinv[i];
  }
}

// The FP32 sessions' alpha/beta: the three 4x4 systems [P v_b; u^T d]
// (v_b = m3_b (1, 1, 1), u = (m3_a, m3_b, m3_c)) share the 3x3 block P, so
// they are solved by block elimination with one inverse of P (the pressure
// tensor, symmetric positive definite: its adjugate over its determinant):
// be_b = (s_b - u.P^-1 r_b) / (d - m3_b u.P^-1 e), al_b = P^-1 r_b - m3_b be_b P^-1 e.
// False (the caller then runs the pivoting solve) when P or a Schur
// complement is degenerate.
__device__ __forceinline__ bool ab_blocks(const double* P, const double* m3, double d, const double* rhs,
                                          double* al, double* be) {
  const double c00 = P[3] * P[5] - P[4] * P[4], c01 = P[2] * P[4] - P[1] * P[5], c02 = P[1] * P[4] - P[2] * P[3];
  const double c11 = P[0] * P[5] - P[2] * P[2], c12 = P[1] * P[2] - P[0] * P[4], c22 = P[0] * P[3] - P[1] * P[1];
  const double det = P[0] * c00 + P[1] * c01 + P[2] * c02;
  if (!(det > 0.0) || !isfinite(det)) return false;
  const double id = 1.0 / det;
  const double i00 = c00 * id, i01 = c01 * id, i02 = c02 * id, i11 = c11 * id, i12 = c12 * id, i22 = c22 * id;
  const double ye0 = i00 + i01 + i02, ye1 = i01 + i11 + i12, ye2 = i02 + i12 + i22;
  const double ue = m3[0] * ye0 + m3[1] * ye1 + m3[2] * ye2;
  for (int b = 0; b < 3; ++b) {
    const double r0 = rhs[3 * b], r1 = rhs[3 * b + 1], r2 = rhs[3 * b + 2];
    const double y0 = i00 * r0 + i01 * r1 + i02 * r2;
    const double y1 = i01 * r0 + i11 * r1 + i12 * r2;
    const double y2 = i02 * r0 + i12 * r1 + i22 * r2;
    const double den = d - m3[b] * ue;
    if (!(fabs(den) > 1e-12 * (fabs(d) + fabs(m3[b] * ue)))) return false;
    const double bb = (rhs[9 + b] - (m3[0] * y0 + m3[1] * y1 + m3[2] * y2)) / den;
    const double f = m3[b] * bb;
    al[3 * b] = y0 - f * ye0;
    al[3 * b + 1] = y1 - f * ye1;
    al[3 * b + 2] = y2 - f * ye2;
    be[b] = bb;
  }
  for (int j = 0; j < 9; ++j) if (!isfinite(al[j])) return false;
  for (int j = 0; j < 3; ++j) if (!isfinite(be[j])) return false;
  return true;
}

// The FP32 sessions' c/gamma (the 9x9 system of src/Fokker_Planck.cpp:590-804)
// by mixed-precision iterative refinement: an LU factorisation of the
// matrix in FP32 (no pivoting: rows 0..5 are the operator c -> P c + c P of
// the positive definite P, rows 6..8 are dominated by their diagonal), then
// residuals b - A x in FP64 with FP32 corrections until the last correction
// is below 1e-13 of the solution -- the FP64 solution, at a fraction of the
// FP64 operations of an FP64 elimination (GB300's FP64 pipe bounds this
// kernel).  False after three corrections without convergence, or on a zero
// or non-finite pivot: the caller then runs the FP64 elimination.
static __device__ __noinline__ bool cg_refined(const double* P, const double* Q, const double* M3, const double* M4,
                                        double DM2, double DM4, const double* b, double* x) {
  const double E = DM4 - DM2 * DM2;
  // rows 6..8 of the matrix in FP64 (rows 0..5 are entries of P and Q)
  double G[27];
  G[0] = Q[0] + 2.0 * M3[0]; G[1] = Q[1] + 4.0 * M3[1]; G[2] = Q[2] + 4.0 * M3[2];
  G[3] = 2.0 * M3[3]; G[4] = 4.0 * M3[4]; G[5] = 2.0 * M3[5];
  G[6] = 2.0 * M4[0] - 2.0 * P[0] * DM2 + E; G[7] = 2.0 * M4[1] - 2.0 * P[1] * DM2;
  G[8] = 2.0 * M4[2] - 2.0 * P[2] * DM2;
  G[9] = 2.0 * M3[1]; G[10] = Q[0] + 4.0 * M3[3]; G[11] = 4.0 * M3[4];
  G[12] = Q[1] + 2.0 * M3[6]; G[13] = Q[2] + 4.0 * M3[7]; G[14] = 2.0 * M3[8];
  G[15] = G[7]; G[16] = 2.0 * M4[3] - 2.0 * P[3] * DM2 + E; G[17] = 2.0 * M4[4] - 2.0 * P[4] * DM2;
  G[18] = 2.0 * M3[2]; G[19] = 4.0 * M3[4]; G[20] = Q[0] + 4.0 * M3[5];
  G[21] = 2.0 * M3[7]; G[22] = Q[1] + 4.0 * M3[8]; G[23] = Q[2] + 2.0 * M3[9];
  G[24] = G[8]; G[25] = G[17]; G[26] = 2.0 * M4[5] - 2.0 * P[5] * DM2 + E;
  const double s03 = P[0] + P[3], s05 = P[0] + P[5], s35 = P[3] + P[5];
  // y = A v in FP64, the rows' nonzeros only
  auto mul = [&](const double* v, double* y) {
    y[0] = 2.0 * (P[0] * v[0] + P[1] * v[1] + P[2] * v[2] + Q[0] * v[6]);
    y[1] = P[1] * v[0] + s03 * v[1] + P[4] * v[2] + P[1] * v[3] + P[2] * v[4] + Q[1] * v[6] + Q[0] * v[7];
    y[2] = P[2] * v[0] + P[4] * v[1] + s05 * v[2] + P[1] * v[4] + P[2] * v[5] + Q[2] * v[6] + Q[0] * v[8];
    y[3] = 2.0 * (P[1] * v[1] + P[3] * v[3] + P[4] * v[4] + Q[1] * v[7]);
    y[4] = P[2] * v[1] + P[1] * v[2] + P[4] * v[3] + s35 * v[4] + P[4] * v[5] + Q[2] * v[7] + Q[1] * v[8];
    y[5] = 2.0 * (P[2] * v[2] + P[4] * v[4] + P[5] * v[5] + Q[2] * v[8]);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      double a = 0.0;
#pragma unroll
      for (int q = 0; q < 9; ++q) a += G[9 * r + q] * v[q];
      y[6 + r] = a;
    }
  };
  // the FP32 matrix, factorised in place (unit lower L below the diagonal,
  // U on and above it, the diagonal holding 1 / U_ii)
  float L[81];
#pragma unroll
  for (int j = 0; j < 81; ++j) L[j] = 0.f;
  const float p0 = (float)P[0], p1 = (float)P[1], p2 = (float)P[2], p3 = (float)P[3], p4 = (float)P[4],
              p5 = (float)P[5], q0 = (float)Q[0], q1 = (float)Q[1], q2 = (float)Q[2];
  L[0] = 2.f * p0; L[1] = 2.f * p1; L[2] = 2.f * p2; L[6] = 2.f * q0;
  L[9] = p1; L[10] = p0 + p3; L[11] = p4; L[12] = p1; L[13] = p2; L[15] = q1; L[16] = q0;
  L[18] = p2; L[19] = p4; L[20] = p0 + p5; L[22] = p1; L[23] = p2; L[24] = q2; L[26] = q0;
  L[28] = 2.f * p1; L[30] = 2.f * p3; L[31] = 2.f * p4; L[34] = 2.f * q1;
  L[37] = p2; L[38] = p1; L[39] = p4; L[40] = p3 + p5; L[41] = p4; L[43] = q2; L[44] = q1;
  L[47] = 2.f * p2; L[49] = 2.f * p4; L[50] = 2.f * p5; L[53] = 2.f * q2;
#pragma unroll
  for (int j = 0; j < 27; ++j) L[54 + j] = (float)G[j];
#pragma unroll
  for (int i = 0; i < 9; ++i) {
    const float piv = L[i * 9 + i];
    if (!(fabsf(piv) > 0.f) || !isfinite(piv)) return false;
    const float inv = 1.0f / piv;
    L[i * 9 + i] = inv;
#pragma unroll
    for (int j = i + 1; j < 9; ++j) {
      const float f = L[j * 9 + i] * inv;
      L[j * 9 + i] = f;
#pragma unroll
      for (int q = i + 1; q < 9; ++q) L[j * 9 + q] = fmaf(-f, L[i * 9 + q], L[j * 9 + q]);
    }
  }
  auto lusolve = [&](float* v) {
#pragma unroll
    for (int i = 1; i < 9; ++i) {
      float a = v[i];
#pragma unroll
      for (int j = 0; j < i; ++j) a = fmaf(-L[i * 9 + j], v[j], a);
      v[i] = a;
    }
#pragma unroll
    for (int i = 8; i >= 0; --i) {
      float a = v[i];
#pragma unroll
      for (int j = i + 1; j < 9; ++j) a = fmaf(-L[i * 9 + j], v[j], a);
      v[i] = a * L[i * 9 + i];
    }
  };
  float v[9];
#pragma unroll
  for (int i = 0; i < 9; ++i) v[i] = (float)b[i];
  lusolve(v);
#pragma unroll
  for (int i = 0; i < 9; ++i) x[i] = (double)v[i];
  for (int it = 0; it < 3; ++it) {
    double ax[9];
    mul(x, ax);
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = (float)(b[i] - ax[i]);
    lusolve(v);
    float dmax = 0.f;
    double xmax = 0.0;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
      x[i] += (double)v[i];
      dmax = fmaxf(dmax, fabsf(v[i]));
      xmax = fmax(xmax, fabs(x[i]));
    }
    if (!isfinite(xmax)) return false;
    if ((double)dmax <= 1e-13 * xmax) return true;
  }
  return false;
}

// One thread per cell: Lambda (src/Main_Functions.cpp:2718-2728),
// alpha/beta (src/Fokker_Planck.cpp:200-587; its 12x12 system is three
// uncoupled 4x4 blocks -- unknowns (alpha_3b..3b+2, beta_b) -- and Gauss_Jordan
// on the 12x12 performs exactly the arithmetic of the three 4x4 solves),
// c/gamma (src/Fokker_Planck.cpp:590-804, 9x9), phi (:2734-2746) and the
// Velocity_FP_parallel constants A1..A3 (src/Fokker_Planck.cpp:1099-1112).
// Launch shape of the per-cell solves: threads per block and blocks resident
// per SM (the register budget).
#ifndef MCPM_SOLVE_T
#define MCPM_SOLVE_T 128
#endif
#ifndef MCPM_SOLVE_MINB
#define MCPM_SOLVE_MINB 1
#endif
template <bool EXACT>
__global__ void __launch_bounds__(MCPM_SOLVE_T, MCPM_SOLVE_MINB)
    k_solve(DevConsts k, double* cell, float* pcell, int with_alpha, int fp_model, uint32_t* status) {
  const int C = k.C;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= C) return;
  auto R = [&](int f) -> double { return cell[(size_t)f * C + c]; };
  auto Rc = [&](int f, int cc) -> double { return cell[(size_t)f * C + cc]; };
  auto W = [&](int f, double v) { cell[(size_t)f * C + c] = v; };
  const double weight = R(MCPM_CF_NUM_INSIDE);
  const int ncnt = (int)weight;
  // ---- moment finalisation, src/Main_Functions.cpp:2563-2593
  double P[6], M3[10], M4[6], M5[3], Q[3] = {0.0, 0.0, 0.0}, Mp[3], DM2, DM4 = 0.0;
  for (int j = 0; j < 3; ++j) Mp[j] = R(CFI_RAW + j);
  for (int j = 0; j < 6; ++j) P[j] = R(CFI_RAW + 3 + j);
  for (int j = 0; j < 10; ++j) M3[j] = R(CFI_RAW + 9 + j);
  for (int j = 0; j < 6; ++j) M4[j] = R(CFI_RAW + 19 + j);
  for (int j = 0; j < 3; ++j) M5[j] = R(CFI_RAW + 25 + j);
  DM2 = R(CFI_RAW + 28);
  if (ncnt > 0) {
    if (EXACT) {
      for (int j = 0; j < 6; ++j) P[j] = P[j] / weight;
      for (int j = 0; j < 10; ++j) M3[j] = M3[j] / weight;
      for (int j = 0; j < 6; ++j) M4[j] = M4[j] / weight;
      for (int j = 0; j < 3; ++j) M5[j] = M5[j] / weight;
      for (int j = 0; j < 3; ++j) Mp[j] = Mp[j] / weight;
      DM2 = DM2 / weight;
    } else {
      const double rw = 1.0 / weight;
      for (int j = 0; j < 6; ++j) P[j] *= rw;
      for (int j = 0; j < 10; ++j) M3[j] *= rw;
      for (int j = 0; j < 6; ++j) M4[j] *= rw;
      for (int j = 0; j < 3; ++j) M5[j] *= rw;
      for (int j = 0; j < 3; ++j) Mp[j] *= rw;
      DM2 *= rw;
    }
    DM4 = M4[0] + M4[3] + M4[5];
    Q[0] = M3[0] + M3[3] + M3[5];
    Q[1] = M3[1] + M3[6] + M3[8];
    Q[2] = M3[2] + M3[7] + M3[9];
  }
  for (int j = 0; j < 6; ++j) W(MCPM_CF_PIJ + j, P[j]);
  for (int j = 0; j < 10; ++j) W(MCPM_CF_M3 + j, M3[j]);
  for (int j = 0; j < 6; ++j) W(MCPM_CF_M4 + j, M4[j]);
  for (int j = 0; j < 3; ++j) W(MCPM_CF_M5 + j, M5[j]);
  for (int j = 0; j < 3; ++j) W(MCPM_CF_Q + j, Q[j]);
  for (int j = 0; j < 3; ++j) W(MCPM_CF_MP + j, Mp[j]);
  W(MCPM_CF_DM2, DM2);
  W(MCPM_CF_DM4, DM4);
  // (the FP32 sessions' variant multiplies by quotients formed once, where
  // the reference divides)
  const double T = EXACT ? k.m * DM2 / (3.0 * k.kb) : DM2 * k.q_T;
  const double n = (k.cell_w ? k.cell_w[c] : 1) * k.Fn * weight / cell_volume(c, k);
  const double iT = EXACT ? 0.0 : 1.0 / T;
  double Ycell;
  if (EXACT) {
    Ycell = ycoll(n, k.b);
  } else {
    const double nb = n * k.b;
    Ycell = 1.0 + nb * (0.625 + nb * (0.2869 + 0.115 * nb));
  }
  W(MCPM_CF_T, T);
  W(MCPM_CF_N, n);
  W(CFI_Y, Ycell);
  // scale_mu(T) (src/Main_Functions.cpp:1970-1973), which the reference
  // evaluates again for Lambda, the c/gamma rhs and the FP constants: once
  const double mu_T = scale_mu(T, k);
  double gst = R(MCPM_CF_GAMMA_ST);
  if (weight > 1e-14) {
    gst = EXACT ? -0.001 * (n * k.b * Ycell / (k.kb * T / k.m)) : -0.001 * (n * k.b * Ycell) * (k.q_m_kb * iT);
    W(MCPM_CF_GAMMA_ST, gst);
  }
  uint32_t bad = 0;
  double Lam = R(MCPM_CF_LAMBDA);
  if (weight > 1e-14) {
    const double mu = mu_T;
    if (EXACT) {
      double tau = 2.0 * mu / (n * k.kb * T);
      double L = (P[0] - DM2 / 3.0) * ((P[3] - DM2 / 3.0) * (P[5] - DM2 / 3.0) - P[4] * P[4]);
      L = L - P[1] * (P[1] * (P[5] - DM2 / 3.0) - P[4] * P[2]);
      L = L + P[2] * (P[1] * P[4] - P[2] * (P[3] - DM2 / 3.0));
      L = -L / (tau * pow(DM2, 4.0));
      Lam = L;
    } else {
      // -det(P - DM2/3) / (tau DM2^4), 1/tau = n kb T / (2 mu)
      const double d3 = DM2 * (1.0 / 3.0);
      const double a0 = P[0] - d3, a3 = P[3] - d3, a5 = P[5] - d3;
      double L = a0 * (a3 * a5 - P[4] * P[4]);
      L = L - P[1] * (P[1] * a5 - P[4] * P[2]);
      L = L + P[2] * (P[1] * P[4] - P[2] * a3);
      const double iD = 1.0 / DM2, iD2 = iD * iD;
      Lam = -L * (n * k.kb * T / (2.0 * mu)) * (iD2 * iD2);
    }
    W(MCPM_CF_LAMBDA, Lam);
  }
  double al[9], be[3];
  for (int j = 0; j < 9; ++j) al[j] = R(MCPM_CF_ALPHA + j);
  for (int j = 0; j < 3; ++j) be[j] = R(MCPM_CF_BETA + j);
  if (fp_model) {
    // ---------------- alpha / beta (FP_dense, step > 0)
    if (with_alpha) {
      if (ncnt < 2) {
        for (int j = 0; j < 9; ++j) al[j] = 0.0;
        for (int j = 0; j < 3; ++j) be[j] = 0.0;
      } else {
        const double pi = 3.141592653589793;  // acos(-1.0), correctly rounded
        double trace = P[0] + P[3] + P[5];
        double dev[6];
        for (int j = 0; j < 6; ++j) dev[j] = P[j];
        dev[0] = dev[0] - (1.0 / 3.0) * trace;
        dev[3] = dev[3] - (1.0 / 3.0) * trace;
        dev[5] = dev[5] - (1.0 / 3.0) * trace;
        double ma = M3[0] + M3[3] + M3[5];
        double mb = M3[1] + M3[6] + M3[8];
        double mc = M3[2] + M3[7] + M3[9];
        double d = M4[0] + M4[3] + M4[5] - DM2 * DM2;
        double Y = Ycell;
        double p_crr = (1.0 + n * k.b * Y);
        double mu_crr = (1.0 + 2.0 * n * k.b * Y / 5.0);
        double k_crr = (1.0 + 3.0 * n * k.b * Y / 5.0);
        double w;
        if (EXACT) {
          w = (4.0 / 9.0) * sqrt(pi) * Y * (n * n) * pow(k.sigma, 4.0) * sqrt(k.m * k.kb * T);
        } else {
          const double s2 = k.sigma * k.sigma;
          w = (4.0 / 9.0) * 1.7724538509055159 * Y * (n * n) * (s2 * s2) * sqrt(k.m * k.kb * T);
        }
        double div_U;
        const int last = C - 1;
        if (EXACT) {
          if (C == 1) div_U = 0.0;
          else if (c == 0) div_U = (Rc(MCPM_CF_U_SPACE + 1, c + 1) - Rc(MCPM_CF_U_SPACE + 1, c)) / k.dy;
          else if (c == k.N1 - 1 || c == last)
            div_U = (Rc(MCPM_CF_U_SPACE + 1, c) - Rc(MCPM_CF_U_SPACE + 1, c - 1)) / k.dy;
          else div_U = (Rc(MCPM_CF_U_SPACE + 1, c + 1) - Rc(MCPM_CF_U_SPACE + 1, c - 1)) / k.dy / 2.0;
        } else {
          if (C == 1) div_U = 0.0;
          else if (c == 0) div_U = (Rc(MCPM_CF_U_SPACE + 1, c + 1) - Rc(MCPM_CF_U_SPACE + 1, c)) * k.q_idy;
          else if (c == k.N1 - 1 || c == last)
            div_U = (Rc(MCPM_CF_U_SPACE + 1, c) - Rc(MCPM_CF_U_SPACE + 1, c - 1)) * k.q_idy;
          else div_U = (Rc(MCPM_CF_U_SPACE + 1, c + 1) - Rc(MCPM_CF_U_SPACE + 1, c - 1)) * (0.5 * k.q_idy);
        }
        W(MCPM_CF_DIVU, div_U);
        double nbY = n * k.b * Y;
        double rhs[12];
        if (!EXACT) {
          // the same terms with the common factors formed once and one
          // division for the two transport corrections:
          // coeff_mu = 0.6012 x^2 / (1 + 0.4 x), coeff_k = 0.2004 x^2 / (1 + 0.6 x)
          const double x2 = nbY * nbY, dmu = 1.0 + 0.4 * nbY, dk = 1.0 + 0.6 * nbY;
          const double id = 1.0 / (dmu * dk);
          const double coeff_mu = (3.0 * 1.002 / 5.0) * x2 * (dk * id), coeff_k = (1.002 / 5.0) * x2 * (dmu * id);
          // w div_U / (m n) with w's factor n^2 cancelled
          const double s2 = k.sigma * k.sigma;
          const double wmn = (4.0 / 9.0) * 1.7724538509055159 * Y * n * (s2 * s2) * sqrt(k.m * k.kb * T) * k.q_im;
          const double pt3 = nbY * trace * (1.0 / 3.0) - wmn * div_U;
          const double cm = 0.4 * nbY + coeff_mu, ck = 0.6 * nbY + coeff_k;
          rhs[0] = cm * dev[0] + pt3 - gst * M4[0];
          rhs[1] = cm * dev[1] - gst * M4[1];
          rhs[2] = cm * dev[2] - gst * M4[2];
          rhs[3] = rhs[1];
          rhs[4] = cm * dev[3] + pt3 - gst * M4[3];
          rhs[5] = cm * dev[4] - gst * M4[4];
          rhs[6] = rhs[2];
          rhs[7] = rhs[5];
          rhs[8] = cm * dev[5] + pt3 - gst * M4[5];
          rhs[9] = ck * ma - gst * M5[0] + gst * (DM2 * ma);
          rhs[10] = ck * mb - gst * M5[1] + gst * (DM2 * mb);
          rhs[11] = ck * mc - gst * M5[2] + gst * (DM2 * mc);
        } else {
        double coeff_mu = 3.0 * 1.002 / 5.0 * (nbY * nbY) / (1 + 2.0 * n * k.b * Y / 5.0);
        double coeff_k = 1.002 * (nbY * nbY) / (1 + 3.0 * n * k.b * Y / 5.0) / 5.0;
        rhs[0] = (mu_crr - 1.0) * dev[0] + (p_crr - 1.0) * trace / 3.0 - w * div_U / (k.m * n) + coeff_mu * dev[0] - gst * M4[0];
        rhs[1] = (mu_crr - 1.0) * dev[1] + coeff_mu * dev[1] - gst * M4[1];
        rhs[2] = (mu_crr - 1.0) * dev[2] + coeff_mu * dev[2] - gst * M4[2];
        rhs[3] = (mu_crr - 1.0) * dev[1] + coeff_mu * dev[1] - gst * M4[1];
        rhs[4] = (mu_crr - 1.0) * dev[3] + (p_crr - 1.0) * trace / 3.0 - w * div_U / (k.m * n) + coeff_mu * dev[3] - gst * M4[3];
        rhs[5] = (mu_crr - 1.0) * dev[4] + coeff_mu * dev[4] - gst * M4[4];
        rhs[6] = (mu_crr - 1.0) * dev[2] + coeff_mu * dev[2] - gst * M4[2];
        rhs[7] = (mu_crr - 1.0) * dev[4] + coeff_mu * dev[4] - gst * M4[4];
        rhs[8] = (mu_crr - 1.0) * dev[5] + (p_crr - 1.0) * trace / 3.0 - w * div_U / (k.m * n) + coeff_mu * dev[5] - gst * M4[5];
        rhs[9] = (k_crr - 1.0) * ma + coeff_k * ma - gst * (M5[0]) + gst * (DM2 * (M3[0] + M3[3] + M3[5]));
        rhs[10] = (k_crr - 1.0) * mb + coeff_k * mb - gst * (M5[1]) + gst * (DM2 * (M3[1] + M3[6] + M3[8]));
        rhs[11] = (k_crr - 1.0) * mc + coeff_k * mc - gst * (M5[2]) + gst * (DM2 * (M3[2] + M3[7] + M3[9]));
        }
        const double m3b[3] = {ma, mb, mc};
        const bool blocks = !EXACT && ab_blocks(P, m3b, d, rhs, al, be);
        for (int blk = 0; blk < 3 && !blocks; ++blk) {
          double A[16], r4[4], x4[4];
          A[0] = P[0]; A[1] = P[1]; A[2] = P[2]; A[3] = m3b[blk];
          A[4] = P[1]; A[5] = P[3]; A[6] = P[4]; A[7] = m3b[blk];
          A[8] = P[2]; A[9] = P[4]; A[10] = P[5]; A[11] = m3b[blk];
          A[12] = ma; A[13] = mb; A[14] = mc; A[15] = d;
          r4[0] = rhs[3 * blk]; r4[1] = rhs[3 * blk + 1]; r4[2] = rhs[3 * blk + 2]; r4[3] = rhs[9 + blk];
          if (EXACT) gauss_jordan<4>(A, r4, x4);
          else gauss_jordan_fast<4>(A, r4, x4);
          al[3 * blk] = x4[0]; al[3 * blk + 1] = x4[1]; al[3 * blk + 2] = x4[2]; be[blk] = x4[3];
        }
        for (int j = 0; j < 9; ++j) if (al[j] != al[j]) bad |= MCPM_ERR_NAN;
        for (int j = 0; j < 3; ++j) if (be[j] != be[j]) bad |= MCPM_ERR_NAN;
      }
      for (int j = 0; j < 9; ++j) W(MCPM_CF_ALPHA + j, al[j]);
      for (int j = 0; j < 3; ++j) W(MCPM_CF_BETA + j, be[j]);
    }
    // ---------------- c / gamma
    double x[9];
    if (ncnt < 2) {
      for (int j = 0; j < 9; ++j) x[j] = 0.0;
    } else {
      double rhs[9];
      for (int j = 0; j < 9; ++j) { rhs[j] = 0.0; x[j] = 0.0; }
      double Pr = 2.0 / 3.0;
      double Y = (k.model == MCPM_MODEL_FP_DENSE) ? Ycell : 1.0;
      const double mu = mu_T;
      for (int j = 0; j < 6; ++j) rhs[j] = -2.0 * Lam * M4[j];
      if (EXACT) {
        double tau = 2.0 * mu / (n * k.kb * T);
        rhs[6] = Y * (3.0 / tau - 2.0 * Pr / tau) * Q[0];
        rhs[7] = Y * (3.0 / tau - 2.0 * Pr / tau) * Q[1];
        rhs[8] = Y * (3.0 / tau - 2.0 * Pr / tau) * Q[2];
      } else {
        const double f = Y * (3.0 - 2.0 * Pr) * (n * k.kb * T / (2.0 * mu));  // Y (3 - 2 Pr) / tau
        rhs[6] = f * Q[0]; rhs[7] = f * Q[1]; rhs[8] = f * Q[2];
      }
      rhs[6] += Lam * (-3.0 * M5[0] + DM2 * Q[0] + 2.0 * (P[0] * Q[0] + P[1] * Q[1] + P[2] * Q[2]));
      rhs[7] += Lam * (-3.0 * M5[1] + DM2 * Q[1] + 2.0 * (P[1] * Q[0] + P[3] * Q[1] + P[4] * Q[2]));
      rhs[8] += Lam * (-3.0 * M5[2] + DM2 * Q[2] + 2.0 * (P[2] * Q[0] + P[4] * Q[1] + P[5] * Q[2]));
      if (EXACT || !cg_refined(P, Q, M3, M4, DM2, DM4, rhs, x)) {
        double A[81];
        for (int j = 0; j < 81; ++j) A[j] = 0.0;
#define AA(r, q) A[(r) * 9 + (q)]
        AA(0, 0) = 2.0 * P[0]; AA(0, 1) = 2.0 * P[1]; AA(0, 2) = 2.0 * P[2]; AA(0, 6) = 2.0 * Q[0];
        AA(1, 0) = P[1]; AA(1, 1) = P[0] + P[3]; AA(1, 2) = P[4]; AA(1, 3) = P[1]; AA(1, 4) = P[2];
        AA(1, 6) = Q[1]; AA(1, 7) = Q[0];
        AA(2, 0) = P[2]; AA(2, 1) = P[4]; AA(2, 2) = P[0] + P[5]; AA(2, 4) = P[1]; AA(2, 5) = P[2];
        AA(2, 6) = Q[2]; AA(2, 8) = Q[0];
        AA(3, 1) = 2.0 * P[1]; AA(3, 3) = 2.0 * P[3]; AA(3, 4) = 2.0 * P[4]; AA(3, 7) = 2.0 * Q[1];
        AA(4, 1) = P[2]; AA(4, 2) = P[1]; AA(4, 3) = P[4]; AA(4, 4) = P[3] + P[5]; AA(4, 5) = P[4];
        AA(4, 7) = Q[2]; AA(4, 8) = Q[1];
        AA(5, 2) = 2.0 * P[2]; AA(5, 4) = 2.0 * P[4]; AA(5, 5) = 2.0 * P[5]; AA(5, 8) = 2.0 * Q[2];
        AA(6, 0) = Q[0] + 2.0 * M3[0]; AA(6, 1) = Q[1] + 4.0 * M3[1]; AA(6, 2) = Q[2] + 4.0 * M3[2];
        AA(6, 3) = 2.0 * M3[3]; AA(6, 4) = 4.0 * M3[4]; AA(6, 5) = 2.0 * M3[5];
        AA(6, 6) = 2.0 * M4[0] - 2.0 * P[0] * DM2; AA(6, 7) = 2.0 * M4[1] - 2.0 * P[1] * DM2;
        AA(6, 8) = 2.0 * M4[2] - 2.0 * P[2] * DM2;
        AA(7, 0) = 2.0 * M3[1]; AA(7, 1) = Q[0] + 4.0 * M3[3]; AA(7, 2) = 4.0 * M3[4];
        AA(7, 3) = Q[1] + 2.0 * M3[6]; AA(7, 4) = Q[2] + 4.0 * M3[7]; AA(7, 5) = 2.0 * M3[8];
        AA(7, 6) = 2.0 * M4[1] - 2.0 * P[1] * DM2; AA(7, 7) = 2.0 * M4[3] - 2.0 * P[3] * DM2;
        AA(7, 8) = 2.0 * M4[4] - 2.0 * P[4] * DM2;
        AA(8, 0) = 2.0 * M3[2]; AA(8, 1) = 4.0 * M3[4]; AA(8, 2) = Q[0] + 4.0 * M3[5];
        AA(8, 3) = 2.0 * M3[7]; AA(8, 4) = Q[1] + 4.0 * M3[8]; AA(8, 5) = Q[2] + 2.0 * M3[9];
        AA(8, 6) = 2.0 * M4[2] - 2.0 * P[2] * DM2; AA(8, 7) = 2.0 * M4[4] - 2.0 * P[4] * DM2;
        AA(8, 8) = 2.0 * M4[5] - 2.0 * P[5] * DM2;
        AA(6, 6) += DM4 - (DM2) * (DM2);
        AA(7, 7) += DM4 - (DM2) * (DM2);
        AA(8, 8) += DM4 - (DM2) * (DM2);
#undef AA
        if (EXACT) gauss_jordan<9>(A, rhs, x);
        else gauss_jordan_fast<9>(A, rhs, x);
      }
    }
    for (int j = 0; j < 6; ++j) W(MCPM_CF_C + j, x[j]);
    for (int j = 0; j < 3; ++j) W(MCPM_CF_GAMMA + j, x[6 + j]);
    // ---------------- Velocity_FP_parallel per-cell constants
    if (ncnt > 1) {
      const double mu = mu_T;
      double Y = (k.model == MCPM_MODEL_FP_DENSE) ? Ycell : 1.0;
      if (EXACT) {
        double tau = 2.0 * mu / (n * k.kb * T);
        tau = tau / Y;
        W(CFI_A1, exp(-k.dt / tau));
        W(CFI_A3, sqrt((1.0 - exp(-2.0 * k.dt / tau)) * k.kb * T / (1.0 * k.m)));
        W(CFI_A2, (1.0 - exp(-k.dt / tau)) * tau);
      } else {
        // the FP32 sessions' record holds these as floats: formed in float
        // (off GB300's FP64 pipe, which bounds this kernel), 1 - e^-x by
        // expm1f so that a small dt / tau keeps its digits
        const float tau = 2.0f * (float)mu / ((float)n * (float)k.kb * (float)T * (float)Y);
        const float x = (float)k.dt / tau;
        W(CFI_A1, (double)expf(-x));
        W(CFI_A3, (double)sqrtf(-expm1f(-2.0f * x) * ((float)T * (float)k.q_kb_m)));
        W(CFI_A2, (double)(-expm1f(-x) * tau));
      }
    }
  }
  // 3 kT / m (the FP32 sessions' record holds it as a float: formed in float)
  const double eq3 = EXACT ? 3.0 * k.kb * T / k.m : (double)(3.0f * (float)T * (float)k.q_kb_m);
  W(CFI_3KT, eq3);
  const double ph0 = al[0] * Mp[0] + al[1] * Mp[1] + al[2] * Mp[2];
  const double ph1 = al[3] * Mp[0] + al[4] * Mp[1] + al[5] * Mp[2];
  W(MCPM_CF_PHI + 0, ph0);
  W(MCPM_CF_PHI + 1, ph1);
  W(MCPM_CF_PHI + 2, al[6] * Mp[0] + al[7] * Mp[1] + al[8] * Mp[2]);
  if (pcell) {
    // the FP32 update kernel's per-cell record
    float* pf = pcell + (size_t)c * PF_STRIDE;
    pf[PF_US0] = (float)R(MCPM_CF_U_SPACE + 0);
    pf[PF_US1] = (float)R(MCPM_CF_U_SPACE + 1);
    pf[PF_US2] = (float)R(MCPM_CF_U_SPACE + 2);
    // Velocity_FP_linear (src/Fokker_Planck.cpp:1262-1264) has no drift:
    // its cells carry zero drift coefficients (c, gamma, Lambda stay in the
    // cell view, where cell_update computed them)
    const bool lin = k.model == MCPM_MODEL_FP_LINEAR;
    pf[PF_A1] = (float)R(CFI_A1); pf[PF_A2] = lin ? 0.f : (float)R(CFI_A2); pf[PF_A3] = (float)R(CFI_A3);
    pf[PF_EQ] = (float)eq3;
    pf[PF_LAM] = lin ? 0.f : (float)Lam;
    for (int j = 0; j < 6; ++j) pf[PF_C0 + j] = lin ? 0.f : (float)R(MCPM_CF_C + j);
    for (int j = 0; j < 3; ++j) {
      pf[PF_G0 + j] = lin ? 0.f : (float)R(MCPM_CF_GAMMA + j);
      pf[PF_Q0 + j] = (float)Q[j];
    }
    for (int j = 0; j < 6; ++j) pf[PF_AL0 + j] = (float)al[j];
    pf[PF_BE0] = (float)be[0]; pf[PF_BE1] = (float)be[1];
    pf[PF_GST] = (float)gst;
    pf[PF_HQ0] = (float)(M3[0] + M3[3] + M3[5]);
    pf[PF_HQ1] = (float)(M3[1] + M3[6] + M3[8]);
    pf[PF_PH0] = (float)ph0; pf[PF_PH1] = (float)ph1;
    pf[PF_N] = (float)ncnt;
    pf[PF_E2] = (float)R(CFI_RAW + 28);
    // Y(n) and n as floats after the records (the FP32 ESMC test reads
    // them for every candidate)
    float* yn = pcell + (size_t)PF_STRIDE * C;
    yn[c] = (float)Ycell;
    yn[C + c] = (float)n;
  }
  raise_status(status, bad);
}

}  // namespace mcpm
