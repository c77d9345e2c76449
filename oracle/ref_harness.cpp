// ref_harness.cpp -- drives the reference's own routines on caller data.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build.py together with the
// reference translation units (src/Main_Functions.cpp, src/Fokker_Planck.cpp,
// src/Math_Func.cpp, src/collisions.cpp, src/FEM.cpp, src/myIO.cpp, ...)
// straight from the reference tree into oracle/_ref/libref.so.  The reference
// is used unmodified; this file only
//   * replaces the translation unit src/random_generator.cpp with a
//     generateGaussianNoise that returns injected draws in call order, so that
//     random_generator (src/Fokker_Planck.cpp:84-90) is reproducible;
//   * supplies solver_pardiso (src/solver_pardiso.cpp needs MKL) as a dense LU
//     with partial pivoting on the CSR matrix compute_SP_2D builds;
//   * stubs dgesv, whose only caller (src/solver.cpp) is dead code;
//   * fills GAS/BOX/CELLS from an mcpm_config and exposes extern "C" calls.
#include "../include/mcpm.h"  // before the reference header: it #defines short names

#include "cpp_headers.h"

#include <fcntl.h>
#include <unistd.h>

#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

// ---------------------------------------------------------------- injected
static std::vector<double> g_inj;
static size_t g_inj_pos = 0;

double generateGaussianNoise(double mu, double sigma) {
  double z = g_inj.empty() ? 0.0 : g_inj[g_inj_pos % g_inj.size()];
  g_inj_pos++;
  return z * sigma + mu;
}

int solver_pardiso(int* ia, int* ja, double* a, int n, double* b, double* x) {
  // CSR with 1-based indices (src/FEM.cpp:120-157) -> dense, LU with partial pivoting
  std::vector<double> A((size_t)n * n, 0.0), r(b, b + n);
  for (int i = 0; i < n; ++i)
    for (int p = ia[i] - 1; p < ia[i + 1] - 1; ++p) A[(size_t)i * n + (ja[p] - 1)] = a[p];
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[(size_t)i * n + k]) > fabs(A[(size_t)piv * n + k])) piv = i;
    if (piv != k) {
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)k * n + j], A[(size_t)piv * n + j]);
      std::swap(r[k], r[piv]);
    }
    for (int i = k + 1; i < n; ++i) {
      double f = A[(size_t)i * n + k] / A[(size_t)k * n + k];
      if (f == 0.0) continue;
      for (int j = k; j < n; ++j) A[(size_t)i * n + j] -= f * A[(size_t)k * n + j];
      r[i] -= f * r[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double s = r[i];
    for (int j = i + 1; j < n; ++j) s -= A[(size_t)i * n + j] * x[j];
    x[i] = s / A[(size_t)i * n + i];
  }
  return 0;
}

extern "C" void dgesv(const int*, const int*, double*, const int*, int*, double*, const int*, int* info) {
  if (info) *info = -1;
}

// ------------------------------------------------------------- stdout gag
struct Quiet {
  int saved;
  Quiet() {
    fflush(stdout);
    saved = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    dup2(devnull, 1);
    close(devnull);
  }
  ~Quiet() {
    fflush(stdout);
    dup2(saved, 1);
    close(saved);
  }
};

struct Ref {
  GAS gas;
  BOX box;
  CELLS* cells;
  int C;
  long N;
  std::vector<double> x3, x3_old, Mp1, Mp2, Mp3, xi1, xi2, xi3, T, rho;
  std::vector<int> color, flag;
};

static const char* model_name(int m) {
  switch (m) {
    case MCPM_MODEL_FP_DENSE: return "FP_dense";
    case MCPM_MODEL_FP_IDEAL_GAS: return "FP_ideal_gas";
    case MCPM_MODEL_ESMC: return "ESMC";
    case MCPM_MODEL_FP_LINEAR: return "FP_linear";
    case MCPM_MODEL_DSMC_VHS: return "DSMC_VHS";
    default: return "none";
  }
}

extern "C" {

void* ref_create(const mcpm_config* c, long N) {
  Quiet q;
  Ref* r = new Ref();
  GAS& g = r->gas;
  BOX& b = r->box;
  g.sigma = c->sigma; g.m = c->m; g.kb = c->kb; g.n = c->n; g.Fn = c->Fn;
  g.T0 = c->T0; g.mu = c->mu; g.visp = c->visp; g.b = c->b; g.delta_t = c->dt;
  g.phi = c->phi; g.eqdist = c->eqdist; g.ast = c->ast; g.bst = c->bst;
  g.long_range = c->long_range; g.model = model_name(c->model); g.N = N;
  g.crref = c->crref;
  g.n_ratio = 1; g.times = 1.0;
  for (int i = 0; i < 3; ++i) {
    b.N[i] = c->n_cells[i]; b.Len[i] = c->length[i];
    b.delta_dim[i] = c->length[i] / c->n_cells[i]; b.direction[i] = c->direction[i];
  }
  b.problem = (c->problem == MCPM_PROBLEM_PERIODIC) ? relaxation : c->problem;
  b.T_wall_1 = c->T_wall[0]; b.T_wall_2 = c->T_wall[1]; b.T_wall_3 = c->T_wall[2]; b.T_wall_4 = c->T_wall[3];
  b.U_wall_1 = c->U_wall[0]; b.U_wall_2 = c->U_wall[1]; b.U_wall_3 = c->U_wall[2]; b.U_wall_4 = c->U_wall[3];
  b.every = 1 << 30; b.after = 1 << 30; b.init_step = 0; b.step = 0;
  b.Ny = 1; b.s = 2.0; b.Ly = 1.0;
  r->C = b.N[0] * b.N[1] * b.N[2];
  r->N = N;
  r->cells = (CELLS*)calloc(r->C, sizeof(CELLS));
  make_cells(&b, r->cells, &g);
  for (int k = 0; k < r->C; ++k) {
    r->cells[k].indices_inside = (int*)malloc(sizeof(int));
    r->cells[k].indices_inside[0] = -1;
  }
  r->x3.assign(N, 0.5 * c->length[2]); r->x3_old = r->x3;
  r->Mp1.assign(N, 0.0); r->Mp2.assign(N, 0.0); r->Mp3.assign(N, 0.0);
  r->xi1.assign(N, 0.0); r->xi2.assign(N, 0.0); r->xi3.assign(N, 0.0);
  r->T.assign(N, 0.0); r->rho.assign(N, 0.0);
  r->color.assign(N, 0); r->flag.assign(N, 0);
  return r;
}

void ref_destroy(void* h) {
  Ref* r = (Ref*)h;
  for (int k = 0; k < r->C; ++k) free(r->cells[k].indices_inside);
  free(r->cells);
  delete r;
}

void ref_set_step(void* h, int step) { ((Ref*)h)->box.step = step; }

void ref_inject_normals(const double* a, const double* b, const double* c, long N) {
  g_inj.assign(a, a + N);
  g_inj.insert(g_inj.end(), b, b + N);
  g_inj.insert(g_inj.end(), c, c + N);
  g_inj_pos = 0;
}

void ref_cell_update(void* h, double* x1, double* x2, double* U1, double* U2, double* U3, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  double* T = r->T.data();
  cell_update(x1, x2, U1, U2, U3, &r->gas, r->cells, &r->box, index, &T, r->rho.data(), r->color.data());
}

void ref_random_generator(void* h, int* index, double* xi1f, double* xi2f, double* xi3f) {
  Quiet q;
  Ref* r = (Ref*)h;
  g_inj_pos = 0;
  random_generator(r->xi1.data(), r->xi2.data(), r->xi3.data(), xi1f, xi2f, xi3f, r->cells, &r->box, &r->gas, index);
}

void ref_velocity_fp(void* h, double* U1, double* U2, double* U3, int* index, double* xi1f, double* xi2f,
                     double* xi3f) {
  Quiet q;
  Ref* r = (Ref*)h;
  // the dispatch of velocity_update, src/Main_Functions.cpp:1565-1570
  if (r->gas.model == "FP_linear")
    Velocity_FP_linear(U1, U2, U3, &r->gas, r->cells, &r->box, index, xi1f, xi2f, xi3f, r->Mp1.data(),
                       r->Mp2.data(), r->Mp3.data());
  else
    Velocity_FP_parallel(U1, U2, U3, &r->gas, r->cells, &r->box, index, xi1f, xi2f, xi3f, r->Mp1.data(),
                         r->Mp2.data(), r->Mp3.data());
}

void ref_long_range(void* h, double* x1, double* x2, double* U2, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  if (r->gas.long_range == 2) {
    // the density-expansion force is inline in velocity_update
    // (src/Main_Functions.cpp:1632-1653): run velocity_update with no
    // collision model so that only its long-range part acts
    const std::string model = r->gas.model;
    r->gas.model = "none";
    Collision cba;
    std::memset(&cba, 0, sizeof(cba));
    std::vector<double> U1(r->N, 0.0), U3(r->N, 0.0), F1(r->N, 0.0), F2(r->N, 0.0), F3(r->N, 0.0);
    velocity_update(U1.data(), U2, U3.data(), x1, x2, r->x3.data(), &r->gas, &r->box, r->cells, index, &cba,
                    r->xi1.data(), r->xi2.data(), r->xi3.data(), r->Mp1.data(), r->Mp2.data(), r->Mp3.data(),
                    F1.data(), F2.data(), F3.data(), r->rho.data(), r->T.data(), r->color.data());
    r->gas.model = model;
    return;
  }
  if (r->gas.long_range == 1) vlasov_taking_the_integral(U2, &r->gas, &r->box, r->cells, index, x1, x2, r->x3.data());
  else if (r->gas.long_range == 3) poisson_solver(U2, x1, x2, r->x3.data(), &r->gas, &r->box, r->cells, index);
}

// the 2-D routines, src/FEM.cpp:249-726 (the reference calls them for its
// 2-D injection problem, src/Main_Functions.cpp:1622, :1656)
void ref_long_range_2d(void* h, double* x1, double* x2, double* U1, double* U2, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  if (r->gas.long_range == 1) compute_Vlasov_2D(&r->gas, &r->box, r->cells, x1, x2, U1, U2, index);
  else if (r->gas.long_range == 3) compute_SP_2D(&r->gas, &r->box, r->cells, x1, x2, U1, U2, index);
}

// nodal densities n_n of the last cell_update, [C][4]
void ref_get_node_density(void* h, double* out) {
  Ref* r = (Ref*)h;
  for (int c = 0; c < r->C; ++c)
    for (int k = 0; k < 4; ++k) out[(size_t)c * 4 + k] = r->cells[c].n_n[k];
}

void ref_dfp_extra_streaming(void* h, double* U1, double* U2, double* U3, double* x1, double* x2, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  DFP_extra_streaming(U1, U2, U3, x1, x2, &r->gas, &r->box, r->cells, index, r->gas.delta_t);
}

void ref_apply_bc(void* h, double* U1, double* U2, double* U3, double* x1, double* x2, double* x1_old,
                  double* x2_old, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  if (r->box.problem == relaxation) return;  // the periodic wrap is not a reference routine
  apply_BC(U1, U2, U3, x1, x2, r->x3.data(), x1_old, x2_old, r->x3_old.data(), &r->gas, &r->box, r->cells, index,
           r->flag.data(), r->xi1.data(), r->xi2.data(), r->xi3.data(), r->xi1.data(), r->xi2.data(), r->xi3.data(),
           r->Mp1.data(), r->Mp2.data(), r->Mp3.data(), r->T.data());
}

void ref_store_old_positions(void* h, double* x1, double* x2, double* x1_old, double* x2_old) {
  Quiet q;
  Ref* r = (Ref*)h;
  store_old_positions(x1, x2, r->x3.data(), x1_old, x2_old, r->x3_old.data(), &r->gas, &r->box);
}

void ref_stream(void* h, double* U1, double* U2, double* U3, double* x1, double* x2, double* x1_old,
                double* x2_old, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  stream_particles(U1, U2, U3, x1, x2, r->x3.data(), x1_old, x2_old, r->x3_old.data(), &r->gas, &r->box,
                   r->cells, index);
}

void ref_esmc(void* h, double* U1, double* U2, double* U3, double* x1, double* x2, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  Collision_ESMC_new3(U1, U2, U3, x1, x2, &r->gas, &r->box, r->cells, index);
}

void ref_dsmc_vhs(void* h, double* U1, double* U2, double* U3, double* x1, double* x2) {
  Quiet q;
  Ref* r = (Ref*)h;
  Collision DSMC;
  std::memset(&DSMC, 0, sizeof(DSMC));
  Collision_DSMC_VHS(U1, U2, U3, x1, x2, &r->gas, &r->box, r->cells, &DSMC);
}

// cell_poly_velocity (src/Main_Functions.cpp:1918), then its running sums
// into out, [C][MCPM_SF_COUNT]
void ref_sample_cells(void* h, double* U1, double* U2, double* U3, int* index, double* out) {
  Quiet q;
  Ref* r = (Ref*)h;
  cell_poly_velocity(U1, U2, U3, r->cells, &r->box, r->box.step, &r->gas, index);
  for (int c = 0; c < r->C; ++c) {
    const CELLS& k = r->cells[c];
    double* o = out + (size_t)c * MCPM_SF_COUNT;
    o[MCPM_SF_WEIGHT] = k.sum_weight;
    for (int i = 0; i < 3; ++i) o[MCPM_SF_M + i] = k.sum_M[i];
    for (int i = 0; i < 6; ++i) o[MCPM_SF_MM + i] = k.sum_MM[i];
    for (int i = 0; i < 10; ++i) o[MCPM_SF_MMM + i] = k.sum_MMM[i];
    for (int i = 0; i < 6; ++i) o[MCPM_SF_MMMM + i] = k.sum_MMMM[i];
  }
}

// readSettingsFile (src/myIO.cpp:1756-3016) on the file at path: the derived
// GAS/BOX values a configuration takes, ints [N0 N1 N2 dir0 dir1 dir2
// problem long_range model N] and doubles [Len0..2 sigma m kb n Fn T0 mu visp
// b delta_t phi eqdist ast bst T_wall1..4 U_wall1..4 crref]
void ref_read_settings(const char* path, long* iv, double* dv) {
  Quiet q;
  GAS g{};
  BOX b{};
  b.file_name = path;
  readSettingsFile(&g, &b);
  int model = -1;
  if (g.model == "none") model = 0;
  else if (g.model == "FP_dense") model = MCPM_MODEL_FP_DENSE;
  else if (g.model == "FP_ideal_gas") model = MCPM_MODEL_FP_IDEAL_GAS;
  else if (g.model == "ESMC") model = MCPM_MODEL_ESMC;
  else if (g.model == "FP_linear") model = MCPM_MODEL_FP_LINEAR;
  else if (g.model == "DSMC_VHS") model = MCPM_MODEL_DSMC_VHS;
  const long ivals[10] = {b.N[0], b.N[1], b.N[2], b.direction[0], b.direction[1], b.direction[2],
                          b.problem, g.long_range, model, (long)g.N};
  for (int i = 0; i < 10; ++i) iv[i] = ivals[i];
  const double dvals[28] = {b.Len[0], b.Len[1], b.Len[2], g.sigma, g.m, g.kb, g.n, g.Fn, g.T0, g.mu,
                            g.visp, g.b, g.delta_t, g.phi, g.eqdist, g.ast, g.bst,
                            b.T_wall_1, b.T_wall_2, b.T_wall_3, b.T_wall_4,
                            b.U_wall_1, b.U_wall_2, b.U_wall_3, b.U_wall_4, g.crref, 0.0, 0.0};
  for (int i = 0; i < 26; ++i) dv[i] = dvals[i];
}

// readSettingsFile then initialization (src/Main_Functions.cpp:4222) on the
// file at path: the reference's initial particles (N of them)
void ref_initialize(const char* path, double* x1, double* x2, double* U1, double* U2, double* U3, long N) {
  Quiet q;
  GAS g{};
  BOX b{};
  b.file_name = path;
  readSettingsFile(&g, &b);
  if ((long)g.N != N) return;
  const int C = b.N[0] * b.N[1] * b.N[2];
  CELLS* cells = (CELLS*)calloc(C, sizeof(CELLS));
  make_cells(&b, cells, &g);
  std::vector<double> x3(N);
  initialization(U1, U2, U3, x1, x2, x3.data(), &g, &b, cells);
  free(cells);
}

void ref_init_omega_max(void* h) {
  // src/main.cpp:250-269
  Ref* r = (Ref*)h;
  double pi = acos(-1);
  for (int num = 0; num < r->C; ++num) {
    double thermal = sqrt(r->gas.kb * r->cells[num].T / r->gas.m);
    r->cells[num].crm = 10.0 * ((thermal));
    r->cells[num].omega_max = 4.0 * pi * r->gas.sigma * r->gas.sigma * r->cells[num].crm * r->cells[num].n * r->gas.delta_t;
    if (r->gas.model == "ESMC") r->cells[num].omega_max = r->cells[num].omega_max * increase_collision_rate(r->gas.n, &r->gas);
  }
}

// cells[].n_ratio of the harness's cells (make_cells sets 1 outside the
// interface problems)
void ref_set_cell_weights(void* h, const int* cw) {
  Ref* r = (Ref*)h;
  for (int c = 0; c < r->C; ++c) r->cells[c].n_ratio = cw[c];
}

// thermostat (src/Main_Functions.cpp:1674) in its live branch, problem
// inverted, on the lists of the last ref_cell_update
void ref_thermostat(void* h, double* U1, double* U2, double* U3, double* x2, int* index, double Tc, double Th,
                    double thermc, double thermh) {
  Quiet q;
  Ref* r = (Ref*)h;
  const int problem = r->box.problem;
  r->box.problem = inverted;
  r->gas.Tc = Tc; r->gas.Th = Th;
  r->box.thermc = thermc; r->box.thermh = thermh;
  thermostat(U1, U2, U3, x2, &r->gas, &r->box, r->cells, index);
  r->box.problem = problem;
}

// inverted_addremove_particles (src/Main_Functions.cpp:1206) against the
// lists of the last ref_cell_update: the particle weights w (N), the cell
// weights cw (C) and n_ratio; the reference frees and re-allocates its
// arrays, so they are handed over as malloc'd copies and the new state is
// copied out (room for cap particles).  Returns the new N (-1: no room).
long ref_addremove(void* h, const double* x1, const double* x2, const double* x1_old, const double* x2_old,
                   const double* U1, const double* U2, const double* U3, const int* index, const int* w,
                   const int* cw, int n_ratio, long cap, double* ox1, double* ox2, double* ox1_old,
                   double* ox2_old, double* oU1, double* oU2, double* oU3, int* ow) {
  Quiet q;
  Ref* r = (Ref*)h;
  const long N = r->gas.N;
  auto dup = [&](const double* a) {
    double* p = (double*)malloc(sizeof(double) * (N > 0 ? N : 1));
    memcpy(p, a, sizeof(double) * N);
    return p;
  };
  auto idup = [&](const int* a) {
    int* p = (int*)malloc(sizeof(int) * (N > 0 ? N : 1));
    if (a) memcpy(p, a, sizeof(int) * N);
    else memset(p, 0, sizeof(int) * N);
    return p;
  };
  double *a1 = dup(x1), *a2 = dup(x2), *a1o = dup(x1_old), *a2o = dup(x2_old);
  double *u1 = dup(U1), *u2 = dup(U2), *u3 = dup(U3);
  double *xi1 = dup(U1), *xi2 = dup(U1), *xi3 = dup(U1), *xf1 = dup(U1), *xf2 = dup(U1), *xf3 = dup(U1);
  double *m1 = dup(U1), *m2 = dup(U1), *m3 = dup(U1);
  int *ix = idup(index), *fl = idup(nullptr), *nr = idup(w), *col = idup(nullptr);
  for (int c = 0; c < r->C; ++c) r->cells[c].n_ratio = cw[c];
  r->gas.n_ratio = n_ratio;
  const int step = r->box.step;
  r->box.step = 1;  // the first call frees no earlier split lists (:1289-1290)
  inverted_addremove_particles(&u1, &u2, &u3, &a1, &a1o, &a2, &a2o, &r->gas, &r->box, r->cells, &ix, &fl, &nr,
                               &xi1, &xi2, &xi3, &xf1, &xf2, &xf3, &m1, &m2, &m3, &col);
  r->box.step = step;
  const long M = (long)r->gas.N;
  if (M <= cap) {
    memcpy(ox1, a1, sizeof(double) * M); memcpy(ox2, a2, sizeof(double) * M);
    memcpy(ox1_old, a1o, sizeof(double) * M); memcpy(ox2_old, a2o, sizeof(double) * M);
    memcpy(oU1, u1, sizeof(double) * M); memcpy(oU2, u2, sizeof(double) * M); memcpy(oU3, u3, sizeof(double) * M);
    memcpy(ow, nr, sizeof(int) * M);
  }
  for (int c = 0; c < r->C; ++c) { free(r->cells[c].id_split_part); r->cells[c].id_split_part = nullptr; }
  free(a1); free(a2); free(a1o); free(a2o); free(u1); free(u2); free(u3);
  free(xi1); free(xi2); free(xi3); free(xf1); free(xf2); free(xf3); free(m1); free(m2); free(m3);
  free(ix); free(fl); free(nr); free(col);
  r->gas.N = N;  // the harness's particle count stays (its side arrays are sized by it)
  return M <= cap ? M : -1;
}

// measure_pressure (src/Main_Functions.cpp:13), then cells[].p_m into out [C]
void ref_measure_pressure(void* h, double* U2, double* x2, double* x2_old, double* out) {
  Quiet q;
  Ref* r = (Ref*)h;
  measure_pressure(U2, x2, x2_old, &r->gas, &r->box, r->cells);
  for (int c = 0; c < r->C; ++c) out[c] = r->cells[c].p_m;
}

// write_post_processing (src/myIO.cpp:597) with the harness's cells: the
// file PostProc/<name>_<lr>_<step>.dat under dir (which must hold PostProc/)
void ref_write_post(void* h, int step, double t_post, const char* dir, const char* name, double* U1, double* U2,
                    double* U3, double* x1, double* x2, double* x2_old, int* index) {
  Quiet q;
  Ref* r = (Ref*)h;
  char cwd[4096];
  if (!getcwd(cwd, sizeof cwd) || chdir(dir) != 0) return;
  const int every = r->box.every, after = r->box.after;
  const double times = r->gas.times;
  r->box.every = 1; r->box.after = 0; r->gas.times = 0.0;
  r->gas.output_name = name;
  r->gas.t_post = t_post;
  int done = 0;
  std::vector<int> nratio(r->N, 1);
  write_post_processing(step, r->cells, &r->box, &done, &r->gas, U1, U2, U3, x1, x2, r->flag.data(), index,
                        r->color.data(), nratio.data(), x2_old);
  r->box.every = every; r->box.after = after; r->gas.times = times;
  if (chdir(cwd) != 0) return;
}

// the console lines of post_processing (src/myIO.cpp:935) into buf
long ref_post_text(void* h, int step, double* U1, double* U2, double* U3, double* x1, double* x2, double* x2_old,
                   int* index, char* buf, long len) {
  Ref* r = (Ref*)h;
  char tmpl[] = "/tmp/mcpm_ref_textXXXXXX";
  const int fd = mkstemp(tmpl);
  if (fd < 0) return -1;
  fflush(stdout);
  const int saved = dup(1);
  dup2(fd, 1);
  const int every = r->box.every, st = r->box.step;
  r->box.every = 1; r->box.step = step;
  int done = 0;
  std::vector<int> nratio(r->N, 1);
  post_processing(step, r->cells, &r->box, &done, &r->gas, U1, U2, U3, x1, x2, r->flag.data(), index,
                  r->color.data(), nratio.data(), x2_old);
  r->box.every = every; r->box.step = st;
  fflush(stdout);
  dup2(saved, 1);
  close(saved);
  const long n = (long)lseek(fd, 0, SEEK_END);
  lseek(fd, 0, SEEK_SET);
  long got = 0;
  if (n > 0 && n < len) got = (long)read(fd, buf, (size_t)n);
  close(fd);
  unlink(tmpl);
  if (got >= 0 && got < len) buf[got] = 0;
  return got;
}

// the CELLS fields of enum mcpm_cell_field, cell-major [C][MCPM_CF_COUNT]
void ref_get_cells(void* h, double* out) {
  Ref* r = (Ref*)h;
  for (int c = 0; c < r->C; ++c) {
    const CELLS& k = r->cells[c];
    double* o = out + (size_t)c * MCPM_CF_COUNT;
    o[MCPM_CF_NUM_INSIDE] = k.num_inside;
    for (int i = 0; i < 3; ++i) o[MCPM_CF_U_SPACE + i] = k.U_space[i];
    for (int i = 0; i < 6; ++i) o[MCPM_CF_PIJ + i] = k.PIJ[i];
    for (int i = 0; i < 10; ++i) o[MCPM_CF_M3 + i] = k.M3[i];
    for (int i = 0; i < 6; ++i) o[MCPM_CF_M4 + i] = k.M4[i];
    for (int i = 0; i < 3; ++i) o[MCPM_CF_M5 + i] = k.M5[i];
    for (int i = 0; i < 3; ++i) o[MCPM_CF_Q + i] = k.Q[i];
    o[MCPM_CF_DM2] = k.DM2;
    o[MCPM_CF_DM4] = k.DM4;
    for (int i = 0; i < 3; ++i) o[MCPM_CF_MP + i] = k.Mp[i];
    o[MCPM_CF_T] = k.T;
    o[MCPM_CF_N] = k.n;
    o[MCPM_CF_GAMMA_ST] = k.gamma_st;
    o[MCPM_CF_LAMBDA] = k.Lambda;
    for (int i = 0; i < 6; ++i) o[MCPM_CF_C + i] = k.c[i];
    for (int i = 0; i < 3; ++i) o[MCPM_CF_GAMMA + i] = k.gamma[i];
    for (int i = 0; i < 9; ++i) o[MCPM_CF_ALPHA + i] = k.alpha[i];
    for (int i = 0; i < 3; ++i) o[MCPM_CF_BETA + i] = k.beta[i];
    for (int i = 0; i < 3; ++i) o[MCPM_CF_PHI + i] = k.phi[i];
    o[MCPM_CF_F2] = k.F2;
    o[MCPM_CF_OMEGA_MAX] = (r->gas.model == "DSMC_VHS") ? k.crm : k.omega_max;
    o[MCPM_CF_DIVU] = k.divU;
    o[MCPM_CF_N_SMOOTH] = k.n_smooth;
    o[MCPM_CF_DN2] = k.dn2;
    o[MCPM_CF_DN3] = k.dn3;
  }
}

}  // extern "C"
