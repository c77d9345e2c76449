/*
 * mcpm_oracle.c -- CPU restatement (FP64) of the reference particle step.
 *
 * TEST INFRASTRUCTURE ONLY (see mcpm_oracle.h).  Built with -O2
 * -ffp-contract=off so that every multiply and add rounds separately, as in
 * the reference built for x86-64 without FMA.  Expressions keep the reference's
 * evaluation order (C evaluates left to right), which is what makes the
 * bit-for-bit comparison against oracle/_ref possible.
 */
#include "mcpm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define CF MCPM_CF_COUNT
#define CELL(s, c, f) ((s)->cell[(size_t)(c) * CF + (f)])

enum { RNG_STREAM_FP = 0, RNG_STREAM_BC = 1, RNG_STREAM_ESMC = 2,
       RNG_STREAM_BIN = 3, RNG_STREAM_ESMC_ACC = 4, RNG_STREAM_ESMC_M = 5,
       RNG_STREAM_DSMC = 6, RNG_STREAM_DSMC_ACC = 7, RNG_STREAM_DSMC_M = 8,
       RNG_STREAM_ADDREM_DEL = 9, RNG_STREAM_ADDREM_NEW = 10 };

struct orc_state {
  mcpm_config cfg;
  int64_t N;
  int N0, N1, C;
  double dx, dy, dz;
  double* cell;      /* [C][CF] */
  int* cnt;          /* num_inside */
  int* off;          /* list offsets (C+1) */
  int* list;         /* per-cell particle ids, ascending */
  int32_t* index;    /* cell of each particle */
  int step;
  int status;
  int rng_mode;
  double* inj;       /* 3N injected normals */
  double* xi;        /* 3N whitened normals (random_generator output) */
  double* nn;        /* [C][4] nodal densities n_n of the last cell_update */
  int32_t* cw;       /* [C] cells[].n_ratio once set, else NULL (1) */
  uint32_t* rinj[RNG_STREAM_ADDREM_NEW + 1];  /* injected words per stream, 4 per row */
  int64_t rinj_rows[RNG_STREAM_ADDREM_NEW + 1];
};

/* ------------------------------------------------------------------ RNG -- */
/* Philox4x32-10, J. K. Salmon et al., "Parallel random numbers: as easy as
   1, 2, 3", SC'11: ten rounds of two 32x32->64 multiplies with the published
   multipliers and Weyl key increments. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)0xD2511F53u * c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
    uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
    uint32_t n1 = (uint32_t)p1;
    uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
    uint32_t n3 = (uint32_t)p0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static void philox(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2,
                   uint32_t c3, uint32_t out[4]) {
  uint32_t ctr[4] = {c0, c1, c2, c3};
  uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
  orc_philox4x32_10(ctr, key, out);
}

static double u01(uint32_t x) { return ((double)x + 0.5) * (1.0 / 4294967296.0); }

/* the four words of a draw of the session's stream c2 with key c0 and
   counter c3: the injected row (c0 + c3) mod rows (mcpm_inject_uniforms),
   else Philox on (c0, c1 = step, c2, c3) */
static void rng(const orc_state* s, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, uint32_t out[4]) {
  if (c2 <= RNG_STREAM_ADDREM_NEW && s->rinj[c2]) {
    const uint32_t* w = s->rinj[c2] + 4 * (((uint64_t)c0 + c3) % (uint64_t)s->rinj_rows[c2]);
    out[0] = w[0]; out[1] = w[1]; out[2] = w[2]; out[3] = w[3];
    return;
  }
  philox(s->cfg.seed, c0, c1, c2, c3, out);
}

static const double TWO_PI = 6.283185307179586476925286766559;

/* four standard normals by two Box-Muller pairs on the four Philox words */
void orc_normals4(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2,
                  uint32_t c3, double z[4]) {
  uint32_t r[4];
  philox(seed, c0, c1, c2, c3, r);
  double a = sqrt(-2.0 * log(u01(r[0])));
  double b = sqrt(-2.0 * log(u01(r[2])));
  z[0] = a * cos(TWO_PI * u01(r[1]));
  z[1] = a * sin(TWO_PI * u01(r[1]));
  z[2] = b * cos(TWO_PI * u01(r[3]));
  z[3] = b * sin(TWO_PI * u01(r[3]));
}

/* orc_normals4 on the session's draw (injected or Philox) */
static void normals4_s(const orc_state* s, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3, double z[4]) {
  uint32_t r[4];
  rng(s, c0, c1, c2, c3, r);
  double a = sqrt(-2.0 * log(u01(r[0])));
  double b = sqrt(-2.0 * log(u01(r[2])));
  z[0] = a * cos(TWO_PI * u01(r[1]));
  z[1] = a * sin(TWO_PI * u01(r[1]));
  z[2] = b * cos(TWO_PI * u01(r[3]));
  z[3] = b * sin(TWO_PI * u01(r[3]));
}

/* uniform integer in [0, n) from one Philox word */
static int pick(uint32_t r, int n) { return (int)(((uint64_t)r * (uint64_t)n) >> 32); }

/* ------------------------------------------------------- small helpers -- */
/* increase_collision_rate, src/Main_Functions.cpp:1906-1915 */
static double Ycoll(const orc_state* s, double n) {
  double nb = n * s->cfg.b;
  return 1.0 + 0.625 * n * s->cfg.b + 0.2869 * pow(nb, 2.0) + 0.115 * pow(nb, 3.0);
}
/* scale_mu, src/Main_Functions.cpp:1970-1973 */
static double scale_mu(const orc_state* s, double T) {
  return s->cfg.mu * pow(T / s->cfg.T0, s->cfg.visp);
}
/* the cell volume exactly as make_cells builds it, src/myIO.cpp:1456-1465 */
static double cell_volume(const orc_state* s, int c) {
  int j = c % s->N0, k = c / s->N0;
  double d0 = (double)j * s->dx, d1 = (double)(j + 1) * s->dx;
  double d2 = (double)k * s->dy, d3 = (double)(k + 1) * s->dy;
  double d4 = 0.0 * s->dz, d5 = 1.0 * s->dz;
  return (d1 - d0) * (d3 - d2) * (d5 - d4);
}


/* cell geometry exactly as make_cells builds it (src/myIO.cpp:1456-1479):
   dx_c = dim[1] - dim[0], centre = (dim[0] + dim[1]) / 2, node k of the
   cell at centre -/+ dx_c / 2 (k = 0 lower left, 1 lower right, 2 upper
   left, 3 upper right) */
typedef struct { double dxc, dyc, cx, cy, xn[4], yn[4]; } cell_geo;
static cell_geo geometry(const orc_state* s, int c) {
  cell_geo g;
  int j = c % s->N0, k = c / s->N0;
  double d0 = (double)j * s->dx, d1 = (double)(j + 1) * s->dx;
  double d2 = (double)k * s->dy, d3 = (double)(k + 1) * s->dy;
  g.dxc = d1 - d0; g.dyc = d3 - d2;
  g.cx = 0.5 * (d0 + d1); g.cy = 0.5 * (d2 + d3);
  g.xn[0] = g.cx - g.dxc / 2.0; g.xn[1] = g.cx + g.dxc / 2.0;
  g.xn[2] = g.cx - g.dxc / 2.0; g.xn[3] = g.cx + g.dxc / 2.0;
  g.yn[0] = g.cy - g.dyc / 2.0; g.yn[1] = g.cy - g.dyc / 2.0;
  g.yn[2] = g.cy + g.dyc / 2.0; g.yn[3] = g.cy + g.dyc / 2.0;
  return g;
}
/* node ids of cell c: id[0] = k (N0+1) + j, id[1] = id[0] + 1,
   id[2] = id[0] + N0 + 1, id[3] = id[2] + 1 (src/myIO.cpp:1448-1451) */
static void node_ids(const orc_state* s, int c, int id[4]) {
  int j = c % s->N0, k = c / s->N0;
  id[0] = k * (s->N0 + 1) + j; id[1] = id[0] + 1;
  id[2] = (k + 1) * (s->N0 + 1) + j; id[3] = id[2] + 1;
}

/* nodal density n_n, src/Main_Functions.cpp:2268-2364: every particle adds
   Fn/volume to the node of its own cell nearest to it, in every cell that
   shares that node; wall nodes are then doubled per wall they lie on. */
#define NN(c, q) s->nn[(size_t)(c) * 4 + (q)]
static void node_density(orc_state* s, const double* x1, const double* x2) {
  const mcpm_config* g = &s->cfg;
  const int N0 = s->N0, N1 = s->N1;
  for (size_t i = 0; i < (size_t)s->C * 4; ++i) s->nn[i] = 0.0;
  for (int64_t i = 0; i < s->N; ++i) {
    int num = s->index[i], j = num % N0, k = num / N0, kk, jj, num2;
    cell_geo cg = geometry(s, num);
#define ADD(c, q) NN(c, q) += g->Fn / cell_volume(s, c)
    if (x1[i] < cg.cx) {
      if (x2[i] < cg.cy) {
        ADD(num, 0);
        kk = k; jj = j - 1; if (jj >= 0) { num2 = kk * N0 + jj; ADD(num2, 1); }
        kk = k - 1; jj = j; if (kk >= 0) { num2 = kk * N0 + jj; ADD(num2, 2); }
        kk = k - 1; jj = j - 1; if (kk >= 0 && jj >= 0) { num2 = kk * N0 + jj; ADD(num2, 3); }
      } else {
        ADD(num, 2);
        kk = k; jj = j - 1; if (jj >= 0) { num2 = kk * N0 + jj; ADD(num2, 3); }
        kk = k + 1; jj = j; if (kk <= N1 - 1) { num2 = kk * N0 + jj; ADD(num2, 0); }
        kk = k + 1; jj = j - 1; if (kk <= N1 - 1 && jj >= 0) { num2 = kk * N0 + jj; ADD(num2, 1); }
      }
    } else {
      if (x2[i] < cg.cy) {
        ADD(num, 1);
        kk = k; jj = j + 1; if (jj <= N0 - 1) { num2 = kk * N0 + jj; ADD(num2, 0); }
        kk = k - 1; jj = j; if (kk >= 0) { num2 = kk * N0 + jj; ADD(num2, 3); }
        kk = k - 1; jj = j + 1; if (kk >= 0 && jj <= N0 - 1) { num2 = kk * N0 + jj; ADD(num2, 2); }
      } else {
        ADD(num, 3);
        kk = k; jj = j + 1; if (jj <= N0 - 1) { num2 = kk * N0 + jj; ADD(num2, 2); }
        kk = k + 1; jj = j; if (kk <= N1 - 1) { num2 = kk * N0 + jj; ADD(num2, 1); }
        kk = k + 1; jj = j + 1; if (kk <= N1 - 1 && jj <= N0 - 1) { num2 = kk * N0 + jj; ADD(num2, 0); }
      }
    }
#undef ADD
  }
  for (int jj = 0; jj < N0; ++jj) { int c = jj; NN(c, 0) = NN(c, 0) * 2.0; NN(c, 1) = NN(c, 1) * 2.0; }
  for (int jj = 0; jj < N0; ++jj) { int c = (N1 - 1) * N0 + jj; NN(c, 2) = NN(c, 2) * 2.0; NN(c, 3) = NN(c, 3) * 2.0; }
  for (int kk = 0; kk < N1; ++kk) { int c = kk * N0; NN(c, 0) = NN(c, 0) * 2.0; NN(c, 2) = NN(c, 2) * 2.0; }
  for (int kk = 0; kk < N1; ++kk) { int c = kk * N0 + N0 - 1; NN(c, 1) = NN(c, 1) * 2.0; NN(c, 3) = NN(c, 3) * 2.0; }
}
void orc_get_node_density(const orc_state* s, double* out) {
  memcpy(out, s->nn, sizeof(double) * (size_t)s->C * 4);
}

/* ----------------------------------------------------------- lifecycle -- */
orc_state* orc_create(const mcpm_config* cfg, int64_t n_particles) {
  orc_state* s = (orc_state*)calloc(1, sizeof(orc_state));
  s->cfg = *cfg;
  s->N = n_particles;
  s->N0 = cfg->n_cells[0];
  s->N1 = cfg->n_cells[1];
  s->C = s->N0 * s->N1;
  s->dx = cfg->length[0] / cfg->n_cells[0];
  s->dy = cfg->length[1] / cfg->n_cells[1];
  s->dz = cfg->length[2] / cfg->n_cells[2];
  s->cell = (double*)calloc((size_t)s->C * CF, sizeof(double));
  s->cnt = (int*)calloc(s->C, sizeof(int));
  s->off = (int*)calloc(s->C + 1, sizeof(int));
  s->list = (int*)calloc(n_particles > 0 ? n_particles : 1, sizeof(int));
  s->index = (int32_t*)calloc(n_particles > 0 ? n_particles : 1, sizeof(int32_t));
  s->inj = (double*)calloc(3 * (n_particles > 0 ? n_particles : 1), sizeof(double));
  s->xi = (double*)calloc(3 * (n_particles > 0 ? n_particles : 1), sizeof(double));
  s->nn = (double*)calloc((size_t)s->C * 4, sizeof(double));
  return s;
}

void orc_destroy(orc_state* s) {
  if (!s) return;
  free(s->cell); free(s->cnt); free(s->off); free(s->list); free(s->index);
  free(s->inj); free(s->xi); free(s->nn); free(s->cw);
  for (int i = 0; i <= RNG_STREAM_ADDREM_NEW; ++i) free(s->rinj[i]);
  free(s);
}

int orc_num_cells(const orc_state* s) { return s->C; }
void orc_set_cell_weights(orc_state* s, const int32_t* cw) {
  if (!s->cw) s->cw = (int32_t*)malloc(sizeof(int32_t) * (size_t)s->C);
  memcpy(s->cw, cw, sizeof(int32_t) * (size_t)s->C);
}
void orc_get_cells(const orc_state* s, double* out) {
  memcpy(out, s->cell, sizeof(double) * (size_t)s->C * CF);
}
void orc_set_cell_field(orc_state* s, int f, const double* v) {
  for (int c = 0; c < s->C; ++c) CELL(s, c, f) = v[c];
}
int orc_get_step(const orc_state* s) { return s->step; }
void orc_set_step(orc_state* s, int step) { s->step = step; }
int orc_status(orc_state* s) { int st = s->status; s->status = 0; return st; }
void orc_set_rng(orc_state* s, int mode) { s->rng_mode = mode; }
/* mcpm_inject_uniforms: n_rows rows of four uniforms as the words
   floor(u 2^32), clamped to [0, 2^32 - 1]; n_rows = 0 restores Philox */
void orc_inject_uniforms(orc_state* s, int stream, int64_t n_rows, const double* u) {
  if (stream < 0 || stream > RNG_STREAM_ADDREM_NEW) return;
  free(s->rinj[stream]);
  s->rinj[stream] = NULL;
  s->rinj_rows[stream] = 0;
  if (n_rows <= 0 || !u) return;
  s->rinj[stream] = (uint32_t*)malloc(sizeof(uint32_t) * 4 * (size_t)n_rows);
  for (int64_t i = 0; i < 4 * n_rows; ++i) {
    const double v = u[i];
    uint32_t w = 0;
    if (v > 0.0) {
      const double t = floor(v * 4294967296.0);
      w = t >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)t;
    }
    s->rinj[stream][i] = w;
  }
  s->rinj_rows[stream] = n_rows;
}
void orc_inject_normals(orc_state* s, const double* a, const double* b,
                        const double* c) {
  for (int64_t i = 0; i < s->N; ++i) {
    s->inj[i] = a[i]; s->inj[s->N + i] = b[i]; s->inj[2 * s->N + i] = c[i];
  }
  s->rng_mode = MCPM_RNG_INJECTED;
}

/* --------------------------------------------------------- Gauss-Jordan -- */
/* maxx_magnittude, src/Math_Func.cpp:107-119: first index of the largest |a| */
static int maxx_magnitude(const double* a, int n) {
  double b = fabs(a[0]);
  int l = 0;
  for (int i = 0; i < n; ++i)
    if (fabs(b) < fabs(a[i])) { b = fabs(a[i]); l = i; }
  return l;
}
/* Scalling, src/Math_Func.cpp:159-163 */
static double scaling(const double* row, int i, int n) {
  int b = maxx_magnitude(row, n);
  return fabs(row[i]) / fabs(row[b]);
}
/* Gauss_Jordan, src/Math_Func.cpp:165-232: forward elimination with scaled
   partial pivoting (full-row updates, reciprocal-then-multiply factor),
   then back substitution. */
void orc_gauss_jordan(double* A, double* RHS, int n, double* x) {
  double z[16];
  for (int i = 0; i < n - 1; ++i) {
    for (int ii = 0; ii < n; ++ii) z[ii] = 0.0;
    int k = 0;
    for (int j = i; j < n; ++j) { z[k] = scaling(&A[j * n], i, n); k++; }
    k = maxx_magnitude(z, n);
    k = i + k;
    if (i != k && k < n) {
      for (int j = 0; j < n; ++j) {
        double b = A[i * n + j]; A[i * n + j] = A[k * n + j]; A[k * n + j] = b;
      }
      double c = RHS[i]; RHS[i] = RHS[k]; RHS[k] = c;
    }
    for (int j = i + 1; j < n; ++j) {
      double Factor = (1.0 / A[i * n + i]) * A[j * n + i];
      for (int kk = 0; kk < n; ++kk) A[j * n + kk] = A[j * n + kk] - Factor * A[i * n + kk];
      RHS[j] = RHS[j] - Factor * RHS[i];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double a = 0;
    for (int j = i + 1; j < n; ++j) a = a + A[i * n + j] * x[j];
    x[i] = (RHS[i] - a) / (A[i * n + i]);
  }
}

/* --------------------------------------------------- Gauss-Legendre tables */
/* The reference hard-codes Gauss-Legendre tables: 50 points printed to 8
   decimals (src/Main_Functions.cpp:3327-3346, :3649-3667, src/FEM.cpp:346-364)
   and 100 points in full precision (src/FEM.cpp:636-637).  Both are the
   Legendre roots and weights on [-1,1]; we compute them by Newton iteration
   and round the 50-point table to 8 decimals as the reference's literals are. */
void orc_gl_table(int n, double* xs, double* ws) {
  for (int i = 0; i < n; ++i) {
    double x = cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5));
    double dp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = n * (x * p1 - p0) / (x * x - 1.0);
      double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-17) break;
    }
    {
      double p0 = 1.0, p1 = x;
      for (int k = 2; k <= n; ++k) {
        double p2 = ((2.0 * k - 1.0) * x * p1 - (k - 1.0) * p0) / k;
        p0 = p1; p1 = p2;
      }
      dp = n * (x * p1 - p0) / (x * x - 1.0);
    }
    /* ascending order */
    xs[n - 1 - i] = x;
    ws[n - 1 - i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
  for (int i = 0; i < n / 2; ++i) { /* exact symmetry */
    double xa = 0.5 * (xs[n - 1 - i] - xs[i]);
    double wa = 0.5 * (ws[n - 1 - i] + ws[i]);
    xs[i] = -xa; xs[n - 1 - i] = xa; ws[i] = wa; ws[n - 1 - i] = wa;
  }
  if (n == 50) {
    for (int i = 0; i < n; ++i) {
      xs[i] = nearbyint(xs[i] * 1e8) / 1e8;
      ws[i] = nearbyint(ws[i] * 1e8) / 1e8;
    }
  }
}

/* ---------------------------------------------------------- cell_update -- */
/* binning, src/Main_Functions.cpp:2231-2266, and the per-cell index lists,
   :2367-2376 (ascending particle id within a cell). */
static void bin_particles(orc_state* s, const double* x1, const double* x2) {
  const mcpm_config* g = &s->cfg;
  for (int c = 0; c < s->C; ++c) s->cnt[c] = 0;
  for (int64_t i = 0; i < s->N; ++i) {
    int j = 0, k;
    if (g->direction[0] == 1) j = (int)floor(x1[i] / s->dx);
    k = (int)floor(x2[i] / s->dy);
    if (k > 0 && k < s->N1 - 1) {
      if (fabs(x2[i] - s->dy * k) < 1e-15 || fabs(x2[i] - s->dy * (k + 1)) < 1e-15) {
        uint32_t r[4];
        rng(s, (uint32_t)i, (uint32_t)s->step, RNG_STREAM_BIN, 0, r);
        int sgn = (u01(r[0]) > 0.5) ? 1 : -1;
        k = (int)floor((x2[i] + 1e-14 * sgn) / s->dy);
      }
    }
    /* the reference exits on an out-of-box particle; a particle on the far
       wall (x == Len, or x/dx rounding up to N) is binned into the last cell */
    if (g->direction[0] == 1 && !(x1[i] >= 0.0 && x1[i] <= g->length[0]))
      s->status |= MCPM_ERR_OUT_OF_BOX;
    if (!(x2[i] >= 0.0 && x2[i] <= g->length[1])) s->status |= MCPM_ERR_OUT_OF_BOX;
    if (j < 0) j = 0;
    if (j > s->N0 - 1) j = s->N0 - 1;
    if (k < 0) k = 0;
    if (k > s->N1 - 1) k = s->N1 - 1;
    int num = k * s->N0 + j;
    s->index[i] = num;
    s->cnt[num]++;
  }
  s->off[0] = 0;
  for (int c = 0; c < s->C; ++c) s->off[c + 1] = s->off[c] + s->cnt[c];
  int* fill = (int*)calloc(s->C, sizeof(int));
  for (int64_t i = 0; i < s->N; ++i) {
    int num = s->index[i];
    s->list[s->off[num] + fill[num]] = (int)i;
    fill[num]++;
  }
  free(fill);
}

/* moments, src/Main_Functions.cpp:2461-2593 */
static void moments(orc_state* s, const double* U1, const double* U2,
                    const double* U3) {
  const mcpm_config* g = &s->cfg;
  for (int num = 0; num < s->C; ++num) {
    double us0 = 0.0, us1 = 0.0, us2 = 0.0, weight = 0.0;
    int n_in = s->cnt[num];
    const int* L = &s->list[s->off[num]];
    for (int i = 0; i < n_in; ++i) {
      int id = L[i];
      double w = 1.0;
      us0 = us0 + U1[id] * w;
      us1 = us1 + U2[id] * w;
      us2 = us2 + U3[id] * w;
      weight += w;
    }
    if (n_in > 0) { us0 = us0 / weight; us1 = us1 / weight; us2 = us2 / weight; }
    double P[6] = {0}, M3[10] = {0}, M4[6] = {0}, M5[3] = {0}, Mp[3] = {0};
    double DM2 = 0.0, DM4 = 0.0, Q[3] = {0};
    for (int i = 0; i < n_in; ++i) {
      int id = L[i];
      double w = 1.0;
      double Mp1 = U1[id] - us0, Mp2 = U2[id] - us1, Mp3 = U3[id] - us2;
      Mp[0] += Mp1 * w; Mp[1] += Mp2 * w; Mp[2] += Mp3 * w;
      P[0] = P[0] + Mp1 * Mp1 * w;
      P[1] = P[1] + Mp1 * Mp2 * w;
      P[2] = P[2] + Mp1 * Mp3 * w;
      P[3] = P[3] + Mp2 * Mp2 * w;
      P[4] = P[4] + Mp2 * Mp3 * w;
      P[5] = P[5] + Mp3 * Mp3 * w;
      double energy = Mp1 * Mp1 + Mp2 * Mp2 + Mp3 * Mp3;
      M3[0] = M3[0] + Mp1 * Mp1 * Mp1 * w;
      M3[1] = M3[1] + Mp1 * Mp1 * Mp2 * w;
      M3[2] = M3[2] + Mp1 * Mp1 * Mp3 * w;
      M3[3] = M3[3] + Mp1 * Mp2 * Mp2 * w;
      M3[4] = M3[4] + Mp1 * Mp2 * Mp3 * w;
      M3[5] = M3[5] + Mp1 * Mp3 * Mp3 * w;
      M3[6] = M3[6] + Mp2 * Mp2 * Mp2 * w;
      M3[7] = M3[7] + Mp2 * Mp2 * Mp3 * w;
      M3[8] = M3[8] + Mp2 * Mp3 * Mp3 * w;
      M3[9] = M3[9] + Mp3 * Mp3 * Mp3 * w;
      M4[0] = M4[0] + Mp1 * Mp1 * energy * w;
      M4[1] = M4[1] + Mp1 * Mp2 * energy * w;
      M4[2] = M4[2] + Mp1 * Mp3 * energy * w;
      M4[3] = M4[3] + Mp2 * Mp2 * energy * w;
      M4[4] = M4[4] + Mp2 * Mp3 * energy * w;
      M4[5] = M4[5] + Mp3 * Mp3 * energy * w;
      M5[0] = M5[0] + Mp1 * energy * energy * w;
      M5[1] = M5[1] + Mp2 * energy * energy * w;
      M5[2] = M5[2] + Mp3 * energy * energy * w;
      DM2 = DM2 + energy * w;
    }
    if (n_in > 0) {
      for (int j = 0; j < 6; ++j) P[j] = P[j] / weight;
      for (int j = 0; j < 10; ++j) M3[j] = M3[j] / weight;
      for (int j = 0; j < 6; ++j) M4[j] = M4[j] / weight;
      for (int j = 0; j < 3; ++j) M5[j] = M5[j] / weight;
      for (int j = 0; j < 3; ++j) Mp[j] = Mp[j] / weight;
      DM2 = DM2 / weight;
      DM4 = M4[0] + M4[3] + M4[5];
      Q[0] = M3[0] + M3[3] + M3[5];
      Q[1] = M3[1] + M3[6] + M3[8];
      Q[2] = M3[2] + M3[7] + M3[9];
    }
    CELL(s, num, MCPM_CF_NUM_INSIDE) = n_in;
    CELL(s, num, MCPM_CF_U_SPACE + 0) = us0;
    CELL(s, num, MCPM_CF_U_SPACE + 1) = us1;
    CELL(s, num, MCPM_CF_U_SPACE + 2) = us2;
    for (int j = 0; j < 6; ++j) CELL(s, num, MCPM_CF_PIJ + j) = P[j];
    for (int j = 0; j < 10; ++j) CELL(s, num, MCPM_CF_M3 + j) = M3[j];
    for (int j = 0; j < 6; ++j) CELL(s, num, MCPM_CF_M4 + j) = M4[j];
    for (int j = 0; j < 3; ++j) CELL(s, num, MCPM_CF_M5 + j) = M5[j];
    for (int j = 0; j < 3; ++j) CELL(s, num, MCPM_CF_Q + j) = Q[j];
    for (int j = 0; j < 3; ++j) CELL(s, num, MCPM_CF_MP + j) = Mp[j];
    CELL(s, num, MCPM_CF_DM2) = DM2;
    CELL(s, num, MCPM_CF_DM4) = DM4;
    double T = g->m * DM2 / (3.0 * g->kb);
    double n = (s->cw ? s->cw[num] : 1) * g->Fn * weight / cell_volume(s, num);
    CELL(s, num, MCPM_CF_T) = T;
    CELL(s, num, MCPM_CF_N) = n;
    double Y = Ycoll(s, n);
    if (weight > 1e-14)
      CELL(s, num, MCPM_CF_GAMMA_ST) = -0.001 * (n * g->b * Y / (g->kb * T / g->m));
  }
}

/* Lambda closed form, src/Main_Functions.cpp:2718-2728 */
static void lambda_cells(orc_state* s) {
  const mcpm_config* g = &s->cfg;
  for (int num = 0; num < s->C; ++num) {
    if (!(CELL(s, num, MCPM_CF_NUM_INSIDE) > 1e-14)) continue;
    const double* P = &CELL(s, num, MCPM_CF_PIJ);
    double DM2 = CELL(s, num, MCPM_CF_DM2), T = CELL(s, num, MCPM_CF_T);
    double n = CELL(s, num, MCPM_CF_N);
    double mu = scale_mu(s, T);
    double tau = 2.0 * mu / (n * g->kb * T);
    double L = (P[0] - DM2 / 3.0) * ((P[3] - DM2 / 3.0) * (P[5] - DM2 / 3.0) - P[4] * P[4]);
    L = L - P[1] * (P[1] * (P[5] - DM2 / 3.0) - P[4] * P[2]);
    L = L + P[2] * (P[1] * P[4] - P[2] * (P[3] - DM2 / 3.0));
    L = -L / (tau * pow(DM2, 4.0));
    CELL(s, num, MCPM_CF_LAMBDA) = L;
  }
}

/* alpha_calculation, src/Fokker_Planck.cpp:200-587 (the live "with bulk
   term" branch).  div_U uses the linear neighbours num-1, num+1
   (src/Fokker_Planck.cpp:443-451); for the last cell of a 2-D grid, where the
   reference reads one past the end of the cell array, the one-sided
   difference of the upper end is used. */
static void alpha_cells(orc_state* s) {
  const mcpm_config* g = &s->cfg;
  const double pi = acos(-1.0);
  double A[144], rhs[12], x[12];
  for (int num = 0; num < s->C; ++num) {
    if (s->cnt[num] < 2) {
      for (int ii = 0; ii < 9; ++ii) CELL(s, num, MCPM_CF_ALPHA + ii) = 0.0;
      for (int ii = 0; ii < 3; ++ii) CELL(s, num, MCPM_CF_BETA + ii) = 0.0;
      continue;
    }
    const double* P = &CELL(s, num, MCPM_CF_PIJ);
    const double* M3 = &CELL(s, num, MCPM_CF_M3);
    const double* M4 = &CELL(s, num, MCPM_CF_M4);
    const double* M5 = &CELL(s, num, MCPM_CF_M5);
    double DM2 = CELL(s, num, MCPM_CF_DM2);
    double n = CELL(s, num, MCPM_CF_N), T = CELL(s, num, MCPM_CF_T);
    double gst = CELL(s, num, MCPM_CF_GAMMA_ST);
    double trace = P[0] + P[3] + P[5];
    double dev[6];
    for (int ii = 0; ii < 6; ++ii) dev[ii] = P[ii];
    dev[0] = dev[0] - (1.0 / 3.0) * trace;
    dev[3] = dev[3] - (1.0 / 3.0) * trace;
    dev[5] = dev[5] - (1.0 / 3.0) * trace;
    double a = M3[0] + M3[3] + M3[5];
    double b = M3[1] + M3[6] + M3[8];
    double c = M3[2] + M3[7] + M3[9];
    double d = M4[0] + M4[3] + M4[5] - DM2 * DM2;
    for (int ii = 0; ii < 144; ++ii) A[ii] = 0.0;
#define AA(r, q) A[(r) * 12 + (q)]
    AA(0, 0) = P[0]; AA(0, 1) = P[1]; AA(0, 2) = P[2]; AA(0, 9) = a;
    AA(1, 0) = P[1]; AA(1, 1) = P[3]; AA(1, 2) = P[4]; AA(1, 9) = a;
    AA(2, 0) = P[2]; AA(2, 1) = P[4]; AA(2, 2) = P[5]; AA(2, 9) = a;
    AA(3, 3) = P[0]; AA(3, 4) = P[1]; AA(3, 5) = P[2]; AA(3, 10) = b;
    AA(4, 3) = P[1]; AA(4, 4) = P[3]; AA(4, 5) = P[4]; AA(4, 10) = b;
    AA(5, 3) = P[2]; AA(5, 4) = P[4]; AA(5, 5) = P[5]; AA(5, 10) = b;
    AA(6, 6) = P[0]; AA(6, 7) = P[1]; AA(6, 8) = P[2]; AA(6, 11) = c;
    AA(7, 6) = P[1]; AA(7, 7) = P[3]; AA(7, 8) = P[4]; AA(7, 11) = c;
    AA(8, 6) = P[2]; AA(8, 7) = P[4]; AA(8, 8) = P[5]; AA(8, 11) = c;
    AA(9, 0) = a; AA(9, 1) = b; AA(9, 2) = c; AA(9, 9) = d;
    AA(10, 3) = a; AA(10, 4) = b; AA(10, 5) = c; AA(10, 10) = d;
    AA(11, 6) = a; AA(11, 7) = b; AA(11, 8) = c; AA(11, 11) = d;
#undef AA
    double Y = Ycoll(s, n);
    double p_crr = (1.0 + n * g->b * Y);
    double mu_crr = (1.0 + 2.0 * n * g->b * Y / 5.0);
    double k_crr = (1.0 + 3.0 * n * g->b * Y / 5.0);
    double w = (4.0 / 9.0) * sqrt(pi) * Y * pow(n, 2.0) * pow(g->sigma, 4.0) * sqrt(g->m * g->kb * T);
    double div_U;
    int last = s->C - 1;
    if (s->C == 1) {
      div_U = 0.0;
    } else if (num == 0) {
      div_U = (CELL(s, num + 1, MCPM_CF_U_SPACE + 1) - CELL(s, num, MCPM_CF_U_SPACE + 1)) / s->dy;
    } else if (num == s->N1 - 1 || num == last) {
      div_U = (CELL(s, num, MCPM_CF_U_SPACE + 1) - CELL(s, num - 1, MCPM_CF_U_SPACE + 1)) / s->dy;
    } else {
      div_U = (CELL(s, num + 1, MCPM_CF_U_SPACE + 1) - CELL(s, num - 1, MCPM_CF_U_SPACE + 1)) / s->dy / 2.0;
    }
    CELL(s, num, MCPM_CF_DIVU) = div_U;
    double coeff_mu = 3.0 * 1.002 / 5.0 * pow(n * g->b * Y, 2.0) / (1 + 2.0 * n * g->b * Y / 5.0);
    double coeff_k = 1.002 * pow(n * g->b * Y, 2.0) / (1 + 3.0 * n * g->b * Y / 5.0) / 5.0;
    rhs[0] = (mu_crr - 1.0) * dev[0] + (p_crr - 1.0) * trace / 3.0 - w * div_U / (g->m * n) + coeff_mu * dev[0] - gst * M4[0];
    rhs[1] = (mu_crr - 1.0) * dev[1] + coeff_mu * dev[1] - gst * M4[1];
    rhs[2] = (mu_crr - 1.0) * dev[2] + coeff_mu * dev[2] - gst * M4[2];
    rhs[3] = (mu_crr - 1.0) * dev[1] + coeff_mu * dev[1] - gst * M4[1];
    rhs[4] = (mu_crr - 1.0) * dev[3] + (p_crr - 1.0) * trace / 3.0 - w * div_U / (g->m * n) + coeff_mu * dev[3] - gst * M4[3];
    rhs[5] = (mu_crr - 1.0) * dev[4] + coeff_mu * dev[4] - gst * M4[4];
    rhs[6] = (mu_crr - 1.0) * dev[2] + coeff_mu * dev[2] - gst * M4[2];
    rhs[7] = (mu_crr - 1.0) * dev[4] + coeff_mu * dev[4] - gst * M4[4];
    rhs[8] = (mu_crr - 1.0) * dev[5] + (p_crr - 1.0) * trace / 3.0 - w * div_U / (g->m * n) + coeff_mu * dev[5] - gst * M4[5];
    rhs[9] = (k_crr - 1.0) * a + coeff_k * a - gst * (M5[0]) + gst * (DM2 * (M3[0] + M3[3] + M3[5]));
    rhs[10] = (k_crr - 1.0) * b + coeff_k * b - gst * (M5[1]) + gst * (DM2 * (M3[1] + M3[6] + M3[8]));
    rhs[11] = (k_crr - 1.0) * c + coeff_k * c - gst * (M5[2]) + gst * (DM2 * (M3[2] + M3[7] + M3[9]));
    orc_gauss_jordan(A, rhs, 12, x);
    for (int ii = 0; ii < 12; ++ii)
      if (x[ii] != x[ii]) s->status |= MCPM_ERR_NAN;
    for (int ii = 0; ii < 9; ++ii) CELL(s, num, MCPM_CF_ALPHA + ii) = x[ii];
    for (int ii = 0; ii < 3; ++ii) CELL(s, num, MCPM_CF_BETA + ii) = x[9 + ii];
  }
}

/* c_gamma_calculation, src/Fokker_Planck.cpp:590-804 */
static void c_gamma_cells(orc_state* s) {
  const mcpm_config* g = &s->cfg;
  double A[81], rhs[9], x[9];
  for (int num = 0; num < s->C; ++num) {
    if (s->cnt[num] < 2) {
      for (int ii = 0; ii < 6; ++ii) CELL(s, num, MCPM_CF_C + ii) = 0.0;
      for (int ii = 0; ii < 3; ++ii) CELL(s, num, MCPM_CF_GAMMA + ii) = 0.0;
      continue;
    }
    const double* P = &CELL(s, num, MCPM_CF_PIJ);
    const double* M3 = &CELL(s, num, MCPM_CF_M3);
    const double* M4 = &CELL(s, num, MCPM_CF_M4);
    const double* M5 = &CELL(s, num, MCPM_CF_M5);
    const double* Q = &CELL(s, num, MCPM_CF_Q);
    double DM2 = CELL(s, num, MCPM_CF_DM2), DM4 = CELL(s, num, MCPM_CF_DM4);
    double n = CELL(s, num, MCPM_CF_N), T = CELL(s, num, MCPM_CF_T);
    double Lam = CELL(s, num, MCPM_CF_LAMBDA);
    for (int ii = 0; ii < 81; ++ii) A[ii] = 0.0;
    for (int ii = 0; ii < 9; ++ii) { rhs[ii] = 0.0; x[ii] = 0.0; }
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
    double Pr = 2.0 / 3.0;
    double Y = (g->model == MCPM_MODEL_FP_DENSE) ? Ycoll(s, n) : 1.0;
    double mu = scale_mu(s, T);
    double tau = 2.0 * mu / (n * g->kb * T);
    for (int ii = 0; ii < 6; ++ii) rhs[ii] = -2.0 * Lam * M4[ii];
    rhs[6] = Y * (3.0 / tau - 2.0 * Pr / tau) * Q[0];
    rhs[7] = Y * (3.0 / tau - 2.0 * Pr / tau) * Q[1];
    rhs[8] = Y * (3.0 / tau - 2.0 * Pr / tau) * Q[2];
    rhs[6] += Lam * (-3.0 * M5[0] + DM2 * Q[0] + 2.0 * (P[0] * Q[0] + P[1] * Q[1] + P[2] * Q[2]));
    rhs[7] += Lam * (-3.0 * M5[1] + DM2 * Q[1] + 2.0 * (P[1] * Q[0] + P[3] * Q[1] + P[4] * Q[2]));
    rhs[8] += Lam * (-3.0 * M5[2] + DM2 * Q[2] + 2.0 * (P[2] * Q[0] + P[4] * Q[1] + P[5] * Q[2]));
    orc_gauss_jordan(A, rhs, 9, x);
    for (int ii = 0; ii < 6; ++ii) CELL(s, num, MCPM_CF_C + ii) = x[ii];
    for (int ii = 0; ii < 3; ++ii) CELL(s, num, MCPM_CF_GAMMA + ii) = x[6 + ii];
  }
}

/* phi = alpha * <M'>, src/Main_Functions.cpp:2734-2746 */
static void phi_cells(orc_state* s) {
  for (int num = 0; num < s->C; ++num) {
    const double* al = &CELL(s, num, MCPM_CF_ALPHA);
    const double* Mp = &CELL(s, num, MCPM_CF_MP);
    CELL(s, num, MCPM_CF_PHI + 0) = al[0] * Mp[0] + al[1] * Mp[1] + al[2] * Mp[2];
    CELL(s, num, MCPM_CF_PHI + 1) = al[3] * Mp[0] + al[4] * Mp[1] + al[5] * Mp[2];
    CELL(s, num, MCPM_CF_PHI + 2) = al[6] * Mp[0] + al[7] * Mp[1] + al[8] * Mp[2];
  }
}

/* Kernel smoothing of cell_update, src/Main_Functions.cpp:2378-2427: at the
   centre of every cell a Gaussian of width h = dy/2, cut at r_cut = 2 dy,
   over the particles of rows k-2..k+2 of its column (a row past a wall
   takes the wall row's particles shifted by whole cells), summed in the
   reference's order (column, row, neighbour row, particle id). */
static void kernel_smoothing(orc_state* s, const double* x2) {
  const double dy = s->dy;
  double r_cut = 2.0 * dy, h = r_cut / 4.0;
  double sqrt_pi = sqrt(2.0 * acos(-1.0));
  int search = (int)floor(r_cut / dy);
  double mb = s->cfg.Fn;
  double s2h2 = pow(1.0 / h / h, 2.0);
  for (int num = 0; num < s->C; ++num) {
    CELL(s, num, MCPM_CF_N_SMOOTH) = 0.0;
    CELL(s, num, MCPM_CF_DN2) = 0.0;
    CELL(s, num, MCPM_CF_DN3) = 0.0;
  }
  for (int j = 0; j < s->N0; ++j)
    for (int k = 0; k < s->N1; ++k) {
      int num = k * s->N0 + j;
      double d2 = (double)k * dy, d3 = (double)(k + 1) * dy;
      double r1 = 0.5 * (d2 + d3);
      for (int kk = k - search; kk <= k + search; ++kk) {
        int kkk = kk < 0 ? 0 : (kk > s->N1 - 1 ? s->N1 - 1 : kk);
        int num2 = kkk * s->N0 + j;
        for (int i = 0; i < s->cnt[num2]; ++i) {
          int64_t id = s->list[s->off[num2] + i];
          double r2 = x2[id] + (kk - kkk) * dy;
          double r1r2 = r2 - r1;
          double rr = fabs(r2 - r1);
          if (rr < r_cut) {
            CELL(s, num, MCPM_CF_N_SMOOTH) += mb / sqrt_pi / h * exp(-rr * rr / h / h / 2.0);
            double W = 1.0 / sqrt_pi / h * exp(-rr * rr / h / h / 2.0);
            CELL(s, num, MCPM_CF_DN2) += mb * W * r1r2 * (-1.0 / h / h);
            CELL(s, num, MCPM_CF_DN3) += mb * W * s2h2 * (3.0 * r1r2 - 1.0 / h / h * r1r2 * r1r2 * r1r2);
          }
        }
      }
    }
}

/* cell_update, src/Main_Functions.cpp:2138-2749, for the uniform Cartesian
   grid.  The kernel-density smoothing (:2378-2427) feeds only long_range 2,
   which is out of scope, and is not computed. */
void orc_cell_update(orc_state* s, const double* x1, const double* x2,
                     const double* U1, const double* U2, const double* U3,
                     int32_t* index) {
  bin_particles(s, x1, x2);
  if (x1) node_density(s, x1, x2);
  if (s->cfg.long_range == MCPM_LR_DENSITY_EXPANSION) kernel_smoothing(s, x2);
  if (index) memcpy(index, s->index, sizeof(int32_t) * (size_t)s->N);
  moments(s, U1, U2, U3);
  lambda_cells(s);
  int m = s->cfg.model;
  if (m == MCPM_MODEL_FP_DENSE || m == MCPM_MODEL_FP_IDEAL_GAS || m == MCPM_MODEL_FP_LINEAR) {
    if (s->step > 0 && m == MCPM_MODEL_FP_DENSE) alpha_cells(s);
    c_gamma_cells(s);
  }
  phi_cells(s);
}

/* ----------------------------------------------------- random_generator -- */
/* src/Fokker_Planck.cpp:20-145: 3 draws per particle, centred per cell, then
   divided by the per-cell RMS when the cell holds more than one particle.
   Sums run in particle order as in the reference. */
void orc_random_generator(orc_state* s, double* x1f, double* x2f, double* x3f) {
  int64_t N = s->N;
  for (int64_t i = 0; i < N; ++i) {
    if (s->rng_mode == MCPM_RNG_INJECTED) {
      x1f[i] = s->inj[i]; x2f[i] = s->inj[N + i]; x3f[i] = s->inj[2 * N + i];
    } else {
      double z[4];
      normals4_s(s, (uint32_t)i, (uint32_t)s->step, RNG_STREAM_FP, 0, z);
      x1f[i] = z[0]; x2f[i] = z[1]; x3f[i] = z[2];
    }
  }
  double* s1 = (double*)calloc(s->C, sizeof(double));
  double* s2 = (double*)calloc(s->C, sizeof(double));
  double* s3 = (double*)calloc(s->C, sizeof(double));
  double* y1 = (double*)malloc(sizeof(double) * (size_t)N);
  double* y2 = (double*)malloc(sizeof(double) * (size_t)N);
  double* y3 = (double*)malloc(sizeof(double) * (size_t)N);
  for (int64_t i = 0; i < N; ++i) {
    int num = s->index[i];
    s1[num] += x1f[i]; s2[num] += x2f[i]; s3[num] += x3f[i];
  }
  for (int64_t i = 0; i < N; ++i) {
    int num = s->index[i];
    y1[i] = x1f[i] - s1[num] / (1.0 * s->cnt[num]);
    y2[i] = x2f[i] - s2[num] / (1.0 * s->cnt[num]);
    y3[i] = x3f[i] - s3[num] / (1.0 * s->cnt[num]);
  }
  for (int c = 0; c < s->C; ++c) { s1[c] = 0.0; s2[c] = 0.0; s3[c] = 0.0; }
  for (int64_t i = 0; i < N; ++i) {
    int num = s->index[i];
    s1[num] += y1[i] * y1[i]; s2[num] += y2[i] * y2[i]; s3[num] += y3[i] * y3[i];
  }
  for (int c = 0; c < s->C; ++c) {
    s1[c] = sqrt(s1[c] / (1.0 * s->cnt[c]));
    s2[c] = sqrt(s2[c] / (1.0 * s->cnt[c]));
    s3[c] = sqrt(s3[c] / (1.0 * s->cnt[c]));
  }
  for (int64_t i = 0; i < N; ++i) {
    int num = s->index[i];
    if (s->cnt[num] > 1) {
      x1f[i] = y1[i] / s1[num]; x2f[i] = y2[i] / s2[num]; x3f[i] = y3[i] / s3[num];
    }
  }
  for (int64_t i = 0; i < N; ++i) {
    s->xi[i] = x1f[i]; s->xi[N + i] = x2f[i]; s->xi[2 * N + i] = x3f[i];
  }
  free(s1); free(s2); free(s3); free(y1); free(y2); free(y3);
}

/* ------------------------------------------------- Velocity_FP_parallel -- */
/* src/Fokker_Planck.cpp:1065-1182: Ornstein-Uhlenbeck step with the cubic
   drift, then per-cell rescaling that restores sum |M'|^2 exactly.
   FP_linear (Velocity_FP_linear, :1186-1283) is the same step without the
   drift, Y = 1; its face-force term F (:1246-1260) is computed but never
   used there and is left out.  Velocity_FP_linear has no one-particle
   guard: such a cell has T = 0 and its tau is 0/0, so the reference stops
   on its NaN check (:1266-1268); here it takes the guarded branch of
   Velocity_FP_parallel (U = U_space, the particle keeps its velocity). */
void orc_velocity_fp(orc_state* s, double* U1, double* U2, double* U3,
                     const double* xi1, const double* xi2, const double* xi3) {
  const mcpm_config* g = &s->cfg;
  int64_t N = s->N;
  double* frac1 = (double*)calloc(s->C, sizeof(double));
  double* frac2 = (double*)calloc(s->C, sizeof(double));
  double* Mp1 = (double*)malloc(sizeof(double) * (size_t)N);
  double* Mp2 = (double*)malloc(sizeof(double) * (size_t)N);
  double* Mp3 = (double*)malloc(sizeof(double) * (size_t)N);
  for (int64_t id = 0; id < N; ++id) {
    int num = s->index[id];
    Mp1[id] = U1[id] - CELL(s, num, MCPM_CF_U_SPACE + 0);
    Mp2[id] = U2[id] - CELL(s, num, MCPM_CF_U_SPACE + 1);
    Mp3[id] = U3[id] - CELL(s, num, MCPM_CF_U_SPACE + 2);
    frac1[num] += Mp1[id] * Mp1[id] + Mp2[id] * Mp2[id] + Mp3[id] * Mp3[id];
  }
  for (int64_t id = 0; id < N; ++id) {
    int num = s->index[id];
    if (s->cnt[num] > 1) {
      double T = CELL(s, num, MCPM_CF_T), n = CELL(s, num, MCPM_CF_N);
      double mu = scale_mu(s, T);
      double tau = 2.0 * mu / (n * g->kb * T);
      double Y = (g->model == MCPM_MODEL_FP_DENSE) ? Ycoll(s, n) : 1.0;
      tau = tau / Y;
      double A1 = exp(-g->dt / tau);
      double A3 = sqrt((1.0 - exp(-2.0 * g->dt / tau)) * g->kb * T / (1.0 * g->m));
      double A2 = (1.0 - exp(-g->dt / tau)) * tau;
      if (g->model == MCPM_MODEL_FP_LINEAR) {
        /* Velocity_FP_linear, src/Fokker_Planck.cpp:1262-1264: no drift */
        Mp1[id] = A1 * Mp1[id] + A3 * xi1[id];
        Mp2[id] = A1 * Mp2[id] + A3 * xi2[id];
        Mp3[id] = A1 * Mp3[id] + A3 * xi3[id];
        if (Mp2[id] != Mp2[id]) s->status |= MCPM_ERR_NAN;
        continue;
      }
      double energy = Mp1[id] * Mp1[id] + Mp2[id] * Mp2[id] + Mp3[id] * Mp3[id];
      const double* c = &CELL(s, num, MCPM_CF_C);
      const double* gm = &CELL(s, num, MCPM_CF_GAMMA);
      const double* Q = &CELL(s, num, MCPM_CF_Q);
      double Lam = CELL(s, num, MCPM_CF_LAMBDA);
      double d0, d1, d2;
      d0 = c[0] * Mp1[id] + c[1] * Mp2[id] + c[2] * Mp3[id];
      d0 += gm[0] * (energy - 3.0 * g->kb * T / g->m);
      d0 += Lam * (Mp1[id] * energy - Q[0]);
      d1 = c[1] * Mp1[id] + c[3] * Mp2[id] + c[4] * Mp3[id];
      d1 += gm[1] * (energy - 3.0 * g->kb * T / g->m);
      d1 += Lam * (Mp2[id] * energy - Q[1]);
      d2 = c[2] * Mp1[id] + c[4] * Mp2[id] + c[5] * Mp3[id];
      d2 += gm[2] * (energy - 3.0 * g->kb * T / g->m);
      d2 += Lam * (Mp3[id] * energy - Q[2]);
      Mp1[id] = A1 * Mp1[id] + A2 * d0 + A3 * xi1[id];
      Mp2[id] = A1 * Mp2[id] + A2 * d1 + A3 * xi2[id];
      Mp3[id] = A1 * Mp3[id] + A2 * d2 + A3 * xi3[id];
    } else {
      Mp1[id] = 0.0; Mp2[id] = 0.0; Mp3[id] = 0.0;
    }
    if (Mp2[id] != Mp2[id]) s->status |= MCPM_ERR_NAN;
  }
  for (int64_t id = 0; id < N; ++id) {
    int num = s->index[id];
    frac2[num] += Mp1[id] * Mp1[id] + Mp2[id] * Mp2[id] + Mp3[id] * Mp3[id];
  }
  for (int64_t id = 0; id < N; ++id) {
    int num = s->index[id];
    const double* Us = &CELL(s, num, MCPM_CF_U_SPACE);
    if (s->cnt[num] > 1) {
      double r = sqrt(fabs(frac1[num] / frac2[num]));
      U1[id] = Mp1[id] * r + Us[0];
      U2[id] = Mp2[id] * r + Us[1];
      U3[id] = Mp3[id] * r + Us[2];
    } else {
      U1[id] = Us[0]; U2[id] = Us[1]; U3[id] = Us[2];
    }
  }
  free(frac1); free(frac2); free(Mp1); free(Mp2); free(Mp3);
}

/* ------------------------------------------------------------------ ESMC -- */
/* Collision_ESMC_new3, src/collisions.cpp:583-720, restated per cell.
   The reference assigns its M = sum_c m_c candidates to cells by sampling
   candidate slots without replacement through a linear prefix scan
   (:631-646); that gives every cell exactly its m_c = floor(omega_max/2 N_c+u)
   candidates, so here each cell simply runs its own m_c candidates.
   Candidates that may touch the same particle are serialised: cells are
   processed in colour classes whose partner neighbourhoods (+-R cells,
   R = ceil(sigma/dx)) are disjoint, candidates of one cell in order.  This
   is the order the GPU uses.  Per candidate, the physics is the
   reference's: partner cell at r_i + sigma e, Y at the midpoint, acceptance
   omega/omega_max > u, no g.e > 0 test, U_i -= (g.e)e, U_j += (g.e)e. */
static void esmc_cell(orc_state* s, int I, const double* x1, const double* x2,
                      double* U1, double* U2, double* U3) {
  const mcpm_config* g = &s->cfg;
  const double pi = acos(-1.0);
  int NI = s->cnt[I];
  uint32_t r[4];
  rng(s, (uint32_t)I, (uint32_t)s->step, RNG_STREAM_ESMC_M, 0, r);
  double om_max = CELL(s, I, MCPM_CF_OMEGA_MAX);
  int mI = (int)floor(0.5 * om_max * (1.0 * NI) + u01(r[0]));
  double omega = 0.0;
  if (NI > 0) {
    for (int k = 0; k < mI; ++k) {
      rng(s, (uint32_t)I, (uint32_t)s->step, RNG_STREAM_ESMC, (uint32_t)k, r);
      int i = s->list[s->off[I] + pick(r[0], NI)];
      double theta = 2.0 * pi * u01(r[1]);
      double cph = 2.0 * u01(r[2]) - 1.0;
      double sph = sqrt(1.0 - cph * cph);
      double dir0 = cos(theta) * sph, dir1 = sin(theta) * sph, dir2 = cph;
      double xx = x1[i] + g->sigma * dir0;
      double yy = x2[i] + g->sigma * dir1;
      int i0 = (int)floor(xx / s->dx), i1 = (int)floor(yy / s->dy);
      int J = i1 * s->N0 + i0;
      if (!(i0 >= 0 && i0 < s->N0 && i1 >= 0 && i1 < s->N1)) continue;
      int NJ = s->cnt[J];
      if (NJ <= 0) continue;
      int j = s->list[s->off[J] + pick(r[3], NJ)];
      if (i == j) continue;
      double xm0 = (x1[i] + x1[j]) / 2.0, xm1 = (x2[i] + x2[j]) / 2.0;
      int m0 = (int)floor(xm0 / s->dx), m1 = (int)floor(xm1 / s->dy);
      if (m0 < 0) m0 = 0; if (m0 > s->N0 - 1) m0 = s->N0 - 1;
      if (m1 < 0) m1 = 0; if (m1 > s->N1 - 1) m1 = s->N1 - 1;
      double Ymid = Ycoll(s, CELL(s, m1 * s->N0 + m0, MCPM_CF_N));
      double g0 = U1[i] - U1[j], g1 = U2[i] - U2[j], g2 = U3[i] - U3[j];
      double gd = g0 * dir0 + g1 * dir1 + g2 * dir2;
      double dummy = 4.0 * pi * g->sigma * g->sigma * gd * Ymid * CELL(s, J, MCPM_CF_N) * g->dt;
      if (dummy - omega > 0.0) omega = dummy;
      uint32_t ra[4];
      rng(s, (uint32_t)I, (uint32_t)s->step, RNG_STREAM_ESMC_ACC, (uint32_t)k, ra);
      if (dummy / om_max > u01(ra[0])) {
        U1[i] = U1[i] - gd * dir0; U2[i] = U2[i] - gd * dir1; U3[i] = U3[i] - gd * dir2;
        U1[j] = U1[j] + gd * dir0; U2[j] = U2[j] + gd * dir1; U3[j] = U3[j] + gd * dir2;
      }
    }
  }
  CELL(s, I, MCPM_CF_OMEGA_MAX) = omega > om_max ? omega : om_max;
}

void orc_esmc(orc_state* s, const double* x1, const double* x2, double* U1,
              double* U2, double* U3) {
  int Rx = (int)ceil(s->cfg.sigma / s->dx), Ry = (int)ceil(s->cfg.sigma / s->dy);
  if (Rx < 1) Rx = 1;
  if (Ry < 1) Ry = 1;
  int Sx = (s->N0 > 1) ? 2 * Rx + 1 : 1, Sy = 2 * Ry + 1;
  for (int cy = 0; cy < Sy; ++cy)
    for (int cx = 0; cx < Sx; ++cx)
      for (int k = cy; k < s->N1; k += Sy)
        for (int j = cx; j < s->N0; j += Sx) esmc_cell(s, k * s->N0 + j, x1, x2, U1, U2, U3);
}

/* -------------------------------------------------------------- DSMC VHS -- */
/* Collision_DSMC_VHS, src/collisions.cpp:2063-2141, restated with
   counter-based draws.  Per cell I with N_I > 1: the reference loops while
   cand < floor(M + u) with a fresh u per test (:2090), which stops after
   floor(M) or floor(M) + 1 candidates with the probabilities of
   floor(M + u); here one u gives that count.  Each candidate takes two
   distinct particles of the cell uniformly (the reference redraws the
   second until it differs, :2092-2096: the same distribution),
   sigma_T = |g|^(2 - 2 visp) crref^(2 visp - 1) (:2102), the running maximum
   of sigma_T, acceptance sigma_T / crm > u (:2106) and on acceptance an
   isotropic relative velocity of the same magnitude about the pair's centre
   of mass (:2107-2127).  Finally crm = max(1.1 max sigma_T, 0.9 crm) (:2135).
   The cell's crm lives in the OMEGA_MAX field. */
static void dsmc_cell(orc_state* s, int I, double* U1, double* U2, double* U3) {
  const mcpm_config* g = &s->cfg;
  const double pi = acos(-1.0);
  int NI = s->cnt[I];
  if (NI <= 1) return;
  uint32_t r[4], ra[4];
  double crm_cell = CELL(s, I, MCPM_CF_OMEGA_MAX);
  rng(s, (uint32_t)I, (uint32_t)s->step, RNG_STREAM_DSMC_M, 0, r);
  double M_cand = pi * g->sigma * g->sigma * ((double)NI * CELL(s, I, MCPM_CF_N)) * crm_cell * g->dt / 2.0;
  int mI = (int)floor(M_cand + u01(r[0]));
  double crm = 0.0;
  double crfac = pow(g->crref, 2.0 * g->visp - 1.0);
  for (int k = 0; k < mI; ++k) {
    rng(s, (uint32_t)I, (uint32_t)s->step, RNG_STREAM_DSMC, (uint32_t)k, r);
    int a = pick(r[0], NI), b = pick(r[1], NI - 1);
    if (b >= a) b += 1;
    int i = s->list[s->off[I] + a], j = s->list[s->off[I] + b];
    double Vr = sqrt((U1[i] - U1[j]) * (U1[i] - U1[j]) + (U2[i] - U2[j]) * (U2[i] - U2[j]) +
                     (U3[i] - U3[j]) * (U3[i] - U3[j]));
    double sigmat = pow(Vr, (2.0 - 2.0 * g->visp)) * crfac;
    if (sigmat - crm > 0.0) crm = sigmat;
    if (sigmat / crm_cell > u01(r[2])) {
      rng(s, (uint32_t)I, (uint32_t)s->step, RNG_STREAM_DSMC_ACC, (uint32_t)k, ra);
      double theta = acos(2.0 * u01(r[3]) - 1.0);
      double phi = 2.0 * pi * u01(ra[0]);
      double v0 = Vr * cos(theta), v1 = Vr * sin(theta) * cos(phi), v2 = Vr * sin(theta) * sin(phi);
      double c0 = 0.5 * (U1[i] + U1[j]), c1 = 0.5 * (U2[i] + U2[j]), c2 = 0.5 * (U3[i] + U3[j]);
      U1[i] = c0 + 0.5 * v0; U2[i] = c1 + 0.5 * v1; U3[i] = c2 + 0.5 * v2;
      U1[j] = c0 - 0.5 * v0; U2[j] = c1 - 0.5 * v1; U3[j] = c2 - 0.5 * v2;
    }
  }
  double x = 1.1 * crm, y = 0.9 * crm_cell;
  CELL(s, I, MCPM_CF_OMEGA_MAX) = x < y ? y : x;
}

void orc_dsmc_vhs(orc_state* s, double* U1, double* U2, double* U3) {
  for (int I = 0; I < s->C; ++I) dsmc_cell(s, I, U1, U2, U3);
}

/* ---------------------------------------------------------- sampling -- */
/* cell_poly_velocity, src/Main_Functions.cpp:1918-1968, in particle-id order:
   adds every particle's raw velocity products to acc, [C][MCPM_SF_COUNT]
   cell-major (the CELLS members sum_weight, sum_M, sum_MM, sum_MMM,
   sum_MMMM). */
void orc_sample_cells(orc_state* s, const double* U1, const double* U2, const double* U3, double* acc) {
  for (int64_t i = 0; i < s->N; ++i) {
    int num = s->index[i];
    double* a = acc + (size_t)num * MCPM_SF_COUNT;
    a[MCPM_SF_WEIGHT] += 1.0;
    a[MCPM_SF_M + 0] += U1[i];
    a[MCPM_SF_M + 1] += U2[i];
    a[MCPM_SF_M + 2] += U3[i];
    a[MCPM_SF_MM + 0] += U1[i] * U1[i];
    a[MCPM_SF_MM + 1] += U1[i] * U2[i];
    a[MCPM_SF_MM + 2] += U1[i] * U3[i];
    a[MCPM_SF_MM + 3] += U2[i] * U2[i];
    a[MCPM_SF_MM + 4] += U2[i] * U3[i];
    a[MCPM_SF_MM + 5] += U3[i] * U3[i];
    int id = 0;
    for (int m = 0; m < 4; ++m)
      for (int n = 0; n < 4 - m; ++n) {
        int l = 3 - m - n;
        a[MCPM_SF_MMM + id] += pow(U1[i], m) * pow(U2[i], n) * pow(U3[i], l);
        id++;
      }
    double energy = U1[i] * U1[i] + U2[i] * U2[i] + U3[i] * U3[i];
    a[MCPM_SF_MMMM + 0] += U1[i] * U1[i] * energy;
    a[MCPM_SF_MMMM + 1] += U1[i] * U2[i] * energy;
    a[MCPM_SF_MMMM + 2] += U1[i] * U3[i] * energy;
    a[MCPM_SF_MMMM + 3] += U2[i] * U2[i] * energy;
    a[MCPM_SF_MMMM + 4] += U2[i] * U3[i] * energy;
    a[MCPM_SF_MMMM + 5] += U3[i] * U3[i] * energy;
  }
}

/* ESMC majorant initialisation, src/main.cpp:250-269 */
void orc_init_omega_max(orc_state* s) {
  const mcpm_config* g = &s->cfg;
  double pi = acos(-1);
  for (int num = 0; num < s->C; ++num) {
    double thermal = sqrt(g->kb * CELL(s, num, MCPM_CF_T) / g->m);
    double crm = 10.0 * (thermal);
    double om = 4.0 * pi * g->sigma * g->sigma * crm * CELL(s, num, MCPM_CF_N) * g->dt;
    if (g->model == MCPM_MODEL_ESMC) om = om * Ycoll(s, g->n);
    /* DSMC_VHS keeps cells[].crm in this field */
    CELL(s, num, MCPM_CF_OMEGA_MAX) = (g->model == MCPM_MODEL_DSMC_VHS) ? crm : om;
  }
}

/* ------------------------------------------------------------ Vlasov 1-D -- */
/* density lookup with the reference's edge clamping */
static double n_lookup(const orc_state* s, int num) {
  if (num > -1 && num < s->N1) return CELL(s, num, MCPM_CF_N);
  if (num < 0) return CELL(s, 0, MCPM_CF_N);
  return CELL(s, s->N1 - 1, MCPM_CF_N);
}

/* vlasov_taking_the_integral, src/Main_Functions.cpp:3582-3942: face
   potentials V_f = sum_{r,phi} (sigma/r)^6 r^2 2pi n(y_f + r cos phi) sin phi
   on the GL(50) x GL(50) grid, r in [eqdist, 3 eqdist], phi in [0, pi]. */
void orc_vlasov_face_potential(orc_state* s, double* V) {
  const mcpm_config* g = &s->cfg;
  double xi[50], wi[50], rr[50], dr[50], ph[50], dph[50];
  orc_gl_table(50, xi, wi);
  double pi = acos(-1);
  double b = 3.0 * g->eqdist, a = 1.0 * g->eqdist, c = 0.0, d = pi;
  for (int i = 0; i < 50; ++i) { rr[i] = (b - a) / 2.0 * xi[i] + (a + b) / 2.0; dr[i] = wi[i] * (b - a) / 2.0; }
  for (int i = 0; i < 50; ++i) { ph[i] = (d - c) / 2.0 * xi[i] + (c + d) / 2.0; dph[i] = wi[i] * (d - c) / 2.0; }
  double int_theta = 2.0 * pi;
  int nf = s->N1 + 1;
  for (int fc = 0; fc < nf; ++fc) {
    V[fc] = 0.0;
    for (int i = 0; i < 50; ++i) {
      double radial_part = -(-pow(g->sigma / rr[i], 6.0)) * rr[i] * rr[i] * int_theta * dr[i];
      for (int ii = 0; ii < 50; ++ii) {
        double y = fc * s->dy + rr[i] * cos(ph[ii]);
        int num = (int)floor(y / s->dy);
        double n = n_lookup(s, num);
        V[fc] += -radial_part * n * sin(ph[ii]) * dph[ii];
      }
    }
  }
}

/* Thompson_3d, src/Math_Func.cpp:28-52 (b lower, c upper diagonal) */
static void thomas(double* a, const double* b, const double* c, double* x,
                   double* RHS, int n) {
  for (int i = 1; i < n; ++i) {
    double Factor = (1.0 / a[i - 1]) * b[i - 1];
    a[i] = a[i] - c[i - 1] * Factor;
    RHS[i] = RHS[i] - Factor * RHS[i - 1];
  }
  for (int i = n - 1; i >= 0; --i) {
    double r = RHS[i];
    if (i != n - 1) r = r - c[i] * x[i + 1];
    x[i] = r / a[i];
  }
}

/* poisson_solver, src/Main_Functions.cpp:3285-3581: screened-Poisson face
   potential with Green's-function Dirichlet values at both walls, minus the
   analytic r < sigma part. x receives the corrected face potential. */
void orc_poisson_faces(orc_state* s, double* x) {
  const mcpm_config* g = &s->cfg;
  int nf = s->N1 + 1;
  double* a = (double*)malloc(sizeof(double) * nf);
  double* b = (double*)malloc(sizeof(double) * nf);
  double* c = (double*)malloc(sizeof(double) * nf);
  double* nj = (double*)malloc(sizeof(double) * nf);
  double* rhs = (double*)malloc(sizeof(double) * nf);
  double xi[50], wi[50], rr[50], dr[50], ph[50], dph[50];
  orc_gl_table(50, xi, wi);
  double pi = acos(-1);
  for (int i = 0; i < nf; ++i) {
    if (i == 0) nj[i] = CELL(s, 0, MCPM_CF_N);
    else if (i == s->N1) nj[i] = CELL(s, s->N1 - 1, MCPM_CF_N);
    else nj[i] = (CELL(s, i, MCPM_CF_N) + CELL(s, i - 1, MCPM_CF_N)) / 2.0;
  }
  for (int i = 0; i < nf; ++i) a[i] = (2.0 + pow(s->dy * g->bst, 2.0));
  for (int i = 0; i < nf - 1; ++i) { b[i] = -1.0; c[i] = -1.0; }
  for (int i = 0; i < nf; ++i) rhs[i] = nj[i] * pow(s->dy, 2.0);
  double bb = 3.0 * g->eqdist, aa = 0.0 * g->eqdist, cc = 0.0, dd = pi;
  for (int i = 0; i < 50; ++i) { rr[i] = (bb - aa) / 2.0 * xi[i] + (aa + bb) / 2.0; dr[i] = wi[i] * (bb - aa) / 2.0; }
  for (int i = 0; i < 50; ++i) { ph[i] = (dd - cc) / 2.0 * xi[i] + (cc + dd) / 2.0; dph[i] = wi[i] * (dd - cc) / 2.0; }
  double V_lw = 0.0, V_uw = 0.0, n = 0.0;
  for (int fc = 0; fc < nf; fc = fc + nf - 1) {
    for (int i = 0; i < 50; ++i) {
      double radial_part = exp(-g->bst * rr[i]) / (2.0) * rr[i] * dr[i];
      for (int ii = 0; ii < 50; ++ii) {
        double y = fc * s->dy + rr[i] * cos(ph[ii]);
        int num = (int)floor(y / s->dy);
        n = n_lookup(s, num);
        if (fc == 0) V_lw += radial_part * n * sin(ph[ii]) * dph[ii];
        if (fc == nf - 1) V_uw += radial_part * n * sin(ph[ii]) * dph[ii];
      }
    }
  }
  c[0] = 0.0; a[0] = 1.0; rhs[0] = V_lw;
  a[nf - 1] = 1.0; rhs[nf - 1] = V_uw; b[nf - 2] = 0.0;
  thomas(a, b, c, x, rhs, nf);
  double dummy = 1.0 - (g->sigma * g->bst + 1.0) * exp(-g->bst * g->sigma);
  dummy = dummy / g->bst / g->bst;
  for (int i = 0; i < nf; ++i) x[i] = x[i] - nj[i] * dummy;
  free(a); free(b); free(c); free(nj); free(rhs);
}

/* long-range dispatch of velocity_update, src/Main_Functions.cpp:1618-1663,
   for the 1-D paths: F2 per cell from the face potential, U2 += F2 dt. */
/* velocity_update's density-expansion force, src/Main_Functions.cpp:1632-1653:
   the gradient sum dn2 of the kernel smoothing scaled by
   4 pi (sigma 2^(1/6))^3 phi / m 2, subtracted (times dt) from U2 except in
   cell 0 and in cell N[1]-1 (the linear cell index against N[1]-1, as the
   reference writes it).  F2 records the kick, -dummyF. */
static void density_expansion(orc_state* s, double* U2) {
  const mcpm_config* g = &s->cfg;
  const double pi = acos(-1);
  for (int num = 0; num < s->C; ++num) {
    double dummyF = CELL(s, num, MCPM_CF_DN2);
    dummyF = dummyF * 4.0 * pi * pow(g->sigma * pow(2.0, 1.0 / 6.0), 3.0) * g->phi / g->m * 2.0;
    CELL(s, num, MCPM_CF_F2) = (num != 0 && num != s->N1 - 1) ? -dummyF : 0.0;
  }
  for (int64_t id = 0; id < s->N; ++id) {
    int num = s->index[id];
    if (num != 0 && num != s->N1 - 1) U2[id] = U2[id] - (-CELL(s, num, MCPM_CF_F2)) * g->dt;
  }
}

void orc_long_range(orc_state* s, double* U2) {
  const mcpm_config* g = &s->cfg;
  if (g->long_range == MCPM_LR_DENSITY_EXPANSION) { density_expansion(s, U2); return; }
  if (g->long_range != MCPM_LR_DIRECT && g->long_range != MCPM_LR_SCREENED_POISSON) return;
  int nf = s->N1 + 1;
  double* V = (double*)malloc(sizeof(double) * nf);
  double coef;
  if (g->long_range == MCPM_LR_DIRECT) { orc_vlasov_face_potential(s, V); coef = g->phi; }
  else { orc_poisson_faces(s, V); coef = g->ast; }
  for (int num = 0; num < s->N1; ++num) {
    int fc = num + 1;
    double F2 = -(V[fc] - V[fc - 1]) / s->dy;
    F2 = F2 / g->m * coef;
    for (int j = 0; j < s->N0; ++j) CELL(s, num * s->N0 + j, MCPM_CF_F2) = F2;
  }
  for (int64_t id = 0; id < s->N; ++id) {
    int num = s->index[id];
    U2[id] = U2[id] + CELL(s, num, MCPM_CF_F2) * g->dt;
  }
  free(V);
}


/* ---------------------------------------------------- 2-D long range -- */
/* shape-function derivatives of the bilinear element, src/FEM.cpp:22-49 */
static double dNxi(int i, double xi, double eta) {
  (void)xi;
  if (i == 0) return eta - 1.0;
  if (i == 1) return 1.0 - eta;
  if (i == 2) return -eta;
  return eta;
}
static double dNeta(int i, double xi, double eta) {
  (void)eta;
  if (i == 0) return xi - 1.0;
  if (i == 1) return -xi;
  if (i == 2) return -xi + 1;
  return xi;
}

/* r, phi, theta quadrature of the 2-D routines: GL(npts) on [a, b] x
   [0, 2 pi] x [0, pi] (src/FEM.cpp:352-371, :657-671) */
typedef struct {
  int n;
  double rr[100], dr[100], ph[100], dph[100], th[100], dth[100];
  double cph[100], sph[100], sth[100];
} sph_quad;
static void sph_quad_make(sph_quad* q, int npts, double a, double b) {
  double xi[100], wi[100];
  double pi = acos(-1.0);
  orc_gl_table(npts, xi, wi);
  q->n = npts;
  double cc = 0.0, dd = 2 * pi, ee = 0.0, ff = pi;
  for (int i = 0; i < npts; ++i) {
    q->rr[i] = (b - a) / 2.0 * xi[i] + (a + b) / 2.0; q->dr[i] = wi[i] * (b - a) / 2.0;
    q->ph[i] = (dd - cc) / 2.0 * xi[i] + (cc + dd) / 2.0; q->dph[i] = wi[i] * (dd - cc) / 2.0;
    q->th[i] = (ff - ee) / 2.0 * xi[i] + (ff + ee) / 2.0; q->dth[i] = wi[i] * (ff - ee) / 2.0;
  }
  for (int i = 0; i < npts; ++i) { q->cph[i] = cos(q->ph[i]); q->sph[i] = sin(q->ph[i]); q->sth[i] = sin(q->th[i]); }
}
/* vlasov_taking_the_integral_2D (src/FEM.cpp:158-202, kind 1) and
   Compute_SP_using_Green_Function (:203-247, kind 3): the potential at
   (xx, yy) from the cell densities, points outside the box taking the
   density of the nearest edge cell. */
static double sphere_integral(const orc_state* s, const sph_quad* q, int kind, double xx, double yy) {
  const mcpm_config* g = &s->cfg;
  double pi = acos(-1);
  double V = 0.0;
  for (int i = 0; i < q->n; ++i) {
    double radial_part = kind == 1 ? pow(g->sigma / q->rr[i], 6.0) * q->rr[i] * q->rr[i] * q->dr[i]
                                   : exp(-g->bst * q->rr[i]) / (4.0 * pi) * q->rr[i] * q->dr[i];
    for (int ii = 0; ii < q->n; ++ii) {
      for (int iii = 0; iii < q->n; ++iii) {
        double x = xx + q->rr[i] * q->cph[ii] * q->sth[iii];
        double y = yy + q->rr[i] * q->sph[ii] * q->sth[iii];
        int j = (int)floor(x / s->dx);
        int k = (int)floor(y / s->dy);
        if (j < 0) j = 0; else if (j > s->N0 - 1) j = s->N0 - 1;
        if (k < 0) k = 0; else if (k > s->N1 - 1) k = s->N1 - 1;
        double n = CELL(s, k * s->N0 + j, MCPM_CF_N);
        V += radial_part * n * q->dph[ii] * q->sth[iii] * q->dth[iii];
      }
    }
  }
  return V;
}
/* the cell and corner through which the node loops of src/FEM.cpp:511-545,
   :675-700 reach node (i, j) */
static void node_cell(const orc_state* s, int i, int j, int* num, int* k) {
  int ii = i, jj = j;
  *k = 0;
  if (i == s->N0) { ii = i - 1; jj = j; *k = 1; }
  if (j == s->N1) { ii = i; jj = j - 1; *k = 2; }
  if (i == s->N0 && j == s->N1) { ii = i - 1; jj = j - 1; *k = 3; }
  *num = jj * s->N0 + ii;
}

/* compute_Vlasov_2D node potentials, src/FEM.cpp:613-701: GL(100)^3 over
   r in [sigma, 3 sigma] at every node */
void orc_vlasov2d_nodes(orc_state* s, double* V) {
  sph_quad q;
  sph_quad_make(&q, 100, 1.0 * s->cfg.sigma, 3.0 * s->cfg.sigma);
  for (int j = 0; j < s->N1 + 1; ++j)
    for (int i = 0; i < s->N0 + 1; ++i) {
      int num, k;
      node_cell(s, i, j, &num, &k);
      cell_geo cg = geometry(s, num);
      V[j * (s->N0 + 1) + i] = sphere_integral(s, &q, 1, cg.xn[k], cg.yn[k]);
    }
}

/* dense LU with partial pivoting: the solve that stands in for PARDISO
   (src/solver_pardiso.cpp:33-158, MKL, not available) */
static void dense_lu_solve(double* A, double* r, int n, double* x) {
  for (int k = 0; k < n; ++k) {
    int piv = k;
    for (int i = k + 1; i < n; ++i)
      if (fabs(A[(size_t)i * n + k]) > fabs(A[(size_t)piv * n + k])) piv = i;
    if (piv != k) {
      for (int j = 0; j < n; ++j) { double t = A[(size_t)k * n + j]; A[(size_t)k * n + j] = A[(size_t)piv * n + j]; A[(size_t)piv * n + j] = t; }
      double t = r[k]; r[k] = r[piv]; r[piv] = t;
    }
    for (int i = k + 1; i < n; ++i) {
      double f = A[(size_t)i * n + k] / A[(size_t)k * n + k];
      if (f == 0.0) continue;
      for (int j = k; j < n; ++j) A[(size_t)i * n + j] -= f * A[(size_t)k * n + j];
      r[i] -= f * r[k];
    }
  }
  for (int i = n - 1; i >= 0; --i) {
    double sm = r[i];
    for (int j = i + 1; j < n; ++j) sm -= A[(size_t)i * n + j] * x[j];
    x[i] = sm / A[(size_t)i * n + i];
  }
}

/* compute_SP_2D node potentials, src/FEM.cpp:249-610: bilinear FEM of
   -lap V + bst^2 V = n_n with the Green's-function values on the walls
   (GL(50)^3 over r in [0, 3 sigma]), minus the analytic near-field part.
   Dense; for small grids only. */
void orc_sp2d_nodes(orc_state* s, double* x) {
  const mcpm_config* g = &s->cfg;
  const int N0 = s->N0, N1 = s->N1, nn = (N0 + 1) * (N1 + 1), nc = s->C;
  static const double dudv[4][4] = {{2.0 / 3.0, -1.0 / 6.0, -1.0 / 6.0, -1.0 / 3.0},
                                    {-1.0 / 6.0, 2.0 / 3.0, -1.0 / 3.0, -1.0 / 6.0},
                                    {-1.0 / 6.0, -1.0 / 3.0, 2.0 / 3.0, -1.0 / 6.0},
                                    {-1.0 / 3.0, -1.0 / 6.0, -1.0 / 6.0, 2.0 / 3.0}};
  static const double uv[4][4] = {{1.0 / 9.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 36.0},
                                  {1.0 / 18.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 18.0},
                                  {1.0 / 18.0, 1.0 / 36.0, 1.0 / 9.0, 1.0 / 18.0},
                                  {1.0 / 36.0, 1.0 / 18.0, 1.0 / 18.0, 1.0 / 9.0}};
  double* A = (double*)calloc((size_t)nn * nn, sizeof(double));
  double* b = (double*)calloc(nn, sizeof(double));
  double lambda2 = pow(g->bst, 2.0);
  for (int i = 0; i < nn; ++i) x[i] = 0.0;
  for (int num = 0; num < nc; ++num) {
    int id[4];
    double v[4];
    node_ids(s, num, id);
    double vol = cell_volume(s, num);
    for (int i = 0; i < 4; ++i) {
      v[i] = 0.0;
      for (int j = 0; j < 4; ++j) v[i] += NN(num, j) * uv[i][j];
    }
    for (int i = 0; i < 4; ++i) {
      for (int j = 0; j < 4; ++j) {
        A[(size_t)id[i] * nn + id[j]] += dudv[i][j];
        A[(size_t)id[i] * nn + id[j]] += lambda2 * uv[i][j] * vol;
      }
      b[id[i]] += v[i] * vol;
    }
  }
  sph_quad q;
  sph_quad_make(&q, 50, 0.0, 3.0 * g->sigma);
  /* Dirichlet rows: lower, upper, left, right wall (:396-455) */
  const int walls[4][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}};
  for (int w = 0; w < 4; ++w) {
    int cnt = w < 2 ? N0 : N1;
    for (int jj = 0; jj < cnt; ++jj) {
      int num = w == 0 ? jj : (w == 1 ? (N1 - 1) * N0 + jj : (w == 2 ? jj * N0 : jj * N0 + N0 - 1));
      int id[4];
      node_ids(s, num, id);
      cell_geo cg = geometry(s, num);
      for (int t = 0; t < 2; ++t) {
        int k = walls[w][t], i = id[k];
        for (int j = 0; j < nn; ++j) A[(size_t)i * nn + j] = 0.0;
        A[(size_t)i * nn + i] = 1.0;
        b[i] = sphere_integral(s, &q, 3, cg.xn[k], cg.yn[k]);
      }
    }
  }
  dense_lu_solve(A, b, nn, x);
  double dummy = 1.0 - (g->sigma * g->bst + 1.0) * exp(-g->bst * g->sigma);
  dummy = dummy / g->bst / g->bst;
  double dummy2 = (-1.0 / 6.0 * pow(g->bst, 3) * pow(g->sigma, 3) - 1.0 / 2.0 * pow(g->bst, 2) * pow(g->sigma, 2) -
                   g->bst * g->sigma + exp(g->bst * g->sigma) - 1) *
                  exp(-g->bst * g->sigma) / pow(g->bst, 4);
  dummy2 = dummy2 / pow(s->dx, 2);
  for (int j = 0; j < N1 + 1; ++j) {
    for (int i = 0; i < N0 + 1; ++i) {
      int id = j * (N0 + 1) + i, ii = i, jj = j, k = 0;
      int ipm[4] = {0, -1, 0, 0}, jpm[4] = {0, 0, 0, -1}, kpm[4] = {1, 0, 2, 0};
      if (i == N0) { ii = i - 1; jj = j; k = 1; kpm[0] = k; }
      if (j == N1) { ii = i; jj = j - 1; k = 2; kpm[2] = k; }
      if (i == N0 && j == N1) { ii = i - 1; jj = j - 1; k = 3; kpm[0] = k; kpm[2] = k; }
      if (i == 0) { ipm[1] = 0; jpm[1] = 0; kpm[1] = 0; }
      if (j == 0) { ipm[3] = 0; jpm[3] = 0; kpm[3] = 0; }
      int num = jj * N0 + ii;
      double d2 = NN(num, k) * dummy;
      double d3 = -4.0 * NN(num, k) * dummy2;
      for (int ll = 0; ll < 4; ++ll) {
        num = (jj + jpm[ll]) * N0 + ii + ipm[ll];
        d3 += NN(num, kpm[ll]) * dummy2;
      }
      x[id] += -(d2 + d3);
    }
  }
  free(A); free(b);
}

/* the kick of compute_Vlasov_2D / compute_SP_2D (src/FEM.cpp:567-578,
   :703-714): bilinear gradient of the node potential at the particle */
static void kick_2d(orc_state* s, const double* V, double coef, const double* x1, const double* x2,
                    double* U1, double* U2) {
  const mcpm_config* g = &s->cfg;
  for (int64_t i = 0; i < s->N; ++i) {
    int num = s->index[i], id[4];
    cell_geo cg = geometry(s, num);
    node_ids(s, num, id);
    double xi = (x1[i] - cg.xn[0]) / cg.dxc;
    double eta = (x2[i] - cg.yn[0]) / cg.dyc;
    double F1 = 0.0, F2 = 0.0;
    for (int j = 0; j < 4; ++j) {
      F1 += dNxi(j, xi, eta) * V[id[j]];
      F2 += dNeta(j, xi, eta) * V[id[j]];
    }
    F1 = F1 / g->m * coef / cg.dxc; F2 = F2 / g->m * coef / cg.dyc;
    U1[i] = U1[i] - F1 * g->dt;
    U2[i] = U2[i] - F2 * g->dt;
  }
}

/* long-range dispatch for 2-D boxes: compute_Vlasov_2D (long_range 1) or
   compute_SP_2D (long_range 3), src/Main_Functions.cpp:1618-1663.  The
   reference reaches them for its 2-D injection problem; here any 2-D box. */
void orc_long_range_2d(orc_state* s, const double* x1, const double* x2, double* U1, double* U2, double* V) {
  const mcpm_config* g = &s->cfg;
  if (g->long_range != MCPM_LR_DIRECT && g->long_range != MCPM_LR_SCREENED_POISSON) return;
  int nn = (s->N0 + 1) * (s->N1 + 1);
  double* W = V ? V : (double*)malloc(sizeof(double) * nn);
  if (g->long_range == MCPM_LR_DIRECT) orc_vlasov2d_nodes(s, W);
  else orc_sp2d_nodes(s, W);
  kick_2d(s, W, g->long_range == MCPM_LR_DIRECT ? g->phi : g->ast, x1, x2, U1, U2);
  if (!V) free(W);
}

/* ------------------------------------------------- DFP_extra_streaming -- */
/* src/Fokker_Planck.cpp:904-946, including its use of U_space[1] in the x1
   heat-flux term (:936). */
void orc_dfp_extra_streaming(orc_state* s, const double* U1, const double* U2,
                             const double* U3, double* x1, double* x2) {
  const mcpm_config* g = &s->cfg;
  double dummy = (g->model == MCPM_MODEL_FP_DENSE) ? 1.0 : 0.0;
  double dt = g->dt;
  for (int64_t ii = 0; ii < s->N; ++ii) {
    int num = s->index[ii];
    const double* Us = &CELL(s, num, MCPM_CF_U_SPACE);
    const double* al = &CELL(s, num, MCPM_CF_ALPHA);
    const double* be = &CELL(s, num, MCPM_CF_BETA);
    const double* M3 = &CELL(s, num, MCPM_CF_M3);
    const double* ph = &CELL(s, num, MCPM_CF_PHI);
    double gst = CELL(s, num, MCPM_CF_GAMMA_ST), T = CELL(s, num, MCPM_CF_T);
    double energy = (U1[ii] - Us[0]) * (U1[ii] - Us[0]) + (U2[ii] - Us[1]) * (U2[ii] - Us[1]) +
                    (U3[ii] - Us[2]) * (U3[ii] - Us[2]);
    if (g->direction[0] == 1) {
      x1[ii] = x1[ii] + dummy * dt * ((U1[ii] - Us[0]) * al[0] + (U2[ii] - Us[1]) * al[1] + (U3[ii] - Us[2]) * al[2] +
                                      be[0] * (energy - 3.0 * g->kb * T / g->m)) +
               dummy * gst * ((U1[ii] - Us[1]) * energy - M3[0] - M3[3] - M3[5]) * dt;
      x1[ii] = x1[ii] - dummy * dt * ph[0];
    }
    if (g->direction[1] == 1) {
      x2[ii] = x2[ii] + dummy * dt * ((U1[ii] - Us[0]) * al[3] + (U2[ii] - Us[1]) * al[4] + (U3[ii] - Us[2]) * al[5] +
                                      be[1] * (energy - 3.0 * g->kb * T / g->m)) +
               dummy * gst * ((U2[ii] - Us[1]) * energy - M3[1] - M3[6] - M3[8]) * dt;
      x2[ii] = x2[ii] - dummy * dt * ph[1];
    }
  }
}

/* ----------------------------------------------------- free flight, BCs -- */
/* Position_FP_ideal_gas, src/Fokker_Planck.cpp:948-969 */
void orc_stream(orc_state* s, double* x1, double* x2, const double* U1,
                const double* U2, const double* U3) {
  (void)U3;
  if (s->cfg.direction[0] == 1)
    for (int64_t i = 0; i < s->N; ++i) x1[i] = x1[i] + s->cfg.dt * U1[i];
  if (s->cfg.direction[1] == 1)
    for (int64_t i = 0; i < s->N; ++i) x2[i] = x2[i] + s->cfg.dt * U2[i];
}

/* store_old_positions, src/Main_Functions.cpp:5736-5760 */
void orc_store_old_positions(orc_state* s, const double* x1, const double* x2,
                             double* x1_old, double* x2_old) {
  if (s->cfg.direction[0] == 1) memcpy(x1_old, x1, sizeof(double) * (size_t)s->N);
  if (s->cfg.direction[1] == 1) memcpy(x2_old, x2, sizeof(double) * (size_t)s->N);
}

/* BC_specular_reflection, src/Main_Functions.cpp:6399-6525 (the wall
   momentum tally gas.M is a diagnostic and is not kept) */
static void bc_specular(orc_state* s, double* x1, double* x2, double* U1, double* U2) {
  const mcpm_config* g = &s->cfg;
  double Tol1 = 1e-16, Tol2 = -1e-16;
  for (int64_t i = 0; i < s->N; ++i) {
    int done = 0, it = 0;
    while (done == 0) {
      if (g->direction[0] == 1) {
        if (x1[i] - g->length[0] > Tol2) { U1[i] = -U1[i]; x1[i] = x1[i] - 2.0 * fabs(x1[i] - g->length[0]); }
        else if (x1[i] < Tol1) { U1[i] = -U1[i]; x1[i] = x1[i] + 2.0 * fabs(x1[i]); }
      }
      if (g->direction[1] == 1) {
        if (x2[i] - g->length[1] > Tol2) { U2[i] = -U2[i]; x2[i] = x2[i] - 2.0 * fabs(x2[i] - g->length[1]); }
        else if (x2[i] < Tol1) { U2[i] = -U2[i]; x2[i] = x2[i] + 2.0 * fabs(x2[i]); }
      }
      done = 1;
      if (g->direction[0] == 1 && (x1[i] - g->length[0] > 0.0 || x1[i] < 0.0)) done = 0;
      if (g->direction[1] == 1 && (x2[i] - g->length[1] > 0.0 || x2[i] < 0.0)) done = 0;
      if (++it > 64) { s->status |= MCPM_ERR_BC_LOOP; break; }
    }
  }
}

/* periodic wrap in the active directions */
static void bc_periodic(orc_state* s, double* x1, double* x2) {
  const mcpm_config* g = &s->cfg;
  for (int64_t i = 0; i < s->N; ++i) {
    if (g->direction[0] == 1) x1[i] = x1[i] - g->length[0] * floor(x1[i] / g->length[0]);
    if (g->direction[1] == 1) x2[i] = x2[i] - g->length[1] * floor(x2[i] / g->length[1]);
  }
}

/* intersect_3D_x / intersect_3D_y, src/Main_Functions.cpp:2757-2806, with
   z_new == z_old (no streaming in z) */
static void intersect_x(double x, double* y, double xo, double yo, double xn, double yn) {
  double n0 = xn - xo, n1 = yn - yo, n2 = 0.0;
  double size = 0.0;
  size += n0 * n0; size += n1 * n1; size += n2 * n2;
  size = sqrt(size);
  n0 = n0 / size; n1 = n1 / size;
  if (fabs(n0) > 1e-16) *y = (n1 / n0) * (x - xo) + yo;
  else *y = yn;
}
static void intersect_y(double* x, double y, double xo, double yo, double xn, double yn) {
  double n0 = xn - xo, n1 = yn - yo, n2 = 0.0;
  double size = 0.0;
  size += n0 * n0; size += n1 * n1; size += n2 * n2;
  size = sqrt(size);
  n0 = n0 / size; n1 = n1 / size;
  if (fabs(n1) > 1e-16) *x = (n0 / n1) * (y - yo) + xo;
  else *x = xn;
}

/* one diffuse re-emission: tangential Maxwellian, normal Rayleigh */
static void wall_draw(const orc_state* s, int64_t i, int call_no, int it, double z[2], double* ray) {
  uint32_t r[4];
  rng(s, (uint32_t)i, (uint32_t)s->step, RNG_STREAM_BC,
         (uint32_t)((call_no << 8) | (it & 0xff)), r);
  *ray = sqrt(-log(u01(r[0])));
  double a = sqrt(-2.0 * log(u01(r[1])));
  z[0] = a * cos(TWO_PI * u01(r[2]));
  z[1] = a * sin(TWO_PI * u01(r[2]));
}

/* BC_thermal_wall_3D, src/Main_Functions.cpp:4917-5250, in 2-D (direction[2]
   = 0): diffuse walls at x = 0 (T_wall_3), x = Len0 (T_wall_4),
   y = sigma (T_wall_1), y = Len1 - sigma (T_wall_2), with re-flight for the
   rest of the step from the wall crossing point. */
/* The reference's diffuse-wall offset epsilon = 1e-15 (:4933) is an absolute
   length meant for SI boxes; where it is below the resolution of the box
   length the offset is 4 ulp(Len) instead (the same rule as the GPU). */
static double wall_eps(double L) { return fmax(1e-15, 4.0 * (nextafter(L, 2.0 * L + 1.0) - L)); }

static void bc_thermal_wall(orc_state* s, int call_no, double* x1, double* x2,
                            double* x1o, double* x2o, double* U1, double* U2, double* U3) {
  const mcpm_config* g = &s->cfg;
  const double ex = wall_eps(g->length[0]), ey = wall_eps(g->length[1]);
  const double L0 = g->length[0], L1 = g->length[1];
  for (int64_t i = 0; i < s->N; ++i) {
    double dt = g->dt;
    int done = 0, it = 0;
    double Ue0 = fabs(x1[i] - x1o[i]) / g->dt;
    double Ue1 = fabs(x2[i] - x2o[i]) / g->dt;
    while (done == 0) {
      double dt_remain = 0.0, xw, yw, tU0, z[2], ray;
      if (it > 20) { s->status |= MCPM_ERR_BC_LOOP; break; }
      if (dt < 1e-15) {
        if (x1[i] < ex) x1[i] = ex;
        else if (x1[i] > L0 - ex) x1[i] = L0 - ex;
        if (x2[i] < ey) x2[i] = ey;
        else if (x2[i] > L1 - ey) x2[i] = L1 - ey;
      }
      /* a particle exactly on an x wall counts as having reached it (the
         reference's > / < leave x == Len neither inside nor outside) */
      if (x1[i] - L0 >= 0.0) { /* right wall */
        xw = L0 - ex;
        if (fabs(x1o[i] - x1[i]) > 1e-15) intersect_x(xw, &yw, x1o[i], x2o[i], x1[i], x2[i]);
        else yw = 0.5 * (x2o[i] + x2[i]);
        tU0 = (fabs(dt - g->dt) < 1e-15) ? Ue0 : U1[i];
        wall_draw(s, i, call_no, it, z, &ray);
        U1[i] = -sqrt(2.0 * g->kb * g->T_wall[3] / (g->m)) * ray;
        U2[i] = sqrt(g->kb * g->T_wall[3] / (g->m)) * z[0] + (1.0 * g->U_wall[3]);
        U3[i] = sqrt(g->kb * g->T_wall[3] / (g->m)) * z[1];
        if (dt > 1e-15) {
          dt_remain = fabs((x1[i] - xw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          x1[i] = xw + dt_remain * U1[i];
          x2[i] = yw + dt_remain * U2[i];
          dt = dt - dt_remain;
          x1o[i] = xw; x2o[i] = yw;
        } else x1[i] = xw;
      } else if (x1[i] <= 0.0) { /* left wall */
        xw = ex;
        if (fabs(x1o[i] - x1[i]) > 1e-15) intersect_x(xw, &yw, x1o[i], x2o[i], x1[i], x2[i]);
        else yw = 0.5 * (x2o[i] + x2[i]);
        tU0 = (fabs(dt - g->dt) < 1e-15) ? Ue0 : U1[i];
        wall_draw(s, i, call_no, it, z, &ray);
        U1[i] = sqrt(2.0 * g->kb * g->T_wall[2] / (g->m)) * ray;
        U2[i] = sqrt(g->kb * g->T_wall[2] / g->m) * z[0] + (1.0 * g->U_wall[2]);
        U3[i] = sqrt(g->kb * g->T_wall[2] / g->m) * z[1];
        if (dt > 1e-15) {
          dt_remain = fabs((x1[i] - xw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          x1[i] = xw + dt_remain * U1[i];
          x2[i] = yw + dt_remain * U2[i];
          dt = dt - dt_remain;
          x1o[i] = xw; x2o[i] = yw;
        } else x1[i] = xw;
      } else if (x2[i] > L1 - g->sigma - ey) { /* upper wall */
        yw = L1 - g->sigma - ey;
        intersect_y(&xw, yw, x1o[i], x2o[i], x1[i], x2[i]);
        tU0 = (fabs(dt - g->dt) < 1e-15) ? Ue1 : U2[i];
        wall_draw(s, i, call_no, it, z, &ray);
        U1[i] = sqrt(g->kb * g->T_wall[1] / (g->m)) * z[0] + (1.0 * g->U_wall[1]);
        U2[i] = -sqrt(2.0 * g->kb * g->T_wall[1] / (g->m)) * ray;
        U3[i] = sqrt(g->kb * g->T_wall[1] / (g->m)) * z[1];
        if (dt > 1e-15) {
          dt_remain = fabs((x2[i] - yw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          x1[i] = xw + dt_remain * U1[i];
          x2[i] = yw + dt_remain * U2[i];
          dt = dt - dt_remain;
          x1o[i] = xw; x2o[i] = yw;
        } else x2[i] = yw;
      } else if (x2[i] < g->sigma + ey) { /* lower wall */
        yw = g->sigma + ey;
        intersect_y(&xw, yw, x1o[i], x2o[i], x1[i], x2[i]);
        tU0 = (fabs(dt - g->dt) < 1e-15) ? Ue1 : U2[i];
        wall_draw(s, i, call_no, it, z, &ray);
        U1[i] = sqrt(g->kb * g->T_wall[0] / (g->m)) * z[0] + (1.0 * g->U_wall[0]);
        U2[i] = sqrt(2.0 * g->kb * g->T_wall[0] / (g->m)) * ray;
        U3[i] = sqrt(g->kb * g->T_wall[0] / g->m) * z[1];
        if (dt > 1e-15) {
          dt_remain = fabs((x2[i] - yw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          x1[i] = xw + dt_remain * U1[i];
          x2[i] = yw + dt_remain * U2[i];
          dt = dt - dt_remain;
          x1o[i] = xw; x2o[i] = yw;
        } else x2[i] = yw;
      }
      if (x1[i] - L0 < 0.0 && x1[i] > 0.0 && x2[i] - L1 < 0.0 && x2[i] > 0.0) done = 1;
      it++;
    }
  }
}

/* BC_wall, src/Main_Functions.cpp:4816-4914: diffuse lower wall at y = 0
   (T_wall_1), specular upper wall, 1-D in y. */
static void bc_wall(orc_state* s, int call_no, double* x2, double* x2o,
                    double* U1, double* U2, double* U3) {
  const mcpm_config* g = &s->cfg;
  const double eps = wall_eps(g->length[1]);
  const double L1 = g->length[1];
  for (int64_t i = 0; i < s->N; ++i) {
    double dt = g->dt;
    int done = 0, it = 0;
    double Ue1 = fabs(x2[i] - x2o[i]) / g->dt;
    while (done == 0) {
      double dt_remain = 0.0, tU0, z[2], ray;
      if (it > 20) { s->status |= MCPM_ERR_BC_LOOP; break; }
      if (dt < 1e-15) {
        if (x2[i] < eps) x2[i] = eps;
        else if (x2[i] > L1 - eps) x2[i] = L1 - eps;
      } else if (x2[i] >= L1) { /* >= / <=: see bc_thermal_wall */
        U2[i] = -U2[i];
        x2[i] = x2[i] - 2.0 * fabs(x2[i] - L1);
      } else if (x2[i] <= 0.0) {
        double yw = eps;
        tU0 = (fabs(dt - g->dt) < 1e-15) ? Ue1 : U2[i];
        wall_draw(s, i, call_no, it, z, &ray);
        U1[i] = sqrt(g->kb * g->T_wall[0] / (g->m)) * z[0] + (1.0 * g->U_wall[0]);
        U2[i] = sqrt(2.0 * g->kb * g->T_wall[0] / (g->m)) * ray;
        U3[i] = sqrt(g->kb * g->T_wall[0] / g->m) * z[1];
        if (dt > 1e-15) {
          dt_remain = fabs((x2[i] - yw) / tU0);
          dt_remain = dt < dt_remain ? dt : dt_remain;
          x2[i] = yw + dt_remain * U2[i];
          dt = dt - dt_remain;
          x2o[i] = yw;
        } else x2[i] = yw;
      }
      if (x2[i] - L1 < 0.0 && x2[i] > 0.0) done = 1;
      it++;
    }
  }
}

/* apply_BC, src/Main_Functions.cpp:1451-1492 */
void orc_apply_bc(orc_state* s, int call_no, double* x1, double* x2,
                  double* x1_old, double* x2_old, double* U1, double* U2, double* U3) {
  switch (s->cfg.problem) {
    case MCPM_PROBLEM_CLOSED_BOX: bc_specular(s, x1, x2, U1, U2); break;
    case MCPM_PROBLEM_COUETTE: bc_thermal_wall(s, call_no, x1, x2, x1_old, x2_old, U1, U2, U3); break;
    case MCPM_PROBLEM_WALL: bc_wall(s, call_no, x2, x2_old, U1, U2, U3); break;
    case MCPM_PROBLEM_PERIODIC: bc_periodic(s, x1, x2); break;
    default: break;
  }
}

/* --------------------------------------------------------------- step -- */
/* one iteration of src/main.cpp:389-669 for the in-scope models */
void orc_step(orc_state* s, double* x1, double* x2, double* x1_old,
              double* x2_old, double* U1, double* U2, double* U3, int32_t* index) {
  int m = s->cfg.model;
  int64_t N = s->N;
  orc_cell_update(s, x1, x2, U1, U2, U3, index);
  /* FP_linear draws as well: the reference's loop leaves its noise arrays
     unfilled for that model (src/main.cpp:442) */
  if (m == MCPM_MODEL_FP_DENSE || m == MCPM_MODEL_FP_IDEAL_GAS || m == MCPM_MODEL_FP_LINEAR) {
    orc_random_generator(s, s->xi, s->xi + N, s->xi + 2 * N);
    orc_velocity_fp(s, U1, U2, U3, s->xi, s->xi + N, s->xi + 2 * N);
  } else if (m == MCPM_MODEL_ESMC) {
    orc_esmc(s, x1, x2, U1, U2, U3);
  } else if (m == MCPM_MODEL_DSMC_VHS) {
    orc_dsmc_vhs(s, U1, U2, U3);
  }
  if (s->cfg.direction[0] == 1 && s->cfg.long_range != MCPM_LR_DENSITY_EXPANSION)
    orc_long_range_2d(s, x1, x2, U1, U2, NULL);
  else orc_long_range(s, U2);
  if (m == MCPM_MODEL_FP_DENSE) orc_dfp_extra_streaming(s, U1, U2, U3, x1, x2);
  orc_apply_bc(s, 0, x1, x2, x1_old, x2_old, U1, U2, U3);
  orc_store_old_positions(s, x1, x2, x1_old, x2_old);
  orc_stream(s, x1, x2, U1, U2, U3);
  orc_apply_bc(s, 1, x1, x2, x1_old, x2_old, U1, U2, U3);
  orc_apply_bc(s, 2, x1, x2, x1_old, x2_old, U1, U2, U3);
  s->step++;
}

/* take the per-cell particle order from the caller (e.g. the GPU's slot
   layout) instead of ascending particle ids; counts must match the binning */
void orc_set_layout(orc_state* s, const int32_t* off, const int32_t* list) {
  for (int c = 0; c <= s->C; ++c) s->off[c] = off[c];
  for (int c = 0; c < s->C; ++c) s->cnt[c] = off[c + 1] - off[c];
  for (int64_t i = 0; i < s->N; ++i) s->list[i] = list[i];
}

/* ------------------------------------------------ interface problems -- */
/* thermostat, src/Main_Functions.cpp:1674-1869: the live branch (problem
   inverted, :1745-1855).  Cells num < N[1] whose centre (make_cells:
   0.5 (dim[2] + dim[3]), src/myIO.cpp:1467) lies below thermc are rescaled
   to Tc, above Len[1] - thermh to Th, for T > 0, over the cell's list. */
void orc_thermostat(orc_state* s, double* U1, double* U2, double* U3,
                    double Tc, double Th, double thermc, double thermh) {
  int ncell = s->N1 < s->C ? s->N1 : s->C;
  for (int num = 0; num < ncell; ++num) {
    int k = num / s->N0;
    double d2 = (double)(k) * s->dy, d3 = (double)(k + 1) * s->dy;
    double yc = 0.5 * (d2 + d3);
    double target;
    if (yc < thermc) target = Tc;
    else if (yc > s->cfg.length[1] - thermh) target = Th;
    else continue;
    double T = CELL(s, num, MCPM_CF_T);
    if (!(T > 0.0)) continue;
    double lamb = sqrt(target / T);
    double us0 = CELL(s, num, MCPM_CF_U_SPACE + 0), us1 = CELL(s, num, MCPM_CF_U_SPACE + 1),
           us2 = CELL(s, num, MCPM_CF_U_SPACE + 2);
    for (int id = 0; id < s->cnt[num]; ++id) {
      int i = s->list[s->off[num] + id];
      U1[i] = lamb * (U1[i] - us0) + us0;
      U2[i] = lamb * (U2[i] - us1) + us1;
      U3[i] = lamb * (U3[i] - us2) + us2;
    }
  }
}

/* inverted_addremove_particles, src/Main_Functions.cpp:1258-1284: the
   flags, in particle order; deletion draws are Philox keyed by the
   particle id and step (the reference: std::mt19937 from random_device) */
void orc_addremove_flags(orc_state* s, const int32_t* w, const int32_t* cw,
                         int n_ratio, int8_t* flag, int64_t* n_kept,
                         int64_t* n_new) {
  double ratio = 1.0 - 1.0 / (n_ratio * 1.0);
  int64_t kept = s->N, split = 0;
  for (int64_t id = 0; id < s->N; ++id) {
    int num = s->index[id];
    if (w[id] > cw[num]) {
      flag[id] = 1;
      split++;
    } else if (w[id] < cw[num]) {
      uint32_t r[4];
      rng(s, (uint32_t)id, (uint32_t)s->step, RNG_STREAM_ADDREM_DEL, 0, r);
      if (u01(r[0]) < ratio) { flag[id] = -1; kept--; }
      else flag[id] = 2;
    } else {
      flag[id] = 0;
    }
  }
  *n_kept = kept;
  *n_new = (int64_t)(n_ratio - 1) * split;
}

/* the velocity spread of the copies per cell, h = 1.06 sig (numb_rem +
   n_ratio)^(-1/5) (src/Main_Functions.cpp:1285-1346) for the given flags:
   the kept weight and counts, the "mean" of the reference's assigning loop
   (the last kept particle's weighted velocity, :1300-1306) over the kept
   weight, and sig (:1312-1327); 0 in cells without split particles */
void orc_addremove_widths(orc_state* s, const double* U1, const double* U2, const double* U3,
                          const int32_t* w, const int32_t* cw, int n_ratio, const int8_t* flag,
                          double* h) {
  int C = s->C;
  int64_t N = s->N;
  int* numb_new = (int*)calloc(C, sizeof(int));
  int* numb_rem = (int*)calloc(C, sizeof(int));
  int* weight = (int*)calloc(C, sizeof(int));
  double* Um = (double*)calloc(3 * (size_t)C, sizeof(double));
  double* sig = (double*)calloc(C, sizeof(double));
#define WEFF(id) (flag[id] == 2 ? cw[s->index[id]] : w[id])
  for (int64_t id = 0; id < N; ++id) {
    int num = s->index[id];
    if (flag[id] == -1) continue;
    weight[num] += WEFF(id);
    if (flag[id] == 1) numb_new[num]++;
    else numb_rem[num]++;
  }
  for (int64_t id = 0; id < N; ++id) {
    if (flag[id] == -1) continue;
    int num = s->index[id];
    Um[num] = U1[id] * WEFF(id);
    Um[C + num] = U2[id] * WEFF(id);
    Um[2 * C + num] = U3[id] * WEFF(id);
  }
  for (int num = 0; num < C; ++num) {
    Um[num] = Um[num] / (1.0 * weight[num]);
    Um[C + num] = Um[C + num] / (1.0 * weight[num]);
    Um[2 * C + num] = Um[2 * C + num] / (1.0 * weight[num]);
  }
  for (int64_t id = 0; id < N; ++id) {
    if (flag[id] == -1) continue;
    int num = s->index[id];
    double energy = (U1[id] - Um[num]) * (U1[id] - Um[num])
                  + (U2[id] - Um[C + num]) * (U2[id] - Um[C + num])
                  + (U3[id] - Um[2 * C + num]) * (U3[id] - Um[2 * C + num]);
    sig[num] = sig[num] + energy * WEFF(id);
  }
  for (int num = 0; num < C; ++num) {
    sig[num] = sqrt(sig[num] / (1.0 * weight[num]));
    h[num] = numb_new[num] ? 1.06 * sig[num] * pow(1.0 * (numb_rem[num] + n_ratio), -1.0 / 5.0) : 0.0;
  }
#undef WEFF
  free(numb_new); free(numb_rem); free(weight); free(Um); free(sig);
}

/* the rest of inverted_addremove_particles (:1285-1445): per cell the kept
   weight and counts, the "mean" of the reference's assigning loop (the last
   kept particle's weighted velocity, :1300-1306) over the kept weight, the
   spread sig (:1312-1327), h = 1.06 sig (numb_rem + n_ratio)^(-1/5) and
   n_ratio - 1 copies per split particle with velocities U + h z; the kept
   particles first in id order, then the copies by split particle id (the
   reference: by cell, then by id within the cell), every weight reset to
   its cell's (:1436-1443, the cell of the last binning). */
void orc_addremove_apply(orc_state* s, const double* x1, const double* x2,
                         const double* x1_old, const double* x2_old,
                         const double* U1, const double* U2, const double* U3,
                         const int32_t* w, const int32_t* cw, int n_ratio,
                         const int8_t* flag, double* x1o, double* x2o,
                         double* x1_oldo, double* x2_oldo, double* U1o,
                         double* U2o, double* U3o, int32_t* w_out) {
  int C = s->C;
  int64_t N = s->N, split = 0, deleted = 0;
  for (int64_t id = 0; id < N; ++id) {
    if (flag[id] == 1) split++;
    if (flag[id] == -1) deleted++;
  }
  if (split == 0 && deleted == 0) {
    for (int64_t id = 0; id < N; ++id) w_out[id] = flag[id] == 2 ? cw[s->index[id]] : w[id];
    return;
  }
  double* h = (double*)calloc(C, sizeof(double));
  orc_addremove_widths(s, U1, U2, U3, w, cw, n_ratio, flag, h);
  int64_t j = 0;
  for (int64_t id = 0; id < N; ++id) {
    if (flag[id] == -1) continue;
    x1o[j] = x1[id]; x2o[j] = x2[id]; x1_oldo[j] = x1_old[id]; x2_oldo[j] = x2_old[id];
    U1o[j] = U1[id]; U2o[j] = U2[id]; U3o[j] = U3[id];
    w_out[j] = cw[s->index[id]];
    j++;
  }
  for (int64_t id = 0; id < N; ++id) {
    if (flag[id] != 1) continue;
    int num = s->index[id];
    for (int c = 0; c < n_ratio - 1; ++c) {
      double z[4];
      normals4_s(s, (uint32_t)id, (uint32_t)s->step, RNG_STREAM_ADDREM_NEW, (uint32_t)c, z);
      U1o[j] = U1[id] + h[num] * z[0];
      U2o[j] = U2[id] + h[num] * z[1];
      U3o[j] = U3[id] + h[num] * z[2];
      x1o[j] = x1[id]; x2o[j] = x2[id]; x1_oldo[j] = x1_old[id]; x2_oldo[j] = x2_old[id];
      w_out[j] = cw[num];
      j++;
    }
  }
  free(h);
}

/* measure_pressure, src/Main_Functions.cpp:13-34: every particle whose
   cell row changed over the step adds Fn m |U2| to p_m of each row index it
   crossed (p_m accumulates, C values) */
void orc_measure_pressure(orc_state* s, const double* U2, const double* x2,
                          const double* x2_old, double* p_m) {
  for (int64_t i = 0; i < s->N; ++i) {
    int numO = (int)floor(x2_old[i] / s->dy);
    int numN = (int)floor(x2[i] / s->dy);
    int num1, num2;
    if (numN > numO) { num1 = numO; num2 = numN; }
    else if (numN < numO) { num1 = numN; num2 = numO; }
    else { num1 = -1; num2 = -1; }
    for (int num = num1; num < num2; num++) p_m[num] += s->cfg.Fn * s->cfg.m * fabs(U2[i]);
  }
}
