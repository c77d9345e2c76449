// reference_surface.cpp -- the reference's own routine signatures for the
// particle loop of src/main.cpp:418-514, over the session C-ABI, so that the
// reference's main loop links against the GPU step unchanged.
//
// The routines take the reference's struct pointers (GAS, BOX, CELLS,
// src/cpp_headers.h:145-347) and address the fields they use by the offsets
// measured from the reference's header (ref_layout.h, written by
// make_layout.py), so this file needs no copy of those structs.  One device
// session follows the reference's arrays:
//   cell_update          uploads the caller's particles (the host arrays
//                        are the state at the start of a step), bins them,
//                        and writes back index[], every CELLS field the
//                        step computes and the per-cell particle lists
//                        (indices_inside, freed and re-allocated as the
//                        reference does, ascending ids);
//   random_generator     draws on the device (the draws stay there);
//   velocity_update      collisions / FP update + long-range kick, then the
//                        velocities back (and F2, omega_max per cell);
//   DFP_extra_streaming, apply_BC, store_old_positions, stream_particles
//                        on the device, each followed by the arrays it
//                        changes (apply_BC: the old positions too, which
//                        diffuse walls move to the wall crossing);
//   measure_pressure     on the device from the caller's x2_old, the crossings
//                        added to cells[].p_m.
// The reference's routines return nothing and stop the program on errors;
// these print the library's message to stderr and exit(1) likewise.  The
// reference is single-threaded: so is this layer (one session, one thread).
// For speed a caller keeps the particles on the device and calls mcpm_step;
// this layer trades that for running the reference's loop as it stands.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/mcpm.h"
#include "ref_layout.h"

struct GAS;
struct BOX;
struct CELLS;
struct Collision;

namespace {

constexpr size_t off_of(size_t o, size_t) { return o; }
constexpr size_t size_of(size_t, size_t s) { return s; }
#define OFF(name) off_of(MCPM_REF_##name)
#define SZ(name) size_of(MCPM_REF_##name)

static_assert(SZ(GAS_N) == sizeof(long) && SZ(GAS_long_range) == sizeof(int) && SZ(GAS_model) == sizeof(std::string),
              "GAS field sizes");
static_assert(SZ(BOX_N) == 3 * sizeof(int) && SZ(BOX_Len) == 3 * sizeof(double) && SZ(BOX_step) == sizeof(int),
              "BOX field sizes");
static_assert(SZ(CELLS_num_inside) == sizeof(int) && SZ(CELLS_indices_inside) == sizeof(int*) &&
                  SZ(CELLS_U_space) == 3 * sizeof(double) && SZ(CELLS_M3) == 10 * sizeof(double) &&
                  SZ(CELLS_alpha) == 9 * sizeof(double),
              "CELLS field sizes");

template <class V> V& at(const void* base, size_t off) {
  return *reinterpret_cast<V*>(reinterpret_cast<char*>(const_cast<void*>(base)) + off);
}
char* cell_ptr(CELLS* cells, int num) { return reinterpret_cast<char*>(cells) + (size_t)num * MCPM_REF_SIZEOF_CELLS; }

struct Shim {
  mcpm_session* s = nullptr;
  mcpm_config cfg{};
  int64_t N = 0;
  int C = 0;
  bool om_synced = false;
  bool press = false;
  std::vector<double> cells;      // [MCPM_CF_COUNT][C]
  std::vector<int32_t> pid, off;  // layout of the last cell_update
} g;

[[noreturn]] void die(const char* where, int rc) {
  fprintf(stderr, "mcpm: %s failed (%d): %s\n", where, rc, g.s ? mcpm_last_error(g.s) : "no session");
  exit(1);
}
void ck(int rc, const char* where) {
  if (rc) die(where, rc);
}

int model_id(const std::string& m) {
  if (m == "FP_dense") return MCPM_MODEL_FP_DENSE;
  if (m == "FP_ideal_gas") return MCPM_MODEL_FP_IDEAL_GAS;
  if (m == "ESMC") return MCPM_MODEL_ESMC;
  if (m == "FP_linear") return MCPM_MODEL_FP_LINEAR;
  if (m == "DSMC_VHS") return MCPM_MODEL_DSMC_VHS;
  if (m == "none") return MCPM_MODEL_NONE;
  return -1;
}

// the session's configuration from the reference's GAS and BOX
mcpm_config config_of(const GAS* gas, const BOX* box) {
  mcpm_config c;
  std::memset(&c, 0, sizeof c);
  for (int i = 0; i < 3; ++i) {
    c.n_cells[i] = at<int>(box, OFF(BOX_N) + i * sizeof(int));
    c.direction[i] = at<int>(box, OFF(BOX_direction) + i * sizeof(int));
    c.length[i] = at<double>(box, OFF(BOX_Len) + i * sizeof(double));
  }
  c.problem = at<int>(box, OFF(BOX_problem));
  // injection (12) runs between the closed box's specular walls (apply_BC,
  // src/Main_Functions.cpp:1487-1489)
  if (c.problem == 12) c.problem = MCPM_PROBLEM_CLOSED_BOX;
  c.model = model_id(at<std::string>(gas, OFF(GAS_model)));
  const int lr = at<int>(gas, OFF(GAS_long_range));
  c.long_range = (lr >= 1 && lr <= 3) ? lr : MCPM_LR_NONE;  // src/Main_Functions.cpp:1612-1617
  const char* prec = getenv("MCPM_COMPAT_PRECISION");
  c.precision = (prec && std::strcmp(prec, "fp32") == 0) ? MCPM_FP32 : MCPM_FP64;
  c.sigma = at<double>(gas, OFF(GAS_sigma));
  c.m = at<double>(gas, OFF(GAS_m));
  c.kb = at<double>(gas, OFF(GAS_kb));
  c.n = at<double>(gas, OFF(GAS_n));
  c.Fn = at<double>(gas, OFF(GAS_Fn));
  c.T0 = at<double>(gas, OFF(GAS_T0));
  c.mu = at<double>(gas, OFF(GAS_mu));
  c.visp = at<double>(gas, OFF(GAS_visp));
  c.b = at<double>(gas, OFF(GAS_b));
  c.dt = at<double>(gas, OFF(GAS_delta_t));
  c.phi = at<double>(gas, OFF(GAS_phi));
  c.eqdist = at<double>(gas, OFF(GAS_eqdist));
  c.ast = at<double>(gas, OFF(GAS_ast));
  c.bst = at<double>(gas, OFF(GAS_bst));
  c.crref = at<double>(gas, OFF(GAS_crref));
  const size_t tw[4] = {OFF(BOX_T_wall_1), OFF(BOX_T_wall_2), OFF(BOX_T_wall_3), OFF(BOX_T_wall_4)};
  const size_t uw[4] = {OFF(BOX_U_wall_1), OFF(BOX_U_wall_2), OFF(BOX_U_wall_3), OFF(BOX_U_wall_4)};
  for (int i = 0; i < 4; ++i) {
    c.T_wall[i] = at<double>(box, tw[i]);
    c.U_wall[i] = at<double>(box, uw[i]);
  }
  c.max_particles = at<long>(gas, OFF(GAS_N));
  c.seed = 0x4D43504Dull;
  return c;
}

bool same_config(const mcpm_config& a, const mcpm_config& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

// a session for this configuration and particle count
void ensure(const GAS* gas, const BOX* box) {
  const mcpm_config c = config_of(gas, box);
  const int64_t N = at<long>(gas, OFF(GAS_N));
  if (g.s && same_config(c, g.cfg)) return;
  if (g.s) mcpm_session_destroy(g.s);
  g.s = nullptr;
  g.cfg = c;
  if (c.model < 0) {
    fprintf(stderr, "mcpm: gas.model is outside the particle step\n");
    exit(1);
  }
  ck(mcpm_session_create(&g.cfg, &g.s), "session_create");
  g.N = N;
  g.C = c.n_cells[0] * c.n_cells[1] * c.n_cells[2];
  g.cells.assign((size_t)MCPM_CF_COUNT * g.C, 0.0);
  g.om_synced = false;
  g.press = false;
}

void download(double* x1, double* x2, double* U1, double* U2, double* U3) {
  ck(mcpm_download_particles(g.s, g.N, x1, x2, U1, U2, U3), "download");
}

// the per-cell fields cell_update computes, into the reference's CELLS
void write_cells(CELLS* cells) {
  ck(mcpm_get_cells(g.s, g.cells.data()), "get_cells");
  const int C = g.C;
  auto F = [&](int f, int c) { return g.cells[(size_t)f * C + c]; };
  struct Arr { size_t off; int field, n; };
  const Arr arrs[] = {
      {OFF(CELLS_U_space), MCPM_CF_U_SPACE, 3}, {OFF(CELLS_PIJ), MCPM_CF_PIJ, 6}, {OFF(CELLS_M3), MCPM_CF_M3, 10},
      {OFF(CELLS_M4), MCPM_CF_M4, 6}, {OFF(CELLS_M5), MCPM_CF_M5, 3}, {OFF(CELLS_Q), MCPM_CF_Q, 3},
      {OFF(CELLS_DM2), MCPM_CF_DM2, 1}, {OFF(CELLS_DM4), MCPM_CF_DM4, 1}, {OFF(CELLS_Mp), MCPM_CF_MP, 3},
      {OFF(CELLS_T), MCPM_CF_T, 1}, {OFF(CELLS_n), MCPM_CF_N, 1}, {OFF(CELLS_gamma_st), MCPM_CF_GAMMA_ST, 1},
      {OFF(CELLS_Lambda), MCPM_CF_LAMBDA, 1}, {OFF(CELLS_c), MCPM_CF_C, 6}, {OFF(CELLS_gamma), MCPM_CF_GAMMA, 3},
      {OFF(CELLS_alpha), MCPM_CF_ALPHA, 9}, {OFF(CELLS_beta), MCPM_CF_BETA, 3}, {OFF(CELLS_phi), MCPM_CF_PHI, 3},
      {OFF(CELLS_divU), MCPM_CF_DIVU, 1}, {OFF(CELLS_n_smooth), MCPM_CF_N_SMOOTH, 1},
      {OFF(CELLS_dn2), MCPM_CF_DN2, 1}, {OFF(CELLS_dn3), MCPM_CF_DN3, 1}};
  for (int c = 0; c < C; ++c) {
    char* k = cell_ptr(cells, c);
    const int n = (int)F(MCPM_CF_NUM_INSIDE, c);
    at<int>(k, OFF(CELLS_num_inside)) = n;
    at<double>(k, OFF(CELLS_weight)) = (double)n;
    for (const Arr& a : arrs)
      for (int j = 0; j < a.n; ++j) at<double>(k, a.off + j * sizeof(double)) = F(a.field + j, c);
  }
}

// the per-cell particle lists (src/Main_Functions.cpp:2367-2376), ascending ids
void write_lists(CELLS* cells) {
  g.pid.resize((size_t)g.N);
  g.off.resize((size_t)g.C + 1);
  ck(mcpm_get_layout(g.s, g.pid.data(), g.off.data()), "get_layout");
  for (int c = 0; c < g.C; ++c) {
    char* k = cell_ptr(cells, c);
    int*& list = at<int*>(k, OFF(CELLS_indices_inside));
    free(list);
    const int n = g.off[c + 1] - g.off[c];
    list = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    std::memcpy(list, g.pid.data() + g.off[c], sizeof(int) * (size_t)n);
    std::sort(list, list + n);
  }
}

void cell_field_to_cells(CELLS* cells, int field, size_t off) {
  ck(mcpm_get_cells(g.s, g.cells.data()), "get_cells");
  for (int c = 0; c < g.C; ++c) at<double>(cell_ptr(cells, c), off) = g.cells[(size_t)field * g.C + c];
}

}  // namespace

// cell_update, src/Main_Functions.cpp:2138-2749 (src/cpp_headers.h:501)
void cell_update(double* x1, double* x2, double* U1, double* U2, double* U3, struct GAS* gas, struct CELLS* cells,
                 struct BOX* box, int* index, double** T, double* rho, int* color) {
  (void)T; (void)rho; (void)color;
  ensure(gas, box);
  g.N = at<long>(gas, OFF(GAS_N));
  ck(mcpm_upload_particles(g.s, g.N, x1, x2, U1, U2, U3), "upload");
  // the cells' weights, where the problem gives some cells other than 1
  std::vector<int32_t> w((size_t)g.C);
  bool any = false;
  for (int c = 0; c < g.C; ++c) {
    w[c] = at<int>(cell_ptr(cells, c), OFF(CELLS_n_ratio));
    any = any || (w[c] != 1 && w[c] != 0);
  }
  if (any) ck(mcpm_set_cell_weights(g.s, w.data()), "set_cell_weights");
  ck(mcpm_set_step(g.s, at<int>(box, OFF(BOX_step))), "set_step");
  ck(mcpm_cell_update(g.s), "cell_update");
  ck(mcpm_get_index(g.s, index), "get_index");
  write_cells(cells);
  write_lists(cells);
}

// random_generator, src/Fokker_Planck.cpp:20-145 (src/cpp_headers.h:362): the
// draws stay on the device for velocity_update
void random_generator(double* xi_1, double* xi_2, double* xi_3, double* xi_1f, double* xi_2f, double* xi_3f,
                      struct CELLS* cells, struct BOX* box, struct GAS* gas, int* index) {
  (void)xi_1; (void)xi_2; (void)xi_3; (void)xi_1f; (void)xi_2f; (void)xi_3f; (void)cells; (void)box; (void)gas;
  (void)index;
  ck(mcpm_random_generator(g.s), "random_generator");
}

// velocity_update, src/Main_Functions.cpp:1538-1673 (src/cpp_headers.h:499)
void velocity_update(double* U1, double* U2, double* U3, double* x1, double* x2, double* x3, struct GAS* gas,
                     struct BOX* box, struct CELLS* cells, int* index, struct Collision* CBA, double* xi_1f,
                     double* xi_2f, double* xi_3f, double* Mp1, double* Mp2, double* Mp3, double* F1, double* F2,
                     double* F3, double* rho, double* T, int* color) {
  (void)x3; (void)gas; (void)box; (void)index; (void)CBA; (void)xi_1f; (void)xi_2f; (void)xi_3f; (void)Mp1;
  (void)Mp2; (void)Mp3; (void)F1; (void)F2; (void)F3; (void)rho; (void)T; (void)color;
  const bool pairs = g.cfg.model == MCPM_MODEL_ESMC || g.cfg.model == MCPM_MODEL_DSMC_VHS;
  const size_t om = g.cfg.model == MCPM_MODEL_DSMC_VHS ? OFF(CELLS_crm) : OFF(CELLS_omega_max);
  if (pairs && !g.om_synced) {
    // the majorant the reference's main initialised (src/main.cpp:250-269)
    std::vector<double> v((size_t)g.C);
    for (int c = 0; c < g.C; ++c) v[c] = at<double>(cell_ptr(cells, c), om);
    ck(mcpm_set_cell_field(g.s, MCPM_CF_OMEGA_MAX, v.data()), "set_cell_field");
    g.om_synced = true;
  }
  ck(mcpm_velocity_update(g.s), "velocity_update");
  download(x1, x2, U1, U2, U3);
  if (pairs) cell_field_to_cells(cells, MCPM_CF_OMEGA_MAX, om);
  if (g.cfg.long_range != MCPM_LR_NONE) cell_field_to_cells(cells, MCPM_CF_F2, OFF(CELLS_F2));
}

// DFP_extra_streaming, src/Fokker_Planck.cpp:904-946 (src/cpp_headers.h:406)
void DFP_extra_streaming(double* U1, double* U2, double* U3, double* x1, double* x2, struct GAS* gas,
                         struct BOX* box, struct CELLS* cells, int* index, double dt) {
  (void)gas; (void)box; (void)cells; (void)index; (void)dt;
  ck(mcpm_dfp_extra_streaming(g.s), "DFP_extra_streaming");
  download(x1, x2, U1, U2, U3);
}

// apply_BC, src/Main_Functions.cpp:1451-1492 (src/cpp_headers.h:498)
void apply_BC(double* U1, double* U2, double* U3, double* x1, double* x2, double* x3, double* x1_old,
              double* x2_old, double* x3_old, struct GAS* gas, struct BOX* box, struct CELLS* cells, int* index,
              int* flag, double* xi_1, double* xi_2, double* xi_3, double* xi_1f, double* xi_2f, double* xi_3f,
              double* Mp1, double* Mp2, double* Mp3, double* T) {
  (void)x3; (void)x3_old; (void)gas; (void)box; (void)cells; (void)index; (void)flag; (void)xi_1; (void)xi_2;
  (void)xi_3; (void)xi_1f; (void)xi_2f; (void)xi_3f; (void)Mp1; (void)Mp2; (void)Mp3; (void)T;
  const bool old = g.cfg.problem == MCPM_PROBLEM_COUETTE || g.cfg.problem == MCPM_PROBLEM_WALL;
  // the walls read the caller's old positions (an upload starts them as the positions)
  if (old) ck(mcpm_set_old_positions(g.s, x1_old, x2_old), "set_old_positions");
  ck(mcpm_apply_bc(g.s), "apply_BC");
  download(x1, x2, U1, U2, U3);
  if (old) ck(mcpm_get_old_positions(g.s, x1_old, x2_old), "get_old_positions");
}

// store_old_positions, src/Main_Functions.cpp:5736-5760 (src/cpp_headers.h:454)
void store_old_positions(double* x1, double* x2, double* x3, double* x1_old, double* x2_old, double* x3_old,
                         struct GAS* gas, struct BOX* box) {
  (void)gas; (void)box;
  ck(mcpm_store_old_positions(g.s), "store_old_positions");
  const size_t b = sizeof(double) * (size_t)g.N;
  std::memcpy(x1_old, x1, b);
  std::memcpy(x2_old, x2, b);
  if (x3 && x3_old) std::memcpy(x3_old, x3, b);
}

// stream_particles, src/Main_Functions.cpp:1494-1521 (src/cpp_headers.h:495)
void stream_particles(double* U1, double* U2, double* U3, double* x1, double* x2, double* x3, double* x1_old,
                      double* x2_old, double* x3_old, struct GAS* gas, struct BOX* box, struct CELLS* cells,
                      int* index) {
  (void)x3; (void)x1_old; (void)x2_old; (void)x3_old; (void)gas; (void)box; (void)cells; (void)index;
  ck(mcpm_stream_particles(g.s), "stream_particles");
  download(x1, x2, U1, U2, U3);
}

// measure_pressure, src/Main_Functions.cpp:13-34 (src/cpp_headers.h:388):
// the crossings between the caller's x2_old and the current positions
void measure_pressure(double* U2, double* x2, double* x2_old, struct GAS* gas, struct BOX* box,
                      struct CELLS* cells) {
  (void)U2; (void)x2; (void)gas; (void)box;
  if (!g.press) {
    ck(mcpm_set_pressure_sampling(g.s, 1), "set_pressure_sampling");
    g.press = true;
  }
  ck(mcpm_set_old_positions(g.s, nullptr, x2_old), "set_old_positions");
  ck(mcpm_reset_pressure(g.s), "reset_pressure");
  ck(mcpm_measure_pressure(g.s), "measure_pressure");
  std::vector<double> p((size_t)g.C);
  ck(mcpm_get_pressure(g.s, p.data()), "get_pressure");
  for (int c = 0; c < g.C; ++c) at<double>(cell_ptr(cells, c), OFF(CELLS_p_m)) += p[c];
}

// ------------------------------------------------------------------ tests
// Plain-C helpers for driving the routines above without the reference's
// header: the structs' sizes and field offsets, zeroed objects with their
// std::string members constructed, string fields, and the session.
namespace {
struct Field { const char* name; size_t off, size; };
#define FLD(T, f) {#T "." #f, OFF(T##_##f), SZ(T##_##f)}
const Field kFields[] = {
    FLD(GAS, N), FLD(GAS, sigma), FLD(GAS, m), FLD(GAS, kb), FLD(GAS, n), FLD(GAS, Fn), FLD(GAS, T0), FLD(GAS, mu),
    FLD(GAS, visp), FLD(GAS, b), FLD(GAS, delta_t), FLD(GAS, phi), FLD(GAS, eqdist), FLD(GAS, ast), FLD(GAS, bst),
    FLD(GAS, crref), FLD(GAS, model), FLD(GAS, long_range), FLD(GAS, Tc), FLD(GAS, Th), FLD(GAS, n_ratio),
    FLD(GAS, T), FLD(BOX, N), FLD(BOX, Len), FLD(BOX, delta_dim), FLD(BOX, direction), FLD(BOX, problem),
    FLD(BOX, T_wall_1), FLD(BOX, T_wall_2), FLD(BOX, T_wall_3), FLD(BOX, T_wall_4), FLD(BOX, U_wall_1),
    FLD(BOX, U_wall_2), FLD(BOX, U_wall_3), FLD(BOX, U_wall_4), FLD(BOX, step), FLD(BOX, thermc), FLD(BOX, thermh),
    FLD(BOX, file_name), FLD(CELLS, num_inside), FLD(CELLS, indices_inside), FLD(CELLS, weight),
    FLD(CELLS, U_space), FLD(CELLS, PIJ), FLD(CELLS, M3), FLD(CELLS, M4), FLD(CELLS, M5), FLD(CELLS, Q),
    FLD(CELLS, DM2), FLD(CELLS, DM4), FLD(CELLS, Mp), FLD(CELLS, T), FLD(CELLS, n), FLD(CELLS, gamma_st),
    FLD(CELLS, Lambda), FLD(CELLS, c), FLD(CELLS, gamma), FLD(CELLS, alpha), FLD(CELLS, beta), FLD(CELLS, phi),
    FLD(CELLS, F2), FLD(CELLS, omega_max), FLD(CELLS, crm), FLD(CELLS, divU), FLD(CELLS, n_smooth),
    FLD(CELLS, dn2), FLD(CELLS, dn3), FLD(CELLS, n_ratio), FLD(CELLS, p_m)};
const size_t kSizes[3] = {MCPM_REF_SIZEOF_GAS, MCPM_REF_SIZEOF_BOX, MCPM_REF_SIZEOF_CELLS};
}  // namespace

extern "C" {
// 0: GAS, 1: BOX, 2: CELLS
int64_t mcpm_compat_sizeof(int32_t which) { return which >= 0 && which < 3 ? (int64_t)kSizes[which] : -1; }
// "GAS.sigma" -> byte offset (size in *size), -1 if unknown
int64_t mcpm_compat_offset(const char* name, int64_t* size) {
  for (const Field& f : kFields)
    if (std::strcmp(f.name, name) == 0) {
      if (size) *size = (int64_t)f.size;
      return (int64_t)f.off;
    }
  return -1;
}
// count zeroed objects of the struct, std::string members constructed
void* mcpm_compat_new(int32_t which, int64_t count) {
  if (which < 0 || which > 2 || count < 1) return nullptr;
  char* p = (char*)calloc((size_t)count, kSizes[which]);
  for (int64_t i = 0; i < count && which < 2; ++i) {
    char* o = p + (size_t)i * kSizes[which];
    if (which == 0) {
      new (o + OFF(GAS_model)) std::string();
    } else {
      new (o + OFF(BOX_file_name)) std::string();
    }
  }
  return p;
}
void mcpm_compat_delete(int32_t which, void* p, int64_t count) {
  if (!p) return;
  for (int64_t i = 0; i < count; ++i) {
    char* o = (char*)p + (size_t)i * kSizes[which];
    if (which == 0) reinterpret_cast<std::string*>(o + OFF(GAS_model))->~basic_string();
    else if (which == 1) reinterpret_cast<std::string*>(o + OFF(BOX_file_name))->~basic_string();
    else free(at<int*>(o, OFF(CELLS_indices_inside)));
  }
  free(p);
}
void mcpm_compat_set_model(void* gas, const char* model) { at<std::string>(gas, OFF(GAS_model)) = model; }
// the routine of that name ("cell_update", ...), for callers without the
// reference's header
void* mcpm_compat_routine(const char* name) {
  struct R { const char* n; void* f; };
  const R rs[] = {{"cell_update", (void*)&cell_update}, {"random_generator", (void*)&random_generator},
                  {"velocity_update", (void*)&velocity_update},
                  {"DFP_extra_streaming", (void*)&DFP_extra_streaming}, {"apply_BC", (void*)&apply_BC},
                  {"store_old_positions", (void*)&store_old_positions},
                  {"stream_particles", (void*)&stream_particles}, {"measure_pressure", (void*)&measure_pressure}};
  for (const R& r : rs)
    if (std::strcmp(r.n, name) == 0) return r.f;
  return nullptr;
}
// the session behind the routines (NULL before the first cell_update)
mcpm_session* mcpm_compat_session(void) { return g.s; }
void mcpm_compat_reset(void) {
  if (g.s) mcpm_session_destroy(g.s);
  g.s = nullptr;
  std::memset(&g.cfg, 0, sizeof g.cfg);
}
}  // extern "C"
