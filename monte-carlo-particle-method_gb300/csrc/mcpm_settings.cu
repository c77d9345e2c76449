// mcpm_settings.cu -- the reference's settings file as an mcpm_config.
//
// readSettingsFile (src/myIO.cpp:1756-3016) reads one "keyword values..."
// line at a time ('#' lines are comments) into GAS/BOX and then derives the
// run's constants: cell sizes, Fn, the hard-sphere or VHS diameter and
// reference speed from the viscosity, b, mu(T0), the mean free path, dt and
// the attraction strength.  This restates that reading and the derivation
// along the path the particle step covers (problems closed_box 1,
// couette_flow 2, wall 11 and injection 12; the step's models), in the
// reference's order of
// operations, so that a run configured by the reference's own files gets
// the constants the reference would use.  Host code only.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <sstream>
#include <string>

#include "../../include/mcpm.h"

namespace {

// the keywords readSettingsFile accepts (src/myIO.cpp:1880-2122); lines with
// any other keyword abort the reference's run
const char* const kKeywords[] = {
    "N", "gp_nn", "N13", "sigc", "alphac", "sigh", "alphah", "n", "nc", "nh", "nvc", "nvh", "nv1", "nv2", "nv3",
    "Tc", "Th", "Tv1", "Tv2", "Tv3", "LcN", "LhN", "LvN", "LvN1", "LvN3", "Lv1", "Lv3", "Nh", "Nv1", "Nv2", "Nv3",
    "long_range", "box_len", "cone_len", "x2_prob", "ghost", "thermc", "thermh", "cone_num_cells", "cone_angles",
    "flatnose", "flatratio", "box_delta_dim", "direction", "U0", "sigma", "weight", "dcones_n", "mass", "steps",
    "dt", "init_step", "model", "output", "movie", "every", "num_realizations", "after", "reset_every",
    "frac_mft", "T", "epsilon", "kb", "num_thr", "mu", "visp", "nualpha", "phi", "phi0", "factor", "n_ratio",
    "problem", "U_wall_1", "U_wall_2", "U_wall_3", "U_wall_4", "U_wall_5", "U_wall_6", "U_wall_7", "T_wall_1",
    "T_wall_2", "T_wall_3", "T_wall_4", "T_wall_5", "T_wall_6", "T_wall_7", "n_wall_4", "n_wall_5", "n_wall_6",
    "n_wall_7", "reset", "drop_dia", "num_cells"};

bool known(const std::string& k) {
  for (const char* w : kKeywords)
    if (k == w) return true;
  return false;
}

// the values the derivation reads, with readSettingsFile's "unset" markers
struct Raw {
  long N = -1;
  int cells[3] = {-1, -1, -1};
  int direction[3] = {0, 0, 0};
  double Len[3] = {-1.0, -1.0, -1.0};
  double delta_dim[3] = {-1.0, -1.0, -1.0};
  double kb = -1.0, sigma = -1.0, T = -1.0, n = -1.0, m = -1.0, dt = -1.0, mu = -1.0, frac_mft = -1.0;
  double epsilon = -1.0, phi = -1.0;
  bool has_visp = false, has_nualpha = false;
  double visp = 0.0, nualpha = 0.0;
  int problem = -1, long_range = 0;
  std::string model;
  double U_wall[4] = {-1.0, -1.0, -1.0, -1.0};
  double T_wall[4] = {-1.0, -1.0, -1.0, -1.0};
  double U0[3] = {-1.0, -1.0, -1.0};
  // problem wall (11): a liquid slab between vapour layers, in units of sigma
  double nc = -1.0, nv1 = 0.0, nv2 = -1.0, Tc = -1.0;
  int LcN = -1, LvN = -1, LvN1 = -1, n_ratio = -1;
  // problem injection (12): a denser disc (the droplet) in a gas at rest
  double nh = -1.0, drop_dia = -1.0;
};

// readSettingsFile's branch for problem wall (src/myIO.cpp:2628-2726): argon's
// diameter, the densities given in sigma^-3, a fixed Fn, the particle counts
// of the lower vapour layer, the liquid slab and the upper vapour layer, and
// the box height they fill; the gas temperature becomes the liquid's
struct WallSetup {
  double sigma, n, Fn, Lv1, Lc, Lv, Len1, T;
  int Nv1, Nc2, Nv2;
  long N;
};

int wall_setup(const Raw& r, WallSetup& w, char* msg, int32_t msg_len);

// readSettingsFile's branch for problem injection (src/myIO.cpp:2727-2760):
// argon's diameter, the densities in sigma^-3, N per cell times the cells,
// the box's x and y lengths in sigma, Fn of the gas density over the box,
// and the droplet's extra particles Nh = floor((nh - nc) pi d^2 / 4 / Fn)
// for a disc of diameter d = drop_dia sigma; the gas temperature becomes Tc
struct InjSetup {
  double sigma, n, Fn, Len0, Len1, drop_dia, T;
  int Nh;
  long N;
};

int inj_setup(const Raw& r, InjSetup& j, char* msg, int32_t msg_len);

int set_msg(char* msg, int32_t len, const char* text, int code) {
  if (msg && len > 0) {
    std::strncpy(msg, text, (size_t)len - 1);
    msg[len - 1] = '\0';
  }
  return code;
}

int model_code(const std::string& m) {
  if (m == "none") return MCPM_MODEL_NONE;
  if (m == "FP_dense") return MCPM_MODEL_FP_DENSE;
  if (m == "FP_ideal_gas") return MCPM_MODEL_FP_IDEAL_GAS;
  if (m == "ESMC") return MCPM_MODEL_ESMC;
  if (m == "FP_linear") return MCPM_MODEL_FP_LINEAR;
  if (m == "DSMC_VHS") return MCPM_MODEL_DSMC_VHS;
  return -1;
}

// reads the file into r, then applies the defaults of src/myIO.cpp:2122-2188
int read_raw(const char* path, Raw& r, char* msg, int32_t msg_len) {
  FILE* f = std::fopen(path, "r");
  if (!f) return set_msg(msg, msg_len, "settings: cannot open the file", MCPM_ERR_ARG);
  char buf[4096];
  int rc = MCPM_OK;
  char err[512] = {0};
  while (std::fgets(buf, sizeof(buf), f)) {
    if (buf[0] == '#') continue;
    std::istringstream iss(buf);
    std::string key;
    // a blank line: the reference re-enters the previous keyword's branch
    // with nothing left to read, which changes nothing
    if (!(iss >> key)) continue;
    if (!known(key)) {
      std::snprintf(err, sizeof(err), "settings: unknown keyword '%s' (src/myIO.cpp:2116-2121)", key.c_str());
      rc = MCPM_ERR_ARG;
      break;
    }
    if (key == "N") iss >> r.N;
    else if (key == "n") iss >> r.n;
    else if (key == "long_range") iss >> r.long_range;
    else if (key == "box_len") iss >> r.Len[0] >> r.Len[1] >> r.Len[2];
    else if (key == "box_delta_dim") iss >> r.delta_dim[0] >> r.delta_dim[1] >> r.delta_dim[2];
    else if (key == "direction") iss >> r.direction[0] >> r.direction[1] >> r.direction[2];
    else if (key == "sigma") iss >> r.sigma;
    else if (key == "mass") iss >> r.m;
    else if (key == "dt") iss >> r.dt;
    else if (key == "model") iss >> r.model;
    else if (key == "frac_mft") iss >> r.frac_mft;
    else if (key == "T") iss >> r.T;
    else if (key == "epsilon") iss >> r.epsilon;
    else if (key == "kb") iss >> r.kb;
    else if (key == "mu") iss >> r.mu;
    else if (key == "visp") r.has_visp = static_cast<bool>(iss >> r.visp);
    else if (key == "nualpha") r.has_nualpha = static_cast<bool>(iss >> r.nualpha);
    else if (key == "phi") iss >> r.phi;
    else if (key == "problem") iss >> r.problem;
    else if (key == "num_cells") iss >> r.cells[0] >> r.cells[1] >> r.cells[2];
    else if (key == "U0") iss >> r.U0[0] >> r.U0[1] >> r.U0[2];
    else if (key == "nc") iss >> r.nc;
    else if (key == "nv1") iss >> r.nv1;
    else if (key == "nv2") iss >> r.nv2;
    else if (key == "Tc") iss >> r.Tc;
    else if (key == "LcN") iss >> r.LcN;
    else if (key == "LvN") iss >> r.LvN;
    else if (key == "LvN1") iss >> r.LvN1;
    else if (key == "n_ratio") iss >> r.n_ratio;
    else if (key == "nh") iss >> r.nh;
    else if (key == "drop_dia") iss >> r.drop_dia;
    else if (key.rfind("U_wall_", 0) == 0 || key.rfind("T_wall_", 0) == 0) {
      const int w = key[7] - '1';
      if (w >= 0 && w < 4) iss >> (key[0] == 'U' ? r.U_wall[w] : r.T_wall[w]);
    }
    // every other keyword belongs to problems, outputs or run control the
    // particle step does not read
  }
  std::fclose(f);
  if (rc) return set_msg(msg, msg_len, err, rc);
  if (r.Len[0] < 0.0) r.Len[0] = r.Len[1] = r.Len[2] = 1.0;  // src/myIO.cpp:2163-2166
  if (r.cells[0] < 1 || r.cells[1] < 1 || r.cells[2] != 1)
    return set_msg(msg, msg_len, "settings: num_cells must be N0 N1 1", MCPM_ERR_ARG);
  if (r.problem < 0) r.problem = 1;
  if (r.problem != 11 && r.N < 1) return set_msg(msg, msg_len, "settings: N (particles) is required", MCPM_ERR_ARG);
  if (r.delta_dim[0] < 0.0 || r.problem == 11 || r.problem == 12) {
    // (problems wall and injection set the cells from the box they derive)
    for (int i = 0; i < 3; ++i) r.delta_dim[i] = r.Len[i] / r.cells[i];
  } else {
    // the session's cells are Len / N: a box_delta_dim that disagrees would
    // give the reference other cells than the step's
    for (int i = 0; i < 2; ++i)
      if (std::fabs(r.delta_dim[i] - r.Len[i] / r.cells[i]) > 1e-12 * std::fabs(r.Len[i] / r.cells[i]))
        return set_msg(msg, msg_len, "settings: box_delta_dim differs from box_len / num_cells", MCPM_ERR_ARG);
  }
  if (r.kb < 0.0) r.kb = 1.38064852 * 1e-23;
  if (r.T < 0.0) r.T = 1.0 / r.kb;
  if (r.sigma < 0.0) r.sigma = 1;
  if (r.n < 0.0) r.n = 1e-3;
  if (r.m < 0.0) r.m = 1.0;
  if (r.U0[0] < 0.0) r.U0[0] = r.U0[1] = r.U0[2] = 1.0;
  for (int i = 0; i < 4; ++i)
    if (r.T_wall[i] < 0) r.T_wall[i] = 1.0;
  if (r.problem != 1 && r.problem != 2 && r.problem != 11 && r.problem != 12)
    return set_msg(msg, msg_len,
                   "settings: only problems closed_box (1), couette_flow (2), wall (11) and injection (12) "
                   "configure the particle step",
                   MCPM_ERR_ARG);
  return MCPM_OK;
}

int inj_setup(const Raw& r, InjSetup& j, char* msg, int32_t msg_len) {
  if (!(r.nc > 0.0) || !(r.nh >= r.nc) || !(r.Tc > 0.0) || !(r.drop_dia >= 0.0))
    return set_msg(msg, msg_len, "settings: problem injection needs nc > 0, nh >= nc, Tc and drop_dia", MCPM_ERR_ARG);
  const double pi = std::acos(-1.0);
  j.sigma = 3.405e-10;
  const double nc = r.nc / std::pow(j.sigma, 3.0);
  const double nh = r.nh / std::pow(j.sigma, 3.0);
  const long N = r.N * r.cells[0] * r.cells[1];
  j.Len0 = r.Len[0] * j.sigma;
  j.Len1 = r.Len[1] * j.sigma;
  j.T = r.Tc;
  j.n = nc;
  j.Fn = j.n * j.Len0 * j.Len1 * r.Len[2] / (1.0 * N);
  j.drop_dia = r.drop_dia * j.sigma;
  j.Nh = (int)std::floor((nh - nc) * pi * j.drop_dia * j.drop_dia / 4.0 / j.Fn);
  j.N = N + j.Nh;
  return MCPM_OK;
}

int wall_setup(const Raw& r, WallSetup& w, char* msg, int32_t msg_len) {
  if (!(r.nc > 0.0) || !(r.nv2 > 0.0) || !(r.Tc > 0.0) || r.LcN < 0 || r.LvN < 0)
    return set_msg(msg, msg_len, "settings: problem wall needs nc, nv2, Tc, LcN and LvN", MCPM_ERR_ARG);
  // LvN1 < 0 (unset) puts the slab below y = 0 in the reference: refused
  if (r.LvN1 < 0 || (r.LvN1 > 0 && !(r.nv1 > 0.0)))
    return set_msg(msg, msg_len, "settings: problem wall needs LvN1 >= 0 (and nv1 when LvN1 > 0)", MCPM_ERR_ARG);
  const double sigma = 3.405e-10;
  const double nc = r.nc / std::pow(sigma, 3.0);
  const double nv1 = r.nv1 / std::pow(sigma, 3.0);
  const double nv2 = r.nv2 / std::pow(sigma, 3.0);
  w.sigma = sigma;
  w.n = nc;
  w.Lc = r.LcN * sigma;
  w.Lv = r.LvN * sigma;
  w.Lv1 = r.LvN1 * sigma;
  const double Lc_ratio = w.Lc;
  const int n_ratio = r.n_ratio < 0 ? (int)std::floor(nc / nv2) : r.n_ratio;
  if (n_ratio < 1) return set_msg(msg, msg_len, "settings: problem wall needs n_ratio >= 1 (or nc >= nv2)", MCPM_ERR_ARG);
  w.Fn = 0.1e+14;
  const int sg1 = r.LvN1 > 0 ? 1 : 0;
  w.Nc2 = (int)std::floor(nc * r.Len[0] * r.Len[2] * (Lc_ratio + 0.5 * (w.Lc - Lc_ratio) * (1 - sg1)) /
                          (1.0 * n_ratio * w.Fn));
  w.Nv1 = (int)std::floor(nv1 * r.Len[0] * r.Len[2] * w.Lv1 / w.Fn);
  w.Nv2 = (int)std::floor(nv2 * r.Len[0] * r.Len[2] * w.Lv / w.Fn);
  w.N = (long)0 + w.Nc2 + 0 + w.Nv1 + w.Nv2;
  w.Len1 = w.Lv + w.Lc + w.Lv1;
  w.T = r.Tc;
  if (w.N < 1) return set_msg(msg, msg_len, "settings: problem wall gives no particles", MCPM_ERR_ARG);
  return MCPM_OK;
}

}  // namespace

extern "C" int mcpm_config_from_settings(const char* path, mcpm_config* out, int64_t* n_particles, char* msg,
                                         int32_t msg_len) {
  if (!path || !out) return set_msg(msg, msg_len, "settings: null argument", MCPM_ERR_ARG);
  Raw r;
  if (int rc = read_raw(path, r, msg, msg_len)) return rc;
  // ---- the derivation, src/myIO.cpp:2213-2900, problems 1, 2 and 11
  const double pi = std::acos(-1.0);
  const int model = model_code(r.model);
  if (model < 0) return set_msg(msg, msg_len, "settings: the model is outside the particle step", MCPM_ERR_ARG);
  if (!r.has_visp) return set_msg(msg, msg_len, "settings: visp is required", MCPM_ERR_ARG);
  const double volume = r.Len[0] * r.Len[1] * r.Len[2];
  const double Fn = r.n * volume / r.N;
  const double thermal = std::sqrt(r.kb * r.T / r.m);
  const double T0 = 273.0;
  if (r.epsilon < 0.0) r.epsilon = 119.8 * r.kb;
  double crref;
  if (std::fabs(r.sigma - 1.0) < 1e-14) {
    crref = thermal;
  } else if (std::fabs(r.visp - 0.5) < 1e-13) {
    // hard spheres: the diameter that gives the viscosity mu at T0
    if (!(r.mu > 0.0)) return set_msg(msg, msg_len, "settings: mu is required to derive sigma", MCPM_ERR_ARG);
    r.sigma = 1.016 * 5.0 * std::sqrt(r.m * r.kb * T0 / pi);
    r.sigma = r.sigma / (16.0 * r.mu);
    r.sigma = std::sqrt(r.sigma);
    crref = thermal;
  } else {
    // variable hard spheres (Bird): diameter and reference speed from mu
    if (!(r.mu > 0.0) || !r.has_nualpha)
      return set_msg(msg, msg_len, "settings: mu and nualpha are required to derive the VHS sigma", MCPM_ERR_ARG);
    const double nu = r.nualpha, w = r.visp;
    r.sigma = 1.016 * 5.0 * (nu + 1.0) * (nu + 2.0) * std::sqrt(r.m * r.kb * T0 / pi);
    r.sigma = r.sigma / ((4.0 * nu) * (5.0 - 2.0 * w) * (7.0 - 2.0 * w) * r.mu);
    r.sigma = std::sqrt(r.sigma);
    const double numer = r.m * std::pow(4.0, w - 1) * 5.0 * (nu + 1.0) * (nu + 2.0) * std::sqrt(pi);
    const double denom = pi * std::pow(r.sigma, 2.0) * nu * (5.0 - 2.0 * w) * (7.0 - 2.0 * w) * 2.0 *
                         std::tgamma(5.0 / 2.0 - w);
    crref = (numer / denom) * std::pow(r.kb * 273.0 / r.m, w) / r.mu;
    crref = std::pow(crref, 1.0 / (w * 2.0 - 1.0));
  }
  double eqdist;
  double Fn_run = Fn;
  long N_run = r.N;
  if (r.problem == 12) {
    // the injection branch, after crref as well (:2727-2760)
    InjSetup js;
    if (int rc = inj_setup(r, js, msg, msg_len)) return rc;
    r.sigma = js.sigma;
    eqdist = js.sigma;
    r.n = js.n;
    Fn_run = js.Fn;
    N_run = js.N;
    r.Len[0] = js.Len0;
    r.Len[1] = js.Len1;
    r.T = js.T;
  } else if (r.problem == 11) {
    // the wall branch replaces the diameter, density, Fn, N, the box height
    // and the temperature after crref is set (:2628-2726)
    WallSetup ws;
    if (int rc = wall_setup(r, ws, msg, msg_len)) return rc;
    r.sigma = ws.sigma;
    eqdist = ws.sigma;
    r.n = ws.n;
    Fn_run = ws.Fn;
    N_run = ws.N;
    r.Len[1] = ws.Len1;
    r.T = ws.T;
  } else {
    eqdist = std::pow(2.0, 1.0 / 6.0) * r.sigma;  // :2820-2822
  }
  const double b = 2 * pi * std::pow(r.sigma, 3) / (3.0);
  const double mu = 5.0 / (16.0 * r.sigma * r.sigma) * std::sqrt(r.m * r.kb * T0 / std::acos(-1.0));
  if (r.dt < 0.0) {
    const double wall_speed = std::fmax(std::sqrt(r.kb * r.T_wall[0] / r.m), std::fmax(r.U_wall[0], r.U_wall[1]));
    const double dy = r.Len[1] / r.cells[1];
    if (model == MCPM_MODEL_DSMC_VHS || model == MCPM_MODEL_ESMC || model == MCPM_MODEL_FP_DENSE) {
      // the mean free path of the VHS/VSS gas, :2836-2839
      if (!r.has_nualpha)
        return set_msg(msg, msg_len, "settings: nualpha is required to derive dt", MCPM_ERR_ARG);
      double lambda = 4.0 * r.nualpha * (5.0 - 2.0 * r.visp) * (7.0 - 2.0 * r.visp);
      lambda = lambda / (5.0 * (r.nualpha + 1.0) * (r.nualpha + 2.0));
      lambda = lambda * std::sqrt(r.m / (2.0 * pi * r.kb * r.T)) * mu / (r.m * r.n);
      const double frac = r.frac_mft < 0.0 ? 0.5 : r.frac_mft;
      r.dt = frac * std::fmin(lambda, dy) / wall_speed;
    } else {
      const double frac = r.frac_mft < 0.0 ? 0.5 : r.frac_mft;
      r.dt = frac * r.Len[1] / r.cells[1] / wall_speed;
    }
  }
  const double phi = r.phi < 0.0 ? -4.0 * r.epsilon : -r.phi * r.epsilon;  // :2900-2905

  mcpm_config c;
  std::memset(&c, 0, sizeof(c));
  for (int i = 0; i < 3; ++i) {
    c.n_cells[i] = r.cells[i];
    c.direction[i] = r.direction[i];
    c.length[i] = r.Len[i];
  }
  // injection's walls are the closed box's specular ones (apply_BC,
  // src/Main_Functions.cpp:1487-1489)
  c.problem = (r.problem == 1 || r.problem == 12) ? MCPM_PROBLEM_CLOSED_BOX
              : r.problem == 2                    ? MCPM_PROBLEM_COUETTE
                                                  : MCPM_PROBLEM_WALL;
  c.model = model;
  // "0 or anything > 3 = no attraction" (src/Main_Functions.cpp:1612-1617)
  c.long_range = (r.long_range >= 1 && r.long_range <= 3) ? r.long_range : MCPM_LR_NONE;
  c.precision = MCPM_FP64;
  c.sigma = r.sigma; c.m = r.m; c.kb = r.kb; c.n = r.n; c.Fn = Fn_run;
  c.T0 = T0; c.mu = mu; c.visp = r.visp; c.b = b; c.dt = r.dt;
  c.phi = phi; c.eqdist = eqdist;
  // the screened-Poisson constants readSettingsFile sets (SI, :2884-2885)
  c.ast = -1.64835851e-28;
  c.bst = 6.91304716e+09;
  for (int i = 0; i < 4; ++i) {
    c.T_wall[i] = r.T_wall[i];
    c.U_wall[i] = r.U_wall[i];
  }
  c.seed = 0x4D43504Dull;
  c.max_particles = N_run;
  c.crref = crref;
  *out = c;
  if (n_particles) *n_particles = N_run;
  return set_msg(msg, msg_len, "", MCPM_OK);
}

// initialization (src/Main_Functions.cpp:4222-4814), its branches for the
// problems above.  Closed box and Couette: positions uniform along the
// streaming directions and at mid-box along the others (:4657-4672).  Wall
// (:4493-4530): x1 as before, x2 uniform in the lower vapour layer for the
// first Nv1 particles, in the liquid slab for the next Nc2, in the upper
// vapour layer for the rest.  Injection (:4627-4643): the gas uniform over
// the box, then the droplet's Nh particles uniform over the central disc.
// Velocities normal about U0 with sqrt(kb T / m),
// T = max(gas.T, max(T_wall_1 + T_wall_2, T_wall_3 + T_wall_4) / 2)
// (:4790-4799; gas.T is Tc for the wall and injection problems).  The reference
// seeds its generator from std::random_device; here a 64-bit Mersenne
// twister seeded by the caller gives the uniforms and Box-Muller pairs the
// normals, so a seed repeats a run on any host.
extern "C" int mcpm_initialize_from_settings(const char* path, uint64_t seed, double* x1, double* x2, double* U1,
                                             double* U2, double* U3, int64_t n_particles, char* msg,
                                             int32_t msg_len) {
  if (!path || !x1 || !x2 || !U1 || !U2 || !U3)
    return set_msg(msg, msg_len, "initialize: null argument", MCPM_ERR_ARG);
  Raw r;
  if (int rc = read_raw(path, r, msg, msg_len)) return rc;
  const bool wall = r.problem == 11, inj = r.problem == 12;
  WallSetup ws{};
  InjSetup js{};
  if (wall) {
    if (int rc = wall_setup(r, ws, msg, msg_len)) return rc;
    r.N = ws.N;
    r.Len[1] = ws.Len1;
    r.T = ws.T;
  } else if (inj) {
    if (int rc = inj_setup(r, js, msg, msg_len)) return rc;
    r.N = js.N;
    r.Len[0] = js.Len0;
    r.Len[1] = js.Len1;
    r.T = js.T;
  }
  if (n_particles != r.N) return set_msg(msg, msg_len, "initialize: n_particles differs from the file's N", MCPM_ERR_ARG);
  std::mt19937_64 gen(seed);
  auto uni = [&]() { return ((double)(gen() >> 11) + 0.5) * (1.0 / 9007199254740992.0); };
  const double two_pi = 2.0 * std::acos(-1.0);
  for (int64_t i = 0; i < r.N; ++i) {
    if (inj) {
      // the gas uniform over the box, then the droplet's Nh particles
      // uniform over the disc at the centre (src/Main_Functions.cpp:4627-4643)
      if (i < r.N - js.Nh) {
        x1[i] = uni() * r.Len[0];
        x2[i] = uni() * r.Len[1];
      } else {
        const double rr = (js.drop_dia / 2.0) * std::sqrt(uni()), th = uni() * two_pi;
        x1[i] = 0.5 * r.Len[0] + rr * std::cos(th);
        x2[i] = 0.5 * r.Len[1] + rr * std::sin(th);
      }
      continue;
    }
    x1[i] = r.direction[0] == 1 ? uni() * r.Len[0] : 0.5 * r.Len[0];
    if (!wall) {
      x2[i] = r.direction[1] == 1 ? uni() * r.Len[1] : 0.5 * r.Len[1];
    } else if (i < ws.Nv1) {
      x2[i] = uni() * ws.Lv1;
    } else if (i < ws.Nv1 + ws.Nc2) {
      // the slab: Lc_ratio = Lc, so the reference's offsets (Lc - Lc_ratio) / 2 vanish
      x2[i] = ws.Lv1 + uni() * ws.Lc;
    } else {
      x2[i] = ws.Lv1 + ws.Lc + uni() * ws.Lv;
    }
  }
  double T = std::fmax(r.T_wall[0] + r.T_wall[1], r.T_wall[2] + r.T_wall[3]) / 2.0;
  T = std::fmax(r.T, T);
  const double sd = std::sqrt(r.kb * T / r.m);
  double* U[3] = {U1, U2, U3};
  for (int64_t i = 0; i < r.N; ++i)
    for (int d = 0; d < 3; ++d) {
      const double a = std::sqrt(-2.0 * std::log(uni())), z = a * std::cos(two_pi * uni());
      U[d][i] = r.U0[d] + sd * z;
    }
  return set_msg(msg, msg_len, "", MCPM_OK);
}
