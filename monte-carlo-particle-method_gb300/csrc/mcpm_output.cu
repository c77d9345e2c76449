// mcpm_output.cu -- the reference's post-processing outputs from the cell
// fields a session keeps (host code).
//
//   write_post_processing  src/myIO.cpp:597-934: one PostProc/<out>_<lr>_<step>.dat
//                          file, a header row of 122 names and one row of 121
//                          values per cell (x outer, y inner, a blank line
//                          after each column of cells)
//   post_processing        src/myIO.cpp:935-965: the console summary lines
//
// The file's layout is a format other tools read, so its columns, their
// order and the printf conversions are the reference's; the face-flux sums
// of its interface problems (update_face_info) and the fields only its
// hybrid and 1-D screened-Poisson paths fill (model, xx, UU, UU0, UUR, UU0R)
// are written as 0, the value they hold in any other run.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mcpm_internal.h"

namespace mcpm {
namespace {

// increase_collision_rate, src/Main_Functions.cpp:1906-1915 (pow kept)
double y_coll(double n, double b) {
  return 1.0 + 0.625 * n * b + 0.2869 * pow(n * b, 2.0) + 0.115 * pow(n * b, 3.0);
}

// the 121 column names without the column-number prefixes that the first
// name and every tenth one up to the 110th carry in the header row
std::vector<std::string> column_names() {
  std::vector<std::string> v;
  auto idx = [&](const char* base, int n, int first = 0) {
    for (int i = first; i < first + n; ++i) v.push_back(std::string(base) + "[" + std::to_string(i) + "]");
  };
  for (const char* s : {"x1", "x2", "dx", "dy", "dz", "tavg", "dt"}) v.push_back(s);
  idx("U_space", 3);
  v.push_back("T");
  v.push_back("n");
  v.push_back("sum_weight");
  idx("sum_M", 3);
  idx("sum_MM", 6);
  idx("sum_MMM", 10);
  idx("sum_T_f", 4);
  idx("sum_M_n", 4);
  idx("sum_M1_f", 6);
  idx("sum_M2_f", 6);
  idx("sum_M3_f", 4);
  idx("sum_N", 2, 2);
  idx("sum_M_np", 6);
  idx("sum_MM_f_1", 6);
  idx("sum_MM_f_2", 6);
  idx("sum_MM_f_3", 6);
  for (const char* s : {"volume", "n_smooth", "N", "ptot", "Fn"}) v.push_back(s);
  idx("sum_MMMM", 6);
  for (const char* s : {"model", "xx", "PIJ[3]", "Q[1]", "F2", "divU", "UU", "UU0", "UUR", "UU0R"}) v.push_back(s);
  for (int i = 1; i <= 9; ++i) v.push_back("alpha" + std::to_string(i));
  for (int i = 1; i <= 3; ++i) v.push_back("beta" + std::to_string(i));
  v.push_back("gamma_st");
  idx("phi", 3);
  v.push_back("p_m");
  v.push_back("p_rep");
  return v;
}

const char* lr_name(int lr) {
  return lr == 1 ? "direct" : lr == 2 ? "denexp" : lr == 3 ? "screened-Poisson" : "noatt";
}

}  // namespace
}  // namespace mcpm

using namespace mcpm;

extern "C" int mcpm_post_processing_write(const mcpm_config* cfg, int32_t step, double t_post, const char* dir,
                                          const char* output_name, const double* cells, const double* samples,
                                          const double* p_m, const int32_t* cell_weights, char* path,
                                          int32_t path_len) {
  if (!cfg || !dir || !output_name || !cells) return MCPM_ERR_ARG;
  const int N0 = cfg->n_cells[0], N1 = cfg->n_cells[1], C = N0 * N1;
  if (N0 < 1 || N1 < 1) return MCPM_ERR_ARG;
  const std::vector<std::string> names = column_names();
  if (names.size() != 121) return MCPM_ERR_STATE;
  char name[4096];
  snprintf(name, sizeof name, "%s/%s_%s_%d.dat", dir, output_name, lr_name(cfg->long_range), step);
  if (path && path_len > 0) snprintf(path, (size_t)path_len, "%s", name);
  FILE* fp = fopen(name, "w");
  if (!fp) return MCPM_ERR_ARG;
  // header: "#variables=" and the first name at width 10, the rest at 20;
  // column k (1-based) carries the prefix "k-" when k is 1 or a multiple of
  // 10 up to 110
  fprintf(fp, "%10s", "#variables=");
  for (int k = 1; k <= 121; ++k) {
    std::string h = names[k - 1];
    if (k == 1 || (k % 10 == 0 && k <= 110)) h = std::to_string(k) + "-" + h;
    fprintf(fp, k == 1 ? "%10s" : "%20s", h.c_str());
  }
  fprintf(fp, "\n");
  auto F = [&](int f, int c) { return cells[(size_t)f * C + c]; };
  auto S = [&](int f, int c) { return samples ? samples[(size_t)f * C + c] : 0.0; };
  const double dx = cfg->length[0] / N0, dy = cfg->length[1] / N1, dz = cfg->length[2] / cfg->n_cells[2];
  for (int i = 0; i < N0; ++i) {
    for (int j = 0; j < N1; ++j) {
      const int num = j * N0 + i;
      // make_cells geometry, src/myIO.cpp:1456-1467
      const double d0 = (double)(i)*dx, d1 = (double)(i + 1) * dx, d2 = (double)(j)*dy, d3 = (double)(j + 1) * dy;
      const double d4 = (double)(0) * dz, d5 = (double)(1) * dz;
      const double n = F(MCPM_CF_N, num), T = F(MCPM_CF_T, num);
      const int nr = cell_weights ? cell_weights[num] : 1;
      double v[121];
      int k = 0;
      v[k++] = 0.5 * (d0 + d1);
      v[k++] = 0.5 * (d2 + d3);
      v[k++] = d1 - d0;
      v[k++] = d3 - d2;
      v[k++] = d5 - d4;
      v[k++] = t_post;
      v[k++] = cfg->dt;
      for (int q = 0; q < 3; ++q) v[k++] = F(MCPM_CF_U_SPACE + q, num);
      v[k++] = T;
      v[k++] = n;
      v[k++] = S(MCPM_SF_WEIGHT, num);
      for (int q = 0; q < 3; ++q) v[k++] = S(MCPM_SF_M + q, num);
      for (int q = 0; q < 6; ++q) v[k++] = S(MCPM_SF_MM + q, num);
      for (int q = 0; q < 10; ++q) v[k++] = S(MCPM_SF_MMM + q, num);
      for (int q = 0; q < 50; ++q) v[k++] = 0.0;  // face sums of the interface problems
      v[k++] = (d1 - d0) * (d3 - d2) * (d5 - d4);
      v[k++] = F(MCPM_CF_N_SMOOTH, num);
      v[k++] = F(MCPM_CF_NUM_INSIDE, num);  // integer column
      v[k++] = n * cfg->kb * T * (1.0 + n * cfg->b * y_coll(n, cfg->b)) - 2.0 * cfg->b * n * n * cfg->phi;
      v[k++] = nr * cfg->Fn;
      for (int q = 0; q < 6; ++q) v[k++] = S(MCPM_SF_MMMM + q, num);
      v[k++] = 0.0;  // model (integer column)
      v[k++] = 0.0;  // xx
      v[k++] = F(MCPM_CF_PIJ + 3, num);
      v[k++] = F(MCPM_CF_Q + 1, num);
      v[k++] = F(MCPM_CF_F2, num);
      v[k++] = F(MCPM_CF_DIVU, num);
      for (int q = 0; q < 4; ++q) v[k++] = 0.0;  // UU UU0 UUR UU0R
      for (int q = 0; q < 9; ++q) v[k++] = F(MCPM_CF_ALPHA + q, num);
      for (int q = 0; q < 3; ++q) v[k++] = F(MCPM_CF_BETA + q, num);
      v[k++] = F(MCPM_CF_GAMMA_ST, num);
      for (int q = 0; q < 3; ++q) v[k++] = F(MCPM_CF_PHI + q, num);
      v[k++] = p_m ? p_m[num] : 0.0;
      v[k++] = n * cfg->kb * T * (1.0 + n * cfg->b * y_coll(n, cfg->b));
      for (int q = 0; q < 121; ++q) {
        if (q == 84 || q == 93) fprintf(fp, "%20d", (int)v[q]);
        else fprintf(fp, "%20e", v[q]);
      }
      fprintf(fp, "\n");
    }
    fprintf(fp, "\n");
  }
  return fclose(fp) == 0 ? MCPM_OK : MCPM_ERR_ARG;
}

// the summary lines of post_processing (src/myIO.cpp:945-965) into buf;
// returns the characters written (the whole text when it fits) or < 0
extern "C" int mcpm_post_processing_text(const mcpm_config* cfg, const double* cells, char* buf, int32_t len) {
  if (!cfg || !cells || !buf || len <= 0) return -MCPM_ERR_ARG;
  const int N0 = cfg->n_cells[0], N1 = cfg->n_cells[1], C = N0 * N1;
  auto F = [&](int f, int c) { return cells[(size_t)f * C + c]; };
  auto T = [&](int c) { return F(MCPM_CF_T, c); };
  auto nc = [&](int c) { return F(MCPM_CF_N, c); };
  auto Ni = [&](int c) { return (int)F(MCPM_CF_NUM_INSIDE, c); };
  auto D2 = [&](int c) { return F(MCPM_CF_DM2, c); };
  std::string out;
  char line[1024];
  double T_avg = 0.0;
  for (int num = 0; num < C; ++num) T_avg += T(num);
  T_avg = T_avg / C;
  if (N1 > 1) {
    const int a = N1 / 2, b = N1 - 2, e = N1 - 1;
    const double s3 = pow(cfg->sigma, 3);
    snprintf(line, sizeof line, "T   = %e,   %e,   %e.... %e ....  %e   %e\n", T(0), T(1), T(2), T(a), T(b), T(e));
    out += line;
    snprintf(line, sizeof line, "N   = %d,   %d,  %d .... %d ....  %d   %d\n", Ni(0), Ni(1), Ni(2), Ni(a), Ni(b),
             Ni(e));
    out += line;
    snprintf(line, sizeof line, "n*sigma^3 = %e,   %e,   %e.... %e ....  %e   %e\n", nc(0) * s3, nc(1) * s3,
             nc(2) * s3, nc(a) * s3, nc(b) * s3, nc(e) * s3);
    out += line;
    // the fourth and fifth values as the reference prints them: n of cell
    // N[1]-2 with DM2 of cell N[1]-1
    snprintf(line, sizeof line, "p   = %e,   %e .... %e ....  %e   %e\n", cfg->m * nc(0) * D2(0) / 3.0,
             cfg->m * nc(1) * D2(1) / 3.0, cfg->m * nc(a) * D2(a) / 3.0, cfg->m * nc(b) * D2(e) / 3.0,
             cfg->m * nc(b) * D2(e) / 3.0);
    out += line;
    snprintf(line, sizeof line, "T_avg = %e\n", T_avg);
    out += line;
    snprintf(line, sizeof line, "(*gas).Fn=%e\n", cfg->Fn);
    out += line;
  } else {
    snprintf(line, sizeof line, "T   = %e\n", T(0));
    out += line;
    snprintf(line, sizeof line, "N   = %d\n", Ni(0));
    out += line;
    snprintf(line, sizeof line, "p   = %e\n", cfg->m * nc(0) * D2(0) / 3.0);
    out += line;
    snprintf(line, sizeof line, "kinetic energy = %e\n", 0.5 * cfg->m * Ni(0) * D2(0));
    out += line;
  }
  snprintf(buf, (size_t)len, "%s", out.c_str());
  return (int)out.size();
}
