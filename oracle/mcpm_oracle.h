/*
 * mcpm_oracle.h -- CPU restatement of the reference particle step (FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against; nothing in the product links it.  Each function follows one
 * reference routine (file:line given per function in mcpm_oracle.c) with the
 * same operation order, so that, built with -ffp-contract=off, it reproduces
 * the reference bit for bit on identical inputs and injected draws.  It is
 * itself pinned against the reference compiled from its own sources
 * (oracle/ref_harness.cpp, built into oracle/_ref/) and against the golden
 * vectors under tests/golden/.
 *
 * Where the reference draws from std::random_device (binning face jitter,
 * ESMC, diffuse walls) the restatement draws from the same counter-based
 * Philox4x32-10 stream the GPU uses, so GPU and oracle see identical draws.
 */
#ifndef MCPM_ORACLE_H
#define MCPM_ORACLE_H
#include <stdint.h>
#include "../include/mcpm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_state orc_state;

orc_state* orc_create(const mcpm_config* cfg, int64_t n_particles);
void orc_destroy(orc_state* s);
int orc_num_cells(const orc_state* s);
/* cells[].n_ratio: the weight in the cell density n = n_ratio Fn N / V
   (src/Main_Functions.cpp:2588); 1 until set */
void orc_set_cell_weights(orc_state* s, const int32_t* cw);
/* [C][MCPM_CF_COUNT] cell-major copy of the per-cell fields */
void orc_get_cells(const orc_state* s, double* out_cell_major);
void orc_set_cell_field(orc_state* s, int field, const double* values);
int orc_get_step(const orc_state* s);
void orc_set_step(orc_state* s, int step);
/* status bits accumulated (enum mcpm_status); cleared by the call */
int orc_status(orc_state* s);

/* injected raw normals, 3 arrays of N (particle-id order); mode 1 = use them */
void orc_inject_normals(orc_state* s, const double* xi1, const double* xi2,
                        const double* xi3);
void orc_set_rng(orc_state* s, int mode);

/* the routines of the step; arrays are the reference's SoA, length N */
void orc_cell_update(orc_state* s, const double* x1, const double* x2,
                     const double* U1, const double* U2, const double* U3,
                     int32_t* index);
void orc_random_generator(orc_state* s, double* xi1f, double* xi2f,
                          double* xi3f);
void orc_velocity_fp(orc_state* s, double* U1, double* U2, double* U3,
                     const double* xi1f, const double* xi2f,
                     const double* xi3f);
void orc_esmc(orc_state* s, const double* x1, const double* x2, double* U1,
              double* U2, double* U3);
void orc_long_range(orc_state* s, double* U2);
void orc_dfp_extra_streaming(orc_state* s, const double* U1, const double* U2,
                             const double* U3, double* x1, double* x2);
void orc_apply_bc(orc_state* s, int call_no, double* x1, double* x2,
                  double* x1_old, double* x2_old, double* U1, double* U2,
                  double* U3);
void orc_store_old_positions(orc_state* s, const double* x1, const double* x2,
                             double* x1_old, double* x2_old);
void orc_stream(orc_state* s, double* x1, double* x2, const double* U1,
                const double* U2, const double* U3);
void orc_init_omega_max(orc_state* s);
void orc_dsmc_vhs(orc_state* s, double* U1, double* U2, double* U3);
void orc_sample_cells(orc_state* s, const double* U1, const double* U2, const double* U3, double* acc);
void orc_set_layout(orc_state* s, const int32_t* off, const int32_t* list);
/* thermostat (src/Main_Functions.cpp:1674-1869) on the lists of the last
   orc_cell_update */
void orc_thermostat(orc_state* s, double* U1, double* U2, double* U3,
                    double Tc, double Th, double thermc, double thermh);
/* inverted_addremove_particles (src/Main_Functions.cpp:1206-1450) in two
   calls: the flags (1 split, -1 deleted, 2 re-weighted, 0 kept) and the
   counts against the cells of the last orc_cell_update, then the new state
   (n_kept + n_new particles: the kept ones in id order, then the copies)
   and weights; with nothing split or deleted the second call only
   re-weights (w_out = w with the cell weight where flag is 2). */
void orc_addremove_flags(orc_state* s, const int32_t* w, const int32_t* cw,
                         int n_ratio, int8_t* flag, int64_t* n_kept,
                         int64_t* n_new);
void orc_addremove_widths(orc_state* s, const double* U1, const double* U2,
                          const double* U3, const int32_t* w, const int32_t* cw,
                          int n_ratio, const int8_t* flag, double* h);
void orc_addremove_apply(orc_state* s, const double* x1, const double* x2,
                         const double* x1_old, const double* x2_old,
                         const double* U1, const double* U2, const double* U3,
                         const int32_t* w, const int32_t* cw, int n_ratio,
                         const int8_t* flag, double* x1o, double* x2o,
                         double* x1_oldo, double* x2_oldo, double* U1o,
                         double* U2o, double* U3o, int32_t* w_out);
/* measure_pressure (src/Main_Functions.cpp:13-34) into p_m[C] (added to) */
void orc_measure_pressure(orc_state* s, const double* U2, const double* x2,
                          const double* x2_old, double* p_m);
/* one iteration of the main loop body; x_old arrays persist across steps */
void orc_step(orc_state* s, double* x1, double* x2, double* x1_old,
              double* x2_old, double* U1, double* U2, double* U3,
              int32_t* index);

/* building blocks exported for unit tests */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
void orc_normals4(uint64_t seed, uint32_t c0, uint32_t c1, uint32_t c2,
                  uint32_t c3, double z[4]);
void orc_gauss_jordan(double* A /* n*n row-major, destroyed */, double* rhs,
                      int n, double* x);
void orc_gl_table(int npts, double* nodes, double* weights);
void orc_vlasov_face_potential(orc_state* s, double* V /* N1+1 */);
void orc_poisson_faces(orc_state* s, double* x /* N1+1 */);
/* 2-D long range: node potentials ((N0+1)(N1+1), node id j (N0+1) + i) and
   the full dispatch (V may be NULL); nodal densities [C][4] */
void orc_get_node_density(const orc_state* s, double* out);
void orc_vlasov2d_nodes(orc_state* s, double* V);
void orc_sp2d_nodes(orc_state* s, double* V);
void orc_long_range_2d(orc_state* s, const double* x1, const double* x2,
                       double* U1, double* U2, double* V);

#ifdef __cplusplus
}
#endif
#endif
