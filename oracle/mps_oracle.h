/*
 * mps_oracle.h - C API of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * The oracle is a plain C++ restatement of OpenMps's time step
 * (src/OpenMps/Computer.hpp, Grid.hpp, Environment.hpp, Particle.hpp) used to
 * check the CUDA path.  Only the tests, the smoke check and the CPU-baseline
 * legs of bench.py load it; the product library never links or calls it.
 *
 * Entry points mirror include/mps.h with an `oracle_` prefix.
 */
#ifndef OPENMPS_GB300_ORACLE_H
#define OPENMPS_GB300_ORACLE_H

#include "../include/mps.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_handle oracle_handle;

int oracle_create(const mps_params* prm, oracle_handle** out);
void oracle_destroy(oracle_handle* h);
const char* oracle_last_error(const oracle_handle* h);
int oracle_num_threads(void);

int oracle_add_particles(oracle_handle* h, int64_t n, const int32_t* type, const double* x,
                         const double* z, const double* u, const double* w, const double* p,
                         const double* nd);
int64_t oracle_particle_count(const oracle_handle* h);
int oracle_get_particles(const oracle_handle* h, int32_t* type, double* x, double* z, double* u,
                         double* w, double* p, double* nd);
int oracle_set_particles(oracle_handle* h, const int32_t* type, const double* x, const double* z,
                         const double* u, const double* w, const double* p, const double* nd);
int oracle_set_wall_positions(oracle_handle* h, const double* wx, const double* wz);
int oracle_set_solver(oracle_handle* h, int32_t criterion, double eps, int32_t max_iters);

int oracle_forward_time(oracle_handle* h, double dt);
int oracle_get_environment(const oracle_handle* h, mps_environment* env);
int oracle_get_stats(const oracle_handle* h, int32_t* cg_iterations, double* rr0, double* rr,
                     int64_t* ppe_nnz, int64_t* neighbor_total);

int oracle_stage_begin_step(oracle_handle* h, double dt);
int oracle_stage_search_neighbor(oracle_handle* h);
int oracle_stage_density(oracle_handle* h);
int oracle_stage_error_correction(oracle_handle* h);
int oracle_stage_explicit(oracle_handle* h);
int oracle_stage_save_x(oracle_handle* h);
int oracle_stage_set_ppe(oracle_handle* h);
int oracle_stage_solve_ppe(oracle_handle* h);
int oracle_stage_assign_pressure(oracle_handle* h);
int oracle_stage_pressure_gradient(oracle_handle* h);
int oracle_stage_dynamic_stabilize(oracle_handle* h);
int oracle_stage_density_variation(oracle_handle* h, double* speed);
double oracle_determine_dt(oracle_handle* h);

int oracle_get_neighbors(const oracle_handle* h, int32_t* counts, int32_t* list, int64_t capacity,
                         int64_t* total);
int oracle_get_ppe(const oracle_handle* h, int64_t* row_ptr, int32_t* col, double* val, double* b,
                   double* x, int64_t capacity, int64_t* nnz);
int oracle_set_ppe_x(oracle_handle* h, const double* x);
int oracle_get_aux(const oracle_handle* h, double* n_without_spp, double* ecs, double* ox,
                   double* oz);
int oracle_set_aux(oracle_handle* h, const double* n_without_spp, const double* ecs,
                   const double* ox, const double* oz);

/* Detail::InvertMatrix<2> (Computer.hpp:323-347): m and out row-major {00, 01, 10, 11}. */
void oracle_gc_invert(const double* m, double val, double* out);

/* Reference CG (Computer.hpp:1359-1429) on a caller CSR system; x: guess in, solution out. */
int oracle_cg_solve_csr(int64_t n, const int64_t* row_ptr, const int32_t* col, const double* val,
                        const double* b, double* x, double eps, int32_t criterion,
                        int32_t max_iters, int32_t* iterations, double* rr0, double* rr);

/* ------------------------------------------------------------------------
 * Three-dimensional oracle (mps_oracle3.cpp): the DIM3 build of the reference.
 * Stages of oracle3_stage: 0 begin step (dt <= 0: DetermineDt), 1 search, 2 density,
 * 3 error correction, 4 explicit forces, 5 SaveX, 6 PPE assembly, 7 PPE solve,
 * 8 pressure (from the PPE or explicit), 9 pressure gradient, 10 dynamic stabilisation.
 * ---------------------------------------------------------------------- */
typedef struct oracle3_handle oracle3_handle;
int oracle3_create(const mps_params* prm, oracle3_handle** out);
void oracle3_destroy(oracle3_handle* h);
const char* oracle3_last_error(const oracle3_handle* h);
int oracle3_add_particles(oracle3_handle* h, int64_t n, const int32_t* type, const double* x, const double* y,
                          const double* z, const double* u, const double* v, const double* w, const double* p,
                          const double* nd);
int64_t oracle3_particle_count(const oracle3_handle* h);
int oracle3_get_particles(const oracle3_handle* h, int32_t* type, double* x, double* y, double* z, double* u,
                          double* v, double* w, double* p, double* nd);
int oracle3_set_particles(oracle3_handle* h, const int32_t* type, const double* x, const double* y,
                          const double* z, const double* u, const double* v, const double* w, const double* p,
                          const double* nd);
int oracle3_set_wall_positions(oracle3_handle* h, const double* wx, const double* wy, const double* wz);
int oracle3_forward_time(oracle3_handle* h, double dt);
int oracle3_get_environment(const oracle3_handle* h, mps_environment* env);
int oracle3_stage(oracle3_handle* h, int32_t stage, double dt);
int oracle3_density_variation(oracle3_handle* h, double* speed);
int oracle3_get_neighbors(const oracle3_handle* h, int32_t* counts, int32_t* list, int64_t capacity,
                          int64_t* total);
int oracle3_get_ppe(const oracle3_handle* h, int64_t* row_ptr, int32_t* col, double* val, double* b, double* x,
                    int64_t capacity, int64_t* nnz);
int oracle3_get_aux(const oracle3_handle* h, double* n_without_spp, double* ecs, double* ox, double* oy, double* oz);
int oracle3_set_aux(oracle3_handle* h, const double* n_without_spp, const double* ecs, const double* ox,
                    const double* oy, const double* oz);
int oracle3_get_stats(const oracle3_handle* h, int32_t* cg_iterations);
/* Detail::InvertMatrix<3> (Computer.hpp:364-422): m and out row-major. */
void oracle3_gc_invert(const double* m, double val, double* out);

#ifdef __cplusplus
}
#endif

#endif
