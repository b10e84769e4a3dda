/*
 * esf_oracle.h - CPU restatement of EULERSF's coupled solid-fluid step.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker that the CUDA path in
 * eulersf_gb300/ is compared against; it is never linked into, loaded by or
 * called from the product. Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / --impl reference legs of bench.py use it.
 *
 * Pinned against the reference's own build (oracle/_ref, made by
 * oracle/Makefile from the unmodified sources) through the fixtures in
 * tests/golden/ (written by tests/golden/make_golden.py).
 *
 * The API mirrors include/eulersf.h with an esfo_ prefix and host pointers
 * everywhere.
 */
#ifndef ESF_ORACLE_H
#define ESF_ORACLE_H
#include "../include/eulersf.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct esfo_scene esfo_scene;

esfo_scene* esfo_create(const esf_grid* grid, const esf_params* params);
void esfo_destroy(esfo_scene* s);
int esfo_params_default(const esf_grid* grid, esf_params* params);
int esfo_add_solid(esfo_scene* s, const esf_solid_desc* d);
int esfo_set_fluid(esfo_scene* s, double density, double viscosity);
int esfo_init(esfo_scene* s);
int esfo_set_max_dt(esfo_scene* s, double max_dt);
int esfo_step(esfo_scene* s, esf_step_report* report);
double esfo_dt(const esfo_scene* s);
int esfo_field_info(const esfo_scene* s, int field, int solid, size_t* count,
                    size_t* elem_bytes);
int esfo_get_field(esfo_scene* s, int field, int solid, void* host, size_t bytes);
int esfo_set_field(esfo_scene* s, int field, int solid, const void* host, size_t bytes);

/* getMatVecMult with a per-node mass inverse (host arrays). */
int esfo_pressure_apply(const esf_grid* g, const double* mass_inv_node,
                        const double* in, double* out);
/* Matrix-free solvePCR with that operator; x is the warm start. */
int esfo_pressure_solve(const esf_grid* g, const double* mass_inv_node,
                        const double* diag, const double* b, double* x, double eps,
                        int max_iterations, int* iterations, double* rel_residual);
/* First n outputs of MERSENNETWISTER seeded with `seed` (MT19937). */
void esfo_mt19937(uint32_t seed, uint32_t* out, long n);

#ifdef __cplusplus
}
#endif
#endif
