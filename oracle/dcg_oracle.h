/*
 * dcg_oracle.h — CPU oracle of the DCGrid simulation step (TEST INFRASTRUCTURE).
 *
 * This library is the correctness oracle and the timed CPU baseline. It is a
 * restatement, in plain C++, of the reference's adaptive-grid step
 * (src/dcgrid/dcgrid_*.cu and src/dcgrid/fluid_simulation_dcgrid.cu) and uniform-grid step
 * (src/uniformgrid/ sources), plus the extensions (buoyancy, temperature/vapor,
 * sphere sources, wind, terrain, field-driven refinement) that the reference
 * does not have and which this oracle defines.
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark may
 * load it. The product library (libdcgrid_gb300.so) never links or calls it.
 *
 * Field arithmetic runs in `float` (precision 0: mirrors the reference's FP32
 * operations one for one, in the same order, without FMA contraction) or in
 * `double` (precision 1: the FP64 oracle). Topology decisions (scores,
 * selection) always use float, as the reference does.
 */
#ifndef DCG_ORACLE_H
#define DCG_ORACLE_H
#include "../include/dcg.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct dcgo_sim dcgo_sim;

int dcgo_create(const dcg_params *params, int32_t mode, int32_t precision,
                dcgo_sim **out);
int dcgo_destroy(dcgo_sim *s);
int dcgo_reset(dcgo_sim *s);
int dcgo_step(dcgo_sim *s, int32_t n);
int dcgo_advect_velocity(dcgo_sim *s);
int dcgo_adapt(dcgo_sim *s);
int dcgo_project(dcgo_sim *s);
int dcgo_project_local(dcgo_sim *s);
int dcgo_advect_scalars(dcgo_sim *s);
int dcgo_add_velocity_noise(dcgo_sim *s, uint64_t seed, float amplitude);
int dcgo_set_threads(int32_t n);
int dcgo_get_info(const dcgo_sim *s, dcg_info *info);
const char *dcgo_last_error_string(const dcgo_sim *s);

/* fields in the canonical layout of dcg_get_field, as double */
int dcgo_get_field(dcgo_sim *s, int32_t field, double *dst);
int dcgo_set_field(dcgo_sim *s, int32_t field, const double *src);
int dcgo_get_dense(dcgo_sim *s, int32_t field, double *dst);

int dcgo_get_topology(dcgo_sim *s, int32_t *pos, uint32_t *parent,
                      uint32_t *child, uint8_t *flags, int64_t *load,
                      int64_t *move_limit);
/* Replaces the block table, rebuilds the lookup table and recomputes every
 * apron entry by a fresh deep lookup. */
int dcgo_set_topology(dcgo_sim *s, const int32_t *pos, const uint32_t *parent,
                      const uint32_t *child, const int64_t *load,
                      const int64_t *move_limit);
/* Installs a reference-format apron table (216 global cell indices per block,
 * -1 = not found) as-is. */
int dcgo_set_apron(dcgo_sim *s, const int64_t *src);
int dcgo_get_apron(dcgo_sim *s, int64_t *dst);
/* Number of apron entries of allocated blocks that differ between the table the
 * reference's incremental refresh maintains and a fresh deep lookup. */
int64_t dcgo_apron_mismatches(dcgo_sim *s);

int dcgo_get_last_adapt(dcgo_sim *s, int64_t *moves, int64_t *n_moves,
                        int64_t *refines, int64_t *n_refines);
/* Applies given decisions instead of selecting: moves = (block, dest subblock)
 * pairs, refines = (subblock, new block) pairs. */
int dcgo_adapt_replay(dcgo_sim *s, const int64_t *moves, int64_t n_moves,
                      const int64_t *refines, int64_t n_refines);
/* Subblock / block scores of the current state (float, 8*B and B entries). */
int dcgo_get_scores(dcgo_sim *s, float *subblock, float *block);
int dcgo_get_stats(dcgo_sim *s, dcg_stats *st);
int dcgo_set_emission(dcgo_sim *s, const double *src);
/* dcg_set_heightmap: terrain from nx*nz heights (x fastest) instead of the
 * value noise, then a reset; heights == NULL with nx = nz = 0 restores it */
int dcgo_set_heightmap(dcgo_sim *s, const float *heights, int32_t nx, int32_t nz);
/* the renderer's ray march on the CPU: width*height*4 values (RGBA) */
int dcgo_render(dcgo_sim *s, const dcg_render_params *rp, double *rgba);
/* FP64 host adjoint of the density path: transpose of the step that produced
 * the current state (flow and topology fixed); lam_em (emission_n^3) is
 * accumulated and may be NULL. */
int dcgo_adjoint_step(dcgo_sim *s, const double *lam_in, double *lam_out, double *lam_em);
/* FP64 host adjoint of one whole step (velocity and scalars, buoyancy, the
 * transposed pressure cascade, sample positions' dependence on the velocity):
 * the simulation holds the state before the step; the step runs, replaying
 * the given adaptation decisions (dcg_get_last_adapt layout) when moves is not
 * NULL, and lam_out receives the adjoint of the state before it given lam_in,
 * that of the state after it; (3 + n_scalars) planes of 64*max_blocks. */
int dcgo_adjoint_step_full(dcgo_sim *s, const double *lam_in, double *lam_out, double *lam_em,
                           const int64_t *moves, int64_t n_moves, const int64_t *refines, int64_t n_refines);
/* transpose of dcgo_get_dense, accumulated into lam_cells */
int dcgo_adjoint_dense(dcgo_sim *s, const double *lam_dense, double *lam_cells);
/* dst takes src's whole state; both created with the same parameters and
 * precision (checkpoints of the host adjoint). */
int dcgo_copy_state(dcgo_sim *dst, const dcgo_sim *src);

#ifdef __cplusplus
}
#endif
#endif
