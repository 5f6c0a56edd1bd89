/*
 * mavi_oracle.h — TEST INFRASTRUCTURE ONLY.
 *
 * CPU FP64 restatement of Mavi.jl's step loop, used by tests/, by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
 * It is never linked into libmavi_cuda.so and nothing on the product path calls
 * it. Each function in mavi_oracle.c cites the reference file:line it follows.
 *
 * Parity status: parity unpinned at the golden-vector level — the reference
 * (Julia) cannot run on these machines and ships no numeric golden vectors for
 * this path. The restatement is pinned by the
 * reference's own self-consistency tests (chunked == all-pairs,
 * threaded == sequential; test/tests_rings/tests_general.jl:16-45) and by
 * closed-form known answers; see tests/test_oracle.py. Parity at the ULP level
 * of Julia's `^` is unpinned.
 *
 * One OracleSys is one Julia `System` (a single replica).
 */
#ifndef MAVI_ORACLE_H
#define MAVI_ORACLE_H

#include <stdint.h>
#include "../include/mavi_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleSys OracleSys;

/* force modes */
#define ORACLE_FORCES_SEQUENTIAL 0   /* calc_forces!(…, ::Sequencial)  src/integration.jl:112-157 */
#define ORACLE_FORCES_THREADED   1   /* calc_forces!(…, ::Threaded)    src/integration.jl:159-194 */
#define ORACLE_FORCES_ALL_PAIRS  2   /* calc_forces!(…, ::Nothing, …)  src/integration.jl:197-224 */

OracleSys* oracle_create(const MaviReplicaParams* p, const double* pos,
                         const double* vel, const double* pol,
                         const int32_t* ring_types, int32_t nthreads,
                         int32_t* status);
void    oracle_destroy(OracleSys* s);
int32_t oracle_set_threads(OracleSys* s, int32_t nthreads);
int32_t oracle_update_chunks(OracleSys* s);
int32_t oracle_chunk_geometry(OracleSys* s, int32_t* rows, int32_t* cols, int32_t* cap);
int32_t oracle_get_chunks(OracleSys* s, int32_t* num_in_chunk, int32_t* chunk_particles);
int32_t oracle_get_neighbors(OracleSys* s, int32_t* counts, int32_t* nbr);
int32_t oracle_calc_forces(OracleSys* s, int32_t mode, int32_t include_walls, double* out);
int64_t oracle_noise_count(OracleSys* s);
int32_t oracle_step(OracleSys* s, int64_t nsteps, int32_t force_mode, const double* noise);
int32_t oracle_get_state(OracleSys* s, double* pos, double* vel, double* pol);
int32_t oracle_set_state(OracleSys* s, const double* pos, const double* vel, const double* pol);
int32_t oracle_energies(OracleSys* s, int32_t pe_mode, double* ke, double* pe);
int32_t oracle_get_time(OracleSys* s, int64_t* num_steps, double* time);
int32_t oracle_set_time(OracleSys* s, int64_t num_steps, double time);
int32_t oracle_get_areas(OracleSys* s, double* areas);
int64_t oracle_count_pairs(OracleSys* s);
int32_t oracle_pair_distribution(OracleSys* s, double r_max, int32_t nbins, uint64_t* counts);
int32_t oracle_rings_neighbors(OracleSys* s, double tol, int32_t type_all, int32_t max_list, int32_t* counts,
                               int32_t* lists);
/* Variable rings ids with sources and sinks, as mavi_rings_sources; the step's
 * noise is num_rings normals then one uniform per random-polarisation box. */
int32_t oracle_rings_sources(OracleSys* s, const int32_t* active_mask, int32_t num_entries,
                             const MaviSourceEntry* entries, const MaviSpawnBox* boxes, const double* spawn_xy,
                             const int32_t* chunk_rc);
int32_t oracle_rings_active(OracleSys* s, int32_t* active_mask, int32_t* uids, int32_t* num_active);
/* Invasion detection, as mavi_rings_invasions_config / mavi_rings_invasions. */
int32_t oracle_rings_invasions_config(OracleSys* s, int32_t enable, int64_t steps_to_update, int32_t num_cols,
                                      int32_t num_rows);
int32_t oracle_rings_invasions(OracleSys* s, MaviInvasion* out, int64_t capacity, int64_t* count,
                               int64_t* last_check);
/* Julia float `div` as used by update_particle_chunk! (src/chunks.jl:129-130). */
double  oracle_julia_div(double x, double y);
/* update_particle_chunk! row/col (1-based, before bounds checks) for a point. */
int32_t oracle_chunk_of(OracleSys* s, double x, double y, int64_t* row, int64_t* col);
int32_t oracle_struct_sizes(int64_t* out);

#ifdef __cplusplus
}
#endif
#endif
