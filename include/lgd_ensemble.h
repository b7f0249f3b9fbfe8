/*
 * lgd_ensemble.h - C ABI for batched ensembles of independent grids.
 *
 * An ensemble of D3Q19 BGK lid-driven cavities of uneven sizes advanced by
 * one persistent kernel launch per time step or per two time steps
 * (temporal blocking), replayed from CUDA graphs.
 * The reference has no ensemble runner; the per-instance semantics are
 * those of one Simulator per grid (parallelization/serialsimulator.h:
 * 76-139) running a D3Q19 cell (collision of
 * src/examples/latticeboltzmann/main.cpp:93-170, pull scheme, bounce-back
 * walls, moving lid beyond y = L-1).
 *
 * Instance layout (download/upload): 19 * L^3 doubles, population-major,
 * f[i * L^3 + (z * L + y) * L + x], directions C, N, E, W, S, T, B, NW, SW,
 * NE, SE, TW, BW, TE, BE, TN, BN, TS, BS (N = +y, E = +x, T = +z).
 *
 * Status codes and lgd_gpu_last_error() are shared with lgd_gpu.h.
 */
#ifndef LGD_ENSEMBLE_H
#define LGD_ENSEMBLE_H

#include <stddef.h>
#include <stdint.h>

#include "lgd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lgd_lbm lgd_lbm;

/* count instances with cube edges edges[j] in [2, 1024] and relaxation rates
 * omegas[j] in (0, 2); lid velocity (lid, 0, 0); precision 4 (FP32) or 8
 * (FP64).  All instances start in equilibrium at rest (f_i = w_i). */
int lgd_lbm_create(int count, const int32_t *edges, const double *omegas, double lid, int precision, lgd_lbm **out);
int lgd_lbm_destroy(lgd_lbm *h);

/* steps time steps of every instance: one persistent launch per step. */
int lgd_lbm_step(lgd_lbm *h, int steps);

/* the same steps with one launch per instance and step (comparison path). */
int lgd_lbm_step_looped(lgd_lbm *h, int steps);

/* Launch shape: tile_rows rows of one z plane per work item, threads per
 * CTA (64..1024, power of two), resident CTAs per SM (clamped to the
 * occupancy limit). */
int lgd_lbm_set_config(lgd_lbm *h, int tile_rows, int threads, int ctas_per_sm);
int lgd_lbm_get_config(lgd_lbm *h, int *tile_rows, int *threads, int *ctas_per_sm);

/* Temporal blocking: depth 1 (one step per launch, the default) or 2 (two
 * steps per launch: each work item is a column of 32 x 8 (shape 0) or
 * 32 x 4 (shape 1) cells of one instance marching z, the first step's
 * populations of the column and a one-cell rim kept in shared memory;
 * results identical to single steps), and the resident CTAs per SM of the
 * two-step kernel (clamped to what fits).  An odd step count ends with one
 * single step.  Plays the role of the pipeline length of the reference's
 * CacheBlockingSimulator (parallelization/cacheblockingsimulator.h:36-56). */
int lgd_lbm_set_time_block(lgd_lbm *h, int depth, int shape, int ctas_per_sm);
int lgd_lbm_get_time_block(lgd_lbm *h, int *depth, int *shape, int *ctas_per_sm);

/* Pattern search over the launch shape of single steps, timing trial_steps
 * steps per candidate with CUDA events, then over the two-step kernel's
 * tile shape and residency; leaves the fastest per step set (read it back
 * with lgd_lbm_get_config and lgd_lbm_get_time_block).  The trial steps
 * advance the ensemble: reset or upload afterwards.  (Precedent: the
 * reference's AutoTuningSimulator with PatternOptimizer,
 * parallelization/autotuningsimulator.h:60-145, misc/patternoptimizer.h:13,
 * which tunes the cache-blocking simulator's pipeline length beside its
 * wavefront, misc/cacheblockingsimulationfactory.h:26-28.) */
int lgd_lbm_tune(lgd_lbm *h, int trial_steps, int *tile_rows, int *threads, int *ctas_per_sm, double *best_ms);

/* Every instance back to equilibrium at rest. */
int lgd_lbm_reset(lgd_lbm *h);

int lgd_lbm_download(lgd_lbm *h, int instance, double *f, size_t bytes);
int lgd_lbm_upload(lgd_lbm *h, int instance, const double *f, size_t bytes);
int lgd_lbm_info(lgd_lbm *h, long long *total_cells, int *work_items);
int lgd_lbm_synchronize(lgd_lbm *h);
int lgd_lbm_stream(lgd_lbm *h, void **stream);
int lgd_lbm_launch_count(lgd_lbm *h, uint64_t *count);

/* Memory path of the kernel (identical results): 0 (default) plain loads
 * and stores; 1 populations read through the read-only data path, results
 * written with evict-first stores. */
int lgd_lbm_set_variant(lgd_lbm *h, int variant);

#ifdef __cplusplus
}
#endif

#endif
