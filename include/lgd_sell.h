/*
 * lgd_sell.h - C ABI for unstructured grids stored as SELL-C-sigma.
 *
 * Builder (host): lays out a sparse adjacency matrix exactly as the
 * reference's ReorderingUnstructuredGrid + SellCSigmaSparseMatrixContainer
 * do, so the arrays can be compared byte for byte or handed over.
 * Device (one handle): the diffusion cell x' = 0.1 x + W x on the
 * physical (sigma-sorted) order, double-buffered.
 *
 * Status codes and lgd_gpu_last_error() are shared with lgd_gpu.h.
 */
#ifndef LGD_SELL_H
#define LGD_SELL_H

#include <stddef.h>
#include <stdint.h>

#include "lgd_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Row order and chunk geometry.  Input: CSR row_ptr[n+1] of the logical
 * matrix.  Output: perm[n] (physical row p holds logical row perm[p]),
 * row_length[rows_padded], chunk_length[n_chunks], chunk_offset[n_chunks+1]
 * with n_chunks = (n-1)/C + 1, rows_padded = n_chunks*C, and *total value
 * slots.  Replaces the sigma-window sort of ReorderingUnstructuredGrid::
 * setWeights (storage/reorderingunstructuredgrid.h:195-252) and the
 * chunk-length/offset pass of InitFromMatrix
 * (storage/sellcsigmasparsematrixcontainer.h:82-127). */
int lgd_sell_plan(int n, const int64_t *row_ptr, int C, int sigma, int32_t *perm, int32_t *row_length,
                  int32_t *chunk_length, int32_t *chunk_offset, int64_t *total);

/* Values and columns (total slots each).  remap_columns = 1: column ids
 * become physical ids (the grid path, storage/reorderingunstructuredgrid.
 * h:254-283); 0: logical ids kept (the bare container).  Replaces
 * InitFromMatrix's value placement (storage/sellcsigmasparsematrixcontainer.
 * h:129-160). */
int lgd_sell_fill(int n, const int64_t *row_ptr, const int32_t *col, const double *w, int C, const int32_t *perm,
                  const int32_t *chunk_offset, int64_t total, int remap_columns, double *values, int32_t *column);

typedef struct lgd_sell lgd_sell;

/* flags */
#define LGD_SELL_EXACT 1   /* separate multiply and add (bit-identical to the
                              reference build); default fuses them (FMA) */
#define LGD_SELL_RENUMBER 2 /* lgd_sell_create_from_csr (host input): number
                              the nodes in reverse Cuthill-McKee order before
                              the build, so that rows near each other read
                              columns near each other; logical order at the
                              boundary stays the caller's (the permutation
                              composes both numberings).  The container
                              orders a row's entries by physical column, as
                              the reference's does, so the renumbered grid
                              adds each row's terms in another order: its
                              values agree with the plain grid's to
                              rounding, not bit for bit, and its arrays
                              differ from the reference's container. */

/* Reverse Cuthill-McKee order of a graph (CSR row_ptr[n+1], col
 * [row_ptr[n]], edges taken in both directions): order[k] = the node that
 * gets number k.  Each connected part starts from a node of least degree;
 * neighbours join the breadth-first sweep by increasing degree.  Host code,
 * no GPU needed. */
int lgd_graph_rcm(int n, const int64_t *row_ptr, const int32_t *col, int32_t *order);

/* Uploads the SELL arrays (chunk_offset[n_chunks+1], row_length
 * [rows_padded], values/column[total] with physical column ids) and
 * allocates the double-buffered node vector.  precision: 8 = FP64, 4 = FP32
 * (values and node values rounded to float).  perm (may be NULL) enables
 * logical-order uploads/downloads.  Replaces the device side of an
 * UnstructuredSoAGrid with its SellCSigmaSparseMatrixContainer
 * (storage/unstructuredsoagrid.h:35-101). */
int lgd_sell_create(int n, int C, int64_t total, const int32_t *chunk_offset, const int32_t *row_length,
                    const double *values, const int32_t *column, const int32_t *perm, int precision, int flags,
                    lgd_sell **out);
int lgd_sell_destroy(lgd_sell *h);

/* Builds the SELL-C-sigma matrix on the GPU from a CSR matrix (row_ptr[n+1],
 * col and w [row_ptr[n]]) and returns a ready handle: the arrays of
 * lgd_sell_plan + lgd_sell_fill with remap_columns = 1, byte for byte, and
 * the permutation kept for logical-order copies.  device_input = 0: the CSR
 * arrays are host memory (copied in); 1: device memory.  Device-path limits:
 * sigma <= LGD_SELL_GPU_MAX_SIGMA and at most LGD_SELL_GPU_MAX_ROW entries per
 * row (LGD_ERR_UNSUPPORTED beyond; the host builder has no limit).  Replaces
 * ReorderingUnstructuredGrid::setWeights with InitFromMatrix
 * (storage/reorderingunstructuredgrid.h:195-284,
 * storage/sellcsigmasparsematrixcontainer.h:82-161), which the reference runs
 * on one host thread. */
#define LGD_SELL_GPU_MAX_SIGMA 4096
#define LGD_SELL_GPU_MAX_ROW 1024
int lgd_sell_create_from_csr(int n, const int64_t *row_ptr, const int32_t *col, const double *w, int C, int sigma,
                             int device_input, int precision, int flags, lgd_sell **out);

/* Copies a handle's matrix back to host arrays (each pointer may be NULL):
 * chunk_offset[n_chunks+1], row_length[rows_padded], values[total] (as FP64),
 * column[total], perm[n] (only if the handle has one); *total gets the slot
 * count.  For checking and for writers that save the matrix. */
int lgd_sell_get_layout(lgd_sell *h, int32_t *chunk_offset, int32_t *row_length, double *values, int32_t *column,
                        int32_t *perm, int64_t *total);

/* Node values (n doubles), current (which = 0) or next (1) buffer;
 * logical = 1 maps through perm (GridBase::get/set on a reordering grid,
 * storage/reorderingunstructuredgrid.h:300-340), 0 uses physical order. */
int lgd_sell_upload_x(lgd_sell *h, int which, int logical, const double *x, size_t bytes);
int lgd_sell_download_x(lgd_sell *h, int which, int logical, double *x, size_t bytes);

/* count time steps x <- 0.1 x + W x, swapping after each.  Replaces
 * UnstructuredUpdateFunctor (storage/unstructuredupdatefunctor.h:121-229)
 * driving the cell's updateLineX over the whole node set. */
int lgd_sell_step(lgd_sell *h, int count);

/* Updates physical rows [row_begin, row_end) into the next buffer, no swap
 * (a one-streak region, including streaks that start or end inside a chunk:
 * the reference peels those with unstructuredLoopPeeler,
 * storage/unstructuredlooppeeler.h:75-126). */
int lgd_sell_update_rows(lgd_sell *h, int row_begin, int row_end);
int lgd_sell_swap(lgd_sell *h);

/* Device address of node-value buffer which (0 current, 1 next): rows_padded
 * values of the handle's precision in physical order (rows_padded = chunks
 * x C; the padding rows hold 0).  For a row-block decomposition over ranks
 * (each rank updates its chunks with lgd_sell_update_rows, the ranks gather
 * every block of the next buffer, then lgd_sell_swap): what the reference's
 * HiParSimulator would do with an unstructured grid's patch links
 * (parallelization/hiparsimulator.h, communication/patchlink.h).  Work on the
 * buffers must be ordered with the handle's stream. */
int lgd_sell_x_device(lgd_sell *h, int which, void **ptr, int64_t *rows_padded);
int lgd_sell_synchronize(lgd_sell *h);
int lgd_sell_stream(lgd_sell *h, void **stream);
int lgd_sell_launch_count(lgd_sell *h, uint64_t *count);

/* Kernel variant (all give identical results): 0 = default, software
 * pipelined four slots deep (matrix entries of the next slots load while
 * the x gathers of the current ones are in flight), CTAs of 128 threads;
 * 1 = two slots per iteration, no pipelining, 256 threads; 2 = pipelined
 * two slots deep, 256 threads; 3 = four deep, 64 threads; 4 = four deep,
 * 256 threads; 5 = eight deep, 64 threads. */
int lgd_sell_set_variant(lgd_sell *h, int variant);

#ifdef __cplusplus
}
#endif

#endif
