/*
 * lgd_gpu.h - C ABI of the GB300 (sm_103a) cell-update library.
 *
 * This is the drop-in boundary for LibGeoDecomp's CUDASimulator<CELL> hot
 * path: plain C types, pointers and sizes only.  Every entry point returns
 * an int status (LGD_OK = 0); on failure lgd_gpu_last_error() gives the
 * message.  No C++ exception crosses this boundary; the C++ host layer
 * (libgeodecomp_gb300/include/libgeodecomp_gb300/gb300simulator.h) turns
 * non-zero codes back into the exceptions the reference throws.
 *
 * Threading: one host thread per handle (the reference's CUDASimulator has
 * no locking either).  All work of a handle runs on that handle's CUDA
 * stream; calls that return data to the host synchronise that stream.
 *
 * Grid layout in host buffers: dense, x-fastest, idx = (z*ny + y)*nx + x,
 * one array per cell member (structure of arrays, the layout libflatarray
 * gives SoA cells, lib/libflatarray/include/libflatarray/detail/macros.hpp:
 * 99-106, minus its size buckets and padding).
 */
#ifndef LGD_GPU_H
#define LGD_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes
 * Reference counterparts: LGD_ERR_INVALID ~ std::invalid_argument /
 * std::logic_error (storage/ headers), LGD_ERR_RANGE ~ std::out_of_range thrown by
 * the size-bucket dispatch (lib/libflatarray/include/libflatarray/macros.hpp:
 * 948-1060), LGD_ERR_CUDA ~ std::runtime_error("CUDA error") from
 * CUDAUtil::checkForError (misc/cudautil.h:48-55). */
#define LGD_OK 0
#define LGD_ERR_INVALID 1
#define LGD_ERR_RANGE 2
#define LGD_ERR_CUDA 3
#define LGD_ERR_NOMEM 4
#define LGD_ERR_TIMEOUT 5
#define LGD_ERR_UNSUPPORTED 6

/* Copies the last error message of the calling thread into buf (always
 * NUL-terminated when len > 0); returns the last status code. */
int lgd_gpu_last_error(char *buf, size_t len);

/* Library version as 10000*major + 100*minor + patch. */
int lgd_gpu_version(void);

/* Number of CUDA devices visible (0 on a machine without a GPU). */
int lgd_gpu_device_count(int *count);

/* ------------------------------------------------------ structured grids
 * Cell kinds compiled into the library.  Each one is the device-side
 * restatement of a Cell class's update()/updateLineX(); the member list is
 * the cell's SoA registration in declaration order.
 *   LGD_CELL_JACOBI7_F64   members {double temp}; von Neumann r=1, 3D;
 *                          temp' = (c+n+s+e+w+t+b) * (1/7) (IEEE FP64,
 *                          bit-identical to the reference's SerialSimulator)
 *   LGD_CELL_JACOBI7_F64_FIX same cell with FP64 values at the ABI; on the
 *                          device the grid is held in 64-bit fixed point,
 *                          value = k * 2^(e - 57), 2^e the smallest power of
 *                          two above the grid's largest |value| and the edge
 *                          cell.  The neighbour sum is exact and is
 *                          multiplied by the same double fl(1/7) as the
 *                          cell's, rounding to the nearest unit, so each step
 *                          adds at most 2^(e - 58) absolute error and nothing
 *                          drifts against the IEEE cell; a temporally blocked
 *                          pass of two steps sums both exactly and rounds
 *                          once (within one unit of two single steps).  e is
 *                          raised when an upload needs it and lowered (an
 *                          exact shift) when the grid's values have shrunk,
 *                          checked after an upload whose maximum lies below
 *                          e's range and every 256 steps, so a
 *                          decaying grid keeps 57 significant bits at its
 *                          maximum; such a check waits for the device.  For
 *                          GPUs whose FP64 pipe, not memory, would bound the
 *                          IEEE kernel.
 *   LGD_CELL_JACOBI7_F32   members {float temp}; same stencil in FP32
 *   LGD_CELL_SUM6_F64      members {double valA, double valB}; valB' = the
 *                          six face neighbours' valA summed in the order
 *                          (0,0,-1) (0,-1,0) (-1,0,0) (1,0,0) (0,1,0) (0,0,1)
 *                          (storage/test/unit/fixedneighborhoodupdatefunctortest.h:
 *                          30-46); valA' = valA
 *   LGD_CELL_GOL_U8        members {uint8 alive}; Moore r=1, 2D; Conway's rule
 *                          (src/examples/gameoflife/main.cpp:35-58)
 *   LGD_CELL_VARCOEF_F32 / _F64  members {u, k}; von Neumann r=1, 3D;
 *                          u' = u + sum_faces 0.5 (k + k_nb)(u_nb - u), faces
 *                          -x,+x,-y,+y,-z,+z; k' = k
 *   LGD_CELL_TEST          one member, a 64-byte lgd_test_record; 1D, 2D or
 *                          3D; the reference's self-validating TestCell
 *                          (misc/testcell.h:205-372): every update checks
 *                          each stencil neighbour as delivered (position
 *                          wrapped by the topology, dimensions, cycle
 *                          counter, edge-cell flag) and the nano step
 *                          (== cycle % nano steps), then counts the cycle;
 *                          any failed check clears `valid`.  desc.flags:
 *                          LGD_TEST_VON_NEUMANN (else Moore r=1) |
 *                          LGD_TEST_NANO_STEPS(n) (n in 1..255); edge[0] =
 *                          the edge cell's valid flag + 2 * its edge flag.
 *                          lgd_gpu_step's k-th update runs nano step
 *                          (nano_step + k) % n.  For conformance tests of
 *                          the simulator, not for speed.
 */
#define LGD_CELL_JACOBI7_F64 1
#define LGD_CELL_JACOBI7_F64_FIX 2
#define LGD_CELL_JACOBI7_F32 3
#define LGD_CELL_SUM6_F64 4
#define LGD_CELL_GOL_U8 5
#define LGD_CELL_VARCOEF_F32 6
#define LGD_CELL_VARCOEF_F64 7
#define LGD_CELL_TEST 8
/* A user's own cell class, one record of record_bytes per cell (array of
 * structures, the reference CUDASimulator's device grid of CELL objects,
 * parallelization/cudasimulator.h:314-429).  The library stores, copies and
 * snapshots the records; the cell's own update() / updateCUDA() runs in a
 * kernel compiled from the cell's source in the caller's translation unit
 * (libgeodecomp_gb300/include/libgeodecomp_gb300/gb300cell.cuh) on the
 * handle's stream.  Created by lgd_gpu_create_records; lgd_gpu_step,
 * region updates, fills, checksums and BOV output are not defined for it. */
#define LGD_CELL_RECORD 9
#define LGD_RECORD_MAX_BYTES 4096

#define LGD_TEST_VON_NEUMANN 1
#define LGD_TEST_NANO_STEPS(n) ((n) << 8)

typedef struct lgd_test_record {
    int32_t pos[3];         /* the cell's own idea of its position (unused axes 0) */
    int32_t dim[3];         /* grid dimensions (unused axes 1) */
    uint32_t cycle;         /* cycleCounter */
    uint8_t edge;           /* isEdgeCell */
    uint8_t valid;          /* isValid */
    uint8_t pad0, pad1;
    float test_value;       /* testValue, carried along */
    int32_t pad[7];
} lgd_test_record;

/* periodic bit d set: axis d (0 = x, 1 = y, 2 = z) wraps (Topologies::Torus);
 * clear: cells outside read the constant edge cell (Topologies::Cube with
 * SoAGrid's edge cell, storage/soagrid.h:578-585, geometry/topologies.h:
 * 263-278). */
typedef struct lgd_grid_desc {
    int dim;            /* 1, 2 or 3 (as the cell kind allows) */
    int nx, ny, nz;     /* cells per axis; nz = 1 for 2D, ny = nz = 1 for 1D */
    int periodic;       /* bit mask, see above */
    int cell;           /* LGD_CELL_* */
    int flags;          /* LGD_CELL_TEST: stencil and nano steps; else 0 */
    double edge[4];     /* edge cell, one value per member */
} lgd_grid_desc;

typedef struct lgd_handle lgd_handle;

/* Allocates the double-buffered device grid.  Replaces the device part of
 * CUDASimulator's constructor (parallelization/cudasimulator.h:314-429:
 * cudaMalloc of the old/new grids, offsets, wrap setup).  Sizes up to
 * 2^31-1 cells per axis; the reference's SoA size buckets stop at 1032
 * per 3D axis (lib/libflatarray/include/libflatarray/api_traits.hpp:120-123)
 * and this library has no such limit. */
int lgd_gpu_create(const lgd_grid_desc *desc, lgd_handle **out);
int lgd_gpu_destroy(lgd_handle *h);

/* A grid of a user's cell records (LGD_CELL_RECORD): desc->cell must be
 * LGD_CELL_RECORD, desc->flags 0 and desc->edge is unused; record_bytes
 * (1 .. LGD_RECORD_MAX_BYTES) is sizeof(CELL) and edge_record the edge cell
 * (Topologies::Cube reads it outside the grid).  Rows of records are pitched
 * to 128 bytes: record (x, y, z) starts at ptr + (z*ny + y) * pitch +
 * x * record_bytes.  Replaces the device allocation of CUDASimulator's
 * constructor for cells without a kernel of their own in this library. */
int lgd_gpu_create_records(const lgd_grid_desc *desc, size_t record_bytes, const void *edge_record,
                           lgd_handle **out);

/* The edge record of a record grid: set_edge_record replaces it (the host
 * grid's setEdge, storage/gridbase.h), edge_record_device gives its device
 * copy for kernels. */
int lgd_gpu_set_edge_record(lgd_handle *h, const void *edge_record, size_t bytes);
int lgd_gpu_edge_record_device(lgd_handle *h, const void **device_edge);

/* The grid's descriptor as created (cell kind, dimensions, periodic axes,
 * flags, edge values), for code that steps a handle it did not create. */
int lgd_gpu_get_desc(lgd_handle *h, lgd_grid_desc *out);

/* Counts kernel launches made on the handle's stream by code outside the
 * library (the record kernels of gb300cell.cuh), for lgd_gpu_launch_count. */
int lgd_gpu_count_launches(lgd_handle *h, uint64_t n);

/* Host <-> device copy of one member of one buffer (which: 0 = current
 * grid, 1 = next grid); bytes must equal nx*ny*nz*sizeof(member).  Replaces
 * the H2D copies of CUDASimulator::run (parallelization/cudasimulator.h:
 * 515-516) and the D2H copy of getGrid (:490-497).  Downloads synchronise. */
int lgd_gpu_upload(lgd_handle *h, int member, int which, const void *host, size_t bytes);
int lgd_gpu_download(lgd_handle *h, int member, int which, void *host, size_t bytes);

/* The same copies from / to dense DEVICE memory of another owner (device
 * pipelines: the surrogate, frameworks holding their own buffers);
 * synchronise the handle's stream.  Not for LGD_CELL_JACOBI7_F64_FIX. */
int lgd_gpu_upload_device(lgd_handle *h, int member, int which, const void *dev, size_t bytes);
int lgd_gpu_download_device(lgd_handle *h, int member, int which, void *dev, size_t bytes);

/* Streak-wise copies for plugins that need part of the grid (reference:
 * GridBase::saveRegion / loadRegion, storage/gridbase.h; the libflatarray
 * streak functors save_functor.hpp / load_functor.hpp).  streaks holds
 * n_streaks * 4 ints (x, y, z, endX); the buffer packs the streaks' cells in
 * order. */
int lgd_gpu_save_region(lgd_handle *h, int member, const int *streaks, int n_streaks, void *host, size_t bytes);
int lgd_gpu_load_region(lgd_handle *h, int member, const int *streaks, int n_streaks, const void *host, size_t bytes);

/* Advances the whole grid count time steps (current -> next, then swap),
 * starting at nano step nano_step.  Replaces CUDASimulator::step's nanoStep
 * loop with its pointer swap (parallelization/cudasimulator.h:467-470) and
 * the kernel2D/kernel3D launch (:566-590).  Asynchronous on the handle's
 * stream. */
int lgd_gpu_step(lgd_handle *h, unsigned nano_step, int count);

/* Updates only the cells of the streaks (n_streaks * 4 ints: x, y, z,
 * endX) from the current grid into the next grid; no swap.  Replaces
 * UpdateFunctor<CELL>()(region, ..., gridOld, &gridNew, nanoStep)
 * (storage/updatefunctor.h:403-428). */
int lgd_gpu_update_region(lgd_handle *h, const int *streaks, int n_streaks, unsigned nano_step);

/* Swaps current and next (the simulator's std::swap of grid pointers,
 * parallelization/serialsimulator.h:137-138). */
int lgd_gpu_swap(lgd_handle *h);

/* Fills one member of one buffer with the library's seeded uniform [0,1)
 * doubles (SplitMix64, value i = top 53 bits of mix(key + (i+1)*GAMMA),
 * key = mix(seed*256 + stream)); FP32 members get the double rounded.
 * Test and benchmark helper: lets large grids be initialised on device. */
int lgd_gpu_fill_uniform(lgd_handle *h, int member, int which, uint64_t seed, int stream);

/* Bernoulli(p) 0/1 fill of a uint8 member from the same stream
 * (value i = 1 if uniform_i < p). */
int lgd_gpu_fill_bernoulli(lgd_handle *h, int member, int which, uint64_t seed, int stream, double p);

/* Fixed-point exponent e of an LGD_CELL_JACOBI7_F64_FIX grid. */
int lgd_gpu_fixed_point_exponent(lgd_handle *h, int *exp);

/* Sets the exponent of a fixed-point grid to e (>= the edge cell's bound):
 * both buffers are rescaled, exactly when e falls (a shift left; values
 * that would not fit return LGD_ERR_RANGE and leave the grid unchanged),
 * rounded to nearest when it rises.  pin != 0 keeps e from now on: the
 * checks after an upload and every 256 steps no longer lower it (an upload
 * whose values need more still raises it).  For grids that exchange raw
 * planes (a z-slab decomposition, lgd_gpu_copy_planes), which need one
 * exponent on every rank. */
int lgd_gpu_set_fixed_point_exponent(lgd_handle *h, int e, int pin);

/* Raw planes of the slowest axis (z for 3D grids, y for 2D, the whole row
 * for 1D) in the device representation, row padding included: planes
 * p0 .. p0 + np - 1 of one member of one buffer to or from buf, which may be
 * host or device memory (bytes = np * plane_bytes, plane_bytes from
 * lgd_gpu_plane_bytes).  The ghost-zone exchange of a slab decomposition
 * (the reference's patch links of HiParSimulator,
 * parallelization/hiparsimulator.h:60-72, communication/patchlink.h).
 * Synchronises the handle's stream. */
int lgd_gpu_plane_bytes(lgd_handle *h, int member, size_t *bytes);
int lgd_gpu_copy_planes(lgd_handle *h, int member, int which, int p0, int np, void *buf, size_t bytes, int to_grid);

/* Kernel variant for the Jacobi cells (results are identical): 0 (default)
 * TMA-staged shared-memory planes on cube grids with a zero edge cell,
 * otherwise variant 5; 1 shared-memory plane tiles loaded by the threads;
 * 2 one cell per lane in registers; 3 / 4 / 5 two cells per lane, 8 / 2 / 4
 * rows per warp, marching in z with register rotation and warp shuffles.
 * Var-coef cells: 0 (default) for FP32 TMA-staged planes of u and k, wrapped
 * neighbours copied into their own areas (3D grids whose non-wrapping axes
 * have zero edge values and, when x wraps, rows of a multiple of 16 bytes),
 * otherwise (and for FP64) variant 2; 1 shared-memory plane tiles; 2 .. 5
 * two cells per lane in registers.  6: the TMA kernel wherever it applies
 * (either cell family), else the default.  For tuning and comparison. */
int lgd_gpu_set_variant(lgd_handle *h, int variant);

/* The handle's CUDA stream (a cudaStream_t), for callers that time or
 * order their own work against the library's. */
int lgd_gpu_stream(lgd_handle *h, void **stream);

/* ------------------------------------------------- allocation-free sum
 * No counterpart in the reference.  Sum of n FP64 values in device memory,
 * written to *d_result (device memory), asynchronously on stream (a
 * cudaStream_t, NULL = the default stream) - the same sum as
 * lgd_gpu_checksum, added in a different order (blocks of 65536 values and
 * a tree on the device), so not bit-identical to it - for callers that must
 * not allocate device memory: a
 * plugin or solver running inside another framework's stream and memory
 * pool, where cudaMalloc/cudaFree would synchronise the device and
 * fragment the pool, or code with a fixed memory budget.  It calls no
 * allocating routine: its block partials live in a fixed 128 KiB device
 * array that every GPU loading the library keeps until the process exits.
 * Hence n <= LGD_SUM_STATIC_MAX_N (larger n returns LGD_ERR_RANGE), and
 * calls that overlap on the GPU (unordered streams) race on that array.
 * The first call on a device looks the array's address up (no
 * allocation); make that first call before any stream capture.  The lookup
 * is repeated when the device's context changes (after a cudaDeviceReset). */
#define LGD_SUM_STATIC_CHUNK 65536
#define LGD_SUM_STATIC_MAX_PARTIALS 16384
#define LGD_SUM_STATIC_MAX_N (1LL << 30)
int lgd_sum_f64_static(const double *d_values, long long n, double *d_result, void *stream);

/* Writes one member of the current grid as a BOV snapshot, straight from
 * the device: header prefix.<step, 5 digits>.bov and raw little-endian
 * data prefix.<step>.data, x fastest, in the format of the reference's
 * SerialBOVWriter (io/serialbovwriter.h, io/bovoutput.h:17-58): DATA_FORMAT
 * DOUBLE, FLOAT or BYTE by the member's type, 2D grids as nz = 1, one
 * brick, one component, VARIABLE the given name.  Fixed-point grids write
 * their FP64 values.  Synchronises the handle's stream. */
int lgd_gpu_write_bov(lgd_handle *h, int member, const char *prefix, unsigned step, const char *variable);

/* Checkpoint snapshots in the file layout of the reference's MPIIOWriter /
 * MPIIOInitializer (io/mpiio.h:85-125 writeRegion, :180-200 offsets;
 * io/mpiiowriter.h, io/mpiioinitializer.h), written and read by one process
 * without MPI: the dimensions as DIM 32-bit ints (x, y[, z]), the step and
 * the maximum step count as 32-bit unsigned, the edge cell, then the cells
 * x fastest.  A cell record is the grid's members in order in their host
 * types, as the reference's sizeof(CELL) record for cells without padding;
 * fixed-point grids hold FP64 values.
 *   lgd_gpu_write_snapshot: writes the current grid (synchronises).
 *   lgd_gpu_read_snapshot: loads a snapshot into the current grid; its
 *     dimensions and edge cell must equal the grid's; returns the stored
 *     step and maximum (either output may be null).
 *   lgd_snapshot_info: the dimensions (dim entries), step and maximum of a
 *     file, for restarting (startStep) before a grid exists. */
int lgd_gpu_write_snapshot(lgd_handle *h, const char *path, unsigned step, unsigned max_steps);
int lgd_gpu_read_snapshot(lgd_handle *h, const char *path, unsigned *step, unsigned *max_steps);
int lgd_snapshot_info(const char *path, int dim, int *dims, unsigned *step, unsigned *max_steps);

/* Sum of one member over the whole grid in FP64 (deterministic order). */
int lgd_gpu_checksum(lgd_handle *h, int member, int which, double *sum);

int lgd_gpu_synchronize(lgd_handle *h);

/* For tests of the timeout path; no counterpart in the reference.  Every
 * wait of the library's kernels on a copy or a peer is bounded (about two
 * seconds of clock cycles); a CTA whose wait runs out sets the handle's
 * error word, waits (bounded) for its own copies in flight and returns, and
 * the next synchronising call returns LGD_ERR_TIMEOUT.  This call bounds the
 * single-step TMA Jacobi kernel's waits at wait_cycles (0 = the default)
 * and, with skip_plane >= 0, makes its first CTA leave that plane's copy
 * unissued, so that one wait runs out on purpose (nothing faults or hangs:
 * the wait returns after wait_cycles).  skip_plane = -1 restores normal
 * steps; a step with a skipped plane leaves incomplete results. */
int lgd_gpu_test_bounded_waits(lgd_handle *h, long long wait_cycles, int skip_plane);

/* Device pointer and row pitch (bytes) of one member of one buffer; the
 * grid is pitched: row (y, z) starts at ptr + ((z*ny + y) * pitch). */
int lgd_gpu_device_ptr(lgd_handle *h, int member, int which, void **ptr, size_t *pitch_bytes);

/* Number of kernel launches this handle has issued (for benchmarking). */
int lgd_gpu_launch_count(lgd_handle *h, uint64_t *count);

/* Temporal blocking depth used by lgd_gpu_step (time steps fused into one
 * pass over memory): 0 = library default (3 for LGD_CELL_JACOBI7_F32, 2 for
 * LGD_CELL_JACOBI7_F64_FIX, 16 for LGD_CELL_GOL_U8 with rows of a multiple
 * of 32 cells, 8 for other Game of Life torus grids, 1 for the others),
 * 1 = one step per pass, 2 .. LGD_TB_MAX_DEPTH.  It applies to
 *   - the FP32 Jacobi cell (at most 4; results bit-identical for every depth)
 *     and the fixed-point Jacobi cell (at most 2: its pass sums two steps
 *     exactly and rounds once) on 3D cube grids with a zero edge cell, under
 *     kernel variants 0 and 6;
 *   - Game of Life on a torus (cells 0 or 1; bit-identical): rows of a
 *     multiple of 32 cells run bit-sliced passes (32 cells per 32-bit word;
 *     depths 2, 4, 6, 8, 12, 16, 24, 32) under kernel variant 0, rows of a
 *     multiple of 16 cells byte passes (depths 2, 4, 6, 8, 12) under variant
 *     0, or 1 to force them; other depths run as the next smaller one.
 * Deeper requests run at the cell's maximum; a count of steps that is not a
 * multiple of the depth ends with shorter passes.  Plays the role of the
 * reference's CacheBlockingSimulator pipelineLength, a wavefront of time steps over
 * z-marching frames (parallelization/cacheblockingsimulator.h:36-56); the
 * reference's CUDASimulator runs one step per launch
 * (parallelization/cudasimulator.h:560-594). */
#define LGD_TB_MAX_DEPTH 32
int lgd_gpu_set_time_block(lgd_handle *h, int depth);

/* Box shape of the temporally blocked passes, for tuning and comparison:
 * 0 = the default for the cell and depth, 1 and 2 = alternatives (Jacobi:
 * warps x rows per warp, see k_tb.cu; Game of Life: strips twice as tall /
 * half as tall); a shape that does not exist for a depth runs the default.
 * Results do not depend on the shape. */
int lgd_gpu_set_time_block_shape(lgd_handle *h, int shape);

#ifdef __cplusplus
}
#endif

#endif
