// Internal declarations shared by the library's translation units.
#ifndef LGD_INTERNAL_H
#define LGD_INTERNAL_H

#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/lgd_gpu.h"

namespace lgd {

// Exceptions used inside the library; lgd_guard() maps them to status codes.
struct Error : std::runtime_error {
    int code;
    Error(int code, const std::string& msg) : std::runtime_error(msg), code(code) {}
};

void set_error(int code, const std::string& msg);
void clear_error();

#define LGD_CHECK_CUDA(expr)                                                               \
    do {                                                                                   \
        cudaError_t lgd_err_ = (expr);                                                     \
        if (lgd_err_ != cudaSuccess) {                                                     \
            throw ::lgd::Error(LGD_ERR_CUDA, std::string("CUDA error: ") +                 \
                               cudaGetErrorString(lgd_err_) + " at " #expr);               \
        }                                                                                  \
    } while (0)

#define LGD_REQUIRE(cond, code, msg)                                                       \
    do {                                                                                   \
        if (!(cond)) {                                                                     \
            throw ::lgd::Error((code), (msg));                                             \
        }                                                                                  \
    } while (0)

// Runs f, converting exceptions into status codes and the thread's last
// error message.
template<typename F>
int guard(F&& f)
{
    try {
        clear_error();
        f();
        return LGD_OK;
    } catch (const Error& e) {
        set_error(e.code, e.what());
        return e.code;
    } catch (const std::bad_alloc&) {
        set_error(LGD_ERR_NOMEM, "host allocation failed");
        return LGD_ERR_NOMEM;
    } catch (const std::exception& e) {
        set_error(LGD_ERR_INVALID, e.what());
        return LGD_ERR_INVALID;
    }
}

// A value set up once per device, with that device current: kernel
// attributes (the dynamic shared-memory limit), occupancy and SM counts
// apply per device, so a process that drives several GPUs sets each up on
// its first use there.
template<typename T>
class PerDevice {
public:
    template<typename F>
    T get(F&& init)
    {
        int dev = 0;
        LGD_CHECK_CUDA(cudaGetDevice(&dev));
        LGD_REQUIRE(dev >= 0 && dev < MAX_DEVICES, LGD_ERR_UNSUPPORTED, "device index above 63");
        std::lock_guard<std::mutex> lock(mutex);
        if (!ready[dev]) {
            value[dev] = init();
            ready[dev] = true;
        }
        return value[dev];
    }

private:
    static const int MAX_DEVICES = 64;
    std::mutex mutex;
    T value[MAX_DEVICES] = {};
    bool ready[MAX_DEVICES] = {};
};

// Throws if the last launch failed to start.
inline void check_launch(const char *what)
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        throw Error(LGD_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e) + " launching " + what);
    }
}

inline int round_up(int v, int m) { return (v + m - 1) / m * m; }

// One structured grid: SoA members, each double-buffered and pitched so
// that every row starts on a 128-byte boundary.
struct Member {
    int elem;           // bytes per element
    bool is_static;     // never written by the cell (one buffer serves both)
    void *buf[2];
};

struct Grid {
    lgd_grid_desc desc;
    int n_members;
    Member m[2];
    size_t pitch_elems;     // row pitch in elements (same for all members of equal size)
    size_t pitch_bytes[2];  // per member
    size_t plane_elems;     // pitch_elems * ny
    int cur;                // index of the current buffer
    int time_block;         // temporal blocking depth (0 = default)
    int tb_shape;           // temporal blocking box shape (0 = default for the cell and depth)
    int fix_exp;            // fixed-point grids: value = k * 2^(fix_exp - LGD_FIX_BITS)
    bool fix_nonneg;        // fixed-point grids: no negative value or edge cell so far
    bool fix_pinned;        // fixed-point grids: the exponent is only raised, never lowered
    int fix_steps_unchecked;    // fixed-point grids: steps since the exponent was last lowered
    unsigned long long *d_fixmax;   // fixed-point grids: [0] max |k| of a check, [1] negative-value flag
    unsigned char *edge_record;     // record grids: the edge cell (host copy, malloc'd)
    void *d_edge_record;            // record grids: the edge cell on the device
    int variant;            // kernel variant where a cell has several (0 = default)
    cudaStream_t stream;
    uint64_t launches;
    int device;
    // scratch for region updates and reductions
    int *d_streaks;
    long long *d_streak_prefix;
    int streak_capacity;
    double *d_partials;
    int partial_capacity;
    // TMA kernel: one tensor map (a 128-byte CUtensorMap) per buffer, the
    // buffer it was built for, and the device error word of bounded waits
    alignas(64) unsigned char tmap[2][128];
    bool tmap_ready[2];
    void *tmap_base[2];
    int *d_err;
    // tests of the timeout path (lgd_gpu_test_bounded_waits): wait bound of
    // the TMA Jacobi kernel (0 = the default) and 1 + the plane whose copy
    // its first CTA leaves unissued (0 = none)
    long long test_wait_cycles;
    int test_skip_plane;
    void *d_stage;          // conversion staging at the boundary (fixed-point grids)
    size_t stage_bytes;
    // fixed-point transfers in row chunks: copies on xfer_stream, the
    // conversions on stream, chunk k handed over by xfer_ev[k] (created on
    // first use)
    cudaStream_t xfer_stream;
    cudaEvent_t xfer_ev[17];
    bool xfer_ready;
    // var-coef TMA kernel: six tensor maps (u and k; main box, row, column)
    // per u buffer and the buffers they were built for
    alignas(64) unsigned char vtmap[2][6 * 128];
    bool vtmap_ready[2];
    void *vtmap_base[2][2];
    // temporal-blocking kernel: one tensor map per buffer (box 64 x rows)
    alignas(64) unsigned char tbmap[2][128];
    bool tbmap_ready[2];
    void *tbmap_base[2];
    int tbmap_rows[2];
};

bool tma_applicable(const Grid& g);
void launch_jacobi7_tma(Grid& g);
bool varcoef_tma_applicable(const Grid& g);
void launch_varcoef_tma(Grid& g);
// temporal blocking (k_tb.cu): depth time steps per pass, 2 .. LGD_TB_MAX_DEPTH
bool tb_applicable(const Grid& g);
int tb_default_depth(const Grid& g);
int tb_max_depth(const Grid& g);
void launch_jacobi7_tb(Grid& g, int depth, int shape);

// cuTensorMapEncodeTiled (tiled, no swizzle, no out-of-bounds NaN fill)
// into a 128-byte map: dtype a CUtensorMapDataType, dims and box innermost
// first, strides in bytes for dimensions 1 .. rank-1
void encode_tensor_map(void *map, int dtype, int rank, void *base, const uint64_t *dims, const uint64_t *strides,
                       const uint32_t *box);

// kernels, one entry per cell family (implemented in k_*.cu)
void launch_jacobi7(Grid& g, int steps);
void launch_gol(Grid& g, int steps);
void launch_varcoef(Grid& g, int steps);
void launch_region(Grid& g, const int *d_streaks, const long long *d_prefix, int n_streaks, long long cells,
                   unsigned nano_step);

// device form of lgd_test_record (LGD_CELL_TEST)
struct TestRec {
    int pos[3];
    int dim[3];
    unsigned cycle;
    unsigned char edge, valid, pad0, pad1;
    float test_value;
    int pad[7];
};
static_assert(sizeof(TestRec) == 64, "test record is 64 bytes");

inline unsigned test_nano_steps(const Grid& g)
{
    const unsigned n = ((unsigned)g.desc.flags >> 8) & 255u;
    return n ? n : 1u;
}
void launch_fill(Grid& g, int member, int which, uint64_t seed, int stream, int mode, double p, int scale_exp);
void launch_checksum(Grid& g, int member, int which, double *out);
void launch_streak_copy(Grid& g, int member, int which, const int *d_streaks, const long long *d_prefix,
                        int n_streaks, long long cells, void *d_packed, bool to_grid);
// the same for a fixed-point grid's current buffer, FP64 values at the boundary
void launch_streak_copy_fix(Grid& g, const int *d_streaks, const long long *d_prefix, int n_streaks, long long cells,
                            double *d_packed, bool to_grid);

// SplitMix64 key derivation shared with the fill kernel
uint64_t stream_key(uint64_t seed, int stream);

}  // namespace lgd

struct lgd_handle {
    lgd::Grid g;
};

#endif
