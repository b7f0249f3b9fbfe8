/*
 * CPU oracle: plain C restatement of the reference's algorithms for the
 * cell-update hot path.  TEST INFRASTRUCTURE ONLY - tests/, the smoke check
 * and bench.py's CPU-baseline leg call it to compare results against; no
 * product code path links or calls it.
 *
 * Pinned against golden fixtures written by running the reference's own
 * SerialSimulator (oracle/_ref/lgd_ref, built from the reference headers by
 * oracle/Makefile) and against the reference's known-answer tests; see
 * tests/test_oracle_golden.py.
 *
 * Arithmetic follows the cells in oracle/ref_driver.cpp operation for
 * operation; build with -ffp-contract=off so products are never fused into
 * the following sums, which keeps the results bit-identical to the
 * reference build.  OpenMP parallelises over planes/rows only; every cell
 * is computed by one thread, so results do not depend on the thread count.
 *
 * Grids are x-fastest, idx = (z * ny + y) * nx + x.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "lbm_d3q19.h"

static void set_threads(int threads)
{
#ifdef _OPENMP
    if (threads > 0) {
        omp_set_num_threads(threads);
    }
#else
    (void)threads;
#endif
}

int lgd_oracle_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static inline long wrap(long i, long n)
{
    return (i < 0) ? i + n : ((i >= n) ? i - n : i);
}

/* ------------------------------------------------------------------ Jacobi-7
 * Reference: the Jacobi-7 cell's updateLineX (oracle/ref_driver.cpp) run by
 * FixedNeighborhoodUpdateFunctor (storage/fixedneighborhoodupdatefunctor.h:
 * 126-256); Cube topology reads the SoAGrid edge cell outside the box
 * (storage/soagrid.h:578-585), Torus wraps (geometry/topologies.h:179-253).
 * new = (c + n + s + e + w + t + b) * (1/7) with n = y-1, s = y+1, e = x+1,
 * w = x-1, t = z+1, b = z-1, summed left to right. */
/* One row of a cube grid whose y and z neighbours all lie inside: the x
 * loop between the row's ends reads no edge value, so the compiler can
 * vectorise it (each lane the same additions in the same order, so the
 * results do not change); the reference's updateLineX vectorises the same
 * loop with libflatarray's short_vec. */
static void jacobi7_inner_row(long nx, double edge, const double *c, const double *n, const double *s,
                              const double *t, const double *b, double *d)
{
    if (nx == 1) {
        d[0] = (c[0] + n[0] + s[0] + edge + edge + t[0] + b[0]) * (1.0 / 7.0);
        return;
    }
    d[0] = (c[0] + n[0] + s[0] + c[1] + edge + t[0] + b[0]) * (1.0 / 7.0);
    for (long x = 1; x < nx - 1; ++x) {
        d[x] = (c[x] + n[x] + s[x] + c[x + 1] + c[x - 1] + t[x] + b[x]) * (1.0 / 7.0);
    }
    d[nx - 1] = (c[nx - 1] + n[nx - 1] + s[nx - 1] + edge + c[nx - 2] + t[nx - 1] + b[nx - 1]) * (1.0 / 7.0);
}

static void jacobi7_step(long nx, long ny, long nz, int torus, double edge,
                         const double *src, double *dst)
{
    long z;
#pragma omp parallel for schedule(static)
    for (z = 0; z < nz; ++z) {
        for (long y = 0; y < ny; ++y) {
            if (!torus && y > 0 && y < ny - 1 && z > 0 && z < nz - 1) {
                const double *c = src + (z * ny + y) * nx;
                jacobi7_inner_row(nx, edge, c, c - nx, c + nx, c + ny * nx, c - ny * nx, dst + (z * ny + y) * nx);
                continue;
            }
            for (long x = 0; x < nx; ++x) {
                double c = src[(z * ny + y) * nx + x];
                double n, s, e, w, t, b;
                if (torus) {
                    n = src[(z * ny + wrap(y - 1, ny)) * nx + x];
                    s = src[(z * ny + wrap(y + 1, ny)) * nx + x];
                    e = src[(z * ny + y) * nx + wrap(x + 1, nx)];
                    w = src[(z * ny + y) * nx + wrap(x - 1, nx)];
                    t = src[(wrap(z + 1, nz) * ny + y) * nx + x];
                    b = src[(wrap(z - 1, nz) * ny + y) * nx + x];
                } else {
                    n = (y > 0) ? src[(z * ny + y - 1) * nx + x] : edge;
                    s = (y < ny - 1) ? src[(z * ny + y + 1) * nx + x] : edge;
                    e = (x < nx - 1) ? src[(z * ny + y) * nx + x + 1] : edge;
                    w = (x > 0) ? src[(z * ny + y) * nx + x - 1] : edge;
                    t = (z < nz - 1) ? src[((z + 1) * ny + y) * nx + x] : edge;
                    b = (z > 0) ? src[((z - 1) * ny + y) * nx + x] : edge;
                }
                dst[(z * ny + y) * nx + x] = (c + n + s + e + w + t + b) * (1.0 / 7.0);
            }
        }
    }
}

int lgd_oracle_jacobi7(int nx, int ny, int nz, int torus, double edge, int steps,
                       double *u, int threads)
{
    size_t cells = (size_t)nx * ny * nz;
    double *tmp = (double *)malloc(cells * sizeof(double));
    if (!tmp) {
        return -1;
    }
    set_threads(threads);
    double *a = u;
    double *b = tmp;
    for (int s = 0; s < steps; ++s) {
        jacobi7_step(nx, ny, nz, torus, edge, a, b);
        double *t = a;
        a = b;
        b = t;
    }
    if (a != u) {
        memcpy(u, a, cells * sizeof(double));
    }
    free(tmp);
    return 0;
}

/* Ping-pong form for timing: steps time steps between caller-owned buffers
 * a (input) and b, no allocation; returns 0 if the result is in a, 1 if in b. */
int lgd_oracle_jacobi7_pp(int nx, int ny, int nz, int torus, double edge, int steps,
                          double *a, double *b, int threads)
{
    set_threads(threads);
    for (int s = 0; s < steps; ++s) {
        if (s % 2 == 0) {
            jacobi7_step(nx, ny, nz, torus, edge, a, b);
        } else {
            jacobi7_step(nx, ny, nz, torus, edge, b, a);
        }
    }
    return steps % 2;
}

/* -------------------------------------------------------------- Game of Life
 * Reference: ConwayCell::update (src/examples/gameoflife/main.cpp:35-58) with
 * uint8 cells on a torus, run by VanillaUpdateFunctor
 * (storage/vanillaupdatefunctor.h:12-35). */
int lgd_oracle_gol(int nx, int ny, int steps, uint8_t *cells, int threads)
{
    size_t n = (size_t)nx * ny;
    uint8_t *tmp = (uint8_t *)malloc(n);
    if (!tmp) {
        return -1;
    }
    set_threads(threads);
    uint8_t *a = cells;
    uint8_t *b = tmp;
    for (int s = 0; s < steps; ++s) {
        long y;
#pragma omp parallel for schedule(static)
        for (y = 0; y < ny; ++y) {
            const uint8_t *rm = a + wrap(y - 1, ny) * nx;
            const uint8_t *r0 = a + y * nx;
            const uint8_t *rp = a + wrap(y + 1, ny) * nx;
            for (long x = 0; x < nx; ++x) {
                long xm = wrap(x - 1, nx);
                long xp = wrap(x + 1, nx);
                int living = rm[xm] + rm[x] + rm[xp] + r0[xm] + r0[xp] + rp[xm] + rp[x] + rp[xp];
                uint8_t self = r0[x];
                b[y * nx + x] = self ? (uint8_t)((living == 2) || (living == 3))
                                     : (uint8_t)(living == 3);
            }
        }
        uint8_t *t = a;
        a = b;
        b = t;
    }
    if (a != cells) {
        memcpy(cells, a, n);
    }
    free(tmp);
    return 0;
}

/* -------------------------------------------------------- SELL-C-sigma build
 * Reference: ReorderingUnstructuredGrid::setWeights (storage/
 * reorderingunstructuredgrid.h:195-284) - stable sort of row lengths,
 * descending, inside windows of SIGMA rows; physical row i holds logical
 * row perm[i] - followed by SellCSigmaSparseMatrixContainer::initFromMatrix
 * (storage/sellcsigmasparsematrixcontainer.h:221-228, 49-161): entries
 * sorted by (physical row, physical column); chunkLength = max row length
 * of the chunk's C rows; chunkOffset[c+1] = chunkOffset[c] + C *
 * chunkLength[c]; entry k of physical row r sits at chunkOffset[r / C] +
 * k * C + r % C; padding is value 0, column 0.
 *
 * Input: CSR in logical ids (row_ptr[n+1], col, w).  The window sort is a
 * stable counting sort per window (equivalent to std::stable_sort with the
 * reference's comparator). */
typedef struct {
    int key;
    int idx;
} lgd_pair;

static int cmp_pair(const void *a, const void *b)
{
    const lgd_pair *pa = (const lgd_pair *)a;
    const lgd_pair *pb = (const lgd_pair *)b;
    if (pa->key != pb->key) {
        return (pa->key < pb->key) ? -1 : 1;
    }
    return (pa->idx < pb->idx) ? -1 : (pa->idx > pb->idx);
}

/* Returns the number of SELL value slots; fills perm[n] (physical ->
 * logical), row_length[rows_padded], chunk_length[n_chunks],
 * chunk_offset[n_chunks + 1]. */
long long lgd_oracle_sell_plan(int n, const int64_t *row_ptr, int C, int sigma,
                               int *perm, int *row_length, int *chunk_length, int *chunk_offset)
{
    int n_chunks = (n - 1) / C + 1;
    int rows_padded = n_chunks * C;
    lgd_pair *win = (lgd_pair *)malloc(sizeof(lgd_pair) * (size_t)sigma);
    if (!win) {
        return -1;
    }
    for (int w0 = 0; w0 < n; w0 += sigma) {
        int cnt = (n - w0 < sigma) ? n - w0 : sigma;
        for (int i = 0; i < cnt; ++i) {
            int r = w0 + i;
            /* descending length, ties by original position (stable) */
            win[i].key = -(int)(row_ptr[r + 1] - row_ptr[r]);
            win[i].idx = r;
        }
        qsort(win, (size_t)cnt, sizeof(lgd_pair), cmp_pair);
        for (int i = 0; i < cnt; ++i) {
            perm[w0 + i] = win[i].idx;
        }
    }
    free(win);
    for (int p = 0; p < rows_padded; ++p) {
        row_length[p] = (p < n) ? (int)(row_ptr[perm[p] + 1] - row_ptr[perm[p]]) : 0;
    }
    long long total = 0;
    for (int c = 0; c < n_chunks; ++c) {
        int m = 0;
        for (int l = 0; l < C; ++l) {
            if (row_length[c * C + l] > m) {
                m = row_length[c * C + l];
            }
        }
        chunk_length[c] = m;
        chunk_offset[c] = (int)total;
        total += (long long)m * C;
    }
    chunk_offset[n_chunks] = (int)total;
    return total;
}

/* Fills values[total] and column[total].  remap_columns = 1 gives the
 * grid path (ReorderingUnstructuredGrid: column ids are physical ids and a
 * row's entries are ordered by physical column); remap_columns = 0 gives
 * the bare container (SellCSigmaSparseMatrixContainer::initFromMatrix on
 * the logical matrix: rows are permuted within sigma windows through
 * chunkRowToReal but column ids stay logical). */
int lgd_oracle_sell_fill(int n, const int64_t *row_ptr, const int32_t *col, const double *w,
                         int C, const int *perm, const int *chunk_offset,
                         long long total, double *values, int32_t *column, int remap_columns)
{
    int *log_to_phys = (int *)malloc(sizeof(int) * (size_t)n);
    int max_deg = 0;
    if (!log_to_phys) {
        return -1;
    }
    for (int p = 0; p < n; ++p) {
        log_to_phys[perm[p]] = p;
        int d = (int)(row_ptr[perm[p] + 1] - row_ptr[perm[p]]);
        if (d > max_deg) {
            max_deg = d;
        }
    }
    memset(values, 0, sizeof(double) * (size_t)total);
    memset(column, 0, sizeof(int32_t) * (size_t)total);
    lgd_pair *row = (lgd_pair *)malloc(sizeof(lgd_pair) * (size_t)(max_deg > 0 ? max_deg : 1));
    if (!row) {
        free(log_to_phys);
        return -1;
    }
    for (int p = 0; p < n; ++p) {
        int r = perm[p];
        int d = (int)(row_ptr[r + 1] - row_ptr[r]);
        for (int k = 0; k < d; ++k) {
            int c = col[row_ptr[r] + k];
            row[k].key = remap_columns ? log_to_phys[c] : c;
            row[k].idx = (int)(row_ptr[r] + k);
        }
        qsort(row, (size_t)d, sizeof(lgd_pair), cmp_pair);
        long long base = chunk_offset[p / C] + p % C;
        for (int k = 0; k < d; ++k) {
            values[base + (long long)k * C] = w[row[k].idx];
            column[base + (long long)k * C] = row[k].key;
        }
    }
    free(row);
    free(log_to_phys);
    return 0;
}

/* --------------------------------------------- SELL-C-sigma diffusion step
 * Reference: the diffusion cell's update (oracle/ref_driver.cpp) driven by
 * UnstructuredUpdateFunctor / UnstructuredNeighborhood (storage/
 * unstructuredneighborhood.h:97-200): acc = sum over the row's rowLength
 * entries in SELL order of x[column] * value; x' = 0.1 * x + acc.  Works in
 * physical order. */
int lgd_oracle_sell_diffusion(int n, int C, const int *chunk_offset, const int *row_length,
                              const double *values, const int32_t *column,
                              int steps, double *x, int threads)
{
    double *tmp = (double *)malloc(sizeof(double) * (size_t)n);
    if (!tmp) {
        return -1;
    }
    set_threads(threads);
    double *a = x;
    double *b = tmp;
    for (int s = 0; s < steps; ++s) {
        long p;
#pragma omp parallel for schedule(static, 4096)
        for (p = 0; p < n; ++p) {
            long long base = chunk_offset[p / C] + p % C;
            double acc = 0.0;
            for (int k = 0; k < row_length[p]; ++k) {
                long long idx = base + (long long)k * C;
                acc += a[column[idx]] * values[idx];
            }
            b[p] = 0.1 * a[p] + acc;
        }
        double *t = a;
        a = b;
        b = t;
    }
    if (a != x) {
        memcpy(x, a, sizeof(double) * (size_t)n);
    }
    free(tmp);
    return 0;
}

/* ------------------------------------------------------------------ D3Q19
 * Reference: the D3Q19 cell in oracle/ref_driver.cpp (collision of
 * src/examples/latticeboltzmann/main.cpp:93-170), on an L^3 fluid box with
 * walls outside and the lid beyond y = L-1.  f is SoA: f[i * L^3 + idx]. */

/* one cell next to a wall: populations from outside bounce back */
static void lbm_cell_wall(const double *a, double *b, size_t cells, long L, long x, long y, long z, double omega,
                          double lid)
{
    const size_t idx = ((size_t)z * L + y) * L + x;
    double self[19];
    double pulled[19];
    double out[19];
    for (int i = 0; i < 19; ++i) {
        self[i] = a[i * cells + idx];
    }
    for (int i = 0; i < 19; ++i) {
        long sx = x - LGD_D3Q19_E[i][0];
        long sy = y - LGD_D3Q19_E[i][1];
        long sz = z - LGD_D3Q19_E[i][2];
        if (sx >= 0 && sx < L && sy >= 0 && sy < L && sz >= 0 && sz < L) {
            pulled[i] = a[i * cells + ((size_t)sz * L + sy) * L + sx];
        } else {
            int fromLid = (y == L - 1) && (LGD_D3Q19_E[i][1] == -1);
            pulled[i] = lgd_d3q19_bounce(self, i, fromLid ? lid : 0.0);
        }
    }
    lgd_d3q19_collide(pulled, omega, out);
    for (int i = 0; i < 19; ++i) {
        b[i * cells + idx] = out[i];
    }
}

/* cells x0 .. x1-1 of a row whose every neighbour lies inside the box: the
 * same pulls without the wall tests, the same collision (the compiler may
 * vectorise the row; each cell's operations and their order are unchanged,
 * as in the reference's vectorised updateLineX) */
static void lbm_row_inner(const double *restrict a, double *restrict b, size_t cells, long L, long y, long z,
                          long x0, long x1, double omega)
{
    const size_t row = ((size_t)z * L + y) * L;
    long x = x0;
    for (; x + 1 < x1; x += 2) {            /* two cells at once */
        const size_t idx = row + x;
        lgd_v2d pulled[19];
        lgd_v2d out[19];
        for (int i = 0; i < 19; ++i) {
            const long off = LGD_D3Q19_E[i][0] + LGD_D3Q19_E[i][1] * L + LGD_D3Q19_E[i][2] * L * L;
            memcpy(&pulled[i], a + i * cells + idx - off, sizeof(lgd_v2d));
        }
        lgd_d3q19_collide_v2(pulled, omega, out);
        for (int i = 0; i < 19; ++i) {
            memcpy(b + i * cells + idx, &out[i], sizeof(lgd_v2d));
        }
    }
    for (; x < x1; ++x) {
        const size_t idx = row + x;
        double pulled[19];
        double out[19];
        for (int i = 0; i < 19; ++i) {
            const long off = LGD_D3Q19_E[i][0] + LGD_D3Q19_E[i][1] * L + LGD_D3Q19_E[i][2] * L * L;
            pulled[i] = a[i * cells + idx - off];
        }
        lgd_d3q19_collide(pulled, omega, out);
        for (int i = 0; i < 19; ++i) {
            b[i * cells + idx] = out[i];
        }
    }
}

int lgd_oracle_lbm(int L, int steps, double omega, double lid, double *f, int threads)
{
    size_t cells = (size_t)L * L * L;
    double *tmp = (double *)malloc(sizeof(double) * 19 * cells);
    if (!tmp) {
        return -1;
    }
    set_threads(threads);
    double *a = f;
    double *b = tmp;
    for (int s = 0; s < steps; ++s) {
        long z;
#pragma omp parallel for schedule(static)
        for (z = 0; z < L; ++z) {
            for (long y = 0; y < L; ++y) {
                if (L >= 3 && z >= 1 && z <= L - 2 && y >= 1 && y <= L - 2) {
                    lbm_cell_wall(a, b, cells, L, 0, y, z, omega, lid);
                    lbm_row_inner(a, b, cells, L, y, z, 1, L - 1, omega);
                    lbm_cell_wall(a, b, cells, L, L - 1, y, z, omega, lid);
                } else {
                    for (long x = 0; x < L; ++x) lbm_cell_wall(a, b, cells, L, x, y, z, omega, lid);
                }
            }
        }
        double *t = a;
        a = b;
        b = t;
    }
    if (a != f) {
        memcpy(f, a, sizeof(double) * 19 * cells);
    }
    free(tmp);
    return 0;
}

/* --------------------------------------- variable-coefficient diffusion
 * Reference: the var-coef cell in oracle/ref_driver.cpp on a torus:
 * u' = u + sum over faces (-x,+x,-y,+y,-z,+z) of 0.5 (k + k_nb)(u_nb - u). */
int lgd_oracle_varcoef(int nx, int ny, int nz, int steps, double *u, const double *k, int threads)
{
    size_t cells = (size_t)nx * ny * nz;
    double *tmp = (double *)malloc(sizeof(double) * cells);
    if (!tmp) {
        return -1;
    }
    set_threads(threads);
    double *a = u;
    double *b = tmp;
    for (int s = 0; s < steps; ++s) {
        long z;
#pragma omp parallel for schedule(static)
        for (z = 0; z < nz; ++z) {
            for (long y = 0; y < ny; ++y) {
                for (long x = 0; x < nx; ++x) {
                    size_t c = ((size_t)z * ny + y) * nx + x;
                    size_t nb[6];
                    nb[0] = ((size_t)z * ny + y) * nx + wrap(x - 1, nx);
                    nb[1] = ((size_t)z * ny + y) * nx + wrap(x + 1, nx);
                    nb[2] = ((size_t)z * ny + wrap(y - 1, ny)) * nx + x;
                    nb[3] = ((size_t)z * ny + wrap(y + 1, ny)) * nx + x;
                    nb[4] = ((size_t)wrap(z - 1, nz) * ny + y) * nx + x;
                    nb[5] = ((size_t)wrap(z + 1, nz) * ny + y) * nx + x;
                    double uc = a[c];
                    double kc = k[c];
                    double flux = 0.5 * (kc + k[nb[0]]) * (a[nb[0]] - uc);
                    for (int q = 1; q < 6; ++q) {
                        flux = flux + 0.5 * (kc + k[nb[q]]) * (a[nb[q]] - uc);
                    }
                    b[c] = uc + flux;
                }
            }
        }
        double *t = a;
        a = b;
        b = t;
    }
    if (a != u) {
        memcpy(u, a, sizeof(double) * cells);
    }
    free(tmp);
    return 0;
}
