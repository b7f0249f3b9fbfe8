/*
 * Reference runner: the workload cells written once against the
 * reference's own Cell / APITraits API and advanced by the reference's
 * SerialSimulator / OpenMPSimulator.  Compiled only in the build container
 * (it needs the reference headers) by oracle/Makefile into oracle/_ref/.
 * It is test infrastructure: tests/golden/gen_golden.py runs it to write
 * the golden fixtures that pin the C restatement in oracle/lgd_oracle.c.
 *
 * Input and output arrays are raw little-endian files; every size comes
 * from the command line.  Logical cell order is x-fastest:
 * idx = (z * ny + y) * nx + x.
 *
 * Reference call paths exercised:
 *   - SoA + updateLineX: SerialSimulator::nanoStep
 *     (parallelization/serialsimulator.h:132-139) -> UpdateFunctor
 *     (storage/updatefunctor.h:97-139) -> FixedNeighborhoodUpdateFunctor
 *     (storage/fixedneighborhoodupdatefunctor.h:265).
 *   - AoS vanilla update(): VanillaUpdateFunctor
 *     (storage/vanillaupdatefunctor.h:12-35), torus via Topology::locate.
 *   - Unstructured SELL-C-sigma: ReorderingUnstructuredGrid::setWeights
 *     (storage/reorderingunstructuredgrid.h:195-284) ->
 *     SellCSigmaSparseMatrixContainer::initFromMatrix
 *     (storage/sellcsigmasparsematrixcontainer.h:221-228) ->
 *     UnstructuredUpdateFunctor (storage/unstructuredupdatefunctor.h:121-132).
 */
#include <libgeodecomp/config.h>
#include <libgeodecomp/geometry/stencils.h>
#include <libgeodecomp/io/serialbovwriter.h>
#include <libgeodecomp/io/simpleinitializer.h>
#include <libgeodecomp/misc/apitraits.h>
#include <libgeodecomp/parallelization/serialsimulator.h>
#include <libgeodecomp/parallelization/openmpsimulator.h>
#include <libgeodecomp/storage/unstructuredgrid.h>
#include <libgeodecomp/storage/unstructuredsoagrid.h>
#include <libgeodecomp/storage/reorderingunstructuredgrid.h>
#include <libgeodecomp/storage/unstructuredlooppeeler.h>
#include <libflatarray/macros.hpp>
#include <libflatarray/short_vec.hpp>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

using namespace LibGeoDecomp;

// ---------------------------------------------------------------- file I/O
template<typename T>
static std::vector<T> readArray(const char *path, std::size_t n)
{
    std::vector<T> ret(n);
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        throw std::runtime_error(std::string("cannot open ") + path);
    }
    std::size_t got = std::fread(ret.data(), sizeof(T), n, f);
    std::fclose(f);
    if (got != n) {
        throw std::runtime_error(std::string("short read on ") + path);
    }
    return ret;
}

template<typename T>
static void writeArray(const char *path, const std::vector<T>& a)
{
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        throw std::runtime_error(std::string("cannot open ") + path);
    }
    std::fwrite(a.data(), sizeof(T), a.size(), f);
    std::fclose(f);
}

static double secondsSince(std::chrono::steady_clock::time_point t0)
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

// ------------------------------------------------- Jacobi-7 (SoA, updateLineX)
// new = (c + n + s + e + w + t + b) * (1/7), von Neumann radius 1.
#define LGD_JACOBI7_BODY(HOOD, ACC)                        \
    ((HOOD[FixedCoord< 0,  0,  0>()] ACC +                 \
      HOOD[FixedCoord< 0, -1,  0>()] ACC +                 \
      HOOD[FixedCoord< 0,  1,  0>()] ACC +                 \
      HOOD[FixedCoord< 1,  0,  0>()] ACC +                 \
      HOOD[FixedCoord<-1,  0,  0>()] ACC +                 \
      HOOD[FixedCoord< 0,  0,  1>()] ACC +                 \
      HOOD[FixedCoord< 0,  0, -1>()] ACC) * (1.0 / 7.0))

template<typename TOPOLOGY_API>
class Jacobi7Cell
{
public:
    class API :
        public APITraits::HasFixedCoordsOnlyUpdate,
        public APITraits::HasUpdateLineX,
        public APITraits::HasStencil<Stencils::VonNeumann<3, 1> >,
        public TOPOLOGY_API,
        public APITraits::HasSoA
    {};

    inline explicit Jacobi7Cell(double v = 0) :
        temp(v)
    {}

    template<typename HOOD_OLD, typename HOOD_NEW>
    static void updateLineX(HOOD_OLD& hoodOld, long indexEnd, HOOD_NEW& hoodNew, long /* nanoStep */)
    {
        for (; hoodOld.index() < indexEnd; hoodOld += 1, hoodNew += 1) {
            hoodNew.temp() = LGD_JACOBI7_BODY(hoodOld, .temp());
        }
    }

    template<typename HOOD>
    void update(const HOOD& hood, int /* nanoStep */)
    {
        temp = LGD_JACOBI7_BODY(hood, .temp);
    }

    double temp;
};

typedef Jacobi7Cell<APITraits::HasCubeTopology<3> > Jacobi7CubeCell;
typedef Jacobi7Cell<APITraits::HasTorusTopology<3> > Jacobi7TorusCell;

LIBFLATARRAY_REGISTER_SOA(Jacobi7CubeCell, ((double)(temp)))
LIBFLATARRAY_REGISTER_SOA(Jacobi7TorusCell, ((double)(temp)))

template<typename CELL>
class ArrayInitializer3D : public SimpleInitializer<CELL>
{
public:
    ArrayInitializer3D(Coord<3> dim, unsigned steps, const std::vector<double> *values) :
        SimpleInitializer<CELL>(dim, steps),
        values(values)
    {}

    virtual void grid(GridBase<CELL, 3> *ret)
    {
        CoordBox<3> box = ret->boundingBox();
        Coord<3> dim = this->gridDimensions();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) {
            std::size_t idx = (std::size_t(i->z()) * dim.y() + i->y()) * dim.x() + i->x();
            ret->set(*i, CELL((*values)[idx]));
        }
    }

private:
    const std::vector<double> *values;
};

template<typename CELL, typename SIM>
static int runJacobi(Coord<3> dim, unsigned steps, const char *in, const char *out, bool timeOnly)
{
    std::size_t n = std::size_t(dim.x()) * dim.y() * dim.z();
    std::vector<double> values = readArray<double>(in, n);
    SIM sim(new ArrayInitializer3D<CELL>(dim, steps, &values));
    auto t0 = std::chrono::steady_clock::now();
    for (unsigned s = 0; s < steps; ++s) {
        sim.step();
    }
    double dt = secondsSince(t0);
    std::printf("{\"seconds\": %.6f, \"glups\": %.6f}\n", dt, 1e-9 * double(n) * steps / dt);
    if (timeOnly) {
        return 0;
    }
    const GridBase<CELL, 3> *grid = sim.getGrid();
    std::vector<double> result(n);
    for (int z = 0; z < dim.z(); ++z) {
        for (int y = 0; y < dim.y(); ++y) {
            for (int x = 0; x < dim.x(); ++x) {
                result[(std::size_t(z) * dim.y() + y) * dim.x() + x] = grid->get(Coord<3>(x, y, z)).temp;
            }
        }
    }
    writeArray(out, result);
    return 0;
}

// The reference's SerialBOVWriter (io/serialbovwriter.h, io/bovoutput.h) on
// the Jacobi cube cell: run() with a writer of period `steps` writes
// prefix.00000.{bov,data} (WRITER_INITIALIZED) and prefix.<steps>.{bov,data}
// (WRITER_STEP_FINISHED, then WRITER_ALL_DONE to the same files).
template<typename CELL>
static int runBov(Coord<3> dim, unsigned steps, const char *in, const char *prefix)
{
    std::size_t n = std::size_t(dim.x()) * dim.y() * dim.z();
    std::vector<double> values = readArray<double>(in, n);
    SerialSimulator<CELL> sim(new ArrayInitializer3D<CELL>(dim, steps, &values));
    sim.addWriter(new SerialBOVWriter<CELL>(Selector<CELL>(&CELL::temp, "temp"), prefix, steps));
    sim.run();
    std::printf("{}\n");
    return 0;
}

// ------------------------------------------------ Game of Life (AoS, uint8)
class ConwayCellU8
{
public:
    class API :
        public APITraits::HasStencil<Stencils::Moore<2, 1> >,
        public APITraits::HasTorusTopology<2>
    {};

    inline explicit ConwayCellU8(unsigned char alive = 0) :
        alive(alive)
    {}

    template<typename COORD_MAP>
    void update(const COORD_MAP& hood, unsigned /* nanoStep */)
    {
        int living = 0;
        for (int y = -1; y < 2; ++y) {
            for (int x = -1; x < 2; ++x) {
                living += hood[Coord<2>(x, y)].alive;
            }
        }
        unsigned char self = hood[Coord<2>(0, 0)].alive;
        living -= self;
        if (self) {
            alive = ((2 <= living) && (living <= 3)) ? 1 : 0;
        } else {
            alive = (living == 3) ? 1 : 0;
        }
    }

    unsigned char alive;
};

class GoLInitializer : public SimpleInitializer<ConwayCellU8>
{
public:
    GoLInitializer(Coord<2> dim, unsigned steps, const std::vector<unsigned char> *values) :
        SimpleInitializer<ConwayCellU8>(dim, steps),
        values(values)
    {}

    virtual void grid(GridBase<ConwayCellU8, 2> *ret)
    {
        CoordBox<2> box = ret->boundingBox();
        for (CoordBox<2>::Iterator i = box.begin(); i != box.end(); ++i) {
            std::size_t idx = std::size_t(i->y()) * dimensions.x() + i->x();
            ret->set(*i, ConwayCellU8((*values)[idx]));
        }
    }

private:
    const std::vector<unsigned char> *values;
};

template<typename SIM>
static int runGoL(Coord<2> dim, unsigned steps, const char *in, const char *out, bool timeOnly)
{
    std::size_t n = std::size_t(dim.x()) * dim.y();
    std::vector<unsigned char> values = readArray<unsigned char>(in, n);
    SIM sim(new GoLInitializer(dim, steps, &values));
    auto t0 = std::chrono::steady_clock::now();
    for (unsigned s = 0; s < steps; ++s) {
        sim.step();
    }
    double dt = secondsSince(t0);
    std::printf("{\"seconds\": %.6f, \"glups\": %.6f}\n", dt, 1e-9 * double(n) * steps / dt);
    if (timeOnly) {
        return 0;
    }
    const GridBase<ConwayCellU8, 2> *grid = sim.getGrid();
    std::vector<unsigned char> result(n);
    for (int y = 0; y < dim.y(); ++y) {
        for (int x = 0; x < dim.x(); ++x) {
            result[std::size_t(y) * dim.x() + x] = grid->get(Coord<2>(x, y)).alive;
        }
    }
    writeArray(out, result);
    return 0;
}

// ---------------------------------------- SELL-C-sigma diffusion x' = 0.1 x + W x
// AoS cell through ReorderingUnstructuredGrid<UnstructuredGrid>; the sum runs
// over the row's entries in SELL order (ascending physical column).
template<int C, int SIGMA>
class SellDiffusionCell
{
public:
    class API :
        public APITraits::HasUnstructuredTopology,
        public APITraits::HasSellType<double>,
        public APITraits::HasSellMatrices<1>,
        public APITraits::HasSellC<C>,
        public APITraits::HasSellSigma<SIGMA>
    {};

    inline explicit SellDiffusionCell(double v = 0) :
        value(v)
    {}

    template<typename HOOD>
    void update(HOOD& hood, unsigned /* nanoStep */)
    {
        double acc = 0.0;
        for (const auto& j: hood.weights(0)) {
            acc += hood[j.first()].value * j.second();
        }
        value = 0.1 * hood[hood.index()].value + acc;
    }

    double value;
};

struct CSRInput
{
    int n;
    std::vector<long long> rowPtr;
    std::vector<int> col;
    std::vector<double> w;
    std::vector<double> x;
};

template<typename CELL>
class SellInitializer : public SimpleInitializer<CELL>
{
public:
    typedef typename GridBase<CELL, 1>::SparseMatrix SparseMatrix;

    SellInitializer(const CSRInput *in, unsigned steps) :
        SimpleInitializer<CELL>(Coord<1>(in->n), steps),
        in(in)
    {}

    virtual void grid(GridBase<CELL, 1> *ret)
    {
        for (int i = 0; i < in->n; ++i) {
            ret->set(Coord<1>(i), CELL(in->x[i]));
        }
        SparseMatrix m;
        m.reserve(in->col.size());
        for (int r = 0; r < in->n; ++r) {
            for (long long k = in->rowPtr[r]; k < in->rowPtr[r + 1]; ++k) {
                m.push_back(std::make_pair(Coord<2>(r, in->col[k]), in->w[k]));
            }
        }
        ret->setWeights(0, m);
    }

private:
    const CSRInput *in;
};

static CSRInput readCSR(int n, long long nnz, const char *rowPtr, const char *col, const char *w, const char *x)
{
    CSRInput in;
    in.n = n;
    in.rowPtr = readArray<long long>(rowPtr, std::size_t(n) + 1);
    in.col = readArray<int>(col, std::size_t(nnz));
    in.w = readArray<double>(w, std::size_t(nnz));
    in.x = readArray<double>(x, std::size_t(n));
    return in;
}

template<int C, int SIGMA, typename SIM>
static int runSell(const CSRInput& in, unsigned steps, const char *out, bool timeOnly)
{
    typedef SellDiffusionCell<C, SIGMA> CELL;
    SIM sim(new SellInitializer<CELL>(&in, steps));
    auto t0 = std::chrono::steady_clock::now();
    for (unsigned s = 0; s < steps; ++s) {
        sim.step();
    }
    double dt = secondsSince(t0);
    std::printf("{\"seconds\": %.6f, \"s_per_step\": %.6f}\n", dt, dt / steps);
    if (timeOnly) {
        return 0;
    }
    const GridBase<CELL, 1> *grid = sim.getGrid();
    std::vector<double> result(in.n);
    for (int i = 0; i < in.n; ++i) {
        result[i] = grid->get(Coord<1>(i)).value;
    }
    writeArray(out, result);
    return 0;
}

// Dump the SELL-C-sigma arrays exactly as the reference builds them for the
// matrix: physical->logical row map, chunkOffset, chunkLength, rowLength,
// values, column.
template<int C, int SIGMA>
static int dumpSell(const CSRInput& in, const char *prefix)
{
    typedef SellDiffusionCell<C, SIGMA> CELL;
    typedef ReorderingUnstructuredGrid<UnstructuredGrid<CELL, 1, double, C, SIGMA> > Grid;
    Region<1> nodes;
    nodes << Streak<1>(Coord<1>(0), in.n);
    Grid grid(nodes);
    SellInitializer<CELL> init(&in, 1);
    // cell values carry their logical id, so data() reveals the physical order
    CSRInput ids = in;
    for (int i = 0; i < in.n; ++i) {
        ids.x[i] = i;
    }
    SellInitializer<CELL> idInit(&ids, 1);
    idInit.grid(&grid);

    std::vector<int> physToLogical(in.n);
    for (int p = 0; p < in.n; ++p) {
        physToLogical[p] = int(grid.data()[p].value);
    }
    const auto& sell = grid.getWeights(0);
    std::string p(prefix);
    writeArray((p + "perm.i32").c_str(), physToLogical);
    writeArray((p + "chunk_offset.i32").c_str(), sell.chunkOffsetVec());
    writeArray((p + "chunk_length.i32").c_str(), sell.chunkLengthVec());
    writeArray((p + "row_length.i32").c_str(), sell.rowLengthVec());
    std::vector<double> values(sell.valuesVec().begin(), sell.valuesVec().end());
    std::vector<int> column(sell.columnVec().begin(), sell.columnVec().end());
    writeArray((p + "values.f64").c_str(), values);
    writeArray((p + "column.i32").c_str(), column);
    return 0;
}

// Dump a bare SellCSigmaSparseMatrixContainer built from the logical matrix
// (no grid reordering): chunkRowToReal, chunkOffset, chunkLength, rowLength,
// values, column.
template<int C, int SIGMA>
static int dumpContainer(const CSRInput& in, const char *prefix)
{
    SellCSigmaSparseMatrixContainer<double, C, SIGMA> sell(in.n);
    std::vector<std::pair<Coord<2>, double> > m;
    for (int r = 0; r < in.n; ++r) {
        for (long long k = in.rowPtr[r]; k < in.rowPtr[r + 1]; ++k) {
            m.push_back(std::make_pair(Coord<2>(r, in.col[k]), in.w[k]));
        }
    }
    sell.initFromMatrix(m);
    std::string p(prefix);
    std::vector<int> perm(sell.chunkRowToRealVec().begin(), sell.chunkRowToRealVec().begin() + in.n);
    writeArray((p + "perm.i32").c_str(), perm);
    writeArray((p + "chunk_offset.i32").c_str(), sell.chunkOffsetVec());
    writeArray((p + "chunk_length.i32").c_str(), sell.chunkLengthVec());
    writeArray((p + "row_length.i32").c_str(), sell.rowLengthVec());
    std::vector<double> values(sell.valuesVec().begin(), sell.valuesVec().end());
    std::vector<int> column(sell.columnVec().begin(), sell.columnVec().end());
    writeArray((p + "values.f64").c_str(), values);
    writeArray((p + "column.i32").c_str(), column);
    return 0;
}

// --------------------------------------------- D3Q19 BGK lid-driven cavity
// Pull scheme on an L^3 fluid box; the walls sit outside the box and are
// represented by the Cube topology's edge cell (state WALL).  A population
// pulled from a wall is bounced back from the cell itself; pulled from the
// lid (y == L) it also gains 6 w_i (e_i . u_lid).  Collision is the
// incompressible BGK form of the reference's LBM example
// (src/examples/latticeboltzmann/main.cpp:93-170).
#include "lbm_d3q19.h"

class D3Q19Cell
{
public:
    class API :
        public APITraits::HasStencil<Stencils::Moore<3, 1> >,
        public APITraits::HasCubeTopology<3>
    {};

    enum State {FLUID = 0, WALL = 1};

    inline explicit D3Q19Cell(int state = WALL, double omega = 1.0, double lid = 0.0) :
        state(state), isTop(0), omega(omega), lid(lid)
    {
        for (int i = 0; i < 19; ++i) {
            f[i] = LGD_D3Q19_W[i];
        }
    }

    template<typename COORD_MAP>
    void update(const COORD_MAP& hood, unsigned /* nanoStep */)
    {
        const D3Q19Cell& self = hood[Coord<3>(0, 0, 0)];
        *this = self;
        if (state != FLUID) {
            return;
        }
        double pulled[19];
        for (int i = 0; i < 19; ++i) {
            const D3Q19Cell& src = hood[Coord<3>(-LGD_D3Q19_E[i][0], -LGD_D3Q19_E[i][1], -LGD_D3Q19_E[i][2])];
            if (src.state == FLUID) {
                pulled[i] = src.f[i];
            } else {
                // the lid is the wall beyond y = L-1; isTop marks the top fluid layer
                bool fromLid = (isTop != 0) && (LGD_D3Q19_E[i][1] == -1);
                pulled[i] = lgd_d3q19_bounce(self.f, i, fromLid ? lid : 0.0);
            }
        }
        lgd_d3q19_collide(pulled, omega, f);
    }

    double f[19];
    int state;
    int isTop;
    double omega;
    double lid;
};

class D3Q19Initializer : public SimpleInitializer<D3Q19Cell>
{
public:
    D3Q19Initializer(int L, unsigned steps, double omega, double lid) :
        SimpleInitializer<D3Q19Cell>(Coord<3>::diagonal(L), steps),
        omega(omega), lid(lid)
    {}

    virtual void grid(GridBase<D3Q19Cell, 3> *ret)
    {
        CoordBox<3> box = ret->boundingBox();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) {
            D3Q19Cell c(D3Q19Cell::FLUID, omega, lid);
            c.isTop = (i->y() == dimensions.y() - 1) ? 1 : 0;
            ret->set(*i, c);
        }
        D3Q19Cell wall(D3Q19Cell::WALL, omega, lid);
        wall.isTop = 0;
        ret->setEdge(wall);
    }

private:
    double omega;
    double lid;
};

template<typename SIM>
static int runLBM(int L, unsigned steps, double omega, double lid, const char *out, bool timeOnly)
{
    SIM sim(new D3Q19Initializer(L, steps, omega, lid));
    auto t0 = std::chrono::steady_clock::now();
    for (unsigned s = 0; s < steps; ++s) {
        sim.step();
    }
    double dt = secondsSince(t0);
    std::size_t n = std::size_t(L) * L * L;
    std::printf("{\"seconds\": %.6f, \"glups\": %.6f}\n", dt, 1e-9 * double(n) * steps / dt);
    if (timeOnly) {
        return 0;
    }
    const GridBase<D3Q19Cell, 3> *grid = sim.getGrid();
    // output: member-major (SoA) f[i][z][y][x]
    std::vector<double> result(19 * n);
    for (int z = 0; z < L; ++z) {
        for (int y = 0; y < L; ++y) {
            for (int x = 0; x < L; ++x) {
                D3Q19Cell c = grid->get(Coord<3>(x, y, z));
                std::size_t idx = (std::size_t(z) * L + y) * L + x;
                for (int i = 0; i < 19; ++i) {
                    result[i * n + idx] = c.f[i];
                }
            }
        }
    }
    writeArray(out, result);
    return 0;
}

// ------------------------------------ variable-coefficient diffusion (torus)
// u' = u + sum_faces kf * (u_nb - u), kf = 0.5 * (k + k_nb); faces in the
// order -x, +x, -y, +y, -z, +z.
class VarCoefCell
{
public:
    class API :
        public APITraits::HasStencil<Stencils::VonNeumann<3, 1> >,
        public APITraits::HasTorusTopology<3>
    {};

    inline explicit VarCoefCell(double u = 0, double k = 0) :
        u(u), k(k)
    {}

    template<typename COORD_MAP>
    void update(const COORD_MAP& hood, unsigned /* nanoStep */)
    {
        const VarCoefCell& c = hood[Coord<3>(0, 0, 0)];
        const VarCoefCell& xm = hood[Coord<3>(-1, 0, 0)];
        const VarCoefCell& xp = hood[Coord<3>( 1, 0, 0)];
        const VarCoefCell& ym = hood[Coord<3>( 0, -1, 0)];
        const VarCoefCell& yp = hood[Coord<3>( 0,  1, 0)];
        const VarCoefCell& zm = hood[Coord<3>( 0, 0, -1)];
        const VarCoefCell& zp = hood[Coord<3>( 0, 0,  1)];
        double flux =
            0.5 * (c.k + xm.k) * (xm.u - c.u) +
            0.5 * (c.k + xp.k) * (xp.u - c.u) +
            0.5 * (c.k + ym.k) * (ym.u - c.u) +
            0.5 * (c.k + yp.k) * (yp.u - c.u) +
            0.5 * (c.k + zm.k) * (zm.u - c.u) +
            0.5 * (c.k + zp.k) * (zp.u - c.u);
        u = c.u + flux;
        k = c.k;
    }

    double u;
    double k;
};

class VarCoefInitializer : public SimpleInitializer<VarCoefCell>
{
public:
    VarCoefInitializer(Coord<3> dim, unsigned steps, const std::vector<double> *u, const std::vector<double> *k) :
        SimpleInitializer<VarCoefCell>(dim, steps), u(u), k(k)
    {}

    virtual void grid(GridBase<VarCoefCell, 3> *ret)
    {
        CoordBox<3> box = ret->boundingBox();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) {
            std::size_t idx = (std::size_t(i->z()) * dimensions.y() + i->y()) * dimensions.x() + i->x();
            ret->set(*i, VarCoefCell((*u)[idx], (*k)[idx]));
        }
    }

private:
    const std::vector<double> *u;
    const std::vector<double> *k;
};

template<typename SIM>
static int runVarCoef(Coord<3> dim, unsigned steps, const char *uIn, const char *kIn, const char *out, bool timeOnly)
{
    std::size_t n = std::size_t(dim.x()) * dim.y() * dim.z();
    std::vector<double> u = readArray<double>(uIn, n);
    std::vector<double> k = readArray<double>(kIn, n);
    SIM sim(new VarCoefInitializer(dim, steps, &u, &k));
    auto t0 = std::chrono::steady_clock::now();
    for (unsigned s = 0; s < steps; ++s) {
        sim.step();
    }
    double dt = secondsSince(t0);
    std::printf("{\"seconds\": %.6f, \"glups\": %.6f}\n", dt, 1e-9 * double(n) * steps / dt);
    if (timeOnly) {
        return 0;
    }
    const GridBase<VarCoefCell, 3> *grid = sim.getGrid();
    std::vector<double> result(n);
    for (int z = 0; z < dim.z(); ++z) {
        for (int y = 0; y < dim.y(); ++y) {
            for (int x = 0; x < dim.x(); ++x) {
                result[(std::size_t(z) * dim.y() + y) * dim.x() + x] = grid->get(Coord<3>(x, y, z)).u;
            }
        }
    }
    writeArray(out, result);
    return 0;
}

// ------------------------------------------------------------------- main
static void usage()
{
    std::fprintf(stderr,
        "usage:\n"
        "  lgd_ref jacobi7 cube|torus NX NY NZ STEPS IN.f64 OUT.f64 serial|omp [time]\n"
        "  lgd_ref gol NX NY STEPS IN.u8 OUT.u8 serial|omp [time]\n"
        "  lgd_ref sell C SIGMA N NNZ STEPS ROWPTR.i64 COL.i32 W.f64 X.f64 OUT.f64 serial|omp [time]\n"
        "  lgd_ref sellbuild C SIGMA N NNZ ROWPTR.i64 COL.i32 W.f64 OUTPREFIX\n"
        "  lgd_ref sellcontainer C SIGMA N NNZ ROWPTR.i64 COL.i32 W.f64 OUTPREFIX\n"
        "  lgd_ref lbm L STEPS OMEGA LID OUT.f64 serial|omp [time]\n"
        "  lgd_ref varcoef NX NY NZ STEPS U.f64 K.f64 OUT.f64 serial|omp [time]\n");
}

#define LGD_SELL_DISPATCH(FUNC, ...)                                             \
    if (c == 32 && sigma == 256) return FUNC<32, 256>(__VA_ARGS__);               \
    if (c == 32 && sigma == 1) return FUNC<32, 1>(__VA_ARGS__);                   \
    if (c == 4 && sigma == 1) return FUNC<4, 1>(__VA_ARGS__);                     \
    if (c == 4 && sigma == 60) return FUNC<4, 60>(__VA_ARGS__);                   \
    if (c == 8 && sigma == 16) return FUNC<8, 16>(__VA_ARGS__);                   \
    if (c == 2 && sigma == 1) return FUNC<2, 1>(__VA_ARGS__);                     \
    if (c == 2 && sigma == 4) return FUNC<2, 4>(__VA_ARGS__);                     \
    if (c == 2 && sigma == 8) return FUNC<2, 8>(__VA_ARGS__);                     \
    if (c == 1 && sigma == 1) return FUNC<1, 1>(__VA_ARGS__);                     \
    throw std::invalid_argument("unsupported (C, SIGMA) combination");

template<int C, int SIGMA>
static int runSellSerial(const CSRInput& in, unsigned steps, const char *out, bool timeOnly)
{
    return runSell<C, SIGMA, SerialSimulator<SellDiffusionCell<C, SIGMA> > >(in, steps, out, timeOnly);
}

template<int C, int SIGMA>
static int runSellOMP(const CSRInput& in, unsigned steps, const char *out, bool timeOnly)
{
    return runSell<C, SIGMA, OpenMPSimulator<SellDiffusionCell<C, SIGMA> > >(in, steps, out, timeOnly);
}

static int dispatch(int argc, char **argv)
{
    if (argc < 2) {
        usage();
        return 2;
    }
    std::string cmd(argv[1]);
    auto isOMP = [](const char *s) { return std::string(s) == "omp"; };
    auto timeOnly = [&](int i) { return argc > i && std::string(argv[i]) == "time"; };

    if (cmd == "jacobi7" && argc >= 10) {
        Coord<3> dim(std::atoi(argv[3]), std::atoi(argv[4]), std::atoi(argv[5]));
        unsigned steps = std::atoi(argv[6]);
        bool torus = std::string(argv[2]) == "torus";
        bool omp = isOMP(argv[9]);
        if (torus) {
            return omp ? runJacobi<Jacobi7TorusCell, OpenMPSimulator<Jacobi7TorusCell> >(dim, steps, argv[7], argv[8], timeOnly(10))
                       : runJacobi<Jacobi7TorusCell, SerialSimulator<Jacobi7TorusCell> >(dim, steps, argv[7], argv[8], timeOnly(10));
        }
        return omp ? runJacobi<Jacobi7CubeCell, OpenMPSimulator<Jacobi7CubeCell> >(dim, steps, argv[7], argv[8], timeOnly(10))
                   : runJacobi<Jacobi7CubeCell, SerialSimulator<Jacobi7CubeCell> >(dim, steps, argv[7], argv[8], timeOnly(10));
    }
    if (cmd == "bov" && argc >= 8) {
        Coord<3> dim(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
        return runBov<Jacobi7CubeCell>(dim, std::atoi(argv[5]), argv[6], argv[7]);
    }
    if (cmd == "gol" && argc >= 8) {
        Coord<2> dim(std::atoi(argv[2]), std::atoi(argv[3]));
        unsigned steps = std::atoi(argv[4]);
        return isOMP(argv[7]) ? runGoL<OpenMPSimulator<ConwayCellU8> >(dim, steps, argv[5], argv[6], timeOnly(8))
                              : runGoL<SerialSimulator<ConwayCellU8> >(dim, steps, argv[5], argv[6], timeOnly(8));
    }
    if (cmd == "sell" && argc >= 13) {
        int c = std::atoi(argv[2]);
        int sigma = std::atoi(argv[3]);
        CSRInput in = readCSR(std::atoi(argv[4]), std::atoll(argv[5]), argv[7], argv[8], argv[9], argv[10]);
        unsigned steps = std::atoi(argv[6]);
        if (isOMP(argv[12])) {
            LGD_SELL_DISPATCH(runSellOMP, in, steps, argv[11], timeOnly(13));
        }
        LGD_SELL_DISPATCH(runSellSerial, in, steps, argv[11], timeOnly(13));
    }
    if (cmd == "sellbuild" && argc >= 10) {
        int c = std::atoi(argv[2]);
        int sigma = std::atoi(argv[3]);
        CSRInput in = readCSR(std::atoi(argv[4]), std::atoll(argv[5]), argv[6], argv[7], argv[8], argv[6]);
        LGD_SELL_DISPATCH(dumpSell, in, argv[9]);
    }
    if (cmd == "sellcontainer" && argc >= 10) {
        int c = std::atoi(argv[2]);
        int sigma = std::atoi(argv[3]);
        CSRInput in = readCSR(std::atoi(argv[4]), std::atoll(argv[5]), argv[6], argv[7], argv[8], argv[6]);
        LGD_SELL_DISPATCH(dumpContainer, in, argv[9]);
    }
    if (cmd == "lbm" && argc >= 8) {
        int L = std::atoi(argv[2]);
        unsigned steps = std::atoi(argv[3]);
        double omega = std::atof(argv[4]);
        double lid = std::atof(argv[5]);
        return isOMP(argv[7]) ? runLBM<OpenMPSimulator<D3Q19Cell> >(L, steps, omega, lid, argv[6], timeOnly(8))
                              : runLBM<SerialSimulator<D3Q19Cell> >(L, steps, omega, lid, argv[6], timeOnly(8));
    }
    if (cmd == "varcoef" && argc >= 10) {
        Coord<3> dim(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
        unsigned steps = std::atoi(argv[5]);
        return isOMP(argv[9]) ? runVarCoef<OpenMPSimulator<VarCoefCell> >(dim, steps, argv[6], argv[7], argv[8], timeOnly(10))
                              : runVarCoef<SerialSimulator<VarCoefCell> >(dim, steps, argv[6], argv[7], argv[8], timeOnly(10));
    }
    usage();
    return 2;
}

int main(int argc, char **argv)
{
    try {
        return dispatch(argc, argv);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "lgd_ref: %s\n", e.what());
        return 1;
    }
}
