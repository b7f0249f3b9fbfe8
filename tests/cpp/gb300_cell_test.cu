// User cells on the device: GB300Simulator<CELL> with cells that no kernel
// of the library restates, each running its own update() (or updateCUDA())
// through gb300cell.cuh - what the reference's CUDASimulator does with any
// cell (parallelization/cudasimulator.h:26-236, storage/cudaupdatefunctor.h).
//
//   - the conformance cases of the reference's CUDASimulator test
//     (parallelization/test/unit/cudasimulatortest.h:66-238) with a
//     self-validating TestCell: against the reference's headers its own
//     TestCell and TestInitializer (misc/testcell.h, io/testinitializer.h);
//     without them, a restatement whose update() performs the same checks;
//   - a Jacobi-7 cell and a Game of Life cell written once against the
//     Cell / APITraits API: bit-identical to the library's compiled kernels
//     for the same rules (LGD_CELL_JACOBI7_F64, LGD_CELL_GOL_U8);
//   - a cell with HasSeparateCUDAUpdate: the device runs updateCUDA();
//   - record grids through the C ABI: snapshots, region copies, the edge
//     record, and the calls that are not defined for records.
//
// Compiled by nvcc; prints OK and exits 0 on success, exits 2 without a GPU.
#include <libgeodecomp_gb300/gb300cell.cuh>
#ifdef LGD_GB300_WITH_REFERENCE
#include <libgeodecomp/io/simpleinitializer.h>
#include <libgeodecomp/io/testinitializer.h>
#include <libgeodecomp/misc/testcell.h>
#endif

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace LibGeoDecomp;

static int failures = 0;
#define EXPECT(cond)                                                          \
    do {                                                                      \
        if (!(cond)) {                                                        \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
            ++failures;                                                       \
        }                                                                     \
    } while (0)

// ------------------------------------------- self-validating test cells
#ifdef LGD_GB300_WITH_REFERENCE
template<int DIM, typename STENCIL, typename TOPOLOGY>
using UserTestCell = TestCell<DIM, STENCIL, TOPOLOGY, TestCellHelpers::EmptyAPI, TestCellHelpers::NoOutput>;
template<typename CELL>
using UserTestInitializer = TestInitializer<CELL>;
#else
template<typename STENCIL, int INDEX>
class CheckNeighbour;

// Restatement of the reference's TestCell (misc/testcell.h:132-372): every
// update copies the cell's own previous state, checks each neighbour the
// stencil names (valid, edge flag as the topology says, same cycle and
// dimensions, position wrapped by the topology) and the nano step, then
// counts the cycle; a failed check clears isValid.
template<int DIM, typename STENCIL, typename TOPOLOGY>
class UserTestCell {
public:
    static const unsigned NANO_STEPS = DIM < 3 ? 27 : 3;
    class API : public APITraits::HasTopology<TOPOLOGY>,
                public APITraits::HasNanoSteps<NANO_STEPS>,
                public APITraits::HasStencil<STENCIL> {};

    __host__ __device__ UserTestCell() : cycleCounter(0), isEdgeCell(false), isValid(false), testValue(666) {}
    __host__ __device__ UserTestCell(const Coord<DIM>& pos, const Coord<DIM>& dim, unsigned cycle = 0,
                                     float value = 666) :
        pos(pos), dimensions(dim), cycleCounter(cycle), isEdgeCell(false), isValid(true), testValue(value)
    {
        isEdgeCell = !inBounds(pos);
    }

    __host__ __device__ bool inBounds(const Coord<DIM>& c) const { return !TOPOLOGY::isOutOfBounds(c, dimensions); }

    template<typename HOOD>
    __host__ __device__ void update(const HOOD& hood, unsigned nanoStep)
    {
        *this = hood[FixedCoord<0, 0, 0>()];
        if (isEdgeCell) {
            isValid = false;
            return;
        }
        Stencils::RepeatCuda<STENCIL::VOLUME, CheckNeighbour, STENCIL>()(&isValid, this, hood);
        if (nanoStep >= NANO_STEPS || nanoStep != cycleCounter % NANO_STEPS) {
            isValid = false;
            return;
        }
        ++cycleCounter;
    }

    __host__ __device__ bool checkNeighbour(const UserTestCell& other, const Coord<DIM>& rel) const
    {
        if (!other.isValid) return false;
        const bool shouldBeEdge = !inBounds(pos + rel);
        if (other.isEdgeCell != shouldBeEdge) return false;
        if (shouldBeEdge) return true;
        return other.cycleCounter == cycleCounter && other.dimensions == dimensions &&
               other.pos == TOPOLOGY::normalize(pos + rel, dimensions);
    }

    Coord<DIM> pos;
    Coord<DIM> dimensions;
    unsigned cycleCounter;
    bool isEdgeCell;
    bool isValid;
    float testValue;
};

template<typename STENCIL, int INDEX>
class CheckNeighbour {
public:
    typedef typename STENCIL::template Coords<INDEX> Rel;
    template<typename CELL, typename HOOD>
    __host__ __device__ void operator()(bool *valid, CELL *cell, const HOOD& hood) const
    {
        *valid &= cell->checkNeighbour(hood[Rel()], Coord<CELL::API::Topology::DIM>(Rel()));
    }
};

// Restatement of the reference's TestInitializer (io/testinitializer.h):
// cell (pos, dims, cycle = startStep * NANO_STEPS, testValue = 1 + index),
// edge cell at position -1 with isEdgeCell set.
template<typename CELL>
class UserTestInitializer : public Initializer<CELL> {
public:
    typedef typename Initializer<CELL>::Topology Topology;
    static const int DIM = Topology::DIM;

    UserTestInitializer(const Coord<DIM>& dim, unsigned maxSteps, unsigned startStep = 0) :
        dimensions(dim), maximumSteps(maxSteps), first(startStep)
    {}

    void grid(GridBase<CELL, DIM> *ret)
    {
        const CoordBox<DIM> box = ret->boundingBox();
        const unsigned cycle = first * CELL::NANO_STEPS;
        for (typename CoordBox<DIM>::Iterator i = box.begin(); i != box.end(); ++i) {
            const Coord<DIM> c = Topology::normalize(*i, dimensions);
            long index = 0;
            for (int d = DIM - 1; d >= 0; --d) index = index * dimensions[d] + c[d];
            ret->set(*i, CELL(c, dimensions, cycle, (float)(1 + index)));
        }
        Coord<DIM> minusOne;
        for (int d = 0; d < DIM; ++d) minusOne[d] = -1;
        CELL edgeCell(minusOne, dimensions);
        edgeCell.isEdgeCell = true;
        ret->setEdge(edgeCell);
    }

    Coord<DIM> gridDimensions() const { return dimensions; }
    unsigned maxSteps() const { return maximumSteps; }
    unsigned startStep() const { return first; }

private:
    Coord<DIM> dimensions;
    unsigned maximumSteps;
    unsigned first;
};
#endif

typedef UserTestCell<1, Stencils::VonNeumann<1, 1>, Topologies::Cube<1>::Topology> Cell1dCube;
typedef UserTestCell<1, Stencils::Moore<1, 1>, Topologies::Torus<1>::Topology> Cell1dTorus;
typedef UserTestCell<2, Stencils::VonNeumann<2, 1>, Topologies::Cube<2>::Topology> Cell2dCube;
typedef UserTestCell<2, Stencils::Moore<2, 1>, Topologies::Torus<2>::Topology> Cell2dTorus;
typedef UserTestCell<3, Stencils::VonNeumann<3, 1>, Topologies::Cube<3>::Topology> Cell3dCube;
typedef UserTestCell<3, Stencils::Moore<3, 1>, Topologies::Torus<3>::Topology> Cell3dTorus;
typedef UserTestCell<3, Stencils::Moore<3, 1>, Topologies::Cube<3>::Topology> Cell3dMooreCube;

// the writer of the reference's test (io/testwriter.h:40-62): the event
// sequence, and at every call all cells valid, none the edge cell, all at
// NANO_STEPS * step cycles
template<typename CELL>
class ConformanceWriter : public Writer<CELL> {
public:
    typedef typename Writer<CELL>::GridType GridType;
    static const int DIM = APITraits::SelectTopology<CELL>::Value::DIM;

    ConformanceWriter(unsigned period, unsigned firstStep, unsigned lastStep) : Writer<CELL>("", period), bad(0)
    {
        steps.push_back(firstStep);
        events.push_back(WRITER_INITIALIZED);
        for (unsigned i = firstStep + period - firstStep % period; i < lastStep; i += period) {
            steps.push_back(i);
            events.push_back(WRITER_STEP_FINISHED);
        }
        steps.push_back(lastStep);
        events.push_back(WRITER_ALL_DONE);
    }

    Writer<CELL> *clone() const { return new ConformanceWriter(*this); }

    void stepFinished(const GridType& grid, unsigned step, WriterEvent event)
    {
        if (steps.empty()) {
            ++bad;
            return;
        }
        if (steps.front() != step || events.front() != event) ++bad;
        steps.erase(steps.begin());
        events.erase(events.begin());
        const unsigned expectedCycle = CELL::NANO_STEPS * step;
        if (!grid.getEdge().isEdgeCell) ++bad;
        const CoordBox<DIM> box = grid.boundingBox();
        for (typename CoordBox<DIM>::Iterator i = box.begin(); i != box.end(); ++i) {
            const CELL c = grid.get(*i);
            if (!c.isValid || c.isEdgeCell || c.cycleCounter != expectedCycle) ++bad;
        }
    }

    bool allEventsDone() const { return steps.empty() && events.empty(); }
    long failures() const { return bad; }

private:
    std::vector<unsigned> steps;
    std::vector<WriterEvent> events;
    long bad;
};

template<typename CELL>
static void runConformance(const Coord<APITraits::SelectTopology<CELL>::Value::DIM>& dim, unsigned startStep,
                           unsigned endStep, unsigned period, Coord<3> blockSize = Coord<3>(128, 4, 1))
{
    static_assert(GB300CellTraits<CELL>::KIND == LGD_CELL_RECORD, "the cell must run its own update()");
    GB300Simulator<CELL> sim(new UserTestInitializer<CELL>(dim, endStep, startStep), blockSize);
    ConformanceWriter<CELL> *writer = new ConformanceWriter<CELL>(period, startStep, endStep);
    sim.addWriter(writer);
    sim.run();
    EXPECT(writer->allEventsDone());
    EXPECT(writer->failures() == 0);
    EXPECT(sim.getStep() == endStep);
}

static void testTestCellConformance()
{
    runConformance<Cell1dCube>(Coord<1>(777), 0, 33, 1);
    runConformance<Cell1dTorus>(Coord<1>(666), 40, 70, 3);
    runConformance<Cell2dCube>(Coord<2>(121, 151), 0, 21, 8);
    runConformance<Cell2dTorus>(Coord<2>(141, 131), 35, 60, 6);
    runConformance<Cell3dCube>(Coord<3>(50, 20, 10), 0, 5, 1);
    runConformance<Cell3dTorus>(Coord<3>(50, 20, 10), 28, 38, 3);
    runConformance<Cell2dCube>(Coord<2>(135, 127), 0, 21, 5, Coord<3>(128, 5, 1));
    runConformance<Cell2dTorus>(Coord<2>(251, 91), 0, 21, 6, Coord<3>(128, 5, 1));
    runConformance<Cell3dCube>(Coord<3>(52, 20, 14), 0, 6, 1, Coord<3>(128, 2, 3));
    runConformance<Cell3dTorus>(Coord<3>(54, 20, 13), 0, 7, 1, Coord<3>(64, 2, 3));
    runConformance<Cell3dMooreCube>(Coord<3>(54, 20, 13), 0, 7, 1, Coord<3>(64, 2, 3));
}

// a failed neighbour check must show: a grid whose cells disagree on their
// positions fails validation after the first step
template<typename CELL>
class ShiftedInitializer : public UserTestInitializer<CELL> {
public:
    typedef typename UserTestInitializer<CELL>::Topology Topology;
    static const int DIM = Topology::DIM;
    ShiftedInitializer(const Coord<DIM>& dim, unsigned steps) : UserTestInitializer<CELL>(dim, steps) {}
    void grid(GridBase<CELL, DIM> *ret)
    {
        UserTestInitializer<CELL>::grid(ret);
        Coord<DIM> c;
        CELL cell = ret->get(c);
        cell.pos[0] += 1;
        ret->set(c, cell);
    }
};

static void testBrokenGridIsDetected()
{
    // one step of a 3D Moore cell is three nano steps: the invalid region
    // grows from the shifted cell by one cell per nano step, to 7^3 cells
    GB300Simulator<Cell3dTorus> sim(new ShiftedInitializer<Cell3dTorus>(Coord<3>(20, 20, 20), 1));
    sim.run();
    const GridBase<Cell3dTorus, 3> *g = sim.getGrid();
    long invalid = 0;
    CoordBox<3> box = g->boundingBox();
    for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) invalid += !g->get(*i).isValid;
    EXPECT(invalid == 7 * 7 * 7);
}

// ------------------------------- cells written once against the Cell API
// Jacobi-7 with the library's operation order: temp' = (c + n + s + e + w +
// t + b) * (1/7), n = y - 1, s = y + 1, e = x + 1, w = x - 1, t = z + 1,
// b = z - 1, constant edge cell
class JacobiUserCell {
public:
    class API : public APITraits::HasCubeTopology<3>, public APITraits::HasStencil<Stencils::VonNeumann<3, 1> > {};

    __host__ __device__ explicit JacobiUserCell(double v = 0) : temp(v) {}

    template<typename HOOD>
    __host__ __device__ void update(const HOOD& hood, unsigned)
    {
        double acc = hood[FixedCoord<0, 0, 0>()].temp;
        acc = acc + hood[FixedCoord<0, -1, 0>()].temp;
        acc = acc + hood[FixedCoord<0, 1, 0>()].temp;
        acc = acc + hood[FixedCoord<1, 0, 0>()].temp;
        acc = acc + hood[FixedCoord<-1, 0, 0>()].temp;
        acc = acc + hood[FixedCoord<0, 0, 1>()].temp;
        acc = acc + hood[FixedCoord<0, 0, -1>()].temp;
        temp = acc * (1.0 / 7.0);
    }

    double temp;
};

// neighbourhood over a dense host array with a constant edge value, for
// running the same update() on the host
class HostHood {
public:
    __host__ __device__ HostHood(const double *a, Coord<3> dim, Coord<3> c, double edge) :
        a(a), dim(dim), c(c), edgeCell(edge)
    {}
    // __host__ __device__ only because update() is; it runs on the host
    template<int X, int Y, int Z>
    __host__ __device__ const JacobiUserCell& operator[](FixedCoord<X, Y, Z>) const
    {
        const int x = c.x() + X, y = c.y() + Y, z = c.z() + Z;
        if (x < 0 || y < 0 || z < 0 || x >= dim.x() || y >= dim.y() || z >= dim.z()) return edgeCell;
        cell = JacobiUserCell(a[((std::size_t)z * dim.y() + y) * dim.x() + x]);
        return cell;
    }

private:
    const double *a;
    Coord<3> dim, c;
    JacobiUserCell edgeCell;
    mutable JacobiUserCell cell;
};

// initial values computed once and shared by every run that is compared
// (a host compiler may contract the formula into FMAs differently at
// different call sites)
static std::vector<double> jacobiInitialValues(Coord<3> dim)
{
    std::vector<double> v((std::size_t)dim.prod());
    for (int z = 0; z < dim.z(); ++z)
        for (int y = 0; y < dim.y(); ++y)
            for (int x = 0; x < dim.x(); ++x) {
                v[((std::size_t)z * dim.y() + y) * dim.x() + x] =
                    std::fmod(0.37 * x + 0.11 * y * y + 0.071 * z + 0.013 * x * z, 1.0);
            }
    return v;
}

class JacobiUserInit : public SimpleInitializer<JacobiUserCell> {
public:
    JacobiUserInit(Coord<3> dim, unsigned steps, double edge, const std::vector<double> *values) :
        SimpleInitializer<JacobiUserCell>(dim, steps), edge(edge), values(values), dim(dim)
    {}
    virtual void grid(GridBase<JacobiUserCell, 3> *ret)
    {
        CoordBox<3> box = ret->boundingBox();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) {
            ret->set(*i, JacobiUserCell((*values)[((std::size_t)i->z() * dim.y() + i->y()) * dim.x() + i->x()]));
        }
        ret->setEdge(JacobiUserCell(edge));
    }

private:
    double edge;
    const std::vector<double> *values;
    Coord<3> dim;
};

static void testJacobiUserCellMatchesCompiledKernel()
{
    const Coord<3> dim(45, 23, 17);
    const unsigned steps = 12;
    const double edgeValue = 0.25;
    const std::vector<double> init = jacobiInitialValues(dim);
    GB300Simulator<JacobiUserCell> sim(new JacobiUserInit(dim, steps, edgeValue, &init));
    sim.run();
    const GridBase<JacobiUserCell, 3> *g = sim.getGrid();

    // the same rule through the library's compiled IEEE kernel
    lgd_grid_desc d;
    std::memset(&d, 0, sizeof(d));
    d.dim = 3;
    d.nx = dim.x();
    d.ny = dim.y();
    d.nz = dim.z();
    d.cell = LGD_CELL_JACOBI7_F64;
    d.edge[0] = edgeValue;
    lgd_handle *h = 0;
    gb300Check(lgd_gpu_create(&d, &h));
    const std::size_t n = (std::size_t)dim.prod();
    std::vector<double> u = init;
    gb300Check(lgd_gpu_upload(h, 0, 0, u.data(), n * 8));
    gb300Check(lgd_gpu_step(h, 0, (int)steps));
    gb300Check(lgd_gpu_download(h, 0, 0, u.data(), n * 8));
    gb300Check(lgd_gpu_destroy(h));
    // and the cell's own update() run on the host over the same grid
    std::vector<double> hostA = init, hostB(n);
    for (unsigned s = 0; s < steps; ++s) {
        for (int z = 0; z < dim.z(); ++z)
            for (int y = 0; y < dim.y(); ++y)
                for (int x = 0; x < dim.x(); ++x) {
                    HostHood hood(hostA.data(), dim, Coord<3>(x, y, z), edgeValue);
                    JacobiUserCell c;
                    c.update(hood, 0);
                    hostB[((std::size_t)z * dim.y() + y) * dim.x() + x] = c.temp;
                }
        hostA.swap(hostB);
    }
    long differ = 0, differHost = 0;
    double maxDiff = 0;
    for (int z = 0; z < dim.z(); ++z)
        for (int y = 0; y < dim.y(); ++y)
            for (int x = 0; x < dim.x(); ++x) {
                const std::size_t i = ((std::size_t)z * dim.y() + y) * dim.x() + x;
                const double a = g->get(Coord<3>(x, y, z)).temp;
                differ += std::memcmp(&a, &u[i], 8) != 0;
                differHost += std::memcmp(&a, &hostA[i], 8) != 0;
                maxDiff = std::max(maxDiff, std::fabs(a - u[i]));
            }
    if (differ || differHost) {
        std::printf("Jacobi user cell: %ld cells differ from the compiled kernel (max %g), %ld from the host run\n",
                    differ, maxDiff, differHost);
    }
    EXPECT(differ == 0);
    EXPECT(differHost == 0);
}

// Conway's rule (src/examples/gameoflife/main.cpp:35-58) on a 2D torus
class LifeUserCell {
public:
    class API : public APITraits::HasTorusTopology<2>, public APITraits::HasStencil<Stencils::Moore<2, 1> > {};

    __host__ __device__ explicit LifeUserCell(unsigned char a = 0) : alive(a) {}

    template<typename HOOD>
    __host__ __device__ void update(const HOOD& hood, unsigned)
    {
        int living = hood[FixedCoord<-1, -1>()].alive + hood[FixedCoord<0, -1>()].alive +
                     hood[FixedCoord<1, -1>()].alive + hood[FixedCoord<-1, 0>()].alive + hood[FixedCoord<1, 0>()].alive +
                     hood[FixedCoord<-1, 1>()].alive + hood[FixedCoord<0, 1>()].alive + hood[FixedCoord<1, 1>()].alive;
        const unsigned char self = hood[FixedCoord<0, 0>()].alive;
        alive = self ? (living == 2 || living == 3) : (living == 3);
    }

    unsigned char alive;
};

class LifeUserInit : public SimpleInitializer<LifeUserCell> {
public:
    LifeUserInit(Coord<2> dim, unsigned steps) : SimpleInitializer<LifeUserCell>(dim, steps) {}
    virtual void grid(GridBase<LifeUserCell, 2> *ret)
    {
        CoordBox<2> box = ret->boundingBox();
        for (CoordBox<2>::Iterator i = box.begin(); i != box.end(); ++i) ret->set(*i, LifeUserCell(alive(i->x(), i->y())));
    }
    static unsigned char alive(int x, int y) { return ((x * 7919u + y * 104729u) * 2654435761u >> 29) < 3; }
};

static void testLifeUserCellMatchesCompiledKernel()
{
    const Coord<2> dim(131, 77);
    const unsigned steps = 40;
    GB300Simulator<LifeUserCell> sim(new LifeUserInit(dim, steps));
    sim.run();
    const GridBase<LifeUserCell, 2> *g = sim.getGrid();
    lgd_grid_desc d;
    std::memset(&d, 0, sizeof(d));
    d.dim = 2;
    d.nx = dim.x();
    d.ny = dim.y();
    d.nz = 1;
    d.periodic = 3;
    d.cell = LGD_CELL_GOL_U8;
    lgd_handle *h = 0;
    gb300Check(lgd_gpu_create(&d, &h));
    std::vector<unsigned char> c((std::size_t)dim.prod());
    for (int y = 0; y < dim.y(); ++y)
        for (int x = 0; x < dim.x(); ++x) c[(std::size_t)y * dim.x() + x] = LifeUserInit::alive(x, y);
    gb300Check(lgd_gpu_upload(h, 0, 0, c.data(), c.size()));
    gb300Check(lgd_gpu_step(h, 0, (int)steps));
    gb300Check(lgd_gpu_download(h, 0, 0, c.data(), c.size()));
    gb300Check(lgd_gpu_destroy(h));
    long differ = 0, alive = 0;
    for (int y = 0; y < dim.y(); ++y)
        for (int x = 0; x < dim.x(); ++x) {
            differ += g->get(Coord<2>(x, y)).alive != c[(std::size_t)y * dim.x() + x];
            alive += c[(std::size_t)y * dim.x() + x];
        }
    EXPECT(differ == 0);
    EXPECT(alive > 0);
}

// HasSeparateCUDAUpdate: the device calls updateCUDA(), the host update()
class SeparateCell {
public:
    class API : public APITraits::HasTorusTopology<1>,
                public APITraits::HasStencil<Stencils::Moore<1, 1> >,
                public APITraits::HasSeparateCUDAUpdate {};

    __host__ __device__ explicit SeparateCell(int v = 0) : value(v) {}

    template<typename HOOD>
    __host__ __device__ void update(const HOOD&, unsigned)
    {
        value = -1;
    }

    template<typename HOOD>
    __host__ __device__ void updateCUDA(const HOOD& hood, unsigned)
    {
        value = hood[FixedCoord<-1>()].value + hood[FixedCoord<1>()].value;
    }

    int value;
};

class SeparateInit : public SimpleInitializer<SeparateCell> {
public:
    SeparateInit() : SimpleInitializer<SeparateCell>(Coord<1>(10), 1) {}
    virtual void grid(GridBase<SeparateCell, 1> *ret)
    {
        for (int x = 0; x < 10; ++x) ret->set(Coord<1>(x), SeparateCell(x));
    }
};

static void testSeparateCUDAUpdate()
{
    GB300Simulator<SeparateCell> sim(new SeparateInit());
    sim.run();
    const GridBase<SeparateCell, 1> *g = sim.getGrid();
    for (int x = 0; x < 10; ++x) {
        EXPECT(g->get(Coord<1>(x)).value == (x + 9) % 10 + (x + 1) % 10);
    }
}

// A record grid through the C ABI: uploads, region copies, snapshots, the
// edge record, and the calls that records do not support.
struct Rec {
    double a;
    int b;
    unsigned char c;
};

static void testRecordGridThroughTheABI()
{
    lgd_grid_desc d;
    std::memset(&d, 0, sizeof(d));
    d.dim = 2;
    d.nx = 19;
    d.ny = 7;
    d.nz = 1;
    d.cell = LGD_CELL_RECORD;
    Rec edge = {-1.5, -7, 3};
    lgd_handle *h = 0;
    gb300Check(lgd_gpu_create_records(&d, sizeof(Rec), &edge, &h));
    std::vector<Rec> recs(19 * 7);
    for (int i = 0; i < 19 * 7; ++i) recs[i] = Rec{i * 0.5, i * 3, (unsigned char)i};
    gb300Check(lgd_gpu_upload(h, 0, 0, recs.data(), recs.size() * sizeof(Rec)));
    std::vector<Rec> back(recs.size());
    gb300Check(lgd_gpu_download(h, 0, 0, back.data(), back.size() * sizeof(Rec)));
    EXPECT(std::memcmp(back.data(), recs.data(), recs.size() * sizeof(Rec)) == 0);
    // one streak (x 3 .. 11 of row 4)
    const int streak[4] = {3, 4, 0, 11};
    std::vector<Rec> part(8);
    gb300Check(lgd_gpu_save_region(h, 0, streak, 1, part.data(), part.size() * sizeof(Rec)));
    EXPECT(std::memcmp(part.data(), &recs[4 * 19 + 3], 8 * sizeof(Rec)) == 0);
    for (auto& p : part) p.b = 1000;
    gb300Check(lgd_gpu_load_region(h, 0, streak, 1, part.data(), part.size() * sizeof(Rec)));
    gb300Check(lgd_gpu_download(h, 0, 0, back.data(), back.size() * sizeof(Rec)));
    EXPECT(back[4 * 19 + 3].b == 1000 && back[4 * 19 + 10].b == 1000 && back[4 * 19 + 11].b == recs[4 * 19 + 11].b);
    // snapshot: header, edge record, records
    const char *path = "gb300_cell_test_snapshot.mpiio";
    gb300Check(lgd_gpu_write_snapshot(h, path, 17, 99));
    std::vector<Rec> zero(recs.size());
    std::memset(zero.data(), 0, zero.size() * sizeof(Rec));
    gb300Check(lgd_gpu_upload(h, 0, 0, zero.data(), zero.size() * sizeof(Rec)));
    unsigned step = 0, maxSteps = 0;
    gb300Check(lgd_gpu_read_snapshot(h, path, &step, &maxSteps));
    gb300Check(lgd_gpu_download(h, 0, 0, zero.data(), zero.size() * sizeof(Rec)));
    EXPECT(step == 17 && maxSteps == 99);
    EXPECT(std::memcmp(zero.data(), back.data(), back.size() * sizeof(Rec)) == 0);
    FILE *f = std::fopen(path, "rb");
    Rec fileEdge;
    EXPECT(f != 0 && std::fseek(f, 2 * 4 + 8, SEEK_SET) == 0 && std::fread(&fileEdge, sizeof(Rec), 1, f) == 1);
    if (f) std::fclose(f);
    std::remove(path);
    EXPECT(std::memcmp(&fileEdge, &edge, sizeof(Rec)) == 0);
    // the edge record on the device follows set_edge_record
    Rec edge2 = {2.5, 11, 9};
    gb300Check(lgd_gpu_set_edge_record(h, &edge2, sizeof(Rec)));
    const void *dev = 0;
    gb300Check(lgd_gpu_edge_record_device(h, &dev));
    Rec onDevice;
    EXPECT(cudaMemcpy(&onDevice, dev, sizeof(Rec), cudaMemcpyDeviceToHost) == cudaSuccess);
    EXPECT(std::memcmp(&onDevice, &edge2, sizeof(Rec)) == 0);
    // not defined for records
    EXPECT(lgd_gpu_step(h, 0, 1) == LGD_ERR_UNSUPPORTED);
    double sum = 0;
    EXPECT(lgd_gpu_checksum(h, 0, 0, &sum) == LGD_ERR_UNSUPPORTED);
    EXPECT(lgd_gpu_fill_uniform(h, 0, 0, 1, 1) == LGD_ERR_INVALID);
    EXPECT(lgd_gpu_write_bov(h, 0, "x", 0, "v") == LGD_ERR_UNSUPPORTED);
    EXPECT(lgd_gpu_set_edge_record(h, &edge2, sizeof(Rec) - 1) == LGD_ERR_INVALID);
    gb300Check(lgd_gpu_destroy(h));
    // creation checks
    EXPECT(lgd_gpu_create(&d, &h) == LGD_ERR_INVALID);
    EXPECT(lgd_gpu_create_records(&d, 0, &edge, &h) == LGD_ERR_INVALID);
    EXPECT(lgd_gpu_create_records(&d, LGD_RECORD_MAX_BYTES + 1, &edge, &h) == LGD_ERR_INVALID);
    EXPECT(lgd_gpu_create_records(&d, sizeof(Rec), 0, &h) == LGD_ERR_INVALID);
}

int main()
{
    int n = 0;
    if (lgd_gpu_device_count(&n) != LGD_OK || n == 0) {
        std::printf("no GPU\n");
        return 2;
    }
    testTestCellConformance();
    testBrokenGridIsDetected();
    testJacobiUserCellMatchesCompiledKernel();
    testLifeUserCellMatchesCompiledKernel();
    testSeparateCUDAUpdate();
    testRecordGridThroughTheABI();
    if (failures) {
        std::printf("%d failure(s)\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
