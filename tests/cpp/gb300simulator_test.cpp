// Conformance test of GB300Simulator<CELL> (drop-in for CUDASimulator) with
// unchanged Initializer / Writer / Steerer plugins.  Mirrors what the
// reference's SerialSimulator and CUDASimulator tests check
// (parallelization/test/unit/serialsimulatortest.h,
// parallelization/test/unit/cudasimulatortest.h:66-238, io/testwriter.h:40-62):
// the event sequence, steering, startStep, the result grid.  Expected grids
// come from a plain CPU loop over the same cell rule.
//
// Builds against include/lgd_gpu.h + libgeodecomp_gb300/include (compat
// declarations) or, with -DLGD_GB300_WITH_REFERENCE, against the reference.
#include <libgeodecomp_gb300/gb300simulator.h>
#ifdef LGD_GB300_WITH_REFERENCE
#include <libgeodecomp/io/simpleinitializer.h>
#include <libgeodecomp/io/testinitializer.h>
#include <libgeodecomp/misc/testcell.h>
#endif

#include <cmath>
#include <cstdio>
#include <cstdlib>
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

// ------------------------------------------------------------ Jacobi cell
class JacobiCell {
public:
    class API : public APITraits::HasCubeTopology<3>,
                public APITraits::HasStencil<Stencils::VonNeumann<3, 1> >,
                public APITraits::HasFixedCoordsOnlyUpdate,
                public APITraits::HasUpdateLineX {};

    explicit JacobiCell(double v = 0) : temp(v) {}
    double temp;
};

namespace LibGeoDecomp {
template<>
class GB300CellTraits<JacobiCell> {
public:
    static const int KIND = LGD_CELL_JACOBI7_F64;
    static const int MEMBERS = 1;
    static std::size_t memberSize(int) { return sizeof(double); }
    static void pack(const JacobiCell& c, int, void *dst) { std::memcpy(dst, &c.temp, sizeof(double)); }
    static void unpack(JacobiCell *c, int, const void *src) { std::memcpy(&c->temp, src, sizeof(double)); }
    static double edgeValue(const JacobiCell& c, int) { return c.temp; }
};
}

static double initialValue(int x, int y, int z)
{
    return std::fmod(0.37 * x + 0.11 * y * y + 0.071 * z + 0.013 * x * z, 1.0);
}

class JacobiInit : public SimpleInitializer<JacobiCell> {
public:
    JacobiInit(Coord<3> dim, unsigned steps, unsigned start = 0) :
        SimpleInitializer<JacobiCell>(dim, steps), start(start)
    {}

    virtual void grid(GridBase<JacobiCell, 3> *ret)
    {
        CoordBox<3> box = ret->boundingBox();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) {
            ret->set(*i, JacobiCell(initialValue(i->x(), i->y(), i->z())));
        }
        ret->setEdge(JacobiCell(0.25));
    }

    unsigned startStep() const { return start; }

private:
    unsigned start;
};

// CPU reference of the Jacobi rule with edge value 0.25
static std::vector<double> cpuJacobi(Coord<3> d, int steps)
{
    const int nx = d.x(), ny = d.y(), nz = d.z();
    std::vector<double> a((std::size_t)nx * ny * nz), b(a.size());
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y)
            for (int x = 0; x < nx; ++x) a[((std::size_t)z * ny + y) * nx + x] = initialValue(x, y, z);
    auto at = [&](const std::vector<double>& v, int x, int y, int z) {
        if (x < 0 || y < 0 || z < 0 || x >= nx || y >= ny || z >= nz) return 0.25;
        return v[((std::size_t)z * ny + y) * nx + x];
    };
    for (int s = 0; s < steps; ++s) {
        for (int z = 0; z < nz; ++z)
            for (int y = 0; y < ny; ++y)
                for (int x = 0; x < nx; ++x) {
                    volatile double acc = at(a, x, y, z);
                    acc = acc + at(a, x, y - 1, z);
                    acc = acc + at(a, x, y + 1, z);
                    acc = acc + at(a, x + 1, y, z);
                    acc = acc + at(a, x - 1, y, z);
                    acc = acc + at(a, x, y, z + 1);
                    acc = acc + at(a, x, y, z - 1);
                    b[((std::size_t)z * ny + y) * nx + x] = acc * (1.0 / 7.0);
                }
        a.swap(b);
    }
    return a;
}

struct Event {
    unsigned step;
    int event;
    double sum;
};

class RecordingWriter : public Writer<JacobiCell> {
public:
    RecordingWriter(unsigned period, std::vector<Event> *log) : Writer<JacobiCell>("rec", period), log(log) {}
    Writer<JacobiCell> *clone() const { return new RecordingWriter(period, log); }

    void stepFinished(const GridType& grid, unsigned step, WriterEvent event)
    {
        double s = 0;
        CoordBox<3> box = grid.boundingBox();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) s += grid.get(*i).temp;
        log->push_back(Event{step, (int)event, s});
    }

private:
    std::vector<Event> *log;
};

class StopSteerer : public Steerer<JacobiCell> {
public:
    StopSteerer(unsigned period, unsigned stopAt, std::vector<Event> *log) :
        Steerer<JacobiCell>(period), stopAt(stopAt), log(log)
    {}

    void nextStep(GridType *grid, const Region<3>&, const Coord<3>&, unsigned step, SteererEvent event, std::size_t,
                  bool, SteererFeedback *feedback)
    {
        log->push_back(Event{step, 100 + (int)event, 0.0});
        if (event == STEERER_NEXT_STEP && step >= stopAt) feedback->endSimulation();
        (void)grid;
    }

private:
    unsigned stopAt;
    std::vector<Event> *log;
};

// sets one cell every time it runs: the change must reach the device
class PokeSteerer : public Steerer<JacobiCell> {
public:
    explicit PokeSteerer(unsigned period) : Steerer<JacobiCell>(period) {}
    void nextStep(GridType *grid, const Region<3>&, const Coord<3>&, unsigned, SteererEvent event, std::size_t, bool,
                  SteererFeedback *)
    {
        if (event == STEERER_NEXT_STEP) grid->set(Coord<3>(1, 2, 3), JacobiCell(1000.0));
    }
};

static void testRunEventsAndResult()
{
    const Coord<3> dim(21, 13, 9);
    std::vector<Event> log;
    GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 12));
    sim.addWriter(new RecordingWriter(5, &log));
    sim.run();
    EXPECT(sim.getStep() == 12);
    // INITIALIZED@0, STEP_FINISHED@5, @10, ALL_DONE@12
    EXPECT(log.size() == 4);
    if (log.size() == 4) {
        EXPECT(log[0].step == 0 && log[0].event == WRITER_INITIALIZED);
        EXPECT(log[1].step == 5 && log[1].event == WRITER_STEP_FINISHED);
        EXPECT(log[2].step == 10 && log[2].event == WRITER_STEP_FINISHED);
        EXPECT(log[3].step == 12 && log[3].event == WRITER_ALL_DONE);
    }
    std::vector<double> ref = cpuJacobi(dim, 12);
    const GridBase<JacobiCell, 3> *g = sim.getGrid();
    std::size_t i = 0;
    int mismatches = 0;
    for (int z = 0; z < dim.z(); ++z)
        for (int y = 0; y < dim.y(); ++y)
            for (int x = 0; x < dim.x(); ++x, ++i) {
                if (g->get(Coord<3>(x, y, z)).temp != ref[i]) ++mismatches;
            }
    EXPECT(mismatches == 0);
}

static void testSteererEndsRunAndStartStep()
{
    const Coord<3> dim(8, 7, 6);
    std::vector<Event> log;
    GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 40, 28));
    sim.addSteerer(new StopSteerer(1, 33, &log));
    sim.run();
    // steps 28..32 run, the steerer asks to stop before step 33 runs
    EXPECT(sim.getStep() == 34);
    EXPECT(!log.empty() && log.front().event == 100 + STEERER_INITIALIZED && log.front().step == 28);
    EXPECT(!log.empty() && log.back().event == 100 + STEERER_ALL_DONE);
}

static void testSteeringReachesDevice()
{
    const Coord<3> dim(6, 6, 6);
    GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 3));
    sim.addSteerer(new PokeSteerer(1));
    sim.step();
    // the poke happened before the step: the neighbours of (1,2,3) see it
    const double n = sim.getGrid()->get(Coord<3>(2, 2, 3)).temp;
    EXPECT(n > 100.0);
}

static void testManualStepsMatchCpu()
{
    const Coord<3> dim(17, 5, 11);
    GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 100));
    for (int s = 0; s < 7; ++s) sim.step();
    std::vector<double> ref = cpuJacobi(dim, 7);
    const GridBase<JacobiCell, 3> *g = sim.getGrid();
    std::size_t i = 0;
    int mismatches = 0;
    for (int z = 0; z < dim.z(); ++z)
        for (int y = 0; y < dim.y(); ++y)
            for (int x = 0; x < dim.x(); ++x, ++i) mismatches += (g->get(Coord<3>(x, y, z)).temp != ref[i]);
    EXPECT(mismatches == 0);
    EXPECT(sim.getStep() == 7);
}

// A writer that reads one cell per call: the view it gets copies one z plane
// per call, not the grid.
class ProbeWriter : public Writer<JacobiCell> {
public:
    ProbeWriter(unsigned period, Coord<3> probe, std::vector<double> *seen) :
        Writer<JacobiCell>("probe", period), probe(probe), seen(seen)
    {}
    Writer<JacobiCell> *clone() const { return new ProbeWriter(period, probe, seen); }
    void stepFinished(const GridType& grid, unsigned, WriterEvent) { seen->push_back(grid.get(probe).temp); }

private:
    Coord<3> probe;
    std::vector<double> *seen;
};

static void testWriterReadsOnlyWhatItTouches()
{
    const Coord<3> dim(19, 11, 17);
    const Coord<3> probe(5, 7, 9);
    std::vector<double> seen;
    GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 9));
    sim.addWriter(new ProbeWriter(3, probe, &seen));
    sim.run();
    // INITIALIZED@0, STEP_FINISHED@3, @6, ALL_DONE@9
    EXPECT(seen.size() == 4);
    const int at[4] = {0, 3, 6, 9};
    for (std::size_t k = 0; k < seen.size() && k < 4; ++k) {
        std::vector<double> ref = cpuJacobi(dim, at[k]);
        EXPECT(seen[k] == ref[((std::size_t)probe.z() * dim.y() + probe.y()) * dim.x() + probe.x()]);
    }
    // the initial grid is on the host; afterwards one plane per call
    const std::size_t plane = (std::size_t)dim.x() * dim.y() * sizeof(double);
    EXPECT(sim.writerBytesFetched() == 3 * plane);
    // getGrid() still gives the whole grid, current
    std::vector<double> ref = cpuJacobi(dim, 9);
    const GridBase<JacobiCell, 3> *g = sim.getGrid();
    int mismatches = 0;
    std::size_t i = 0;
    for (int z = 0; z < dim.z(); ++z)
        for (int y = 0; y < dim.y(); ++y)
            for (int x = 0; x < dim.x(); ++x, ++i) mismatches += (g->get(Coord<3>(x, y, z)).temp != ref[i]);
    EXPECT(mismatches == 0);
}

// BOV snapshots straight from the device: at the start and every 4 steps,
// the data file holds the grid of that step
static void testBovWriterFromDevice()
{
    const Coord<3> dim(12, 9, 7);
    const std::string prefix = "gb300_bov_test";
    {
        GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 8));
        sim.addWriter(new GB300BOVWriter<JacobiCell>(&sim, 0, "temp", prefix, 4));
        sim.run();
    }
    const std::size_t n = (std::size_t)dim.x() * dim.y() * dim.z();
    const int at[3] = {0, 4, 8};
    for (int k = 0; k < 3; ++k) {
        char name[128];
        std::snprintf(name, sizeof(name), "%s.%05d.data", prefix.c_str(), at[k]);
        std::vector<double> got(n);
        FILE *f = std::fopen(name, "rb");
        EXPECT(f != nullptr);
        if (!f) continue;
        EXPECT(std::fread(got.data(), sizeof(double), n, f) == n);
        std::fclose(f);
        std::remove(name);
        std::snprintf(name, sizeof(name), "%s.%05d.bov", prefix.c_str(), at[k]);
        EXPECT(std::remove(name) == 0);
        EXPECT(got == cpuJacobi(dim, at[k]));
    }
}

// Checkpoints and restart, as the reference's MPIIOWriter / MPIIOInitializer
// tests check them (io/test/parallel_mpi_1/mpiiowritertest.h,
// io/test/parallel_mpi_2/mpiioinitializertest.h): files named prefix +
// 5-digit step + ".mpiio" at steps 0, 4, ..., 20 and the last step 21, each
// with its step and the maximum in the header and the grid of that step;
// a simulation restarted from step 12 starts there and ends with the grid
// of the uninterrupted run.
static void testSnapshotWriterAndRestart()
{
    const Coord<3> dim(12, 9, 7);
    const std::string prefix = "gb300_snapshot_test";
    const std::size_t n = (std::size_t)dim.x() * dim.y() * dim.z();
    {
        GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 21));
        GB300SnapshotWriter<JacobiCell> *writer = new GB300SnapshotWriter<JacobiCell>(&sim, prefix, 4, 21);
        EXPECT(writer->filename(1234) == prefix + "01234.mpiio");
        sim.addWriter(writer);
        sim.run();
    }
    const unsigned at[7] = {0, 4, 8, 12, 16, 20, 21};
    for (int k = 0; k < 7; ++k) {
        char name[128];
        std::snprintf(name, sizeof(name), "%s%05u.mpiio", prefix.c_str(), at[k]);
        int dims[3] = {0, 0, 0};
        unsigned step = 99, maxSteps = 99;
        EXPECT(lgd_snapshot_info(name, 3, dims, &step, &maxSteps) == LGD_OK);
        EXPECT(dims[0] == 12 && dims[1] == 9 && dims[2] == 7);
        EXPECT(step == at[k] && maxSteps == 21);
        // header: 3 ints, 2 unsigned, the edge cell; then the cells
        std::vector<double> got(n + 1);
        FILE *f = std::fopen(name, "rb");
        EXPECT(f != nullptr);
        if (!f) continue;
        EXPECT(std::fseek(f, 20, SEEK_SET) == 0);
        EXPECT(std::fread(got.data(), sizeof(double), n + 1, f) == n + 1);
        EXPECT(std::fgetc(f) == EOF);
        std::fclose(f);
        EXPECT(got[0] == 0.25);
        EXPECT(std::vector<double>(got.begin() + 1, got.end()) == cpuJacobi(dim, (int)at[k]));
    }
    {
        GB300Simulator<JacobiCell> sim(new GB300SnapshotInitializer<JacobiCell>(prefix + "00012.mpiio"));
        EXPECT(sim.getStep() == 12);
        sim.run();
        EXPECT(sim.getStep() == 21);
        const GridBase<JacobiCell, 3> *grid = sim.getGrid();
        const std::vector<double> expect = cpuJacobi(dim, 21);
        bool same = true;
        for (int z = 0; z < dim.z(); ++z)
            for (int y = 0; y < dim.y(); ++y)
                for (int x = 0; x < dim.x(); ++x) {
                    same &= grid->get(Coord<3>(x, y, z)).temp == expect[((std::size_t)z * dim.y() + y) * dim.x() + x];
                }
        EXPECT(same);
        EXPECT(grid->getEdge().temp == 0.25);
    }
    for (int k = 0; k < 7; ++k) {
        char name[128];
        std::snprintf(name, sizeof(name), "%s%05u.mpiio", prefix.c_str(), at[k]);
        EXPECT(std::remove(name) == 0);
    }
}

// gatherStatistics(): SerialSimulator's categories, filled - total time
// covers compute, input and output, compute the device's work
static void testStatistics()
{
    const Coord<3> dim(64, 48, 40);
    std::vector<Event> log;
    GB300Simulator<JacobiCell> sim(new JacobiInit(dim, 30));
    sim.addWriter(new RecordingWriter(10, &log));
    sim.run();
    EXPECT(log.size() == 4);
    const std::vector<Chronometer> stats = sim.gatherStatistics();
    EXPECT(stats.size() == 1);
    const Chronometer& c = stats[0];
    EXPECT(c.interval<TimeTotal>() > 0);
    EXPECT(c.interval<TimeCompute>() > 0);
    EXPECT(c.interval<TimeOutput>() > 0);
    EXPECT(c.interval<TimeInput>() >= 0);
    EXPECT(c.interval<TimeCompute>() + c.interval<TimeInput>() + c.interval<TimeOutput>() <=
           c.interval<TimeTotal>() * 1.001 + 1e-6);
}

static void testBadBlockSizeThrows()
{
    bool thrown = false;
    try {
        GB300Simulator<JacobiCell> sim(new JacobiInit(Coord<3>(4, 4, 4), 1), Coord<3>(0, 1, 1));
    } catch (const std::invalid_argument&) {
        thrown = true;
    }
    EXPECT(thrown);
}

// ------------------------------------------- self-validating test cells
// The conformance cases of the reference's CUDASimulator test
// (parallelization/test/unit/cudasimulatortest.h:66-238): TestCell grids in
// 1D, 2D and 3D, cube and torus, odd sizes, start steps other than 0 and
// the block sizes of its multi-wavefront cases.  Every cell checks every
// neighbour it is handed (position, dimensions, cycle, edge flag) and the
// nano step on the device (LGD_CELL_TEST); the writer asserts the event
// sequence and, at every call, that all cells are valid, none claims to be
// the edge cell and all counted NANO_STEPS * step cycles
// (io/testwriter.h:40-62, misc/testhelper.h:144-182).  Against the
// reference's headers the cell and initializer are the reference's own
// TestCell and TestInitializer; without them, restatements of both.
#ifdef LGD_GB300_WITH_REFERENCE
template<int DIM, typename STENCIL, typename TOPOLOGY>
using GBTestCell = TestCell<DIM, STENCIL, TOPOLOGY, TestCellHelpers::EmptyAPI, TestCellHelpers::NoOutput>;
template<typename CELL>
using GBTestInitializer = TestInitializer<CELL>;
#else
template<int DIM, typename STENCIL, typename TOPOLOGY>
class GBTestCell {
public:
    static const unsigned NANO_STEPS = DIM < 3 ? 27 : 3;
    class API : public APITraits::HasTopology<TOPOLOGY>,
                public APITraits::HasNanoSteps<NANO_STEPS>,
                public APITraits::HasStencil<STENCIL> {};

    GBTestCell() : cycleCounter(0), isEdgeCell(false), isValid(false), testValue(666) {}
    GBTestCell(const Coord<DIM>& pos, const Coord<DIM>& dim, unsigned cycle = 0, float value = 666) :
        pos(pos), dimensions(dim), cycleCounter(cycle), isEdgeCell(false), isValid(true), testValue(value)
    {}
    bool valid() const { return isValid; }
    bool edgeCell() const { return isEdgeCell; }

    Coord<DIM> pos;
    Coord<DIM> dimensions;
    unsigned cycleCounter;
    bool isEdgeCell;
    bool isValid;
    float testValue;
};

template<typename CELL>
class GBTestInitializer : public Initializer<CELL> {
public:
    typedef typename Initializer<CELL>::Topology Topology;
    static const int DIM = Topology::DIM;

    GBTestInitializer(const Coord<DIM>& dim, unsigned maxSteps, unsigned startStep = 0) :
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

typedef GBTestCell<1, Stencils::VonNeumann<1, 1>, Topologies::Cube<1>::Topology> TestCell1dCube;
typedef GBTestCell<1, Stencils::Moore<1, 1>, Topologies::Torus<1>::Topology> TestCell1dTorus;
typedef GBTestCell<2, Stencils::VonNeumann<2, 1>, Topologies::Cube<2>::Topology> TestCell2dCube;
typedef GBTestCell<2, Stencils::Moore<2, 1>, Topologies::Torus<2>::Topology> TestCell2dTorus;
typedef GBTestCell<3, Stencils::VonNeumann<3, 1>, Topologies::Cube<3>::Topology> TestCell3dCube;
typedef GBTestCell<3, Stencils::Moore<3, 1>, Topologies::Torus<3>::Topology> TestCell3dTorus;
// the SoA test cells (Moore, 3D), whose cases are fixme in the reference's
// test (cudasimulatortest.h:211-239)
#ifdef LGD_GB300_WITH_REFERENCE
typedef TestCell<3, Stencils::Moore<3, 1>, Topologies::Cube<3>::Topology, TestCellHelpers::SoAAPI,
                 TestCellHelpers::NoOutput> TestCellSoA3dCube;
typedef TestCell<3, Stencils::Moore<3, 1>, Topologies::Torus<3>::Topology, TestCellHelpers::SoAAPI,
                 TestCellHelpers::NoOutput> TestCellSoA3dTorus;
#else
typedef GBTestCell<3, Stencils::Moore<3, 1>, Topologies::Cube<3>::Topology> TestCellSoA3dCube;
typedef TestCell3dTorus TestCellSoA3dTorus;
#endif

namespace LibGeoDecomp {
template<> class GB300CellTraits<TestCell1dCube> : public GB300TestCellTraits<TestCell1dCube> {};
template<> class GB300CellTraits<TestCell1dTorus> : public GB300TestCellTraits<TestCell1dTorus> {};
template<> class GB300CellTraits<TestCell2dCube> : public GB300TestCellTraits<TestCell2dCube> {};
template<> class GB300CellTraits<TestCell2dTorus> : public GB300TestCellTraits<TestCell2dTorus> {};
template<> class GB300CellTraits<TestCell3dCube> : public GB300TestCellTraits<TestCell3dCube> {};
template<> class GB300CellTraits<TestCell3dTorus> : public GB300TestCellTraits<TestCell3dTorus> {};
template<> class GB300CellTraits<TestCellSoA3dCube> : public GB300TestCellTraits<TestCellSoA3dCube> {};
#ifdef LGD_GB300_WITH_REFERENCE
template<> class GB300CellTraits<TestCellSoA3dTorus> : public GB300TestCellTraits<TestCellSoA3dTorus> {};
#endif
}

template<typename CELL>
class ConformanceWriter : public Writer<CELL> {
public:
    typedef typename Writer<CELL>::GridType GridType;
    static const int DIM = APITraits::SelectTopology<CELL>::Value::DIM;

    ConformanceWriter(unsigned period, unsigned firstStep, unsigned lastStep) :
        Writer<CELL>("", period), bad(0)
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
        if (!grid.getEdge().isEdgeCell || !grid.getEdge().isValid) ++bad;
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
    GB300Simulator<CELL> sim(new GBTestInitializer<CELL>(dim, endStep, startStep), blockSize);
    ConformanceWriter<CELL> *writer = new ConformanceWriter<CELL>(period, startStep, endStep);
    sim.addWriter(writer);
    sim.run();
    EXPECT(writer->allEventsDone());
    EXPECT(writer->failures() == 0);
    EXPECT(sim.getStep() == endStep);
}

static void testTestCellConformance()
{
    runConformance<TestCell1dCube>(Coord<1>(777), 0, 33, 1);
    runConformance<TestCell1dTorus>(Coord<1>(666), 40, 70, 3);
    runConformance<TestCell2dCube>(Coord<2>(121, 151), 0, 21, 8);
    runConformance<TestCell2dTorus>(Coord<2>(141, 131), 35, 60, 6);
    runConformance<TestCell3dCube>(Coord<3>(50, 20, 10), 0, 5, 1);
    runConformance<TestCell3dTorus>(Coord<3>(50, 20, 10), 28, 38, 3);
    // the multiple-wavefront cases (block sizes are validated, the library
    // picks its own launch shapes)
    runConformance<TestCell2dCube>(Coord<2>(135, 127), 0, 21, 5, Coord<3>(128, 5, 1));
    runConformance<TestCell2dTorus>(Coord<2>(251, 91), 0, 21, 6, Coord<3>(128, 5, 1));
    runConformance<TestCell3dCube>(Coord<3>(52, 20, 14), 0, 6, 1, Coord<3>(128, 2, 3));
    runConformance<TestCell3dTorus>(Coord<3>(54, 20, 13), 0, 7, 1, Coord<3>(64, 2, 3));
    // the SoA cells, with the writer the reference's test leaves out
    runConformance<TestCellSoA3dCube>(Coord<3>(54, 20, 13), 0, 7, 1, Coord<3>(64, 2, 3));
    runConformance<TestCellSoA3dTorus>(Coord<3>(54, 20, 13), 0, 7, 1, Coord<3>(64, 2, 3));
}

// Failures made on the host (no device fault): a Writer that throws in the
// middle of run(), an Initializer that throws while filling the grid, and
// one whose grid is empty.  The exception reaches the caller, the simulator
// is destroyed cleanly, and the library keeps working afterwards.
class ThrowingWriter : public Writer<JacobiCell> {
public:
    explicit ThrowingWriter(unsigned at) : Writer<JacobiCell>("throw", 1), at(at) {}
    Writer<JacobiCell> *clone() const { return new ThrowingWriter(at); }
    void stepFinished(const GridType&, unsigned step, WriterEvent)
    {
        if (step == at) throw std::runtime_error("writer failed on purpose");
    }

private:
    unsigned at;
};

class ThrowingInit : public JacobiInit {
public:
    ThrowingInit() : JacobiInit(Coord<3>(8, 8, 8), 4) {}
    void grid(GridBase<JacobiCell, 3> *) { throw std::runtime_error("initializer failed on purpose"); }
};

static void testHostFailuresPropagate()
{
    bool thrown = false;
    {
        GB300Simulator<JacobiCell> sim(new JacobiInit(Coord<3>(16, 12, 10), 10));
        sim.addWriter(new ThrowingWriter(6));
        try {
            sim.run();
        } catch (const std::runtime_error& e) {
            thrown = std::string(e.what()) == "writer failed on purpose";
        }
        EXPECT(thrown);
        EXPECT(sim.getStep() == 6);
    }
    thrown = false;
    try {
        GB300Simulator<JacobiCell> sim(new ThrowingInit());
    } catch (const std::runtime_error& e) {
        thrown = std::string(e.what()) == "initializer failed on purpose";
    }
    EXPECT(thrown);
    thrown = false;
    try {
        GB300Simulator<JacobiCell> sim(new JacobiInit(Coord<3>(0, 4, 4), 3));
    } catch (const std::exception&) {
        thrown = true;
    }
    EXPECT(thrown);
    // the library still works after the failures
    GB300Simulator<JacobiCell> sim(new JacobiInit(Coord<3>(12, 9, 7), 5));
    sim.run();
    const GridBase<JacobiCell, 3> *grid = sim.getGrid();
    const std::vector<double> expect = cpuJacobi(Coord<3>(12, 9, 7), 5);
    EXPECT(grid->get(Coord<3>(3, 4, 5)).temp == expect[(5 * 9 + 4) * 12 + 3]);
}

// ----------------------------------------------------- Game of Life (2D torus)
class LifeCell {
public:
    class API : public APITraits::HasTorusTopology<2>, public APITraits::HasStencil<Stencils::Moore<2, 1> > {};
    explicit LifeCell(unsigned char a = 0) : alive(a) {}
    unsigned char alive;
};

namespace LibGeoDecomp {
template<>
class GB300CellTraits<LifeCell> {
public:
    static const int KIND = LGD_CELL_GOL_U8;
    static const int MEMBERS = 1;
    static std::size_t memberSize(int) { return 1; }
    static void pack(const LifeCell& c, int, void *dst) { *(unsigned char *)dst = c.alive; }
    static void unpack(LifeCell *c, int, const void *src) { c->alive = *(const unsigned char *)src; }
    static double edgeValue(const LifeCell& c, int) { return c.alive; }
};
}

class GliderInit : public SimpleInitializer<LifeCell> {
public:
    GliderInit() : SimpleInitializer<LifeCell>(Coord<2>(37, 29), 4 * 37) {}
    virtual void grid(GridBase<LifeCell, 2> *ret)
    {
        const int g[5][2] = {{1, 0}, {2, 1}, {0, 2}, {1, 2}, {2, 2}};
        for (int i = 0; i < 5; ++i) ret->set(Coord<2>(g[i][0] + 3, g[i][1] + 4), LifeCell(1));
    }
};

static void testGliderCrossesTorus()
{
    // a glider moves (1, 1) every 4 generations; after 4 * 37 * 29 / gcd...
    // use 4 * 37 generations: it moves 37 cells in x (one full turn) and 37
    // in y (= 8 mod 29)
    GB300Simulator<LifeCell> sim(new GliderInit());
    sim.run();
    const GridBase<LifeCell, 2> *g = sim.getGrid();
    const int gl[5][2] = {{1, 0}, {2, 1}, {0, 2}, {1, 2}, {2, 2}};
    int alive = 0, onGlider = 0;
    CoordBox<2> box = g->boundingBox();
    for (CoordBox<2>::Iterator i = box.begin(); i != box.end(); ++i) alive += g->get(*i).alive;
    for (int i = 0; i < 5; ++i) {
        onGlider += g->get(Coord<2>((gl[i][0] + 3 + 37) % 37, (gl[i][1] + 4 + 37) % 29)).alive;
    }
    EXPECT(alive == 5);
    EXPECT(onGlider == 5);
}

int main()
{
    int n = 0;
    if (lgd_gpu_device_count(&n) != LGD_OK || n == 0) {
        std::printf("no GPU\n");
        return 2;
    }
    testRunEventsAndResult();
    testSteererEndsRunAndStartStep();
    testSteeringReachesDevice();
    testManualStepsMatchCpu();
    testBadBlockSizeThrows();
    testWriterReadsOnlyWhatItTouches();
    testBovWriterFromDevice();
    testSnapshotWriterAndRestart();
    testGliderCrossesTorus();
    testTestCellConformance();
    testStatistics();
    testHostFailuresPropagate();
    if (failures) {
        std::printf("%d failure(s)\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
