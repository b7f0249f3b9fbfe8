// GB300Simulator<CELL>: drop-in for LibGeoDecomp's CUDASimulator<CELL>
// (parallelization/cudasimulator.h:298-596) on top of the C ABI in
// include/lgd_gpu.h.
//
// The Simulator / MonolithicSimulator surface, the plugin calls and their
// order are those of the reference's single-node simulators
// (parallelization/serialsimulator.h:48-180): Steerers run before a step
// when stepNum % period == 0 (and with STEERER_INITIALIZED / ALL_DONE around
// run()), Writers get WRITER_INITIALIZED at the start step,
// WRITER_STEP_FINISHED when step % period == 0 and WRITER_ALL_DONE at
// maxSteps; SteererFeedback::endSimulation() stops run(); startStep() is
// honoured.  The simulator owns the Initializer, Writers and Steerers.
// gatherStatistics() reports SerialSimulator's chronometer categories
// (total, compute, input, output; serialsimulator.h:78-164), compute time
// including the device's (the reference's CUDASimulator leaves them 0).
//
// Differences from CUDASimulator, all on the host <-> device path:
//   - Writers get a read-only view that copies planes of the grid to the
//     host when they touch them; Steerers and getGrid() get the whole grid,
//     copied only when the device has moved on (the reference copies the
//     whole grid every time a writer asks, :490-497);
//   - after Steerers ran, the host grid is uploaded again, so steering
//     changes reach the device (the reference leaves this as a fixme,
//     :450-454);
//   - blockSize is accepted for signature compatibility and validated; the
//     library picks its own launch shapes;
//   - run() hands the steps between two plugin calls to the library in one
//     call (which may fuse them into fewer passes over memory); the plugin
//     calls themselves are unchanged.
//
// A cell runs on the device in one of two ways; the cell class and its API
// traits stay as they are either way:
//   - bound to a kernel compiled into the library by specialising
//     GB300CellTraits<CELL> (see below): the fast paths (TMA plane rings,
//     temporal blocking), for the cells the library restates;
//   - any other cell runs its own update() / updateCUDA() on the device, as
//     under the reference's CUDASimulator: the translation unit includes
//     gb300cell.cuh and is compiled by nvcc; the grid is a record grid
//     (LGD_CELL_RECORD, one sizeof(CELL) record per cell).
//
// Build with -DLGD_GB300_WITH_REFERENCE and the reference's include paths to
// plug into a LibGeoDecomp application; without it the declarations in
// compat.h stand in for the reference's.
#ifndef LGD_GB300_SIMULATOR_H
#define LGD_GB300_SIMULATOR_H

#ifdef LGD_GB300_WITH_REFERENCE
#include <libgeodecomp/io/initializer.h>
#include <libgeodecomp/io/steerer.h>
#include <libgeodecomp/io/writer.h>
#include <libgeodecomp/parallelization/monolithicsimulator.h>
#include <libgeodecomp/storage/displacedgrid.h>
#else
#include "compat.h"
#endif

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "lgd_gpu.h"

namespace LibGeoDecomp {

// Binding of a cell class to a cell kind of the GPU library.  A
// specialisation provides
//   static const int KIND;                        LGD_CELL_* of lgd_gpu.h
//   static const int MEMBERS;                     SoA members, in the kind's order
//   static std::size_t memberSize(int m);         bytes of member m
//   static void pack(const CELL& c, int m, void *dst);     member m -> dst
//   static void unpack(CELL *c, int m, const void *src);   src -> member m
//   static double edgeValue(const CELL& c, int m);         member m as double
// Without a specialisation the cell is a record cell: its grid holds the
// CELL objects themselves and its own update() runs on the device
// (gb300cell.cuh).
template<typename CELL>
class GB300CellTraits {
public:
    static const int KIND = LGD_CELL_RECORD;
    static const int MEMBERS = 1;
    static std::size_t memberSize(int) { return sizeof(CELL); }
    static void pack(const CELL& c, int, void *dst) { std::memcpy(dst, static_cast<const void *>(&c), sizeof(CELL)); }
    static void unpack(CELL *c, int, const void *src) { std::memcpy(static_cast<void *>(c), src, sizeof(CELL)); }
    static double edgeValue(const CELL&, int) { return 0.0; }
};

// Advances a device grid: compiled kinds through lgd_gpu_step; record cells
// through their own update() in a kernel that gb300cell.cuh defines (a
// translation unit with a record cell must include it and be compiled by
// nvcc; otherwise GB300DeviceStep<CELL, true> stays incomplete).
template<typename CELL, bool RECORD = (GB300CellTraits<CELL>::KIND == LGD_CELL_RECORD)>
struct GB300DeviceStep {
    static void run(lgd_handle *h, unsigned nanoStep, int count);
};

template<typename CELL>
struct GB300DeviceStep<CELL, true>;

// Optional in a binding: static int descFlags() - the grid descriptor's
// flags (cell kinds that take some, LGD_CELL_TEST); 0 when absent.
template<typename TRAITS>
class GB300DescFlags {
    template<typename U>
    static char probe(decltype(&U::descFlags));
    template<typename U>
    static long probe(...);
    template<typename U, bool HAS>
    struct Get {
        static int value() { return U::descFlags(); }
    };
    template<typename U>
    struct Get<U, false> {
        static int value() { return 0; }
    };

public:
    static int value() { return Get<TRAITS, sizeof(probe<TRAITS>(0)) == 1>::value(); }
};

// Binding of a self-validating test cell to LGD_CELL_TEST: any class with
// the members of the reference's TestCell (misc/testcell.h:159-164: pos,
// dimensions, cycleCounter, isEdgeCell, isValid, testValue), its stencil
// (Moore or von Neumann, radius 1) and NANO_STEPS.  Specialise
// GB300CellTraits<TestCellType> by deriving from it.
template<typename CELL>
class GB300TestCellTraits {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    typedef typename APITraits::SelectStencil<CELL>::Value Stencil;
    static const int DIM = Topology::DIM;
    static const int KIND = LGD_CELL_TEST;
    static const int MEMBERS = 1;
    static std::size_t memberSize(int) { return sizeof(lgd_test_record); }
    static int descFlags()
    {
        const bool vonNeumann = (DIM > 1) && (Stencil::VOLUME == 2 * DIM + 1);
        return (vonNeumann ? LGD_TEST_VON_NEUMANN : 0) | LGD_TEST_NANO_STEPS((int)CELL::NANO_STEPS);
    }
    static void pack(const CELL& c, int, void *dst)
    {
        lgd_test_record r;
        std::memset(&r, 0, sizeof(r));
        for (int a = 0; a < 3; ++a) {
            r.pos[a] = a < DIM ? c.pos[a] : 0;
            r.dim[a] = a < DIM ? c.dimensions[a] : 1;
        }
        r.cycle = c.cycleCounter;
        r.edge = c.isEdgeCell ? 1 : 0;
        r.valid = c.isValid ? 1 : 0;
        r.test_value = c.testValue;
        std::memcpy(dst, &r, sizeof(r));
    }
    static void unpack(CELL *c, int, const void *src)
    {
        lgd_test_record r;
        std::memcpy(&r, src, sizeof(r));
        for (int a = 0; a < DIM; ++a) {
            c->pos[a] = r.pos[a];
            c->dimensions[a] = r.dim[a];
        }
        c->cycleCounter = r.cycle;
        c->isEdgeCell = r.edge != 0;
        c->isValid = r.valid != 0;
        c->testValue = r.test_value;
    }
    static double edgeValue(const CELL& c, int) { return (c.isValid ? 1.0 : 0.0) + (c.isEdgeCell ? 2.0 : 0.0); }
};

// Maps a non-zero status of the C ABI to the exception the reference throws
// in the same situation.
inline void gb300Check(int rc)
{
    if (rc == LGD_OK) return;
    char msg[512];
    lgd_gpu_last_error(msg, sizeof(msg));
    switch (rc) {
    case LGD_ERR_INVALID:
        throw std::invalid_argument(msg);
    case LGD_ERR_RANGE:
        throw std::out_of_range(msg);
    case LGD_ERR_UNSUPPORTED:
        throw std::logic_error(msg);
    default:
        throw std::runtime_error(std::string("CUDA error: ") + msg);
    }
}

template<typename CELL, bool RECORD>
void GB300DeviceStep<CELL, RECORD>::run(lgd_handle *h, unsigned nanoStep, int count)
{
    gb300Check(lgd_gpu_step(h, nanoStep, count));
}

// Read-only view of the device grid handed to Writers.  A Writer that
// reads part of the grid moves only that part: cells reach the host grid
// plane by plane (3D: one z plane, 2D: a band of 64 rows, 1D: the line) on
// first touch, through the library's streak copy (lgd_gpu_save_region),
// and every plane is invalidated after a device step.  The reference's
// CUDASimulator copies the whole grid for every writer call
// (parallelization/cudasimulator.h:490-497).
template<typename CELL, typename HostGrid>
class GB300WriterView : public GridBase<CELL, HostGrid::DIM> {
public:
    static const int DIM = HostGrid::DIM;
    static const int BAND = 64;             // rows per 2D band
    typedef GB300CellTraits<CELL> Traits;

    GB300WriterView(lgd_handle *const *handle, HostGrid *grid, const CoordBox<DIM>& box) :
        handle(handle), grid(grid), box(box), valid(planes(), 1), fetched(0)
    {}

    void invalidate() { std::fill(valid.begin(), valid.end(), 0); }
    void markAllValid() { std::fill(valid.begin(), valid.end(), 1); }
    bool allValid() const { return std::find(valid.begin(), valid.end(), 0) == valid.end(); }
    // bytes copied from the device by this view so far
    std::size_t bytesFetched() const { return fetched; }

    virtual CELL get(const Coord<DIM>& c) const
    {
        fetchFor(c);
        return grid->get(c);
    }
    virtual void set(const Coord<DIM>&, const CELL&) { readOnly(); }
    virtual void setEdge(const CELL&) { readOnly(); }
    virtual const CELL& getEdge() const { return grid->getEdge(); }
    virtual CoordBox<DIM> boundingBox() const { return grid->boundingBox(); }

#ifdef LGD_GB300_WITH_REFERENCE
    virtual void resize(const CoordBox<DIM>&) { readOnly(); }
    virtual void set(const Streak<DIM>&, const CELL *) { readOnly(); }
    virtual void get(const Streak<DIM>& s, CELL *cells) const
    {
        fetchFor(s.origin);
        grid->get(s, cells);
    }
    virtual void saveRegion(std::vector<CELL> *buffer, const Region<DIM>& region,
                            const Coord<DIM>& offset = Coord<DIM>()) const
    {
        for (typename Region<DIM>::StreakIterator i = region.beginStreak(); i != region.endStreak(); ++i) {
            fetchFor(i->origin + offset);
        }
        grid->saveRegion(buffer, region, offset);
    }

protected:
    virtual void saveMemberImplementation(char *target, MemoryLocation::Location targetLocation,
                                          const Selector<CELL>& selector,
                                          const typename Region<DIM>::StreakIterator& begin,
                                          const typename Region<DIM>::StreakIterator& end) const
    {
        Region<DIM> region;
        for (typename Region<DIM>::StreakIterator i = begin; i != end; ++i) {
            fetchFor(i->origin);
            region << *i;
        }
        grid->saveMember(target, targetLocation, selector, region);
    }
    virtual void loadMemberImplementation(const char *, MemoryLocation::Location, const Selector<CELL>&,
                                          const typename Region<DIM>::StreakIterator&,
                                          const typename Region<DIM>::StreakIterator&)
    {
        readOnly();
    }
#endif

private:
    lgd_handle *const *handle;      // the simulator's handle (it may be re-created)
    HostGrid *grid;
    CoordBox<DIM> box;
    mutable std::vector<char> valid;
    mutable std::size_t fetched;

    static void readOnly() { throw std::logic_error("the writers' view of a GB300 grid is read-only"); }

    int planes() const
    {
        if (DIM == 3) return box.dimensions[2];
        if (DIM == 2) return (box.dimensions[1] + BAND - 1) / BAND;
        return 1;
    }

    void fetchFor(const Coord<DIM>& c) const
    {
        for (int d = 0; d < DIM; ++d) {
            if (c[d] < box.origin[d] || c[d] >= box.origin[d] + box.dimensions[d]) return;   // the edge cell
        }
        const int p = (DIM == 3) ? c[2] - box.origin[2] : (DIM == 2) ? (c[1] - box.origin[1]) / BAND : 0;
        if (!valid[p]) fetchPlane(p);
    }

    // every row of plane p, all members, in one streak copy per member
    void fetchPlane(int p) const
    {
        const int nx = box.dimensions[0];
        const int ny = DIM > 1 ? box.dimensions[1] : 1;
        const int y0 = (DIM == 2) ? p * BAND : 0;
        const int y1 = (DIM == 2) ? std::min(ny, y0 + BAND) : ny;
        const int z = (DIM == 3) ? p : 0;
        std::vector<int> streaks;
        for (int y = y0; y < y1; ++y) {
            streaks.push_back(0);
            streaks.push_back(y);
            streaks.push_back(z);
            streaks.push_back(nx);
        }
        const int rows = y1 - y0;
        const std::size_t cells = (std::size_t)rows * nx;
        std::vector<std::vector<char> > bufs(Traits::MEMBERS);
        for (int m = 0; m < Traits::MEMBERS; ++m) {
            bufs[m].resize(cells * Traits::memberSize(m));
            gb300Check(lgd_gpu_save_region(*handle, m, streaks.data(), rows, bufs[m].data(), bufs[m].size()));
            fetched += bufs[m].size();
        }
        // rows are contiguous along x in the host grid
        std::size_t i = 0;
        for (int y = y0; y < y1; ++y) {
            Coord<DIM> c = box.origin;
            if (DIM > 1) c[1] += y;
            if (DIM > 2) c[2] += z;
            CELL *row = &(*grid)[c];
            for (int x = 0; x < nx; ++x, ++i) {
                for (int m = 0; m < Traits::MEMBERS; ++m) {
                    Traits::unpack(&row[x], m, &bufs[m][i * Traits::memberSize(m)]);
                }
            }
        }
        valid[p] = 1;
    }
};

template<typename CELL>
class GB300Simulator : public MonolithicSimulator<CELL> {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    static const int DIM = Topology::DIM;
    static const unsigned NANO_STEPS = APITraits::SelectNanoSteps<CELL>::VALUE;
    typedef GridBase<CELL, DIM> GridBaseType;
    typedef DisplacedGrid<CELL, Topology> HostGrid;
    typedef typename Steerer<CELL>::SteererFeedback SteererFeedback;
    typedef GB300CellTraits<CELL> Traits;

    explicit GB300Simulator(Initializer<CELL> *initializer, Coord<3> blockSize = Coord<3>(128, DIM < 3 ? 1 : 4, 1)) :
        MonolithicSimulator<CELL>(initializer),
        handle(0),
        hostGrid(0),
        view(0)
    {
        if (blockSize.x() <= 0 || blockSize.y() <= 0 || blockSize.z() <= 0) {
            throw std::invalid_argument("blockSize must be positive");
        }
        this->stepNum = initializer->startStep();
        box = initializer->gridBox();
        simArea << box;
        // a failing Initializer or device leaves nothing behind (the base
        // class still owns and deletes the Initializer)
        try {
            hostGrid = new HostGrid(box);
            initializer->grid(hostGrid);
            view = new WriterView(&handle, hostGrid, box);
            createDevice();
            upload();
        } catch (...) {
            if (handle) lgd_gpu_destroy(handle);
            delete view;
            delete hostGrid;
            throw;
        }
    }

    virtual ~GB300Simulator()
    {
        if (handle) lgd_gpu_destroy(handle);
        delete view;
        delete hostGrid;
    }

    virtual void step()
    {
        SteererFeedback feedback;
        step(&feedback);
    }

    virtual void step(SteererFeedback *feedback)
    {
        handleInput(STEERER_NEXT_STEP, feedback);
        {
            // compute time includes the device's: the scope waits for it
            TimeCompute t(&this->chronometer);
            for (unsigned i = 0; i < NANO_STEPS; ++i) {
                GB300DeviceStep<CELL>::run(handle, i, 1);
            }
            gb300Check(lgd_gpu_synchronize(handle));
        }
        view->invalidate();
        ++this->stepNum;
        WriterEvent event = WRITER_STEP_FINISHED;
        if (this->stepNum == this->initializer->maxSteps()) {
            event = WRITER_ALL_DONE;
        }
        handleOutput(event);
    }

    virtual void run()
    {
        TimeTotal t(&this->chronometer);
        this->initializer->grid(hostGrid);
        view->markAllValid();
        this->stepNum = this->initializer->startStep();
        if (edgeChanged()) {
            if (Traits::KIND == LGD_CELL_RECORD) {
                gb300Check(lgd_gpu_set_edge_record(handle, &hostGrid->getEdge(), sizeof(CELL)));
                std::memcpy(edgeRecord.data(), static_cast<const void *>(&hostGrid->getEdge()), sizeof(CELL));
            } else {
                gb300Check(lgd_gpu_destroy(handle));
                handle = 0;
                createDevice();
            }
        }
        upload();
        for (std::size_t i = 0; i < this->steerers.size(); ++i) {
            this->steerers[i]->setRegion(simArea);
        }
        SteererFeedback feedback;
        handleInput(STEERER_INITIALIZED, &feedback);
        handleOutput(WRITER_INITIALIZED);
        while (this->stepNum < this->initializer->maxSteps()) {
            if (feedback.simulationEnded()) break;
            advanceQuietSteps();
            step(&feedback);
        }
        handleInput(STEERER_ALL_DONE, &feedback);
    }

    virtual const GridBaseType *getGrid()
    {
        download();
        return hostGrid;
    }

    // The library handle, for callers that want the device grid directly.
    lgd_handle *deviceHandle() { return handle; }

    // Bytes the Writers' view has copied from the device (Writers that read
    // part of the grid move only that part).
    std::size_t writerBytesFetched() const { return view->bytesFetched(); }

private:
    typedef GB300WriterView<CELL, HostGrid> WriterView;
    lgd_handle *handle;
    HostGrid *hostGrid;
    WriterView *view;       // the host grid's validity, plane by plane
    CoordBox<DIM> box;
    Region<DIM> simArea;
    double edge[4];
    std::vector<unsigned char> edgeRecord;      // record cells: the edge cell's bytes

    void createDevice()
    {
        lgd_grid_desc d;
        std::memset(&d, 0, sizeof(d));
        d.dim = DIM;
        d.nx = box.dimensions[0];
        d.ny = DIM > 1 ? box.dimensions[1] : 1;
        d.nz = DIM > 2 ? box.dimensions[2] : 1;
        d.periodic = (Topology::template WrapsAxis<0>::VALUE ? 1 : 0) |
                     (Topology::template WrapsAxis<1>::VALUE ? 2 : 0) |
                     (Topology::template WrapsAxis<2>::VALUE ? 4 : 0);
        d.cell = Traits::KIND;
        d.flags = GB300DescFlags<Traits>::value();
        if (Traits::KIND == LGD_CELL_RECORD) {
            const CELL& e = hostGrid->getEdge();
            edgeRecord.resize(sizeof(CELL));
            std::memcpy(edgeRecord.data(), static_cast<const void *>(&e), sizeof(CELL));
            gb300Check(lgd_gpu_create_records(&d, sizeof(CELL), edgeRecord.data(), &handle));
        } else {
            for (int m = 0; m < Traits::MEMBERS && m < 4; ++m) {
                d.edge[m] = Traits::edgeValue(hostGrid->getEdge(), m);
                edge[m] = d.edge[m];
            }
            gb300Check(lgd_gpu_create(&d, &handle));
        }
    }

    bool edgeChanged() const
    {
        bool changed = false;
        if (Traits::KIND == LGD_CELL_RECORD) {
            changed = std::memcmp(edgeRecord.data(), static_cast<const void *>(&hostGrid->getEdge()), sizeof(CELL)) != 0;
        } else {
            for (int m = 0; m < Traits::MEMBERS && m < 4; ++m) {
                changed |= Traits::edgeValue(hostGrid->getEdge(), m) != edge[m];
            }
        }
        return changed;
    }

    // Rows of the host grid: cells are contiguous along x in the host grid
    // (the reference's Grid and DisplacedGrid store the box x fastest), so a
    // row is one pointer; the members are packed row by row through the
    // binding's inline pack/unpack, and record cells are copied whole.
    std::size_t rows() const
    {
        return (std::size_t)(DIM > 1 ? box.dimensions[1] : 1) * (DIM > 2 ? box.dimensions[2] : 1);
    }

    CELL *rowPointer(std::size_t r)
    {
        Coord<DIM> c = box.origin;
        if (DIM > 1) c[1] += (int)(r % (std::size_t)box.dimensions[1]);
        if (DIM > 2) c[2] += (int)(r / (std::size_t)box.dimensions[1]);
        return &(*hostGrid)[c];
    }

    // host grid -> dense member arrays -> device (current buffer)
    void upload()
    {
        const std::size_t n = box.size();
        const std::size_t nx = (std::size_t)box.dimensions[0];
        std::vector<char> buf;
        for (int m = 0; m < Traits::MEMBERS; ++m) {
            const std::size_t sz = Traits::memberSize(m);
            buf.resize(n * sz);
            char *dst = buf.data();
            for (std::size_t r = 0; r < rows(); ++r) {
                const CELL *row = rowPointer(r);
                if (Traits::KIND == LGD_CELL_RECORD) {
                    std::memcpy(dst, static_cast<const void *>(row), nx * sizeof(CELL));
                    dst += nx * sizeof(CELL);
                } else {
                    for (std::size_t x = 0; x < nx; ++x, dst += sz) Traits::pack(row[x], m, dst);
                }
            }
            gb300Check(lgd_gpu_upload(handle, m, 0, buf.data(), buf.size()));
        }
        view->markAllValid();
    }

    // the whole grid to the host (unless every plane is there already)
    void download()
    {
        if (view->allValid()) return;
        const std::size_t n = box.size();
        const std::size_t nx = (std::size_t)box.dimensions[0];
        std::vector<char> buf;
        for (int m = 0; m < Traits::MEMBERS; ++m) {
            const std::size_t sz = Traits::memberSize(m);
            buf.resize(n * sz);
            gb300Check(lgd_gpu_download(handle, m, 0, buf.data(), buf.size()));
            const char *src = buf.data();
            for (std::size_t r = 0; r < rows(); ++r) {
                CELL *row = rowPointer(r);
                if (Traits::KIND == LGD_CELL_RECORD) {
                    std::memcpy(static_cast<void *>(row), src, nx * sizeof(CELL));
                    src += nx * sizeof(CELL);
                } else {
                    for (std::size_t x = 0; x < nx; ++x, src += sz) Traits::unpack(&row[x], m, src);
                }
            }
        }
        view->markAllValid();
    }

    // Steps before the next one that calls a plugin: no Steerer runs before
    // them (stepNum % period != 0), no Writer after them (step % period !=
    // 0) and none of them is the last.  Those steps go to the library in
    // one call, which may fuse several of them into one pass over memory
    // (temporal blocking); the plugins see exactly the calls that
    // step-by-step execution makes.  Cells with several nano steps keep one
    // call per step.
    void advanceQuietSteps()
    {
        if (NANO_STEPS != 1) return;
        const unsigned s = this->stepNum;
        unsigned next = this->initializer->maxSteps() - 1;     // the last step announces ALL_DONE
        for (std::size_t i = 0; i < this->steerers.size(); ++i) {
            const unsigned p = this->steerers[i]->getPeriod();
            next = std::min(next, (s + p - 1) / p * p);                // stepNum % p == 0
        }
        for (std::size_t i = 0; i < this->writers.size(); ++i) {
            const unsigned p = this->writers[i]->getPeriod();
            next = std::min(next, (s + 1 + p - 1) / p * p - 1);        // (stepNum + 1) % p == 0
        }
        if (next <= s) return;
        {
            TimeCompute t(&this->chronometer);
            GB300DeviceStep<CELL>::run(handle, 0, (int)std::min<unsigned>(next - s, 1u << 30));
            gb300Check(lgd_gpu_synchronize(handle));
        }
        this->stepNum = next;
        view->invalidate();
    }

    void handleInput(SteererEvent event, SteererFeedback *feedback)
    {
        TimeInput t(&this->chronometer);
        bool called = false;
        for (std::size_t i = 0; i < this->steerers.size(); ++i) {
            if ((event != STEERER_NEXT_STEP) || (this->stepNum % this->steerers[i]->getPeriod() == 0)) {
                if (!called) download();
                called = true;
                this->steerers[i]->nextStep(hostGrid, simArea, this->gridDim, this->getStep(), event, 0, true,
                                            feedback);
            }
        }
        if (called) upload();   // steering changes reach the device
    }

    void handleOutput(WriterEvent event)
    {
        TimeOutput t(&this->chronometer);
        for (std::size_t i = 0; i < this->writers.size(); ++i) {
            if ((event != WRITER_STEP_FINISHED) || ((this->getStep() % this->writers[i]->getPeriod()) == 0)) {
                this->writers[i]->stepFinished(*view, this->getStep(), event);   // planes on demand
            }
        }
    }
};

// Writer plugin that writes BOV snapshots of one member straight from the
// device grid of a GB300Simulator (lgd_gpu_write_bov): the format of the
// reference's SerialBOVWriter (io/serialbovwriter.h), without copying the
// grid into host cells first.  The simulator owns the writer (addWriter),
// so the pointer it keeps stays valid.
template<typename CELL>
class GB300BOVWriter : public Writer<CELL> {
public:
    typedef typename Writer<CELL>::GridType GridType;

    GB300BOVWriter(GB300Simulator<CELL> *sim, int member, const std::string& variable, const std::string& prefix,
                   unsigned period) :
        Writer<CELL>(prefix, period), sim(sim), member(member), variable(variable)
    {}

    Writer<CELL> *clone() const { return new GB300BOVWriter(sim, member, variable, this->prefix, this->period); }

    void stepFinished(const GridType&, unsigned step, WriterEvent event)
    {
        if ((event == WRITER_STEP_FINISHED) && (step % this->period != 0)) return;
        gb300Check(lgd_gpu_write_bov(sim->deviceHandle(), member, this->prefix.c_str(), step, variable.c_str()));
    }

private:
    GB300Simulator<CELL> *sim;
    int member;
    std::string variable;
};

// Checkpoints straight from the device grid of a GB300Simulator
// (lgd_gpu_write_snapshot), in the file layout and under the file names of
// the reference's MPIIOWriter (io/mpiiowriter.h: prefix + 5-digit step +
// ".mpiio", written at WRITER_INITIALIZED, every period-th step and
// WRITER_ALL_DONE; io/mpiio.h:85-125 for the layout), by one process
// without MPI.  GB300SnapshotInitializer restarts from such a file.
template<typename CELL>
class GB300SnapshotWriter : public Writer<CELL> {
public:
    typedef typename Writer<CELL>::GridType GridType;

    GB300SnapshotWriter(GB300Simulator<CELL> *sim, const std::string& prefix, unsigned period, unsigned maxSteps) :
        Writer<CELL>(prefix, period), sim(sim), maxSteps(maxSteps)
    {}

    Writer<CELL> *clone() const { return new GB300SnapshotWriter(sim, this->prefix, this->period, maxSteps); }

    void stepFinished(const GridType&, unsigned step, WriterEvent event)
    {
        if ((event == WRITER_STEP_FINISHED) && (step % this->period != 0)) return;
        gb300Check(lgd_gpu_write_snapshot(sim->deviceHandle(), filename(step).c_str(), step, maxSteps));
    }

    std::string filename(unsigned step) const
    {
        char buf[16];
        std::snprintf(buf, sizeof(buf), "%05u", step);
        return this->prefix + buf + ".mpiio";
    }

private:
    GB300Simulator<CELL> *sim;
    unsigned maxSteps;
};

// Restart from a checkpoint: the reference's MPIIOInitializer
// (io/mpiioinitializer.h) read by one process without MPI.  The
// dimensions, start step and maximum come from the file's header, the grid
// and its edge cell from the cell records (sizeof(CELL) bytes each, the
// reference's record for cells without padding, at header + index *
// sizeof(CELL), index x fastest; io/mpiio.h:28-66 readRegion).
template<typename CELL>
class GB300SnapshotInitializer : public Initializer<CELL> {
public:
    typedef typename Initializer<CELL>::Topology Topology;
    static const int DIM = Topology::DIM;

    explicit GB300SnapshotInitializer(const std::string& filename) :
        file(filename)
    {
        int dims[3] = {1, 1, 1};
        gb300Check(lgd_snapshot_info(file.c_str(), DIM, dims, &currentStep, &maximumSteps));
        for (int d = 0; d < DIM; ++d) dimensions[d] = dims[d];
    }

    void grid(GridBase<CELL, DIM> *target)
    {
        const size_t header = 4 * DIM + 8;
        const size_t cells = (size_t)dimensions.prod();
        std::vector<unsigned char> bytes(header + (cells + 1) * sizeof(CELL));
        FILE *f = std::fopen(file.c_str(), "rb");
        if (!f) throw std::runtime_error("cannot open " + file);
        const bool ok = std::fread(bytes.data(), 1, bytes.size(), f) == bytes.size();
        std::fclose(f);
        if (!ok) throw std::runtime_error("snapshot shorter than its header says: " + file);
        CELL cell;
        std::memcpy(static_cast<void *>(&cell), &bytes[header], sizeof(CELL));
        target->setEdge(cell);
        const unsigned char *data = &bytes[header + sizeof(CELL)];
        const CoordBox<DIM> box = target->boundingBox();
        for (size_t i = 0; i < cells; ++i) {
            const Coord<DIM> c = coordOf(i);
            if (!box.inBounds(c)) continue;
            std::memcpy(static_cast<void *>(&cell), data + i * sizeof(CELL), sizeof(CELL));
            target->set(c, cell);
        }
    }

    Coord<DIM> gridDimensions() const { return dimensions; }
    unsigned maxSteps() const { return maximumSteps; }
    unsigned startStep() const { return currentStep; }

private:
    std::string file;
    unsigned currentStep;
    unsigned maximumSteps;
    Coord<DIM> dimensions;

    Coord<DIM> coordOf(size_t i) const
    {
        Coord<DIM> c;
        for (int d = 0; d < DIM; ++d) {
            c[d] = (int)(i % (size_t)dimensions[d]);
            i /= (size_t)dimensions[d];
        }
        return c;
    }
};

}  // namespace LibGeoDecomp

#endif
