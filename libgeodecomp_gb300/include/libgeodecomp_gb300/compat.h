// Host-side mirror of the part of LibGeoDecomp's public API that
// GB300Simulator and its plugins touch, for builds without the reference's
// headers (the reference library is header-only C++ and may not be
// installed where the GPU library runs).  Names, signatures and event
// semantics follow the reference so that plugin code compiles unchanged
// against either:
//   Coord / CoordBox / Streak / Region      geometry/coord.h, coordbox.h,
//                                           streak.h, region.h
//   FixedCoord                              geometry/fixedcoord.h
//   Topologies::Cube / Torus, WrapsAxis     geometry/topologies.h:179-278
//   Stencils::Moore / VonNeumann            geometry/stencils.h:182-227
//   APITraits (topology, nano steps, tags)  misc/apitraits.h:69-836
//   GridBase, DisplacedGrid                 storage/gridbase.h:71,
//                                           storage/displacedgrid.h:116
//   Initializer, SimpleInitializer          io/initializer.h:22-71,
//                                           io/simpleinitializer.h
//   Writer, WriterEvent                     io/writer.h:14-90
//   Steerer, SteererEvent, SteererFeedback  io/steerer.h:11-140
//   Simulator, MonolithicSimulator          parallelization/simulator.h:28-106,
//                                           parallelization/monolithicsimulator.h:16-52
// Only what a single-node simulator needs is here: no MPI, no HPX, no
// serialisation, no region algebra beyond streak lists.  What a cell's
// update() uses (Coord, FixedCoord, the topologies' normalize and
// isOutOfBounds, the stencils' Coords and RepeatCuda) is callable on the
// device when nvcc compiles it, as in the reference, so one cell source
// runs on the host and, through gb300cell.cuh, on the GPU.
#ifndef LGD_GB300_COMPAT_H
#define LGD_GB300_COMPAT_H

#include <algorithm>
#include <chrono>
#include <cstddef>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#ifdef __CUDACC__
#define LGD_COMPAT_HD __host__ __device__
#else
#define LGD_COMPAT_HD
#endif

namespace LibGeoDecomp {

template<typename T>
struct SharedPtr {
    typedef std::shared_ptr<T> Type;
};

// ------------------------------------------------------------- FixedCoord
// A compile-time offset (the stencils' neighbour positions).
template<int DIM_X = 0, int DIM_Y = 0, int DIM_Z = 0>
class FixedCoord {
public:
    static const int X = DIM_X;
    static const int Y = DIM_Y;
    static const int Z = DIM_Z;
    LGD_COMPAT_HD FixedCoord() {}
};

// ------------------------------------------------------------------ Coord
template<int DIM>
class Coord;

template<>
class Coord<1> {
public:
    LGD_COMPAT_HD explicit Coord(int x = 0) { c[0] = x; }
    template<int X, int Y, int Z>
    LGD_COMPAT_HD explicit Coord(FixedCoord<X, Y, Z>) { c[0] = X; }
    LGD_COMPAT_HD int x() const { return c[0]; }
    LGD_COMPAT_HD int& operator[](int i) { return c[i]; }
    LGD_COMPAT_HD int operator[](int i) const { return c[i]; }
    LGD_COMPAT_HD long prod() const { return c[0]; }
    LGD_COMPAT_HD bool operator==(const Coord& o) const { return c[0] == o.c[0]; }
    LGD_COMPAT_HD bool operator!=(const Coord& o) const { return !(*this == o); }
    LGD_COMPAT_HD Coord operator+(const Coord& o) const { return Coord(c[0] + o.c[0]); }
    LGD_COMPAT_HD Coord operator-(const Coord& o) const { return Coord(c[0] - o.c[0]); }
    LGD_COMPAT_HD static Coord diagonal(int v) { return Coord(v); }

private:
    int c[1];
};

template<>
class Coord<2> {
public:
    LGD_COMPAT_HD explicit Coord(int x = 0, int y = 0) { c[0] = x; c[1] = y; }
    template<int X, int Y, int Z>
    LGD_COMPAT_HD explicit Coord(FixedCoord<X, Y, Z>) { c[0] = X; c[1] = Y; }
    LGD_COMPAT_HD int x() const { return c[0]; }
    LGD_COMPAT_HD int y() const { return c[1]; }
    LGD_COMPAT_HD int& operator[](int i) { return c[i]; }
    LGD_COMPAT_HD int operator[](int i) const { return c[i]; }
    LGD_COMPAT_HD long prod() const { return (long)c[0] * c[1]; }
    LGD_COMPAT_HD bool operator==(const Coord& o) const { return c[0] == o.c[0] && c[1] == o.c[1]; }
    LGD_COMPAT_HD bool operator!=(const Coord& o) const { return !(*this == o); }
    LGD_COMPAT_HD Coord operator+(const Coord& o) const { return Coord(c[0] + o.c[0], c[1] + o.c[1]); }
    LGD_COMPAT_HD Coord operator-(const Coord& o) const { return Coord(c[0] - o.c[0], c[1] - o.c[1]); }
    LGD_COMPAT_HD static Coord diagonal(int v) { return Coord(v, v); }

private:
    int c[2];
};

template<>
class Coord<3> {
public:
    LGD_COMPAT_HD explicit Coord(int x = 0, int y = 0, int z = 0) { c[0] = x; c[1] = y; c[2] = z; }
    template<int X, int Y, int Z>
    LGD_COMPAT_HD explicit Coord(FixedCoord<X, Y, Z>) { c[0] = X; c[1] = Y; c[2] = Z; }
    LGD_COMPAT_HD int x() const { return c[0]; }
    LGD_COMPAT_HD int y() const { return c[1]; }
    LGD_COMPAT_HD int z() const { return c[2]; }
    LGD_COMPAT_HD int& operator[](int i) { return c[i]; }
    LGD_COMPAT_HD int operator[](int i) const { return c[i]; }
    LGD_COMPAT_HD long prod() const { return (long)c[0] * c[1] * c[2]; }
    LGD_COMPAT_HD bool operator==(const Coord& o) const
    {
        return c[0] == o.c[0] && c[1] == o.c[1] && c[2] == o.c[2];
    }
    LGD_COMPAT_HD bool operator!=(const Coord& o) const { return !(*this == o); }
    LGD_COMPAT_HD Coord operator+(const Coord& o) const { return Coord(c[0] + o.c[0], c[1] + o.c[1], c[2] + o.c[2]); }
    LGD_COMPAT_HD Coord operator-(const Coord& o) const { return Coord(c[0] - o.c[0], c[1] - o.c[1], c[2] - o.c[2]); }
    LGD_COMPAT_HD static Coord diagonal(int v) { return Coord(v, v, v); }

private:
    int c[3];
};

// --------------------------------------------------------------- CoordBox
template<int DIM>
class CoordBox {
public:
    class Iterator {
    public:
        Iterator(const Coord<DIM>& origin, const Coord<DIM>& dim, const Coord<DIM>& cursor) :
            origin(origin), dim(dim), cursor(cursor)
        {}
        const Coord<DIM>& operator*() const { return cursor; }
        const Coord<DIM> *operator->() const { return &cursor; }
        bool operator!=(const Iterator& o) const { return cursor != o.cursor; }
        bool operator==(const Iterator& o) const { return cursor == o.cursor; }
        Iterator& operator++()
        {
            for (int d = 0; d < DIM; ++d) {
                ++cursor[d];
                if (cursor[d] < origin[d] + dim[d] || d == DIM - 1) {
                    return *this;
                }
                cursor[d] = origin[d];
            }
            return *this;
        }

    private:
        Coord<DIM> origin;
        Coord<DIM> dim;
        Coord<DIM> cursor;
    };

    explicit CoordBox(const Coord<DIM>& origin = Coord<DIM>(), const Coord<DIM>& dimensions = Coord<DIM>()) :
        origin(origin), dimensions(dimensions)
    {}

    bool inBounds(const Coord<DIM>& c) const
    {
        for (int d = 0; d < DIM; ++d) {
            if (c[d] < origin[d] || c[d] >= origin[d] + dimensions[d]) return false;
        }
        return true;
    }

    std::size_t size() const { return (std::size_t)dimensions.prod(); }

    Iterator begin() const { return Iterator(origin, dimensions, origin); }

    Iterator end() const
    {
        if (dimensions.prod() == 0) return begin();
        Coord<DIM> c = origin;
        c[DIM - 1] = origin[DIM - 1] + dimensions[DIM - 1];
        return Iterator(origin, dimensions, c);
    }

    Coord<DIM> origin;
    Coord<DIM> dimensions;
};

// ---------------------------------------------------------- Streak, Region
template<int DIM>
class Streak {
public:
    Streak(const Coord<DIM>& origin = Coord<DIM>(), int endX = 0) : origin(origin), endX(endX) {}
    int length() const { return endX - origin.x(); }
    Coord<DIM> origin;
    int endX;
};

// A region as an ordered list of streaks (no overlap handling).
template<int DIM>
class Region {
public:
    typedef typename std::vector<Streak<DIM> >::const_iterator StreakIterator;

    Region& operator<<(const Streak<DIM>& s)
    {
        if (s.endX > s.origin.x()) streaks.push_back(s);
        return *this;
    }

    Region& operator<<(const CoordBox<DIM>& box)
    {
        if (box.size() == 0) return *this;
        Coord<DIM> row = box.origin;
        CoordBox<DIM> rows = box;
        rows.dimensions[0] = 1;
        for (typename CoordBox<DIM>::Iterator i = rows.begin(); i != rows.end(); ++i) {
            *this << Streak<DIM>(*i, i->x() + box.dimensions.x());
        }
        (void)row;
        return *this;
    }

    StreakIterator beginStreak() const { return streaks.begin(); }
    StreakIterator endStreak() const { return streaks.end(); }
    std::size_t numStreaks() const { return streaks.size(); }

    std::size_t size() const
    {
        std::size_t n = 0;
        for (StreakIterator i = beginStreak(); i != endStreak(); ++i) n += i->length();
        return n;
    }

private:
    std::vector<Streak<DIM> > streaks;
};

// ------------------------------------------------------------- topologies
namespace Topologies {

template<int DIMENSIONS, bool WRAP>
class TopologyTemplate {
public:
    static const int DIM = DIMENSIONS;
    template<int D>
    class WrapsAxis {
    public:
        static const bool VALUE = WRAP && (D < DIMENSIONS);
    };

    // wraps coordinates into the grid on periodic axes
    LGD_COMPAT_HD static Coord<DIM> normalize(Coord<DIM> c, const Coord<DIM>& dim)
    {
        for (int d = 0; d < DIM; ++d) {
            if (WRAP) c[d] = ((c[d] % dim[d]) + dim[d]) % dim[d];
        }
        return c;
    }

    // outside the grid on a non-periodic axis (the edge cell's positions)
    LGD_COMPAT_HD static bool isOutOfBounds(const Coord<DIM>& c, const Coord<DIM>& dim)
    {
        bool out = false;
        for (int d = 0; d < DIM; ++d) {
            out |= !WRAP && (c[d] < 0 || c[d] >= dim[d]);
        }
        return out;
    }
};

template<int DIM>
class Cube {
public:
    typedef TopologyTemplate<DIM, false> Topology;
};

template<int DIM>
class Torus {
public:
    typedef TopologyTemplate<DIM, true> Topology;
};

}  // namespace Topologies

namespace Stencils {
// lattice points with |x_1| + ... + |x_d| <= r, and (2 r + 1)^d
constexpr int vonNeumannVolume(int d, int r)
{
    if (d == 0) return 1;
    int n = 0;
    for (int k = -r; k <= r; ++k) n += vonNeumannVolume(d - 1, r - (k < 0 ? -k : k));
    return n;
}
constexpr int mooreVolume(int d, int r) { return d == 0 ? 1 : (2 * r + 1) * mooreVolume(d - 1, r); }

// Offset `axis` of the index-th point of a stencil: the points of the
// (2r + 1)^d box in x-fastest order (the reference's Moore order), keeping
// only |x| + |y| + |z| <= r for von Neumann stencils.
constexpr int stencilOffset(int dim, int r, bool diamond, int index, int axis)
{
    const int w = 2 * r + 1;
    const int box = mooreVolume(dim, r);
    int seen = -1;
    for (int i = 0; i < box; ++i) {
        const int x = i % w - r;
        const int y = dim > 1 ? (i / w) % w - r : 0;
        const int z = dim > 2 ? i / (w * w) - r : 0;
        const int l1 = (x < 0 ? -x : x) + (y < 0 ? -y : y) + (z < 0 ? -z : z);
        if (diamond && l1 > r) continue;
        if (++seen == index) return axis == 0 ? x : axis == 1 ? y : z;
    }
    return 0;
}

template<int DIMENSIONS, int RAD>
class VonNeumann {
public:
    static const int DIM = DIMENSIONS;
    static const int RADIUS = RAD;
    static const int VOLUME = vonNeumannVolume(DIMENSIONS, RAD);
    template<int INDEX>
    class Coords : public FixedCoord<stencilOffset(DIMENSIONS, RAD, true, INDEX, 0),
                                     stencilOffset(DIMENSIONS, RAD, true, INDEX, 1),
                                     stencilOffset(DIMENSIONS, RAD, true, INDEX, 2)> {};
};

template<int DIMENSIONS, int RAD>
class Moore {
public:
    static const int DIM = DIMENSIONS;
    static const int RADIUS = RAD;
    static const int VOLUME = mooreVolume(DIMENSIONS, RAD);
    template<int INDEX>
    class Coords : public FixedCoord<stencilOffset(DIMENSIONS, RAD, false, INDEX, 0),
                                     stencilOffset(DIMENSIONS, RAD, false, INDEX, 1),
                                     stencilOffset(DIMENSIONS, RAD, false, INDEX, 2)> {};
};

// TEMPLATE<PARAM, I>()(cargo...) for I = 0 .. NUM - 1, on host and device
template<int NUM, template<class C, int I> class TEMPLATE, class PARAM>
class RepeatCuda {
public:
    template<typename... CARGO>
    LGD_COMPAT_HD void operator()(CARGO... cargo) const
    {
        RepeatCuda<NUM - 1, TEMPLATE, PARAM>()(cargo...);
        TEMPLATE<PARAM, NUM - 1>()(cargo...);
    }
};

template<template<class C, int I> class TEMPLATE, class PARAM>
class RepeatCuda<0, TEMPLATE, PARAM> {
public:
    template<typename... CARGO>
    LGD_COMPAT_HD void operator()(CARGO...) const {}
};

template<int NUM, template<class C, int I> class TEMPLATE, class PARAM>
class Repeat : public RepeatCuda<NUM, TEMPLATE, PARAM> {};
}  // namespace Stencils

// -------------------------------------------------------------- APITraits
class APITraits {
public:
    template<typename CELL, typename HAS = void>
    class SelectTopology {
    public:
        typedef Topologies::Cube<2>::Topology Value;
    };

    template<typename CELL>
    class SelectTopology<CELL, typename CELL::API::SupportsTopology> {
    public:
        typedef typename CELL::API::Topology Value;
    };

    template<typename CELL, typename HAS = void>
    class SelectNanoSteps {
    public:
        static const unsigned VALUE = 1;
    };

    template<typename CELL>
    class SelectNanoSteps<CELL, typename CELL::API::SupportsNanoSteps> {
    public:
        static const unsigned VALUE = CELL::API::NANO_STEPS;
    };

    template<typename TOPOLOGY>
    class HasTopology {
    public:
        typedef void SupportsTopology;
        typedef TOPOLOGY Topology;
    };

    template<int DIM>
    class HasCubeTopology : public HasTopology<typename Topologies::Cube<DIM>::Topology> {};

    template<int DIM>
    class HasTorusTopology : public HasTopology<typename Topologies::Torus<DIM>::Topology> {};

    template<unsigned N>
    class HasNanoSteps {
    public:
        typedef void SupportsNanoSteps;
        static const unsigned NANO_STEPS = N;
    };

    template<typename STENCIL>
    class HasStencil {
    public:
        typedef void SupportsStencil;
        typedef STENCIL Stencil;
    };

    template<typename CELL, typename HAS = void>
    class SelectStencil {
    public:
        typedef Stencils::Moore<2, 1> Value;
    };

    template<typename CELL>
    class SelectStencil<CELL, typename CELL::API::SupportsStencil> {
    public:
        typedef typename CELL::API::Stencil Value;
    };

    class TrueType {};
    class FalseType {};

    // a cell with this trait runs updateCUDA() instead of update() on the
    // device (misc/apitraits.h:814-836)
    class HasSeparateCUDAUpdate {
    public:
        typedef void SupportsSeparateCUDAUpdate;
    };

    template<typename CELL, typename HAS = void>
    class SelectSeparateCUDAUpdate {
    public:
        typedef FalseType Value;
    };

    template<typename CELL>
    class SelectSeparateCUDAUpdate<CELL, typename CELL::API::SupportsSeparateCUDAUpdate> {
    public:
        typedef TrueType Value;
    };

    class HasSoA {};
    class HasUpdateLineX {};
    class HasFixedCoordsOnlyUpdate {};
};

// ------------------------------------------------------------------ grids
template<typename CELL, int DIMENSIONS>
class GridBase {
public:
    static const int DIM = DIMENSIONS;
    typedef CELL CellType;

    virtual ~GridBase() {}
    virtual void set(const Coord<DIM>& c, const CELL& cell) = 0;
    virtual CELL get(const Coord<DIM>& c) const = 0;
    virtual void setEdge(const CELL& cell) = 0;
    virtual const CELL& getEdge() const = 0;
    virtual CoordBox<DIM> boundingBox() const = 0;
    Coord<DIM> dimensions() const { return boundingBox().dimensions; }
};

// Host grid with the cells in x-fastest order plus one edge cell.
template<typename CELL, typename TOPOLOGY = Topologies::Cube<2>::Topology, bool TOPOLOGICALLY_CORRECT = false>
class DisplacedGrid : public GridBase<CELL, TOPOLOGY::DIM> {
public:
    static const int DIM = TOPOLOGY::DIM;

    explicit DisplacedGrid(const CoordBox<DIM>& box = CoordBox<DIM>(), const CELL& defaultCell = CELL(),
                           const CELL& edgeCell = CELL()) :
        box(box), cells(box.size(), defaultCell), edge(edgeCell)
    {}

    void set(const Coord<DIM>& c, const CELL& cell) { cells[index(c)] = cell; }
    CELL get(const Coord<DIM>& c) const { return cells[index(c)]; }
    CELL& operator[](const Coord<DIM>& c) { return cells[index(c)]; }
    const CELL& operator[](const Coord<DIM>& c) const { return cells[index(c)]; }
    void setEdge(const CELL& cell) { edge = cell; }
    const CELL& getEdge() const { return edge; }
    CoordBox<DIM> boundingBox() const { return box; }
    CELL *data() { return cells.data(); }
    const CELL *data() const { return cells.data(); }

private:
    CoordBox<DIM> box;
    std::vector<CELL> cells;
    CELL edge;

    std::size_t index(const Coord<DIM>& c) const
    {
        std::size_t i = 0;
        for (int d = DIM - 1; d >= 0; --d) {
            const int v = c[d] - box.origin[d];
            if (v < 0 || v >= box.dimensions[d]) throw std::out_of_range("coordinate outside the grid");
            i = i * box.dimensions[d] + v;
        }
        return i;
    }
};

// ------------------------------------------------------------ Initializer
template<typename CELL>
class Initializer {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    typedef CELL Cell;
    static const unsigned NANO_STEPS = APITraits::SelectNanoSteps<CELL>::VALUE;
    static const int DIM = Topology::DIM;

    virtual ~Initializer() {}
    virtual void grid(GridBase<CELL, DIM> *target) = 0;
    virtual CoordBox<DIM> gridBox() { return CoordBox<DIM>(Coord<DIM>(), gridDimensions()); }
    virtual Coord<DIM> gridDimensions() const = 0;
    virtual unsigned startStep() const = 0;
    virtual unsigned maxSteps() const = 0;
};

template<typename CELL>
class SimpleInitializer : public Initializer<CELL> {
public:
    typedef typename Initializer<CELL>::Topology Topology;
    static const int DIM = Topology::DIM;

    explicit SimpleInitializer(const Coord<DIM>& dimensions, const unsigned steps = 300) :
        dimensions(dimensions), steps(steps)
    {}

    Coord<DIM> gridDimensions() const { return dimensions; }
    unsigned maxSteps() const { return steps; }
    unsigned startStep() const { return 0; }

protected:
    Coord<DIM> dimensions;
    unsigned steps;
};

// ----------------------------------------------------------------- Writer
enum WriterEvent {
    WRITER_INITIALIZED,
    WRITER_STEP_FINISHED,
    WRITER_ALL_DONE
};

template<typename CELL>
class Writer {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    static const int DIM = Topology::DIM;
    typedef GridBase<CELL, DIM> GridType;

    Writer(const std::string& prefix, const unsigned period) : prefix(prefix), period(period)
    {
        if (period == 0) throw std::invalid_argument("period must be positive");
    }

    virtual ~Writer() {}
    virtual Writer *clone() const = 0;
    virtual void stepFinished(const GridType& grid, unsigned step, WriterEvent event) = 0;
    unsigned getPeriod() const { return period; }
    const std::string& getPrefix() const { return prefix; }

protected:
    std::string prefix;
    unsigned period;
};

// ---------------------------------------------------------------- Steerer
enum SteererEvent {
    STEERER_INITIALIZED,
    STEERER_NEXT_STEP,
    STEERER_ALL_DONE
};

template<typename CELL>
class Steerer {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    typedef GridBase<CELL, Topology::DIM> GridType;
    typedef Coord<Topology::DIM> CoordType;

    class SteererFeedback {
    public:
        SteererFeedback() : simulationEnd(false) {}
        void endSimulation() { simulationEnd = true; }
        bool simulationEnded() { return simulationEnd; }

    private:
        bool simulationEnd;
    };

    explicit Steerer(const unsigned period) : period(period) {}
    virtual ~Steerer() {}
    virtual void setRegion(const Region<Topology::DIM>& newRegion) { region = newRegion; }
    virtual void nextStep(GridType *grid, const Region<Topology::DIM>& validRegion, const CoordType& globalDimensions,
                          unsigned step, SteererEvent event, std::size_t rank, bool lastCall,
                          SteererFeedback *feedback) = 0;
    unsigned getPeriod() const { return period; }

protected:
    Region<Topology::DIM> region;
    unsigned period;
};

// ------------------------------------------------------------ Chronometer
// Accumulated wall time per category, with the reference's category ids
// and names (misc/chronometer.h:142-150) and scoped timers that add the
// time between their construction and destruction.
class Chronometer {
public:
    static const std::size_t NUM_INTERVALS = 9;

    Chronometer() : totalTimes(NUM_INTERVALS, 0.0) {}

    double operator[](std::size_t i) const { return totalTimes[i]; }
    double& operator[](std::size_t i) { return totalTimes[i]; }
    double interval(std::size_t i) const { return totalTimes[i]; }
    template<typename INTERVAL>
    double interval() const { return totalTimes[INTERVAL::ID]; }
    void reset() { std::fill(totalTimes.begin(), totalTimes.end(), 0.0); }

    Chronometer& operator+=(const Chronometer& other)
    {
        for (std::size_t i = 0; i < NUM_INTERVALS; ++i) totalTimes[i] += other.totalTimes[i];
        return *this;
    }

private:
    std::vector<double> totalTimes;
};

namespace ChronometerHelpers {
template<int EVENT_ID>
class ScopedEvent {
public:
    static const int ID = EVENT_ID;
    explicit ScopedEvent(Chronometer *chrono) : chrono(chrono), start(std::chrono::steady_clock::now()) {}
    ~ScopedEvent()
    {
        (*chrono)[ID] += std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    }

private:
    Chronometer *chrono;
    std::chrono::steady_clock::time_point start;
};
}  // namespace ChronometerHelpers

#define LGD_COMPAT_EVENT(NAME, EVENT_ID)                                                 \
    class NAME : public ChronometerHelpers::ScopedEvent<EVENT_ID> {                     \
    public:                                                                              \
        explicit NAME(Chronometer *c) : ChronometerHelpers::ScopedEvent<EVENT_ID>(c) {}  \
    };
LGD_COMPAT_EVENT(TimeTotal, 0)
LGD_COMPAT_EVENT(TimeCompute, 1)
LGD_COMPAT_EVENT(TimeComputeInner, 2)
LGD_COMPAT_EVENT(TimeComputeGhost, 3)
LGD_COMPAT_EVENT(TimePatchAccepters, 4)
LGD_COMPAT_EVENT(TimePatchProviders, 5)
LGD_COMPAT_EVENT(TimeCommunication, 6)
LGD_COMPAT_EVENT(TimeInput, 7)
LGD_COMPAT_EVENT(TimeOutput, 8)
#undef LGD_COMPAT_EVENT

// -------------------------------------------------------------- Simulator

template<typename CELL>
class Simulator {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    static const int DIM = Topology::DIM;
    static const unsigned NANO_STEPS = APITraits::SelectNanoSteps<CELL>::VALUE;
    typedef GridBase<CELL, DIM> GridType;
    typedef typename SharedPtr<Initializer<CELL> >::Type InitPtr;
    typedef typename SharedPtr<Steerer<CELL> >::Type SteererPtr;
    typedef std::vector<SteererPtr> SteererVector;

    explicit Simulator(Initializer<CELL> *initializer) :
        stepNum(0), initializer(initializer), gridDim(initializer->gridDimensions())
    {}

    virtual ~Simulator() {}
    virtual void step() = 0;
    virtual void run() = 0;
    virtual unsigned getStep() const { return stepNum; }
    virtual InitPtr getInitializer() const { return initializer; }
    virtual void addSteerer(Steerer<CELL> *steerer) { steerers.push_back(SteererPtr(steerer)); }
    virtual std::vector<Chronometer> gatherStatistics() = 0;

protected:
    Chronometer chronometer;
    unsigned stepNum;
    InitPtr initializer;
    SteererVector steerers;
    Coord<DIM> gridDim;
};

template<typename CELL>
class MonolithicSimulator : public Simulator<CELL> {
public:
    typedef typename SharedPtr<Writer<CELL> >::Type WriterPtr;
    typedef std::vector<WriterPtr> WriterVector;

    explicit MonolithicSimulator(Initializer<CELL> *initializer) : Simulator<CELL>(initializer) {}
    virtual const typename Simulator<CELL>::GridType *getGrid() = 0;
    virtual void addWriter(Writer<CELL> *writer) { writers.push_back(WriterPtr(writer)); }
    std::vector<Chronometer> gatherStatistics() { return std::vector<Chronometer>(1, this->chronometer); }

protected:
    WriterVector writers;
};

}  // namespace LibGeoDecomp

#endif
