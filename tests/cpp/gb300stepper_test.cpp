// GB300SlabStepper<CELL> (the slab stepper in the role of the reference's
// CUDAStepper): ranks as threads of one process, each with its own slab
// and device grid, ghost planes through an in-process link.  Their owned
// slabs together equal a single grid's result bit for bit - Jacobi-7 in
// IEEE FP64 and in fixed point (pinned exponent), Game of Life on a torus
// cut along y (two ranks: each the other's lower and upper neighbour), and
// a record cell running its own update() - for uneven step counts.
//
// Compiled by nvcc (the record cell); prints OK and exits 0 on success,
// exits 2 without a GPU.
#include <libgeodecomp_gb300/gb300cell.cuh>
#include <libgeodecomp_gb300/gb300stepper.h>

#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

using namespace LibGeoDecomp;

static int failures = 0;
static std::mutex failMutex;
#define EXPECT(cond)                                                          \
    do {                                                                      \
        if (!(cond)) {                                                        \
            std::lock_guard<std::mutex> lock(failMutex);                      \
            std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #cond);    \
            ++failures;                                                       \
        }                                                                     \
    } while (0)

// ------------------------------------------------------ in-process link
class Hub {
public:
    explicit Hub(int ranks) : ranks(ranks), arrived(0), generation(0), partial(0), reduced(0) {}
    int ranks;
    std::mutex m;
    std::condition_variable cv;
    std::map<std::pair<int, int>, std::deque<std::vector<unsigned char> > > box;
    int arrived, generation;
    double partial, reduced;
};

class ThreadLink : public GB300GhostLink {
public:
    ThreadLink(Hub *hub, int rank) : hub(hub), rank(rank) {}
    void send(int peer, const void *data, std::size_t bytes)
    {
        std::lock_guard<std::mutex> lock(hub->m);
        const unsigned char *p = static_cast<const unsigned char *>(data);
        hub->box[std::make_pair(rank, peer)].push_back(std::vector<unsigned char>(p, p + bytes));
        hub->cv.notify_all();
    }
    void receive(int peer, void *data, std::size_t bytes)
    {
        std::unique_lock<std::mutex> lock(hub->m);
        std::deque<std::vector<unsigned char> >& q = hub->box[std::make_pair(peer, rank)];
        hub->cv.wait(lock, [&] { return !q.empty(); });
        if (q.front().size() != bytes) throw std::runtime_error("message size mismatch");
        std::memcpy(data, q.front().data(), bytes);
        q.pop_front();
    }
    double maxOverRanks(double v)
    {
        std::unique_lock<std::mutex> lock(hub->m);
        const int gen = hub->generation;
        hub->partial = hub->arrived == 0 ? v : std::max(hub->partial, v);
        if (++hub->arrived == hub->ranks) {
            hub->reduced = hub->partial;
            hub->arrived = 0;
            ++hub->generation;
            hub->cv.notify_all();
        } else {
            hub->cv.wait(lock, [&] { return hub->generation != gen; });
        }
        return hub->reduced;
    }

private:
    Hub *hub;
    int rank;
};

// ------------------------------------------------------------------ cells
class JacobiCell {
public:
    class API : public APITraits::HasCubeTopology<3>, public APITraits::HasStencil<Stencils::VonNeumann<3, 1> > {};
    explicit JacobiCell(double v = 0) : temp(v) {}
    double temp;
};

class JacobiFixCell : public JacobiCell {
public:
    explicit JacobiFixCell(double v = 0) : JacobiCell(v) {}
};

template<typename CELL>
class JacobiTraits {
public:
    static const int MEMBERS = 1;
    static std::size_t memberSize(int) { return sizeof(double); }
    static void pack(const CELL& c, int, void *dst) { std::memcpy(dst, &c.temp, sizeof(double)); }
    static void unpack(CELL *c, int, const void *src) { std::memcpy(&c->temp, src, sizeof(double)); }
    static double edgeValue(const CELL& c, int) { return c.temp; }
};

class LifeCell {
public:
    class API : public APITraits::HasTorusTopology<2>, public APITraits::HasStencil<Stencils::Moore<2, 1> > {};
    explicit LifeCell(unsigned char a = 0) : alive(a) {}
    unsigned char alive;
};

// a record cell: its own update() on the device (3D torus, von Neumann)
class AverageCell {
public:
    class API : public APITraits::HasTorusTopology<3>, public APITraits::HasStencil<Stencils::VonNeumann<3, 1> > {};
    __host__ __device__ explicit AverageCell(float v = 0) : v(v) {}
    template<typename HOOD>
    __host__ __device__ void update(const HOOD& hood, unsigned)
    {
        v = 0.5f * hood[FixedCoord<0, 0, 0>()].v +
            0.125f * (hood[FixedCoord<0, 0, -1>()].v + hood[FixedCoord<0, 0, 1>()].v + hood[FixedCoord<0, -1, 0>()].v +
                      hood[FixedCoord<0, 1, 0>()].v);
    }
    float v;
};

namespace LibGeoDecomp {
template<>
class GB300CellTraits<JacobiCell> : public JacobiTraits<JacobiCell> {
public:
    static const int KIND = LGD_CELL_JACOBI7_F64;
};
template<>
class GB300CellTraits<JacobiFixCell> : public JacobiTraits<JacobiFixCell> {
public:
    static const int KIND = LGD_CELL_JACOBI7_F64_FIX;
};
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

// deterministic values of a global coordinate, set for whatever box the
// target grid covers (one initializer serves the slabs and the whole grid)
template<typename CELL>
class ValueInit : public SimpleInitializer<CELL> {
public:
    static const int DIM = APITraits::SelectTopology<CELL>::Value::DIM;
    ValueInit(Coord<DIM> dim, unsigned steps) : SimpleInitializer<CELL>(dim, steps) {}
    virtual void grid(GridBase<CELL, DIM> *ret)
    {
        const CoordBox<DIM> box = ret->boundingBox();
        for (typename CoordBox<DIM>::Iterator i = box.begin(); i != box.end(); ++i) {
            unsigned h = 2166136261u;
            for (int d = 0; d < DIM; ++d) h = (h ^ (unsigned)(*i)[d]) * 16777619u;
            ret->set(*i, make(h));
        }
        ret->setEdge(CELL());
    }
    static CELL make(unsigned h);
};
template<> JacobiCell ValueInit<JacobiCell>::make(unsigned h) { return JacobiCell((h % 100003) / 100003.0); }
template<> JacobiFixCell ValueInit<JacobiFixCell>::make(unsigned h) { return JacobiFixCell((h % 100003) / 100003.0); }
template<> LifeCell ValueInit<LifeCell>::make(unsigned h) { return LifeCell((h >> 7) % 10 < 3); }
template<> AverageCell ValueInit<AverageCell>::make(unsigned h) { return AverageCell((float)((h % 1009) / 1009.0)); }

// The single grid: the same stepper with one rank (one library grid, no
// ghost zones, the same steps per call - fixed-point passes of two steps
// round differently from two single steps, so the pass structure must
// match), and for the exact cells also GB300Simulator one step at a time.
template<typename CELL>
static std::vector<CELL> singleRun(Coord<APITraits::SelectTopology<CELL>::Value::DIM> dim, unsigned steps,
                                   unsigned ghost, bool simulator)
{
    static const int DIM = APITraits::SelectTopology<CELL>::Value::DIM;
    std::vector<CELL> out;
    if (simulator) {
        GB300Simulator<CELL> sim(new ValueInit<CELL>(dim, steps));
        for (unsigned s = 0; s < steps; ++s) sim.step();
        const GridBase<CELL, DIM> *g = sim.getGrid();
        CoordBox<DIM> box = g->boundingBox();
        for (typename CoordBox<DIM>::Iterator c = box.begin(); c != box.end(); ++c) out.push_back(g->get(*c));
    } else {
        GB300SlabStepper<CELL> st(new ValueInit<CELL>(dim, steps), 0, 1, ghost, 0);
        st.update(steps / 3);
        st.update(steps - steps / 3);
        const GridBase<CELL, DIM> *g = st.getGrid();
        CoordBox<DIM> box = g->boundingBox();
        for (typename CoordBox<DIM>::Iterator c = box.begin(); c != box.end(); ++c) out.push_back(g->get(*c));
    }
    return out;
}

template<typename CELL>
static long countDiffer(const std::vector<CELL>& a, const std::vector<CELL>& b)
{
    if (a.size() != b.size()) return -1;
    long differ = 0;
    for (std::size_t i = 0; i < a.size(); ++i) {
        differ += std::memcmp(static_cast<const void *>(&a[i]), static_cast<const void *>(&b[i]), sizeof(CELL)) != 0;
    }
    return differ;
}

template<typename CELL>
static void compareSlabs(Coord<APITraits::SelectTopology<CELL>::Value::DIM> dim, int ranks, unsigned ghost,
                         unsigned steps, bool fixedPoint)
{
    static const int DIM = APITraits::SelectTopology<CELL>::Value::DIM;
    Hub hub(ranks);
    std::vector<std::vector<CELL> > parts(ranks);
    std::vector<unsigned> exchanges(ranks), stepsDone(ranks);
    std::vector<int> exponents(ranks);
    std::vector<std::thread> threads;
    for (int r = 0; r < ranks; ++r) {
        threads.push_back(std::thread([&, r] {
            try {
                ThreadLink link(&hub, r);
                GB300SlabStepper<CELL> st(new ValueInit<CELL>(dim, steps), r, ranks, ghost, &link);
                if (fixedPoint) gb300Check(lgd_gpu_fixed_point_exponent(st.deviceHandle(), &exponents[r]));
                st.update(steps / 3);
                st.update(steps - steps / 3);
                const GridBase<CELL, DIM> *g = st.getGrid();
                CoordBox<DIM> box = g->boundingBox();
                for (typename CoordBox<DIM>::Iterator c = box.begin(); c != box.end(); ++c) {
                    parts[r].push_back(g->get(*c));
                }
                exchanges[r] = st.exchangeCount();
                stepsDone[r] = st.currentStep();
            } catch (const std::exception& e) {
                std::lock_guard<std::mutex> lock(failMutex);
                std::printf("rank %d: %s\n", r, e.what());
                ++failures;
            }
        }));
    }
    for (std::size_t t = 0; t < threads.size(); ++t) threads[t].join();
    std::vector<CELL> whole;
    for (int r = 0; r < ranks; ++r) whole.insert(whole.end(), parts[r].begin(), parts[r].end());
    const long differ = countDiffer(whole, singleRun<CELL>(dim, steps, ghost, false));
    if (differ) std::printf("%ld cells differ from the single grid\n", differ);
    EXPECT(differ == 0);
    if (!fixedPoint) {
        const long differSim = countDiffer(whole, singleRun<CELL>(dim, steps, ghost, true));
        if (differSim) std::printf("%ld cells differ from GB300Simulator\n", differSim);
        EXPECT(differSim == 0);
    }
    for (int r = 0; r < ranks; ++r) {
        EXPECT(stepsDone[r] == steps);
        EXPECT(exchanges[r] >= steps / ghost);
        if (fixedPoint) EXPECT(exponents[r] == exponents[0]);
    }
}

// arguments the stepper refuses, each with std::invalid_argument and no
// leaked initializer (the stepper owns and deletes it either way)
static void testStepperErrors()
{
    struct Case {
        int rank, ranks;
        unsigned ghost;
        bool link;
    };
    const Case cases[] = {
        {2, 2, 4, false},     // rank outside the world
        {0, 0, 4, false},     // no ranks
        {0, 2, 4, false},     // several ranks without a link
        {0, 2, 0, true},      // ghost width zero
        {0, 3, 16, true},     // 30 planes over 3 ranks: fewer planes than the ghost width
    };
    Hub hub(3);
    for (const Case& c : cases) {
        ThreadLink link(&hub, 0);
        bool threw = false;
        try {
            GB300SlabStepper<JacobiCell> st(new ValueInit<JacobiCell>(Coord<3>(8, 8, 30), 4), c.rank, c.ranks, c.ghost,
                                            c.link ? &link : 0);
        } catch (const std::invalid_argument&) {
            threw = true;
        }
        EXPECT(threw);
    }
}

int main()
{
    int n = 0;
    if (lgd_gpu_device_count(&n) != LGD_OK || n == 0) {
        std::printf("no GPU\n");
        return 2;
    }
    compareSlabs<JacobiCell>(Coord<3>(45, 21, 30), 3, 4, 19, false);
    compareSlabs<JacobiFixCell>(Coord<3>(64, 20, 33), 2, 4, 22, true);
    compareSlabs<LifeCell>(Coord<2>(70, 41), 2, 6, 31, false);
    compareSlabs<LifeCell>(Coord<2>(64, 60), 4, 5, 23, false);
    compareSlabs<AverageCell>(Coord<3>(20, 16, 24), 3, 3, 14, false);
    testStepperErrors();
    if (failures) {
        std::printf("%d failure(s)\n", failures);
        return 1;
    }
    std::printf("OK\n");
    return 0;
}
