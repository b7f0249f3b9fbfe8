// Jacobi-7 heat diffusion through the drop-in, as a LibGeoDecomp user
// writes it: a cell class with its API traits, a SimpleInitializer, a
// Writer, and GB300Simulator<CELL> where the application had
// CUDASimulator<CELL> (parallelization/cudasimulator.h:298-596).
//
//   jacobi3d_dropin [edge] [steps]
//
// edge^3 cells, U[0,1) initial values (the library's seeded SplitMix64,
// the same numbers as lgd_gpu_fill_uniform with seed 42, stream 1), a
// constant zero boundary; steps time steps.  Prints one JSON line: the
// wall time of GB300Simulator::run() - the initializer filling the host
// grid, the upload, the steps, and a writer reading every cell at
// WRITER_ALL_DONE - and of the steps alone, with the writer's checksum.
// The cell is bound to the library's fixed-point Jacobi kernel (two steps
// per pass over memory).
#include <libgeodecomp_gb300/gb300simulator.h>

#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

using namespace LibGeoDecomp;

class JacobiCell {
public:
    class API : public APITraits::HasCubeTopology<3>, public APITraits::HasStencil<Stencils::VonNeumann<3, 1> > {};
    explicit JacobiCell(double v = 0) : temp(v) {}
    double temp;
};

namespace LibGeoDecomp {
// the binding to the library's Jacobi kernels (one double member)
template<>
class GB300CellTraits<JacobiCell> {
public:
    static const int KIND = LGD_CELL_JACOBI7_F64_FIX;
    static const int MEMBERS = 1;
    static std::size_t memberSize(int) { return sizeof(double); }
    static void pack(const JacobiCell& c, int, void *dst) { std::memcpy(dst, &c.temp, sizeof(double)); }
    static void unpack(JacobiCell *c, int, const void *src) { std::memcpy(&c->temp, src, sizeof(double)); }
    static double edgeValue(const JacobiCell& c, int) { return c.temp; }
};
}

// SplitMix64 uniform doubles: value i = top 53 bits of mix(key + (i + 1) *
// GAMMA), key = mix(seed * 256 + stream)
static uint64_t mix(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

class UniformInit : public SimpleInitializer<JacobiCell> {
public:
    UniformInit(int edge, unsigned steps) : SimpleInitializer<JacobiCell>(Coord<3>(edge, edge, edge), steps) {}
    virtual void grid(GridBase<JacobiCell, 3> *ret)
    {
        const uint64_t key = mix(42ull * 256 + 1);
        const CoordBox<3> box = ret->boundingBox();
        const Coord<3> d = box.dimensions;
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) {
            const uint64_t idx = ((uint64_t)i->z() * d.y() + i->y()) * d.x() + i->x();
            const double v = (double)(mix(key + (idx + 1) * 0x9E3779B97F4A7C15ull) >> 11) * (1.0 / 9007199254740992.0);
            ret->set(*i, JacobiCell(v));
        }
        ret->setEdge(JacobiCell(0.0));
    }
};

class ChecksumWriter : public Writer<JacobiCell> {
public:
    ChecksumWriter(unsigned period, double *sum) : Writer<JacobiCell>("sum", period), sum(sum) {}
    Writer<JacobiCell> *clone() const { return new ChecksumWriter(period, sum); }
    void stepFinished(const GridType& grid, unsigned, WriterEvent event)
    {
        if (event != WRITER_ALL_DONE) return;
        double s = 0;
        const CoordBox<3> box = grid.boundingBox();
        for (CoordBox<3>::Iterator i = box.begin(); i != box.end(); ++i) s += grid.get(*i).temp;
        *sum = s;
    }

private:
    double *sum;
};

// times the steps alone: from WRITER_INITIALIZED (before the first step)
// to WRITER_ALL_DONE (after the last one)
class StepClock : public Writer<JacobiCell> {
public:
    StepClock(unsigned period, std::chrono::steady_clock::time_point *start, double *seconds) :
        Writer<JacobiCell>("clock", period), start(start), seconds(seconds)
    {}
    Writer<JacobiCell> *clone() const { return new StepClock(period, start, seconds); }
    void stepFinished(const GridType&, unsigned, WriterEvent event)
    {
        if (event == WRITER_INITIALIZED) *start = std::chrono::steady_clock::now();
        if (event == WRITER_ALL_DONE) {
            *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - *start).count();
        }
    }

private:
    std::chrono::steady_clock::time_point *start;
    double *seconds;
};

int main(int argc, char **argv)
{
    const int edge = argc > 1 ? std::atoi(argv[1]) : 512;
    const unsigned steps = argc > 2 ? (unsigned)std::atoi(argv[2]) : 100;
    int n = 0;
    if (lgd_gpu_device_count(&n) != LGD_OK || n == 0) {
        std::printf("{\"error\": \"no GPU\"}\n");
        return 2;
    }
    double sum = 0, stepSeconds = 0, total = 0;
    std::chrono::steady_clock::time_point stepStart;
    const auto t0 = std::chrono::steady_clock::now();
    {
        GB300Simulator<JacobiCell> sim(new UniformInit(edge, steps));
        sim.addWriter(new StepClock(steps, &stepStart, &stepSeconds));
        sim.addWriter(new ChecksumWriter(steps, &sum));
        const auto t1 = std::chrono::steady_clock::now();
        sim.run();
        total = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
    }
    const double construct = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count() - total;
    const double cells = (double)edge * edge * edge;
    std::printf("{\"cells\": %.0f, \"steps\": %u, \"run_s\": %.4f, \"steps_s\": %.4f, \"construct_s\": %.4f, "
                "\"glups_run\": %.3f, \"glups_steps\": %.3f, \"checksum\": %.17g}\n",
                cells, steps, total, stepSeconds, construct, cells * steps / total * 1e-9,
                cells * steps / stepSeconds * 1e-9, sum);
    return 0;
}
