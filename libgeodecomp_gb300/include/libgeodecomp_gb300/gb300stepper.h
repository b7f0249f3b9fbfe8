// GB300SlabStepper<CELL>: one rank's slab of a grid on this rank's GPU,
// with ghost zones exchanged through a link the application provides.
//
// This plays the role of the reference's CUDAStepper inside
// HiParSimulator (parallelization/nesting/cudastepper.h:195-420): a node
// advances its part of the grid on its GPU and trades ghost zones of width
// G (ghostZoneWidth, parallelization/hiparsimulator.h:60-72) with its
// neighbours every G updates through patch links
// (communication/patchlink.h).  Here the grid is cut along its slowest axis
// (z in 3D, y in 2D) into even slabs, the ghost zones are whole planes, the
// library's kernels advance the slab and its ghost zones together (a
// slab's owned planes stay exact for G updates because wrong values spread
// one plane per update from the ghost zone's outer face), and the link
// carries raw planes (the device representation, lgd_gpu_copy_planes).
// Results equal a single grid's bit for bit; fixed-point cells keep one
// pinned exponent on every rank.
//
// The link is the application's transport (MPI, sockets, or threads of
// one process): per exchange the stepper posts the planes it sends to each
// neighbour, receives the neighbours' planes and finishes; at construction
// it calls maxOverRanks once to agree on a fixed-point exponent.  Partition
// managers, load balancing and the nesting of steppers are out of scope.
#ifndef LGD_GB300_STEPPER_H
#define LGD_GB300_STEPPER_H

#include <algorithm>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "gb300simulator.h"

namespace LibGeoDecomp {

// Transport between the ranks of a slab decomposition.  An exchange posts
// every send first, then receives, then finishes: send() must not wait for
// the peer to receive (copy the data or post a non-blocking send, as
// MPI_Isend does), so rings of ranks cannot deadlock.  Between a pair of
// ranks messages arrive in the order they were sent.
class GB300GhostLink {
public:
    virtual ~GB300GhostLink() {}
    virtual void send(int peer, const void *data, std::size_t bytes) = 0;
    // the next message from `peer`, `bytes` long, into data (host memory)
    virtual void receive(int peer, void *data, std::size_t bytes) = 0;
    // completes this exchange's sends (their buffers may be reused after)
    virtual void finish() {}
    // the maximum of v over all ranks
    virtual double maxOverRanks(double v) = 0;
};

template<typename CELL>
class GB300SlabStepper {
public:
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    static const int DIM = Topology::DIM;
    static const unsigned NANO_STEPS = APITraits::SelectNanoSteps<CELL>::VALUE;
    typedef GB300CellTraits<CELL> Traits;
    typedef DisplacedGrid<CELL, Topology> HostGrid;

    // init fills the global grid's cells of this rank's slab (its
    // gridDimensions() are the global ones) and the edge cell; the stepper
    // owns it, as the reference's simulators own their initializers.  link
    // may be null for a single rank.
    GB300SlabStepper(Initializer<CELL> *init, int rank, int ranks, unsigned ghostWidth, GB300GhostLink *link) :
        initializer(init), link(link), rank(rank), ranks(ranks), ghost(ghostWidth), handle(0), since(ghostWidth),
        exchanges(0), step(init->startStep()), nano(0), nanoDone(0), hostGrid(0)
    {
        static_assert(DIM == 2 || DIM == 3, "slabs cut 2D and 3D grids");
        try {
            if (ranks < 1 || rank < 0 || rank >= ranks) throw std::invalid_argument("rank outside the world");
            if (ghostWidth < 1) throw std::invalid_argument("ghost width must be at least one plane");
            if (ranks > 1 && !link) throw std::invalid_argument("several ranks need a link");
            global = init->gridDimensions();
            const int n = global[DIM - 1];
            const int base = n / ranks, extra = n % ranks;
            p0 = rank * base + std::min(rank, extra);
            p1 = p0 + base + (rank < extra ? 1 : 0);
            const bool wraps = Topology::template WrapsAxis<DIM - 1>::VALUE;
            lower = (ranks == 1) ? -1 : (rank > 0 ? rank - 1 : (wraps ? ranks - 1 : -1));
            upper = (ranks == 1) ? -1 : (rank < ranks - 1 ? rank + 1 : (wraps ? 0 : -1));
            if (ranks > 1 && (unsigned)(p1 - p0) < ghostWidth) {
                throw std::invalid_argument("every rank needs at least ghostWidth planes");
            }
            ghostLo = lower >= 0 ? (int)ghost : 0;
            ghostHi = upper >= 0 ? (int)ghost : 0;
            // the owned slab on the host
            Coord<DIM> origin;
            Coord<DIM> dim = global;
            origin[DIM - 1] = p0;
            dim[DIM - 1] = p1 - p0;
            owned = CoordBox<DIM>(origin, dim);
            hostGrid = new HostGrid(owned);
            init->grid(hostGrid);
            // a wrapping cut axis wraps locally too: with one rank it is the
            // whole axis; with several every face is a ghost face, and what
            // lies beyond a ghost zone never reaches the owned planes
            // between two exchanges, so the torus fast paths stay in use
            createDevice(wraps);
            upload();
        } catch (...) {
            if (handle) lgd_gpu_destroy(handle);
            delete hostGrid;
            delete initializer;
            throw;
        }
    }

    ~GB300SlabStepper()
    {
        if (handle) lgd_gpu_destroy(handle);
        delete hostGrid;
        delete initializer;
    }

    // Advances the slab by `steps` time steps (NANO_STEPS updates each),
    // exchanging ghost zones every `ghostWidth` updates.
    void update(unsigned steps)
    {
        unsigned long long left = (unsigned long long)steps * NANO_STEPS;
        while (left > 0) {
            if (since >= ghost) exchangeGhosts();
            const unsigned k = (unsigned)std::min<unsigned long long>(left, ghost - since);
            GB300DeviceStep<CELL>::run(handle, nano, (int)k);
            nano = (nano + k) % NANO_STEPS;
            since += k;
            left -= k;
            const unsigned long long done = (unsigned long long)k + nanoDone;
            step += (unsigned)(done / NANO_STEPS);
            nanoDone = (unsigned)(done % NANO_STEPS);
        }
        gb300Check(lgd_gpu_synchronize(handle));
    }

    unsigned currentStep() const { return step; }
    const CoordBox<DIM>& ownedBox() const { return owned; }
    unsigned exchangeCount() const { return exchanges; }
    lgd_handle *deviceHandle() { return handle; }

    // The owned cells as they are now (copied from the device).
    const GridBase<CELL, DIM> *getGrid()
    {
        download();
        return hostGrid;
    }

private:
    Initializer<CELL> *initializer;
    GB300GhostLink *link;
    int rank, ranks;
    unsigned ghost;
    lgd_handle *handle;
    unsigned since;                 // updates since the last exchange
    unsigned exchanges;
    unsigned step;
    unsigned nano;                  // nano step of the next update
    unsigned nanoDone;              // updates of the current step done
    Coord<DIM> global;
    int p0, p1, lower, upper, ghostLo, ghostHi;
    CoordBox<DIM> owned;
    HostGrid *hostGrid;
    std::vector<unsigned char> sendBuf, recvBuf;

    int localPlanes() const { return ghostLo + (p1 - p0) + ghostHi; }

    // cells of one plane of the cut axis
    std::size_t planeCells() const { return (std::size_t)global[0] * (DIM == 3 ? global[1] : 1); }

    // rows of the owned box in the host grid, which stores x fastest (the
    // reference's DisplacedGrid): row r starts at rowPointer(r), nx cells
    std::size_t ownedRows() const
    {
        return (std::size_t)owned.dimensions[1] * (DIM == 3 ? (std::size_t)owned.dimensions[2] : 1);
    }

    CELL *rowPointer(std::size_t r)
    {
        Coord<DIM> c = owned.origin;
        c[1] += (int)(r % (std::size_t)owned.dimensions[1]);
        if (DIM == 3) c[2] += (int)(r / (std::size_t)owned.dimensions[1]);
        return &(*hostGrid)[c];
    }

    void createDevice(bool cutAxisWraps)
    {
        lgd_grid_desc d;
        std::memset(&d, 0, sizeof(d));
        d.dim = DIM;
        d.nx = global[0];
        d.ny = DIM == 3 ? global[1] : localPlanes();
        d.nz = DIM == 3 ? localPlanes() : 1;
        d.periodic = (Topology::template WrapsAxis<0>::VALUE ? 1 : 0) |
                     (DIM == 3 && Topology::template WrapsAxis<1>::VALUE ? 2 : 0);
        if (cutAxisWraps) d.periodic |= 1 << (DIM - 1);
        d.cell = Traits::KIND;
        d.flags = GB300DescFlags<Traits>::value();
        if (Traits::KIND == LGD_CELL_RECORD) {
            gb300Check(lgd_gpu_create_records(&d, sizeof(CELL), static_cast<const void *>(&hostGrid->getEdge()),
                                              &handle));
        } else {
            for (int m = 0; m < Traits::MEMBERS && m < 4; ++m) d.edge[m] = Traits::edgeValue(hostGrid->getEdge(), m);
            gb300Check(lgd_gpu_create(&d, &handle));
        }
    }

    // owned cells -> the local grid's owned planes (the ghost planes follow
    // from the first exchange); fixed-point grids first agree on one pinned
    // exponent, the one the whole grid's maximum needs
    void upload()
    {
        const std::size_t cells = planeCells() * (std::size_t)localPlanes();
        const std::size_t nx = (std::size_t)owned.dimensions[0];
        if (Traits::KIND == LGD_CELL_JACOBI7_F64_FIX) {
            double m = 0.0;
            for (std::size_t r = 0; r < ownedRows(); ++r) {
                const CELL *row = rowPointer(r);
                for (std::size_t x = 0; x < nx; ++x) {
                    double v;
                    Traits::pack(row[x], 0, &v);
                    m = std::max(m, std::fabs(v));
                }
            }
            m = link ? link->maxOverRanks(m) : m;
            int e = 0;
            if (m > 0) std::frexp(m, &e);
            gb300Check(lgd_gpu_set_fixed_point_exponent(handle, e, 1));
        }
        for (int m = 0; m < Traits::MEMBERS; ++m) {
            const std::size_t sz = Traits::memberSize(m);
            std::vector<char> buf(cells * sz);
            char *dst = buf.data() + (std::size_t)ghostLo * planeCells() * sz;
            for (std::size_t r = 0; r < ownedRows(); ++r) {
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
        since = ghost;
    }

    void download()
    {
        const std::size_t cells = planeCells() * (std::size_t)localPlanes();
        for (int m = 0; m < Traits::MEMBERS; ++m) {
            const std::size_t sz = Traits::memberSize(m);
            std::vector<char> buf(cells * sz);
            gb300Check(lgd_gpu_download(handle, m, 0, buf.data(), buf.size()));
            const char *src = buf.data() + (std::size_t)ghostLo * planeCells() * sz;
            const std::size_t nx = (std::size_t)owned.dimensions[0];
            for (std::size_t r = 0; r < ownedRows(); ++r) {
                CELL *row = rowPointer(r);
                if (Traits::KIND == LGD_CELL_RECORD) {
                    std::memcpy(static_cast<void *>(row), src, nx * sizeof(CELL));
                    src += nx * sizeof(CELL);
                } else {
                    for (std::size_t x = 0; x < nx; ++x, src += sz) Traits::unpack(&row[x], m, src);
                }
            }
        }
    }

    // The ghost planes of every member from the neighbours, the lower side
    // first.  With two ranks on a wrapping axis the neighbour is both the
    // lower and the upper one, and its first message (its lower-side
    // planes) fills this rank's upper ghost zone.
    void exchangeGhosts()
    {
        if (ranks == 1 || (lower < 0 && upper < 0)) {
            since = 0;
            return;
        }
        const int mine = p1 - p0;
        struct Side {
            int peer, send0, recv0;
        };
        std::vector<Side> sides;
        if (lower >= 0) sides.push_back({lower, ghostLo, 0});
        if (upper >= 0) sides.push_back({upper, ghostLo + mine - (int)ghost, ghostLo + mine});
        const bool samePeer = sides.size() == 2 && sides[0].peer == sides[1].peer;
        for (int m = 0; m < Traits::MEMBERS; ++m) {
            std::size_t planeBytes = 0;
            gb300Check(lgd_gpu_plane_bytes(handle, m, &planeBytes));
            const std::size_t bytes = planeBytes * ghost;
            sendBuf.resize(bytes * sides.size());
            recvBuf.resize(bytes * sides.size());
            for (std::size_t k = 0; k < sides.size(); ++k) {
                gb300Check(lgd_gpu_copy_planes(handle, m, 0, sides[k].send0, (int)ghost, &sendBuf[k * bytes], bytes, 0));
                link->send(sides[k].peer, &sendBuf[k * bytes], bytes);
            }
            for (std::size_t k = 0; k < sides.size(); ++k) {
                const std::size_t r = samePeer ? sides.size() - 1 - k : k;
                link->receive(sides[k].peer, &recvBuf[r * bytes], bytes);
            }
            link->finish();
            for (std::size_t k = 0; k < sides.size(); ++k) {
                gb300Check(lgd_gpu_copy_planes(handle, m, 0, sides[k].recv0, (int)ghost, &recvBuf[k * bytes], bytes, 1));
            }
        }
        ++exchanges;
        since = 0;
    }
};

}  // namespace LibGeoDecomp

#endif
