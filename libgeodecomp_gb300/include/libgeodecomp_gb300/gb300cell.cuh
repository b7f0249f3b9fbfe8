// gb300cell.cuh: a user's own cell class on the GPU.
//
// The reference's CUDASimulator<CELL> runs any cell whose update(hood,
// nanoStep) (or, with APITraits::HasSeparateCUDAUpdate, updateCUDA) is a
// __device__ function: kernel2D/kernel3D walk the grid and call it through
// CUDAUpdateFunctor with a neighbourhood object that maps FixedCoord offsets
// to cells (parallelization/cudasimulator.h:26-236,
// storage/cudaupdatefunctor.h:14-45, misc/apitraits.h:814-836).  This
// header does the same for GB300Simulator: include it from a translation
// unit that nvcc compiles, and a cell without a GB300CellTraits binding to
// one of the library's compiled kernels runs its own update() on the device:
//
//   #include <libgeodecomp_gb300/gb300cell.cuh>
//   class MyCell { ... __host__ __device__ void update(const HOOD& hood,
//                  unsigned nanoStep) { ... hood[FixedCoord<0, -1, 0>()] ... } };
//   GB300Simulator<MyCell> sim(new MyInitializer);   // runs MyCell::update
//
// The grid is the library's record grid (LGD_CELL_RECORD: one sizeof(CELL)
// record per cell, rows pitched to 128 bytes, double buffered); Writers,
// Steerers, snapshots and the statistics work as for the compiled kernels.
// The cell must be copyable as bytes (the reference copies cells between
// host and device with cudaMemcpy as well).
//
// Device side, per step: one thread per x, marching y (2D) or z (3D) over a
// chunk of rows, calls the cell's update() on the new grid's record with a
// neighbourhood over the old grid: hood[FixedCoord<X, Y, Z>()] and
// hood[Coord<DIM>] give the cell at that offset, wrapped on periodic axes,
// the edge cell (staged in shared memory) outside the others - what the
// reference's SoA and AoS grids deliver (storage/fixedneighborhood.h:36-120,
// storage/displacedgrid.h:324-330).  Offsets up to the grid's size wrap any
// number of times.
#ifndef LGD_GB300_CELL_CUH
#define LGD_GB300_CELL_CUH

#include <cuda_runtime.h>

#include <stdexcept>
#include <string>

#include "gb300simulator.h"

namespace LibGeoDecomp {

namespace GB300CellDevice {

__device__ __forceinline__ int wrapAxis(int i, int n)
{
    i = (i < 0) ? i + n : i - n;
    if ((unsigned)i >= (unsigned)n) i = ((i % n) + n) % n;
    return i;
}

// The neighbourhood a cell's update() receives on the device.
template<typename CELL, int DIM, bool WX, bool WY, bool WZ>
class Hood {
public:
    __device__ __forceinline__ Hood(const unsigned char *base, long pitch, int nx, int ny, int nz, const CELL *edge) :
        base(base), pitch(pitch), nx(nx), ny(ny), nz(nz), x(0), y(0), z(0), edge(edge)
    {}

    __device__ __forceinline__ void moveTo(int cx, int cy, int cz)
    {
        x = cx;
        y = cy;
        z = cz;
    }

    template<int X, int Y, int Z>
    __device__ __forceinline__ const CELL& operator[](FixedCoord<X, Y, Z>) const
    {
        return at(X, DIM > 1 ? Y : 0, DIM > 2 ? Z : 0);
    }

    __device__ __forceinline__ const CELL& operator[](const Coord<DIM>& c) const
    {
        return at(c[0], DIM > 1 ? c[1] : 0, DIM > 2 ? c[2] : 0);
    }

private:
    const unsigned char *base;
    long pitch;
    int nx, ny, nz;
    int x, y, z;
    const CELL *edge;

    __device__ __forceinline__ const CELL& at(int dx, int dy, int dz) const
    {
        int xn = x + dx;
        int yn = y + dy;
        int zn = z + dz;
        if (dx != 0 && (unsigned)xn >= (unsigned)nx) {
            if (!WX) return *edge;
            xn = wrapAxis(xn, nx);
        }
        if (DIM > 1 && dy != 0 && (unsigned)yn >= (unsigned)ny) {
            if (!WY) return *edge;
            yn = wrapAxis(yn, ny);
        }
        if (DIM > 2 && dz != 0 && (unsigned)zn >= (unsigned)nz) {
            if (!WZ) return *edge;
            zn = wrapAxis(zn, nz);
        }
        return *reinterpret_cast<const CELL *>(base + ((long)zn * ny + yn) * pitch + (long)xn * (long)sizeof(CELL));
    }
};

// CUDAUpdateFunctor's choice between update() and updateCUDA()
template<typename CELL, typename HOOD>
__device__ __forceinline__ void runUpdate(CELL& cell, const HOOD& hood, unsigned nanoStep, APITraits::FalseType)
{
    cell.update(hood, nanoStep);
}

template<typename CELL, typename HOOD>
__device__ __forceinline__ void runUpdate(CELL& cell, const HOOD& hood, unsigned nanoStep, APITraits::TrueType)
{
    cell.updateCUDA(hood, nanoStep);
}

// One step of the whole grid: thread (x, row band) marches `chunk` rows of
// y (2D) or z (3D); 1D grids have one cell per thread.
template<typename CELL, int DIM, bool WX, bool WY, bool WZ>
__global__ void __launch_bounds__(128)
stepKernel(const unsigned char *__restrict__ oldBase, unsigned char *__restrict__ newBase, long pitch, int nx, int ny,
           int nz, int chunk, const CELL *__restrict__ edgeDevice, unsigned nanoStep)
{
    // the edge cell, once per CTA, as 4-byte words where its size allows
    __shared__ __align__(16) unsigned char edgeBytes[sizeof(CELL)];
    if (sizeof(CELL) % 4 == 0) {
        for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < (int)(sizeof(CELL) / 4); i += blockDim.x * blockDim.y) {
            reinterpret_cast<unsigned *>(edgeBytes)[i] = reinterpret_cast<const unsigned *>(edgeDevice)[i];
        }
    } else {
        for (int i = threadIdx.x + threadIdx.y * blockDim.x; i < (int)sizeof(CELL); i += blockDim.x * blockDim.y) {
            edgeBytes[i] = reinterpret_cast<const unsigned char *>(edgeDevice)[i];
        }
    }
    __syncthreads();
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nx) return;
    Hood<CELL, DIM, WX, WY, WZ> hood(oldBase, pitch, nx, ny, nz, reinterpret_cast<const CELL *>(edgeBytes));
    typedef typename APITraits::SelectSeparateCUDAUpdate<CELL>::Value Separate;
    int y0, y1, z0, z1;
    if (DIM == 3) {
        y0 = blockIdx.y * blockDim.y + threadIdx.y;
        if (y0 >= ny) return;
        y1 = y0 + 1;
        z0 = blockIdx.z * chunk;
        z1 = ::min(z0 + chunk, nz);
    } else if (DIM == 2) {
        y0 = (blockIdx.y * blockDim.y + threadIdx.y) * chunk;
        y1 = ::min(y0 + chunk, ny);
        z0 = 0;
        z1 = 1;
    } else {
        y0 = 0;
        y1 = 1;
        z0 = 0;
        z1 = 1;
    }
    for (int z = z0; z < z1; ++z) {
        for (int y = y0; y < y1; ++y) {
            hood.moveTo(x, y, z);
            CELL& target = *reinterpret_cast<CELL *>(newBase + ((long)z * ny + y) * pitch + (long)x * (long)sizeof(CELL));
            runUpdate(target, hood, nanoStep, Separate());
        }
    }
}

inline void check(int rc)
{
    gb300Check(rc);
}

}  // namespace GB300CellDevice

// Steps of a record grid: count updates of the whole grid, the k-th with
// nano step (nanoStep + k) % NANO_STEPS, each one launch on the handle's
// stream followed by the buffer swap (CUDASimulator::step's nano-step loop,
// parallelization/cudasimulator.h:467-470, 560-594).
template<typename CELL>
struct GB300DeviceStep<CELL, true> {
    typedef typename APITraits::SelectTopology<CELL>::Value Topology;
    static const int DIM = Topology::DIM;
    static const bool WX = Topology::template WrapsAxis<0>::VALUE;
    static const bool WY = DIM > 1 && Topology::template WrapsAxis<1>::VALUE;
    static const bool WZ = DIM > 2 && Topology::template WrapsAxis<2>::VALUE;
    static const unsigned NANO_STEPS = APITraits::SelectNanoSteps<CELL>::VALUE;

    static void run(lgd_handle *h, unsigned nanoStep, int count)
    {
        using GB300CellDevice::check;
        lgd_grid_desc d;
        check(lgd_gpu_get_desc(h, &d));
        if (d.cell != LGD_CELL_RECORD || d.dim != DIM) {
            throw std::invalid_argument("the handle is not a record grid of this cell's dimension");
        }
        void *streamPtr = 0;
        const void *edge = 0;
        check(lgd_gpu_stream(h, &streamPtr));
        check(lgd_gpu_edge_record_device(h, &edge));
        cudaStream_t stream = (cudaStream_t)streamPtr;
        dim3 block, grid;
        int chunk = 1;
        if (DIM == 3) {
            block = dim3(32, 4, 1);
            grid = dim3((d.nx + 31) / 32, (d.ny + 3) / 4, 1);
            // about 16 CTAs per SM of a 152-SM GPU in all, chunks of z planes
            const long long xy = (long long)grid.x * grid.y;
            const long long split = std::max(1LL, std::min((long long)d.nz, (152LL * 16 + xy - 1) / xy));
            chunk = (int)((d.nz + split - 1) / split);
            grid.z = (unsigned)((d.nz + chunk - 1) / chunk);
        } else if (DIM == 2) {
            block = dim3(128, 1, 1);
            grid = dim3((d.nx + 127) / 128, 1, 1);
            const long long split = std::max(1LL, std::min((long long)d.ny, (152LL * 16 + grid.x - 1) / grid.x));
            chunk = (int)((d.ny + split - 1) / split);
            grid.y = (unsigned)((d.ny + chunk - 1) / chunk);
        } else {
            block = dim3(128, 1, 1);
            grid = dim3((d.nx + 127) / 128, 1, 1);
        }
        for (int k = 0; k < count; ++k) {
            void *oldPtr = 0;
            void *newPtr = 0;
            size_t pitch = 0;
            check(lgd_gpu_device_ptr(h, 0, 0, &oldPtr, &pitch));
            check(lgd_gpu_device_ptr(h, 0, 1, &newPtr, &pitch));
            const unsigned nano = (unsigned)((nanoStep + (unsigned)k) % NANO_STEPS);
            GB300CellDevice::stepKernel<CELL, DIM, WX, WY, WZ><<<grid, block, 0, stream>>>(
                (const unsigned char *)oldPtr, (unsigned char *)newPtr, (long)pitch, d.nx, d.ny, d.nz, chunk,
                (const CELL *)edge, nano);
            const cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                throw std::runtime_error(std::string("CUDA error: ") + cudaGetErrorString(e) +
                                         " launching the cell's update kernel");
            }
            check(lgd_gpu_count_launches(h, 1));
            check(lgd_gpu_swap(h));
        }
    }
};

}  // namespace LibGeoDecomp

#endif
