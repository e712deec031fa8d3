// nk_noalloc.cu — nk_picard_change_noalloc: the Picard change measure of a velocity pair, computed with no
// device allocation.
//
// Some hosts cannot let a library call cudaMalloc or cudaFree at the moment they need a result.  A model
// driving its own time loop inside a framework that pools device memory (a Julia CUDA.jl or PyTorch caching
// allocator sized to the whole device) gets OOM from a stray cudaMalloc, and cudaFree synchronises the
// device in the middle of that loop.  For those callers this entry point keeps its scratch (one partial sum
// per thread block plus the blocks' arrival counter) in a statically sized __device__ array of this
// library.  Every GPU that loads the library holds that array until the process exits.
//
// The computation is the reduction of k_picard_end (one thread per cell, 32 x 8 blocks, per-block partials
// summed in block order by the last block to arrive).  On the same velocities it gives the same
// ||(u, v) - (u_prev, v_prev)|| and ||(u, v)|| that nk_picard_solve reports as picard_change and
// picard_norm, read from caller memory in the interior layout of nk_problem_get_field.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "nk_internal.cuh"

constexpr int NOALLOC_SCRATCH_HEADER = 256;   // the arrival counter, padded so the partials start 256-byte aligned
constexpr size_t NOALLOC_SCRATCH_BYTES = NOALLOC_SCRATCH_HEADER + sizeof(double2) * (size_t)NK_NOALLOC_MAX_BLOCKS;

// The scratch (262,400 bytes): bytes [0, 4) the arrival counter of the grid reduction, which must be zero when
// a launch starts; bytes [256, 256 + 16 * NK_NOALLOC_MAX_BLOCKS) one (sum of squared changes, sum of squares)
// pair per block.  In host code this name is only a handle for cudaGetSymbolAddress, not a device address.
static __device__ __align__(256) unsigned char noalloc_scratch[NOALLOC_SCRATCH_BYTES];

namespace {

constexpr int MAX_DEVICES = 64;

std::mutex setup_mutex;
void* scratch_address[MAX_DEVICES] = {};   // device address of noalloc_scratch, per CUDA ordinal

__global__ void k_picard_change_noalloc(int Nx, int Ny, int u_stride, const double* __restrict__ u,
                                        const double* __restrict__ v, const double* __restrict__ u_prev,
                                        const double* __restrict__ v_prev, unsigned char* scratch, double* out) {
    int i = blockIdx.x * nk::BX + threadIdx.x, j = blockIdx.y * nk::BY + threadIdx.y;
    double dd = 0.0, xx = 0.0;
    if (i < Nx && j < Ny) {
        size_t ku = (size_t)j * u_stride + i, kv = (size_t)j * Nx + i;
        double bx = u[ku], by = v[kv];
        double ax = u_prev[ku] + (-1.0) * bx;
        double ay = v_prev[kv] + (-1.0) * by;
        dd = ax * ax + ay * ay;
        xx = bx * bx + by * by;
    }
    double tdd, txx;
    unsigned int* ticket = reinterpret_cast<unsigned int*>(scratch);
    double2* partials = reinterpret_cast<double2*>(scratch + NOALLOC_SCRATCH_HEADER);
    if (nk::grid_sum2(dd, xx, partials, ticket, tdd, txx) && threadIdx.x == 0 && threadIdx.y == 0) {
        out[0] = sqrt(tdd);
        out[1] = sqrt(txx);
    }
}

struct NoAllocError {
    nk_status status;
    std::string message;
};

// Device address of the scratch on the current device `device`, looked up on the first call there.
void* scratch_on(int device) {
    if (device < 0 || device >= MAX_DEVICES)
        throw NoAllocError{NK_BAD_ARGUMENT, "nk_picard_change_noalloc: device ordinal " + std::to_string(device) +
                                                " beyond the " + std::to_string(MAX_DEVICES) + " supported"};
    std::lock_guard<std::mutex> lock(setup_mutex);
    if (!scratch_address[device]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, noalloc_scratch);
        if (e != cudaSuccess || !ptr)
            throw NoAllocError{NK_CUDA_ERROR, std::string("nk_picard_change_noalloc: cudaGetSymbolAddress: ") +
                                                  cudaGetErrorString(e)};
        scratch_address[device] = ptr;
    }
    return scratch_address[device];
}

}  // namespace

extern "C" nk_status nk_picard_change_noalloc(nk_context* ctx, const nk_grid_desc* grid, const double* u,
                                              const double* v, const double* u_prev, const double* v_prev,
                                              double* change_and_norm, void* stream) {
    if (!ctx) return NK_BAD_ARGUMENT;
    try {
        if (!grid || !u || !v || !u_prev || !v_prev || !change_and_norm)
            throw NoAllocError{NK_BAD_ARGUMENT, "nk_picard_change_noalloc: null grid or device pointer"};
        if (grid->Nx <= 0 || grid->Ny <= 0)
            throw NoAllocError{NK_BAD_ARGUMENT, "nk_picard_change_noalloc: Nx and Ny must be positive"};
        bool tx = grid->topology_x == NK_BOUNDED || grid->topology_x == NK_PERIODIC;
        bool ty = grid->topology_y == NK_BOUNDED || grid->topology_y == NK_PERIODIC;
        if (!tx || !ty) throw NoAllocError{NK_BAD_ARGUMENT, "nk_picard_change_noalloc: unknown topology"};
        long long bx = (grid->Nx + nk::BX - 1) / nk::BX, by = (grid->Ny + nk::BY - 1) / nk::BY;
        if (bx * by > NK_NOALLOC_MAX_BLOCKS)
            throw NoAllocError{NK_BAD_ARGUMENT,
                               "nk_picard_change_noalloc: a " + std::to_string(grid->Nx) + " x " +
                                   std::to_string(grid->Ny) + " grid needs " + std::to_string(bx * by) +
                                   " reduction blocks of 32 x 8 cells; the static scratch holds " +
                                   std::to_string(NK_NOALLOC_MAX_BLOCKS) + " (e.g. 2048 x 2048 cells)"};
        cudaError_t e = cudaSetDevice(ctx->device);
        if (e != cudaSuccess)
            throw NoAllocError{NK_CUDA_ERROR, std::string("cudaSetDevice: ") + cudaGetErrorString(e)};
        unsigned char* scratch = static_cast<unsigned char*>(scratch_on(ctx->device));
        cudaStream_t s = static_cast<cudaStream_t>(stream);
        int u_stride = grid->topology_x == NK_BOUNDED ? grid->Nx + 1 : grid->Nx;
        // the arrival counter must start at zero; the partials are written before they are read
        e = cudaMemsetAsync(scratch, 0, sizeof(unsigned int), s);
        if (e != cudaSuccess)
            throw NoAllocError{NK_CUDA_ERROR, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e)};
        nk::LaunchDims d = nk::dims2d(grid->Nx, grid->Ny);
        k_picard_change_noalloc<<<d.grid, d.block, 0, s>>>(grid->Nx, grid->Ny, u_stride, u, v, u_prev, v_prev,
                                                           scratch, change_and_norm);
        nk::count_launch();
        e = cudaGetLastError();
        if (e != cudaSuccess)
            throw NoAllocError{NK_CUDA_ERROR, std::string("k_picard_change_noalloc launch: ") +
                                                  cudaGetErrorString(e)};
        return NK_OK;
    } catch (const NoAllocError& f) {
        ctx->error = f.message;
        return f.status;
    } catch (const std::exception& x) {
        ctx->error = x.what();
        return NK_CUDA_ERROR;
    }
}
