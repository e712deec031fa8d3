// nk_internal.cuh — shared device definitions of libnunatak_gb300.
//
// Device layout.  Every two-dimensional field of an Nx x Ny grid is stored in one pitched array of
// (Ny + 1) rows of `pitch` >= Nx + 1 elements, x fastest; element (i, j), 0-based, is
//   cell (i, j) for a Center-Center field, the west face of cell (i, j) for a Face-Center field,
//   the south face for a Center-Face field, the south-west corner for a Face-Face field.
// Index i = Nx holds the east wall face (Bounded x), row j = Ny the north wall face (Bounded y).
// A velocity vector stores (u, v) of the same (i, j) interleaved as one 16-byte (8-byte in FP32) pair,
// so one load brings both components of a cell; the coefficients of the operator are one packed record
// per (i, j): (eta_H at the centre, eta_H at the south-west corner, beta_u, beta_v).
//
// Halo semantics.  Oceananigans fills halos by a periodic wrap or, for cell-centred data in a Bounded
// direction, by copying the edge value.  The kernels read the same values through index maps: wrap()
// for Periodic directions, clamp() for Bounded ones.  Face data in a Bounded direction is never read
// unmasked outside 0..N, so clamping it is equivalent.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/nunatak_gb300.h"

// Device context of the C ABI: the CUDA ordinal made current by every call, and the last error message.
struct nk_context {
    int device = 0;
    std::string error;
    cudaStream_t stream = nullptr;   // records the reference event
    cudaEvent_t ref = nullptr;       // time origin of nk_solve_stats::device_start_ms / device_end_ms
};

namespace nk {

constexpr int BX = 32;   // thread-block tile of the 2-D kernels: BX x BY cells
constexpr int BY = 8;
constexpr int BLOCK_THREADS = BX * BY;

// Mask bits of the operator (one byte per (i, j)).
constexpr uint8_t U_INACTIVE = 1;   // u point is a wall or ice free (and not prescribed): identity row, zero in strain rates
constexpr uint8_t V_INACTIVE = 2;
constexpr uint8_t U_WALL = 4;       // wall (peripheral) only: the viscosity masks walls, not ice-free points
constexpr uint8_t V_WALL = 8;
// Prescribed velocity (the Dirichlet extension; the reference has none): an identity row whose value, held fixed
// at the prescribed one, still enters the strain rates.  U_INACTIVE is cleared on such a face, so the reads of the
// strain rates test U_INACTIVE alone and the rows test U_IDENTITY.
constexpr uint8_t U_DIRICHLET = 16;
constexpr uint8_t V_DIRICHLET = 32;
constexpr uint8_t U_IDENTITY = U_INACTIVE | U_DIRICHLET;
constexpr uint8_t V_IDENTITY = V_INACTIVE | V_DIRICHLET;

template <typename T> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };
template <typename T> struct Vec4;
template <> struct Vec4<double> { using type = double4; };
template <> struct Vec4<float> { using type = float4; };

// Grid of one multigrid level as the kernels see it.  Metric arrays hold indices -2 .. N+2 (the pointer
// is offset by 2): dxc(i) = cell width of centre i, dxf(i) = centre spacing at face i (west of centre i).
template <typename T>
struct DevGrid {
    int Nx, Ny, pitch;
    int px, py;                         // periodic flags
    const T* dxc; const T* dxf; const T* dyc; const T* dyf;      // spacings
    const T* rdxc; const T* rdxf; const T* rdyc; const T* rdyf;  // their reciprocals
    // A batched launch (gridDim.z slots of identical problems whose device arenas lie slot_stride bytes apart):
    // slot z of a block shifts every pointer by z * slot_stride and stops when its Picard flag p_done (slot 0's,
    // shifted the same way) is set.  Zero and null outside a batch.
    long long slot_stride = 0;
    const int* p_done = nullptr;
    // Every spacing of the level equal (dxc = dxf = dyc = dyf = h over the whole metric range, a regular square grid):
    // h, else 0.  The column-marching walk then takes the closed form of the stencil on such a grid.
    T h = T(0);

    __device__ __forceinline__ int idx(int i, int j) const { return j * pitch + i; }
    __device__ __forceinline__ static int wrap(int i, int n) { return i < 0 ? i + n : (i >= n ? i - n : i); }
    __device__ __forceinline__ static int clampi(int i, int lo, int hi) { return i < lo ? lo : (i > hi ? hi : i); }
    // index maps with halo semantics
    __device__ __forceinline__ int cx(int i) const { return px ? wrap(i, Nx) : clampi(i, 0, Nx - 1); }
    __device__ __forceinline__ int cy(int j) const { return py ? wrap(j, Ny) : clampi(j, 0, Ny - 1); }
    __device__ __forceinline__ int fx(int i) const { return px ? wrap(i, Nx) : clampi(i, 0, Nx); }
    __device__ __forceinline__ int fy(int j) const { return py ? wrap(j, Ny) : clampi(j, 0, Ny); }
    __device__ __forceinline__ int c_idx(int i, int j) const { return idx(cx(i), cy(j)); }   // Center-Center
    __device__ __forceinline__ int u_idx(int i, int j) const { return idx(fx(i), cy(j)); }   // Face-Center
    __device__ __forceinline__ int v_idx(int i, int j) const { return idx(cx(i), fy(j)); }   // Center-Face
    __device__ __forceinline__ int ff_idx(int i, int j) const { return idx(fx(i), fy(j)); }  // Face-Face
    // inactive_cell and peripheral_node (Oceananigans Grids/inactive_node.jl) for Bounded directions
    __device__ __forceinline__ bool out_x(int i) const { return !px && (i < 0 || i >= Nx); }
    __device__ __forceinline__ bool out_y(int j) const { return !py && (j < 0 || j >= Ny); }
    __device__ __forceinline__ bool peripheral_fc(int i, int j) const { return out_y(j) || out_x(i) || out_x(i - 1); }
    __device__ __forceinline__ bool peripheral_cf(int i, int j) const { return out_x(i) || out_y(j) || out_y(j - 1); }
    __device__ __forceinline__ bool peripheral_ff(int i, int j) const { return out_x(i) || out_x(i - 1) || out_y(j) || out_y(j - 1); }
    __device__ __forceinline__ T Az_fc(int i, int j) const { return dxf[i] * dyc[j]; }
    __device__ __forceinline__ T Az_cf(int i, int j) const { return dxc[i] * dyf[j]; }
    __device__ __forceinline__ T Az_cc(int i, int j) const { return dxc[i] * dyc[j]; }
};

// A velocity prescribed at the u face (i, j) / v face (i, j).  Prescribable faces are those of the solved rows,
// (i, j) in 0..Nx-1 x 0..Ny-1 (wrapped when periodic): the west and south boundary faces of a Bounded direction
// and every interior face, but not the east / north boundary faces, which no row of the operator solves.
__device__ __forceinline__ bool prescribed_u(const DevGrid<double>& g, const double2* ud, int i, int j) {
    if (!ud || (!g.px && (i < 0 || i >= g.Nx)) || (!g.py && (j < 0 || j >= g.Ny))) return false;
    return !isnan(ud[g.idx(g.px ? g.wrap(i, g.Nx) : i, g.py ? g.wrap(j, g.Ny) : j)].x);
}
__device__ __forceinline__ bool prescribed_v(const DevGrid<double>& g, const double2* ud, int i, int j) {
    if (!ud || (!g.px && (i < 0 || i >= g.Nx)) || (!g.py && (j < 0 || j >= g.Ny))) return false;
    return !isnan(ud[g.idx(g.px ? g.wrap(i, g.Nx) : i, g.py ? g.wrap(j, g.Ny) : j)].y);
}

// Per-solve scalars of conjugate gradients and Picard, device resident.
struct SolverScalars {
    double rho;          // r . z of the current step
    double rho_new;
    double alpha, beta;
    double pq;
    double rr;           // r . r
    double rz_old;       // r_new . z_old (flexible conjugate gradients)
    double r0, tol, rnorm;
    double picard_dd, picard_xx;   // ||x - x_prev||^2, ||x||^2
    double reltol, abstol;
    int it, done, done_next, status;
    int fixed, iterations, maxiter, flexible;
    unsigned int ticket;           // last-block counter of the fused reductions
    unsigned int ticket2;
    // Picard (picard.jl:63-90), evaluated on the device between the conjugate-gradient solves
    double p_reltol, p_abstol, p_D, p_X;
    int p_fixed, p_iterations, p_maxiter, p_it;
    int p_done, it_total, cg_unconverged;
    int r32_exp;                   // mixed precision: the FP32 residual in the V-cycle is r 2^-r32_exp, z = z32 2^r32_exp
    int r32_exp_next;              // exponent the next k_cg_update scales its residual with (from the latest ‖r‖)
    int zold_exp;                  // mixed precision: z_old = zold32 2^zold_exp (the exponent of the z32 it copies)
};

// Binary exponent that brings a residual of norm `norm` near 1 before it is rounded to FP32.  Scaling by a power of
// two is exact, so the multigrid (linear and homogeneous from a zero guess) gives the same digits as unscaled,
// but right-hand sides of any magnitude stay clear of FP32 overflow and of its subnormal range.  Evaluated by
// one thread per kernel (it costs FP64 instructions); the cells apply it with scale_pow2.
__device__ __forceinline__ int residual_exponent(double norm) {
    return (norm > 0.0 && isfinite(norm)) ? ilogb(norm) : 0;
}

// x 2^k by an integer add to the exponent field (no FP64 instruction): exact for normal x and results.  Zeros,
// infinities and NaNs pass through; subnormal x and results below the normal range flush to a signed zero,
// results above it become infinite.
__device__ __forceinline__ double scale_pow2(double x, int k) {
    long long b = __double_as_longlong(x);
    int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0x7ff || k == 0) return x;
    long long sign = b & (long long)0x8000000000000000ULL;
    int en = ex + k;
    if (ex == 0 || en <= 0) return __longlong_as_double(sign);
    if (en >= 0x7ff) return __longlong_as_double(sign | 0x7ff0000000000000LL);
    return __longlong_as_double(b + ((long long)k << 52));
}

// ---- warp / block reductions (fixed order, so results do not depend on scheduling) --------------------
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum over the block of up to two values; result valid in thread 0.  `sh` holds 2 * 32 doubles.
__device__ __forceinline__ void block_sum2(double& a, double& b, double* sh) {
    int lane = threadIdx.x + threadIdx.y * blockDim.x;
    int w = lane >> 5, l = lane & 31;
    int nw = (blockDim.x * blockDim.y + 31) >> 5;
    a = warp_sum(a);
    b = warp_sum(b);
    if (l == 0) { sh[w] = a; sh[32 + w] = b; }
    __syncthreads();
    if (w == 0) {
        a = l < nw ? sh[l] : 0.0;
        b = l < nw ? sh[32 + l] : 0.0;
        a = warp_sum(a);
        b = warp_sum(b);
    }
    __syncthreads();
}

// Deterministic grid-wide reduction of two values: every block writes its partial sums, the last block
// to arrive sums the partials in index order (fixed partition + fixed tree) and returns true in all its
// threads with the totals in `ta`, `tb`.  `partials` holds 2 * gridDim entries.
__device__ __forceinline__ bool grid_sum2(double a, double b, double2* partials, unsigned int* ticket,
                                          double& ta, double& tb) {
    __shared__ double sh[64];
    __shared__ bool last;
    block_sum2(a, b, sh);
    int nblocks = gridDim.x * gridDim.y;
    int bid = blockIdx.x + blockIdx.y * gridDim.x;
    int tid = threadIdx.x + threadIdx.y * blockDim.x;
    if (tid == 0) {
        partials[bid] = make_double2(a, b);
        __threadfence();
        unsigned int t = atomicAdd(ticket, 1u);
        last = (t == (unsigned int)nblocks - 1);
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    int nt = blockDim.x * blockDim.y;
    double sa = 0.0, sb = 0.0;
    // k = tid, tid + nt, ... in order; eight L2 reads issued before their adds (the partials of the other blocks
    // are not in this SM's L1, so __ldcg), which keeps the summation order and overlaps the read latencies
    for (int base = tid; base < nblocks; base += 8 * nt) {
        double2 p[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            int k = base + u * nt;
            p[u] = k < nblocks ? __ldcg(&partials[k]) : make_double2(0.0, 0.0);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (base + u * nt < nblocks) {
                sa += p[u].x;
                sb += p[u].y;
            }
        }
    }
    block_sum2(sa, sb, sh);
    if (tid == 0) { *ticket = 0u; }
    ta = sa;
    tb = sb;
    return true;   // totals valid in thread 0
}

// ---- batched launches ------------------------------------------------------------------------------------
// `p` moved by d bytes (null stays null): the same buffer in another slot of a batch.  Q is a pointer type,
// restrict-qualified or not (anything else fails the casts).
template <typename Q>
__device__ __forceinline__ void shift_ptr(Q& p, long long d) {
    if (p) p = reinterpret_cast<Q>(reinterpret_cast<unsigned long long>(p) + (unsigned long long)d);
}
template <typename T>
__device__ __forceinline__ void rebase(DevGrid<T>& g, long long d) {
    shift_ptr(g.dxc, d); shift_ptr(g.dxf, d); shift_ptr(g.dyc, d); shift_ptr(g.dyf, d);
    shift_ptr(g.rdxc, d); shift_ptr(g.rdxf, d); shift_ptr(g.rdyc, d); shift_ptr(g.rdyf, d);
    shift_ptr(g.p_done, d);
}
template <typename Q>
__device__ __forceinline__ void rebase(Q& p, long long d) { shift_ptr(p, d); }   // a pointer (restrict-qualified or not)
// The byte shift of this block's slot; false when the slot has stopped (its Picard flag is set).
template <typename T>
__device__ __forceinline__ bool batch_slot(const DevGrid<T>& g, long long& d) {
    d = 0;
    if (!g.slot_stride) return true;
    d = (long long)blockIdx.z * g.slot_stride;
    const int* pd = g.p_done;
    shift_ptr(pd, d);
    return !*(volatile const int*)pd;
}
inline __device__ void rebase_all(long long) {}
template <typename A, typename... Rest>
__device__ __forceinline__ void rebase_all(long long d, A& a, Rest&... rest) {
    rebase(a, d);
    rebase_all(d, rest...);
}
// First statement of every kernel of the solve: under a batched launch, stop for a finished slot and move the
// listed views and pointers (G's grid first) to this block's slot.
#define NK_BATCH_ENTER(G, ...)                                              \
    {                                                                       \
        long long nk_slot_shift_;                                           \
        if (!::nk::batch_slot((G), nk_slot_shift_)) return;                  \
        if (nk_slot_shift_) ::nk::rebase_all(nk_slot_shift_, __VA_ARGS__);   \
    }

// ---- host side helpers ------------------------------------------------------------------------------------
// Slots of the batched launch being captured on this host thread (1 outside); the grid helpers below give every
// launch that many z blocks.
int batch_slots();
void set_batch_slots(int n);
// Sets the slot count for the lifetime of the scope (graph capture of a batch).
struct BatchScope {
    explicit BatchScope(int n) { set_batch_slots(n); }
    ~BatchScope() { set_batch_slots(1); }
    BatchScope(const BatchScope&) = delete;
    BatchScope& operator=(const BatchScope&) = delete;
};
// Kernels launched by the library in this process (instrumentation; every launch site calls count_launch()).
void count_launch();
void count_launches(long long n);
void set_capturing(bool on);
long long launch_count();

// ---- host side helpers (continued) ------------------------------------------------------------------------------
struct LaunchDims {
    dim3 grid, block;
};
// The per-iteration CG vector kernels give each thread VEC_ROWS cells of one column (rows j, j + BY, ...):
// the thread sums its cells before the block reduction, whose FP64 butterfly then costs a quarter per cell.
constexpr int VEC_ROWS = 4;
inline LaunchDims vec_dims(int nx, int ny) {
    LaunchDims d;
    d.block = dim3(BX, BY);
    d.grid = dim3((nx + BX - 1) / BX, (ny + BY * VEC_ROWS - 1) / (BY * VEC_ROWS), batch_slots());
    return d;
}
inline LaunchDims dims2d(int nx, int ny) {
    LaunchDims d;
    d.block = dim3(BX, BY);
    d.grid = dim3((nx + BX - 1) / BX, (ny + BY - 1) / BY, batch_slots());
    return d;
}

}  // namespace nk
