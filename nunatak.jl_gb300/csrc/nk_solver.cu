// nk_solver.cu — operator apply, operator masks and diagonals, and the fused conjugate-gradient kernels.
//
// Conjugate gradients restate src/Solvers/conjugate_gradient.jl:158-223 with the vector operations of
// src/Solvers/velocity_vector.jl:48-141 fused into the kernels that produce their operands:
//   step k:  apply   q = A p,  alpha = rho / p.q                       (one kernel + fused dot)
//            update  x += alpha p, r -= alpha q [, z = r / diag], dots (one kernel + fused dots)
//            [multigrid: z = V-cycle(r), then the r.z dot]
//            xpby    p = z + beta p, commit the stopping decision        (one kernel)
// Every dot is a deterministic two-stage reduction (fixed block partition and tree); its result stays
// on the device, so no step needs a host synchronisation.  Every kernel of a step first reads the
// device `done` flag and returns when the solve has stopped, so steps can be launched in batches (or
// replayed from a CUDA graph) past convergence at the cost of empty launches.
#include <atomic>
#include <cmath>

#include "nk_kernels.cuh"

namespace nk {

static std::atomic<long long> g_launches{0};
static thread_local bool g_capturing = false;   // launches recorded into a graph are counted when the graph runs
void count_launch() { if (!g_capturing) g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void set_capturing(bool on) { g_capturing = on; }
static thread_local int g_batch_slots = 1;
int batch_slots() { return g_batch_slots; }
void set_batch_slots(int n) { g_batch_slots = n < 1 ? 1 : n; }
long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

// ---- layout conversion --------------------------------------------------------------------------------
__global__ void k_pack(double* dst, int pitch, int plane, int stride, int offset, const double* __restrict__ src, int nx, int ny,
                       int planes) {
    long long n = (long long)nx * ny * planes;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nx);
        long long r = t / nx;
        int j = (int)(r % ny);
        int k = (int)(r / ny);
        dst[((long long)k * plane + (long long)j * pitch + i) * stride + offset] = src[t];
    }
}
__global__ void k_unpack(double* __restrict__ dst, const double* src, int pitch, int plane, int stride, int offset, int nx, int ny,
                         int planes) {
    long long n = (long long)nx * ny * planes;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n; t += (long long)gridDim.x * blockDim.x) {
        int i = (int)(t % nx);
        long long r = t / nx;
        int j = (int)(r % ny);
        int k = (int)(r / ny);
        dst[t] = src[((long long)k * plane + (long long)j * pitch + i) * stride + offset];
    }
}
__global__ void k_fill(double* dst, int count, double value) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < count; t += gridDim.x * blockDim.x) dst[t] = value;
}

static int blocks_for(long long n) {
    long long b = (n + 255) / 256;
    return (int)(b > 4096 ? 4096 : (b < 1 ? 1 : b));
}

void launch_pack(double* dst, int pitch, int plane, int stride, int offset, const double* src, int nx, int ny, int planes,
                 cudaStream_t s) {
    k_pack<<<blocks_for((long long)nx * ny * planes), 256, 0, s>>>(dst, pitch, plane, stride, offset, src, nx, ny, planes); count_launch();
}
void launch_unpack(double* dst, const double* src, int pitch, int plane, int stride, int offset, int nx, int ny, int planes,
                   cudaStream_t s) {
    k_unpack<<<blocks_for((long long)nx * ny * planes), 256, 0, s>>>(dst, src, pitch, plane, stride, offset, nx, ny, planes); count_launch();
}
void launch_fill(double* dst, int count, double value, cudaStream_t s) {
    k_fill<<<blocks_for(count), 256, 0, s>>>(dst, count, value); count_launch();
}

// ---- operator, masks, diagonals ---------------------------------------------------------------------------
template <int R>
__global__ void __launch_bounds__(32 * STRIP_WARPS) k_apply(OpView<double> o, const double2* __restrict__ p, double2* __restrict__ q) {
    int i, j0;
    strip_origin<R>(i, j0);
    if (j0 >= o.g.Ny) return;   // whole warp
    strip_apply<R>(o, p, i, j0, [](int) { return NoExtra{}; }, [&](int k, double2 a, double2, NoExtra) { q[k] = a; });
}
void launch_apply(const OpView<double>& o, const double2* p, double2* q, cudaStream_t s) {
    int rows = strip_rows(o.g.Nx, o.g.Ny, 8);
    LaunchDims d = strip_dims(o.g.Nx, o.g.Ny, rows);
    with_strip_rows(rows, [&](auto r) { k_apply<decltype(r)::value><<<d.grid, d.block, 0, s>>>(o, p, q); });
    count_launch();
}

// inactiveᶠᶜᶜ / inactiveᶜᶠᶜ with η̄H (strain_rates.jl:2-3, smooth_ice_mask.jl:72-73) and the wall bits; `ud` (the
// fine level only) marks prescribed faces as identity rows that keep their value (U_DIRICHLET / V_DIRICHLET)
template <typename T>
__global__ void k_mask(OpView<T> o, uint8_t* mask, const double2* ud) {
    NK_BATCH_ENTER(o.g, o, mask, ud)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    const DevGrid<T>& g = o.g;
    if (i > g.Nx || j > g.Ny) return;
    uint8_t m = 0;
    bool wu = g.peripheral_fc(i, j), wv = g.peripheral_cf(i, j);
    bool fu = (o.coef[g.c_idx(i - 1, j)].x + o.coef[g.c_idx(i, j)].x) == T(0);
    bool fv = (o.coef[g.c_idx(i, j - 1)].x + o.coef[g.c_idx(i, j)].x) == T(0);
    if (wu) m |= U_WALL;
    if (wv) m |= V_WALL;
    if (wu || fu) m |= U_INACTIVE;
    if (wv || fv) m |= V_INACTIVE;
    if (ud && i < g.Nx && j < g.Ny) {   // the faces of the solved rows (prescribed_u / prescribed_v)
        double2 d = ud[g.idx(i, j)];
        if (!isnan(d.x)) m = (m & ~U_INACTIVE) | U_DIRICHLET;
        if (!isnan(d.y)) m = (m & ~V_INACTIVE) | V_DIRICHLET;
    }
    mask[g.idx(i, j)] = m;
}
template <typename T>
void launch_mask(const OpView<T>& o, uint8_t* mask, cudaStream_t s, const double2* ud) {
    LaunchDims d = dims2d(o.g.Nx + 1, o.g.Ny + 1);
    k_mask<T><<<d.grid, d.block, 0, s>>>(o, mask, ud); count_launch();
}
template void launch_mask<double>(const OpView<double>&, uint8_t*, cudaStream_t, const double2*);
template void launch_mask<float>(const OpView<float>&, uint8_t*, cudaStream_t, const double2*);

// x = val on the prescribed faces (those where ud is finite): the identity rows' values before a solve
__global__ void k_impose_prescribed(DevGrid<double> g, double2* x, const double2* __restrict__ ud, const double2* __restrict__ val) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;   // the faces of the solved rows (prescribed_u / prescribed_v)
    int k = g.idx(i, j);
    double2 d = ud[k];
    bool cu = !isnan(d.x), cv = !isnan(d.y);
    if (!(cu || cv)) return;
    double2 v = x[k], w = val[k];
    if (cu) v.x = w.x;
    if (cv) v.y = w.y;
    x[k] = v;
}
void launch_impose_prescribed(const DevGrid<double>& g, double2* x, const double2* ud, const double2* val, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_impose_prescribed<<<d.grid, d.block, 0, s>>>(g, x, ud, val); count_launch();
}

__global__ void k_inverse_diagonal(OpView<double> o, double2* invd) {
    NK_BATCH_ENTER(o.g, o, invd)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= o.g.Nx || j >= o.g.Ny) return;
    uint8_t m = o.mask[o.g.idx(i, j)];
    invd[o.g.idx(i, j)] = make_double2(1.0 / x_diagonal(o, i, j, m), 1.0 / y_diagonal(o, i, j, m));
}
void launch_inverse_diagonal(const OpView<double>& o, double2* invd, cudaStream_t s) {
    LaunchDims d = dims2d(o.g.Nx, o.g.Ny);
    k_inverse_diagonal<<<d.grid, d.block, 0, s>>>(o, invd); count_launch();
}

template <typename T>
__global__ void k_inverse_row_sum(OpView<T> o, typename Vec2<T>::type* irs) {
    NK_BATCH_ENTER(o.g, o, irs)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= o.g.Nx || j >= o.g.Ny) return;
    uint8_t m = o.mask[o.g.idx(i, j)];
    typename Vec2<T>::type r;   // zero on prescribed rows: the point smoothers keep their value there
    r.x = (m & U_DIRICHLET) ? T(0) : T(1) / x_row_sum(o, i, j, m);
    r.y = (m & V_DIRICHLET) ? T(0) : T(1) / y_row_sum(o, i, j, m);
    irs[o.g.idx(i, j)] = r;
}
template <typename T>
void launch_inverse_row_sum(const OpView<T>& o, typename Vec2<T>::type* irs, cudaStream_t s) {
    LaunchDims d = dims2d(o.g.Nx, o.g.Ny);
    k_inverse_row_sum<T><<<d.grid, d.block, 0, s>>>(o, irs); count_launch();
}
template void launch_inverse_row_sum<double>(const OpView<double>&, double2*, cudaStream_t);
template void launch_inverse_row_sum<float>(const OpView<float>&, float2*, cudaStream_t);

// ---- conjugate gradients ------------------------------------------------------------------------------------
__device__ __forceinline__ int read_done(const SolverScalars* sc) { return *(volatile const int*)&sc->done; }

__device__ __forceinline__ int stop_after(const SolverScalars* sc, double rnorm, int it) {
    if (!isfinite(rnorm)) return 1;
    if (sc->fixed) return it >= sc->iterations;
    return !(rnorm > sc->tol && it < sc->maxiter);
}

// conjugate_gradient!, conjugate_gradient.jl:165-171: r = b - A x, z = M r, p = z, rho = r.z
template <int R>
__global__ void __launch_bounds__(32 * STRIP_WARPS) k_cg_init(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    int i, j0;
    strip_origin<R>(i, j0);
    double rz = 0.0, rr = 0.0;
    if (j0 < v.o.g.Ny) {   // warps below the grid still take part in the block reduction
        strip_apply<R>(v.o, (const double2*)v.x, i, j0, [&](int k) { return v.b[k]; }, [&](int k, double2 q, double2, const double2& b) {
            double2 r = make_double2(b.x - q.x, b.y - q.y);
            v.r[k] = r;   // the FP32 copy for the multigrid follows in k_cg_scale_r32, once ‖r0‖ is known
            rr += r.x * r.x + r.y * r.y;
            if (v.precond != NK_PRECONDITIONER_MULTIGRID) {
                double2 z = r;
                if (v.precond == NK_PRECONDITIONER_DIAGONAL) {
                    double2 d = v.invd[k];
                    z = make_double2(r.x * d.x, r.y * d.y);
                }
                v.z[k] = z;
                v.p[k] = z;
                rz += r.x * z.x + r.y * z.y;
            }
        });
    }
    double trz, trr;
    if (grid_sum2(rz, rr, v.partials, &v.sc->ticket, trz, trr) && threadIdx.x == 0 && threadIdx.y == 0) {
        SolverScalars* sc = v.sc;
        double r0 = sqrt(trr);
        sc->rr = trr;
        sc->r0 = r0;
        sc->rnorm = r0;
        sc->r32_exp = residual_exponent(r0);
        sc->r32_exp_next = sc->r32_exp;
        sc->tol = fmax(sc->reltol * r0, sc->abstol);
        sc->it = 0;
        sc->rho = trz;
        sc->status = isfinite(r0) ? NK_OK : NK_NONFINITE;
        int done = sc->fixed ? (sc->iterations <= 0) : !(r0 > sc->tol && 0 < sc->maxiter);
        if (!isfinite(r0)) done = 1;
        sc->done = done;
        sc->done_next = done;
        if (v.cond && v.precond != NK_PRECONDITIONER_MULTIGRID) cudaGraphSetConditional(v.cond, done ? 0u : 1u);
    }
}
void launch_cg_init(const CGView& v, cudaStream_t s) {
    int rows = strip_rows(v.o.g.Nx, v.o.g.Ny, 8);
    LaunchDims d = strip_dims(v.o.g.Nx, v.o.g.Ny, rows);
    with_strip_rows(rows, [&](auto r) { k_cg_init<decltype(r)::value><<<d.grid, d.block, 0, s>>>(v); });
    count_launch();
}

// mixed precision start: the FP32 copy of r0 for the first V-cycle, scaled by 2^-e with e the exponent of ‖r0‖
__global__ void k_cg_scale_r32(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    int e = v.sc->r32_exp;   // set with ‖r0‖ by the last block of k_cg_init
    if (i < v.o.g.Nx && j < v.o.g.Ny) {
        int k = v.o.g.idx(i, j);
        double2 r = v.r[k];
        v.r32[k] = make_float2((float)scale_pow2(r.x, -e), (float)scale_pow2(r.y, -e));
    }
}
void launch_cg_scale_r32(const CGView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx, v.o.g.Ny);
    k_cg_scale_r32<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// multigrid start: p = z, rho = r.z (and z_old = z for flexible conjugate gradients)
__global__ void k_cg_init_finish(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    int i = blockIdx.x * BX + threadIdx.x, j0 = blockIdx.y * BY * VEC_ROWS + threadIdx.y;
    double rz = 0.0;
#pragma unroll
    for (int row = 0; row < VEC_ROWS; ++row) {
        int j = j0 + row * BY;
        if (i < v.o.g.Nx && j < v.o.g.Ny) {
            int k = v.o.g.idx(i, j);
            double2 z, r = v.r[k];
            if (v.z32) {
                float2 f = v.z32[k];
                int ze = v.sc->r32_exp;
                z = make_double2(scale_pow2((double)f.x, ze), scale_pow2((double)f.y, ze));
                if (v.zold32) v.zold32[k] = f;
            } else {
                z = v.z[k];
            }
            v.p[k] = z;
            if (v.zold) v.zold[k] = z;
            rz += r.x * z.x + r.y * z.y;
        }
    }
    double trz, dummy;
    if (grid_sum2(rz, 0.0, v.partials, &v.sc->ticket, trz, dummy) && threadIdx.x == 0 && threadIdx.y == 0) {
        v.sc->rho = trz;
        v.sc->zold_exp = v.sc->r32_exp;   // the exponent of the z32 now in zold32
        if (v.cond) cudaGraphSetConditional(v.cond, v.sc->done ? 0u : 1u);
    }
}
void launch_cg_init_finish(const CGView& v, cudaStream_t s) {
    LaunchDims d = vec_dims(v.o.g.Nx, v.o.g.Ny);
    k_cg_init_finish<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// conjugate_gradient_step!, conjugate_gradient.jl:209-212: q = A p, alpha = rho / p.q (0 if p.q = 0)
template <int R>
__global__ void __launch_bounds__(32 * STRIP_WARPS) k_cg_apply(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    if (read_done(v.sc)) return;
    int i, j0;
    strip_origin<R>(i, j0);
    double pq = 0.0;
    if (j0 < v.o.g.Ny) {   // warps below the grid still take part in the block reduction
        strip_apply<R>(v.o, (const double2*)v.p, i, j0, [](int) { return NoExtra{}; }, [&](int k, double2 q, double2 p, NoExtra) {
            v.q[k] = q;
            pq += p.x * q.x + p.y * q.y;
        });
    }
    double tpq, dummy;
    if (grid_sum2(pq, 0.0, v.partials, &v.sc->ticket, tpq, dummy) && threadIdx.x == 0 && threadIdx.y == 0) {
        SolverScalars* sc = v.sc;
        sc->pq = tpq;
        sc->alpha = (tpq == 0.0) ? 0.0 : sc->rho / tpq;
        if (tpq < 0.0 && sc->status == NK_OK) sc->status = NK_BREAKDOWN;
    }
}
void launch_cg_apply(const CGView& v, cudaStream_t s) {
    int rows = strip_rows(v.o.g.Nx, v.o.g.Ny, 8);
    LaunchDims d = strip_dims(v.o.g.Nx, v.o.g.Ny, rows);
    with_strip_rows(rows, [&](auto r) { k_cg_apply<decltype(r)::value><<<d.grid, d.block, 0, s>>>(v); });
    count_launch();
}

// conjugate_gradient_step!, conjugate_gradient.jl:214-219 and the stopping test of :193-197
__global__ void k_cg_update(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    if (read_done(v.sc)) return;
    int i = blockIdx.x * BX + threadIdx.x, j0 = blockIdx.y * BY * VEC_ROWS + threadIdx.y;
    double alpha = v.sc->alpha;
    // FP32 copy of the new residual scaled by the exponent of the previous norm (read before the last block
    // replaces it)
    int r32_exp = v.sc->r32_exp_next;
    double rz = 0.0, rr = 0.0;
#pragma unroll
    for (int row = 0; row < VEC_ROWS; ++row) {
        int j = j0 + row * BY;
        if (i < v.o.g.Nx && j < v.o.g.Ny) {
            int k = v.o.g.idx(i, j);
            double2 p = v.p[k], q = v.q[k], x = v.x[k], r = v.r[k];
            x.x = x.x + alpha * p.x;
            x.y = x.y + alpha * p.y;
            r.x = r.x + (-alpha) * q.x;
            r.y = r.y + (-alpha) * q.y;
            v.x[k] = x;
            v.r[k] = r;
            if (v.r32) v.r32[k] = make_float2((float)scale_pow2(r.x, -r32_exp), (float)scale_pow2(r.y, -r32_exp));
            rr += r.x * r.x + r.y * r.y;
            if (v.precond != NK_PRECONDITIONER_MULTIGRID) {
                double2 z = r;
                if (v.precond == NK_PRECONDITIONER_DIAGONAL) {
                    double2 d = v.invd[k];
                    z = make_double2(r.x * d.x, r.y * d.y);
                }
                v.z[k] = z;
                rz += r.x * z.x + r.y * z.y;
            }
        }
    }
    double trz, trr;
    if (grid_sum2(rz, rr, v.partials, &v.sc->ticket, trz, trr) && threadIdx.x == 0 && threadIdx.y == 0) {
        SolverScalars* sc = v.sc;
        sc->rr = trr;
        double rn = sqrt(trr);
        sc->r32_exp = r32_exp;
        sc->r32_exp_next = residual_exponent(rn);
        sc->rnorm = rn;
        int it = sc->it + 1;
        sc->it = it;
        if (v.precond != NK_PRECONDITIONER_MULTIGRID) {
            double rho = sc->rho;
            sc->beta = (rho == 0.0) ? 0.0 : trz / rho;
            sc->rho = trz;
        }
        if (!isfinite(rn)) sc->status = NK_NONFINITE;
        int stop = stop_after(sc, rn, it);
        sc->done_next = stop;
        if (stop && !sc->fixed && !(rn <= sc->tol)) sc->cg_unconverged += 1;
    }
}
void launch_cg_update(const CGView& v, cudaStream_t s) {
    LaunchDims d = vec_dims(v.o.g.Nx, v.o.g.Ny);
    k_cg_update<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// after z = V-cycle(r): rho_new = r.z; beta = rho_new / rho, or the flexible (Polak-Ribière) form
// beta = (r.z - r.z_old) / rho when the preconditioner varies between steps
__global__ void k_cg_dots_after_precondition(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    if (read_done(v.sc)) return;
    int i = blockIdx.x * BX + threadIdx.x, j0 = blockIdx.y * BY * VEC_ROWS + threadIdx.y;
    double rz = 0.0, rzo = 0.0;
#pragma unroll
    for (int row = 0; row < VEC_ROWS; ++row) {
        int j = j0 + row * BY;
        if (i < v.o.g.Nx && j < v.o.g.Ny) {
            int k = v.o.g.idx(i, j);
            double2 r = v.r[k], z;
            if (v.z32) {
                float2 f = v.z32[k];
                int ze = v.sc->r32_exp;
                z = make_double2(scale_pow2((double)f.x, ze), scale_pow2((double)f.y, ze));
            } else {
                z = v.z[k];
            }
            rz += r.x * z.x + r.y * z.y;
            if (v.zold32) {
                float2 fo = v.zold32[k];
                int zo_e = v.sc->zold_exp;
                double2 zo = make_double2(scale_pow2((double)fo.x, zo_e), scale_pow2((double)fo.y, zo_e));
                rzo += r.x * zo.x + r.y * zo.y;
            } else if (v.zold) {
                double2 zo = v.zold[k];
                rzo += r.x * zo.x + r.y * zo.y;
            }
        }
    }
    double trz, trzo;
    if (grid_sum2(rz, rzo, v.partials, &v.sc->ticket, trz, trzo) && threadIdx.x == 0 && threadIdx.y == 0) {
        SolverScalars* sc = v.sc;
        double rho = sc->rho;
        double num = sc->flexible ? (trz - trzo) : trz;
        sc->beta = (rho == 0.0) ? 0.0 : num / rho;
        sc->rho = trz;
        sc->rz_old = trzo;
    }
}
void launch_cg_dots_after_precondition(const CGView& v, cudaStream_t s) {
    LaunchDims d = vec_dims(v.o.g.Nx, v.o.g.Ny);
    k_cg_dots_after_precondition<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// xpby!(z, beta, p), conjugate_gradient.jl:220; the last block commits the stopping decision
__global__ void k_cg_xpby(CGView v) {
    NK_BATCH_ENTER(v.o.g, v)
    if (read_done(v.sc)) return;
    int i = blockIdx.x * BX + threadIdx.x, j0 = blockIdx.y * BY * VEC_ROWS + threadIdx.y;
    double beta = v.sc->beta;
    int ze = v.sc->r32_exp;
#pragma unroll
    for (int row = 0; row < VEC_ROWS; ++row) {
        int j = j0 + row * BY;
        if (i < v.o.g.Nx && j < v.o.g.Ny) {
            int k = v.o.g.idx(i, j);
            double2 z, p = v.p[k];
            if (v.z32) {   // z = z32 2^e, as k_cg_dots_after_precondition formed it; z_old keeps z32 itself
                float2 f = v.z32[k];
                z = make_double2(scale_pow2((double)f.x, ze), scale_pow2((double)f.y, ze));
                if (v.zold32) v.zold32[k] = f;
            } else {
                z = v.z[k];
            }
            p.x = z.x + beta * p.x;
            p.y = z.y + beta * p.y;
            v.p[k] = p;
            if (v.zold) v.zold[k] = z;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        unsigned int n = gridDim.x * gridDim.y;
        unsigned int t = atomicAdd(&v.sc->ticket2, 1u);
        if (t == n - 1) {
            v.sc->ticket2 = 0u;
            v.sc->zold_exp = v.sc->r32_exp;   // the exponent of the z32 now in zold32
            int d = v.sc->done_next;
            v.sc->done = d;
            if (v.cond) cudaGraphSetConditional(v.cond, d ? 0u : 1u);
        }
    }
}
void launch_cg_xpby(const CGView& v, cudaStream_t s) {
    LaunchDims d = vec_dims(v.o.g.Nx, v.o.g.Ny);
    k_cg_xpby<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// precondition!(z, ::StressBalanceDiagonalPreconditioner, r, ...) over size(z.u), size(z.v)
__global__ void k_precondition_diagonal(DevGrid<double> g, double2* z, const double2* __restrict__ r, const double2* __restrict__ invd) {
    NK_BATCH_ENTER(g, g, z, r, invd)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    double2 o = z[k], rr = r[k];
    bool has_u = j < g.Ny && (i < g.Nx || !g.px);
    bool has_v = i < g.Nx && (j < g.Ny || !g.py);
    bool inside = i < g.Nx && j < g.Ny;
    double2 d = inside ? invd[k] : make_double2(1.0, 1.0);
    if (has_u) o.x = (i < g.Nx) ? rr.x * d.x : rr.x;
    if (has_v) o.y = (j < g.Ny) ? rr.y * d.y : rr.y;
    z[k] = o;
}
void launch_precondition_diagonal(const DevGrid<double>& g, double2* z, const double2* r, const double2* invd, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx + 1, g.Ny + 1);
    k_precondition_diagonal<<<d.grid, d.block, 0, s>>>(g, z, r, invd); count_launch();
}

// ---- Picard -------------------------------------------------------------------------------------------------
__global__ void k_copy_range(DevGrid<double> g, double2* dst, const double2* __restrict__ src) {
    NK_BATCH_ENTER(g, g, dst, src)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    dst[g.idx(i, j)] = src[g.idx(i, j)];
}
void launch_copy_range(const DevGrid<double>& g, double2* dst, const double2* src, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_copy_range<<<d.grid, d.block, 0, s>>>(g, dst, src); count_launch();
}

// picard_solve! loop head (picard.jl:71-79): Δ = ∞, X = 0, iteration = 0.  Batched (stride ≠ 0): block z starts
// slot z, whose scalars lie z * stride bytes after `sc`, unless the slot holds no request (p_done set).
__global__ void k_picard_begin(SolverScalars* sc, unsigned long long cond, long long stride) {
    if (stride) {
        shift_ptr(sc, (long long)blockIdx.z * stride);
        if (*(volatile const int*)&sc->p_done) return;
    }
    sc->p_it = 0;
    sc->p_D = INFINITY;
    sc->p_X = 0.0;
    sc->it_total = 0;
    sc->cg_unconverged = 0;
    sc->status = NK_OK;
    int run = sc->p_fixed ? (sc->p_iterations > 0) : (sc->p_maxiter > 0);
    sc->p_done = !run;
    if (cond) cudaGraphSetConditional(cond, run ? 1u : 0u);
}
void launch_picard_begin(SolverScalars* sc, unsigned long long cond, long long stride, cudaStream_t s) {
    k_picard_begin<<<dim3(1, 1, batch_slots()), 1, 0, s>>>(sc, cond, stride); count_launch();
}

// The loop conditions of a batched graph, one warp over the slots' scalars: Picard goes on while a slot is still
// iterating (cg = 0), conjugate gradients while a slot still iterating has not stopped (cg = 1).  `counter` counts
// the loop bodies that will run (the launch count of the solve).
__global__ void k_batch_condition(const SolverScalars* sc, long long stride, int slots, int cg, unsigned long long cond, int* counter) {
    int more = 0;
    for (int z = threadIdx.x; z < slots; z += 32) {
        const SolverScalars* t = sc;
        shift_ptr(t, (long long)z * stride);
        int going = !*(volatile const int*)&t->p_done;
        if (cg) going = going && !*(volatile const int*)&t->done;
        more |= going;
    }
    more = __any_sync(0xffffffffu, more);
    if (threadIdx.x == 0) {
        cudaGraphSetConditional(cond, more ? 1u : 0u);
        if (more && counter) *counter += 1;
    }
}
void launch_batch_condition(const SolverScalars* sc, long long stride, int slots, int cg, unsigned long long cond, int* counter,
                            cudaStream_t s) {
    k_batch_condition<<<1, 32, 0, s>>>(sc, stride, slots, cg, cond, counter); count_launch();
}

// end of one Picard iteration (picard.jl:83-86): x⁻ = x⁻ - x, Δ = ‖x⁻‖, X = ‖x‖, then the loop test of :79
__global__ void k_picard_end(DevGrid<double> g, double2* xprev, const double2* __restrict__ x, SolverScalars* sc, double2* partials,
                             unsigned long long cond) {
    NK_BATCH_ENTER(g, g, xprev, x, sc, partials)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    double dd = 0.0, xx = 0.0;
    if (i < g.Nx && j < g.Ny) {
        int k = g.idx(i, j);
        double2 a = xprev[k], b = x[k];
        a.x = a.x + (-1.0) * b.x;
        a.y = a.y + (-1.0) * b.y;
        xprev[k] = a;
        dd = a.x * a.x + a.y * a.y;
        xx = b.x * b.x + b.y * b.y;
    }
    double tdd, txx;
    if (grid_sum2(dd, xx, partials, &sc->ticket, tdd, txx) && threadIdx.x == 0 && threadIdx.y == 0) {
        double D = sqrt(tdd), X = sqrt(txx);
        sc->picard_dd = tdd;
        sc->picard_xx = txx;
        sc->p_D = D;
        sc->p_X = X;
        int it = sc->p_it + 1;
        sc->p_it = it;
        sc->it_total += sc->it;
        int more = sc->p_fixed ? (it < sc->p_iterations) : (D > fmax(sc->p_reltol * X, sc->p_abstol) && it < sc->p_maxiter);
        if (!isfinite(D) || sc->status == NK_NONFINITE) {
            sc->status = NK_NONFINITE;
            more = 0;
        }
        sc->p_done = !more;
        if (cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
    }
}
void launch_picard_end(const DevGrid<double>& g, double2* xprev, const double2* x, SolverScalars* sc, double2* partials,
                       unsigned long long cond, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_picard_end<<<d.grid, d.block, 0, s>>>(g, xprev, x, sc, partials, cond); count_launch();
}

// End of one Picard iteration under the viscosity-change rule (NK_VISCOSITY_CONVERGENCE, an extension):
// Δ = ‖η̄H - η̄H⁻‖ between this iteration's coefficients and the previous iteration's (Δ = ∞ at the first),
// X = ‖η̄H‖, then η̄H⁻ = η̄H and the same loop test as k_picard_end.
__global__ void k_picard_end_viscosity(DevGrid<double> g, const double4* __restrict__ coef, double* eta_prev, SolverScalars* sc,
                                       double2* partials, unsigned long long cond) {
    NK_BATCH_ENTER(g, g, coef, eta_prev, sc, partials)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    double dd = 0.0, xx = 0.0;
    if (i < g.Nx && j < g.Ny) {
        int k = g.idx(i, j);
        double e = coef[k].x, d = e - eta_prev[k];
        eta_prev[k] = e;
        dd = d * d;
        xx = e * e;
    }
    double tdd, txx;
    if (grid_sum2(dd, xx, partials, &sc->ticket, tdd, txx) && threadIdx.x == 0 && threadIdx.y == 0) {
        double D = sc->p_it == 0 ? INFINITY : sqrt(tdd), X = sqrt(txx);
        sc->picard_dd = tdd;
        sc->picard_xx = txx;
        sc->p_D = D;
        sc->p_X = X;
        int it = sc->p_it + 1;
        sc->p_it = it;
        sc->it_total += sc->it;
        int more = D > fmax(sc->p_reltol * X, sc->p_abstol) && it < sc->p_maxiter;
        if (isnan(D) || !isfinite(X) || sc->status == NK_NONFINITE) {
            sc->status = NK_NONFINITE;
            more = 0;
        }
        sc->p_done = !more;
        if (cond) cudaGraphSetConditional(cond, more ? 1u : 0u);
    }
}
void launch_picard_end_viscosity(const DevGrid<double>& g, const double4* coef, double* eta_prev, SolverScalars* sc, double2* partials,
                                 unsigned long long cond, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_picard_end_viscosity<<<d.grid, d.block, 0, s>>>(g, coef, eta_prev, sc, partials, cond); count_launch();
}

// ---- vector helpers under the done predicate -------------------------------------------------------------------
__global__ void k_copy_vec(DevGrid<double> g, double2* dst, const double2* __restrict__ src, const int* done) {
    NK_BATCH_ENTER(g, g, dst, src, done)
    if (done && *(volatile const int*)done) return;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    dst[g.idx(i, j)] = src[g.idx(i, j)];
}
void launch_copy_vec(const DevGrid<double>& g, double2* dst, const double2* src, const int* done, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_copy_vec<<<d.grid, d.block, 0, s>>>(g, dst, src, done); count_launch();
}

__global__ void k_to_float(DevGrid<double> g, const double2* __restrict__ src, float2* dst, const int* done) {
    NK_BATCH_ENTER(g, g, src, dst, done)
    if (done && *(volatile const int*)done) return;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    double2 a = src[g.idx(i, j)];
    dst[g.idx(i, j)] = make_float2((float)a.x, (float)a.y);
}
void launch_to_float(const DevGrid<double>& g, const double2* src, float2* dst, const int* done, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_to_float<<<d.grid, d.block, 0, s>>>(g, src, dst, done); count_launch();
}
__global__ void k_to_double(DevGrid<double> g, const float2* __restrict__ src, double2* dst, const int* done) {
    NK_BATCH_ENTER(g, g, src, dst, done)
    if (done && *(volatile const int*)done) return;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    float2 a = src[g.idx(i, j)];
    dst[g.idx(i, j)] = make_double2((double)a.x, (double)a.y);
}
void launch_to_double(const DevGrid<double>& g, const float2* src, double2* dst, const int* done, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_to_double<<<d.grid, d.block, 0, s>>>(g, src, dst, done); count_launch();
}
__global__ void k_coef_to_float(DevGrid<double> g, const double4* __restrict__ src, float4* dst) {
    NK_BATCH_ENTER(g, g, src, dst)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    double4 a = src[g.idx(i, j)];
    dst[g.idx(i, j)] = make_float4((float)a.x, (float)a.y, (float)a.z, (float)a.w);
}
void launch_coef_to_float(const DevGrid<double>& g, const double4* src, float4* dst, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx + 1, g.Ny + 1);
    k_coef_to_float<<<d.grid, d.block, 0, s>>>(g, src, dst); count_launch();
}

}  // namespace nk
