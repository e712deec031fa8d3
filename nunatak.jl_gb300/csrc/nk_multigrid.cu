// nk_multigrid.cu — geometric multigrid V-cycle kernels, in FP64 (plain solve) or FP32 (mixed solve).
//
// Restates src/StressBalances/multigrid_preconditioner.jl: semi-coarsening levels, rediscretised
// coarse coefficients (:331-344), ℓ1-Jacobi point smoother (:213-219) and y-line ℓ1-block Jacobi
// smoother (:231-259), C-grid restriction (:264-318, :346-352) and prolongation (:286-327, :354-360).
// Indices here are 0-based: coarse point I0 gathers fine points 2 I0 + a.
//
// The point smoother reads x from one buffer and writes the next iterate into another, so one kernel
// does a whole Jacobi sweep (the reference computes q = A x in one launch, then x += (b - q) / rowsum).
// Every kernel takes the conjugate-gradient `done` flag and returns once the solve has stopped.
#include "nk_kernels.cuh"

namespace nk {

__device__ __forceinline__ bool stopped(const int* done) { return done && *(volatile const int*)done; }

// ---- restriction / prolongation index rules (0-based) ------------------------------------------------------
__device__ __forceinline__ void offsets(bool face, int c, int& a0, int& a1) {
    if (c == 1) { a0 = 0; a1 = 0; } else if (face) { a0 = -1; a1 = 1; } else { a0 = -1; a1 = 2; }
}
__device__ __forceinline__ int wrapn(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }
// restriction_index (multigrid_preconditioner.jl:268-271)
__device__ __forceinline__ int ridx(int I, int a, int Nf, bool periodic, bool face, int c) {
    if (c == 1) return I;
    int i = 2 * I + a;
    if (periodic) return wrapn(i, Nf);
    if (face) return i < 0 ? 0 : i;
    return i < 0 ? 0 : (i > Nf - 1 ? Nf - 1 : i);
}
// restriction_weight (:273-283)
template <typename T>
__device__ __forceinline__ T rweight(int I, int a, int Nc, bool periodic, bool face, int c) {
    if (c == 1) return T(1);
    if (face) {
        if (!periodic && 2 * I + a < 0) return T(0);
        return a == 0 ? T(1) : T(1) / T(2);
    }
    T w = (a == 0 || a == 1) ? T(3) / T(4) : T(1) / T(4);
    if (periodic) return w;
    bool outside = (I == 0 && a == -1) || (I == Nc - 1 && a == 2);
    bool folded = (I == 0 && a == 0) || (I == Nc - 1 && a == 1);
    w = w + (folded ? T(1) / T(4) : T(0));
    return outside ? T(0) : w;
}
// parents (:286-305)
template <typename T>
__device__ __forceinline__ void parents(int i, int Nc, bool periodic, bool face, int c, int& I1, int& I2, T& w1, T& w2) {
    if (c == 1) { I1 = i; I2 = i; w1 = T(1); w2 = T(0); return; }
    int I = i / 2;
    bool odd1 = (i % 2) == 0;   // the 1-based index i + 1 is odd
    if (face) {
        int up = periodic ? wrapn(I + 1, Nc) : I + 1;
        I1 = I; I2 = odd1 ? I : up;
        w1 = odd1 ? T(1) : T(1) / T(2);
        w2 = odd1 ? T(0) : T(1) / T(2);
    } else {
        int Ip = odd1 ? I - 1 : I + 1;
        I1 = I;
        I2 = periodic ? wrapn(Ip, Nc) : (Ip < 0 ? 0 : (Ip > Nc - 1 ? Nc - 1 : Ip));
        w1 = T(3) / T(4); w2 = T(1) / T(4);
    }
}

// ---- coarse coefficients (_coarsen_coefficients!, :331-344), accumulated in FP64 ---------------------------------
template <typename T, typename TF>
__global__ void k_coarsen(OpView<T> co, int cxf, int cyf, DevGrid<TF> fg, const typename Vec4<TF>::type* __restrict__ fcoef,
                          typename Vec4<T>::type* ccoef) {
    NK_BATCH_ENTER(co.g, co, fg, fcoef, ccoef)
    const DevGrid<T>& cg = co.g;
    int I = blockIdx.x * BX + threadIdx.x, J = blockIdx.y * BY + threadIdx.y;
    if (I >= cg.Nx || J >= cg.Ny) return;
    int i0 = cxf * I, j0 = cyf * J;
    double S = 0.0;
    for (int a = 0; a < cxf; ++a)
        for (int b = 0; b < cyf; ++b) S += (double)fg.Az_cc(i0 + a, j0 + b) * (double)fcoef[fg.idx(i0 + a, j0 + b)].x;
    double su = 0.0, sv = 0.0;
    int a0, a1, b0, b1;
    offsets(true, cxf, a0, a1);
    offsets(false, cyf, b0, b1);
    for (int a = a0; a <= a1; ++a)
        for (int b = b0; b <= b1; ++b) {
            int i = ridx(I, a, fg.Nx, fg.px, true, cxf), j = ridx(J, b, fg.Ny, fg.py, false, cyf);
            double w = rweight<double>(I, a, cg.Nx, fg.px, true, cxf) * rweight<double>(J, b, cg.Ny, fg.py, false, cyf);
            su += w * ((double)fg.Az_fc(i, j) * (double)fcoef[fg.idx(i, j)].z);
        }
    offsets(false, cxf, a0, a1);
    offsets(true, cyf, b0, b1);
    for (int a = a0; a <= a1; ++a)
        for (int b = b0; b <= b1; ++b) {
            int i = ridx(I, a, fg.Nx, fg.px, false, cxf), j = ridx(J, b, fg.Ny, fg.py, true, cyf);
            double w = rweight<double>(I, a, cg.Nx, fg.px, false, cxf) * rweight<double>(J, b, cg.Ny, fg.py, true, cyf);
            sv += w * ((double)fg.Az_cf(i, j) * (double)fcoef[fg.idx(i, j)].w);
        }
    int k = cg.idx(I, J);
    typename Vec4<T>::type c = ccoef[k];
    c.x = (T)(S / (double)cg.Az_cc(I, J));
    c.z = (T)(su / (double)cg.Az_fc(I, J));
    c.w = (T)(sv / (double)cg.Az_cf(I, J));
    ccoef[k] = c;
}
template <typename T, typename TF>
void launch_coarsen(const LevelView<T>& coarse, const DevGrid<TF>& fine_g, const typename Vec4<TF>::type* fine_coef,
                    typename Vec4<T>::type* coarse_coef, cudaStream_t s) {
    LaunchDims d = dims2d(coarse.o.g.Nx, coarse.o.g.Ny);
    k_coarsen<T, TF><<<d.grid, d.block, 0, s>>>(coarse.o, coarse.cx, coarse.cy, fine_g, fine_coef, coarse_coef); count_launch();
    launch_corners<T>(coarse.o.g, coarse_coef, s);
}
template void launch_coarsen<double, double>(const LevelView<double>&, const DevGrid<double>&, const double4*, double4*, cudaStream_t);
template void launch_coarsen<float, double>(const LevelView<float>&, const DevGrid<double>&, const double4*, float4*, cudaStream_t);
template void launch_coarsen<float, float>(const LevelView<float>&, const DevGrid<float>&, const float4*, float4*, cudaStream_t);

// ---- per-point operations (shared by the grid-wide kernels and the fused coarse V-cycle) -------------------
// ℓ1-Jacobi update of one cell (_smooth!, :213-219); `first`: x_in = 0, so A x_in = 0 and x_out = b / rowsum
template <typename T>
__device__ __forceinline__ void smooth_point_at(const LevelView<T>& L, const typename Vec2<T>::type* __restrict__ xin,
                                                typename Vec2<T>::type* __restrict__ xout, bool first, int i, int j) {
    using V2 = typename Vec2<T>::type;
    int k = L.o.g.idx(i, j);
    V2 b = L.b[k], w = L.irs[k], out;
    if (first) {
        out.x = b.x * w.x;
        out.y = b.y * w.y;
    } else {
        V2 q = apply_at(L.o, xin, i, j);
        V2 x = xin[k];
        out.x = x.x + (b.x - q.x) * w.x;
        out.y = x.y + (b.y - q.y) * w.y;
    }
    xout[k] = out;
}

// q = A x, or the residual q = b - A x
template <typename T>
__device__ __forceinline__ void apply_or_residual_at(const LevelView<T>& L, const typename Vec2<T>::type* __restrict__ x,
                                                     typename Vec2<T>::type* __restrict__ q, bool residual, int i, int j) {
    using V2 = typename Vec2<T>::type;
    int k = L.o.g.idx(i, j);
    V2 a = apply_at(L.o, x, i, j);
    if (residual) {
        V2 b = L.b[k];
        a.x = b.x - a.x;
        a.y = b.y - a.y;
    }
    q[k] = a;
}

// restrict (:307-318) of one coarse point with the fine and coarse masks (_restrict!, :346-352).
// first_out != nullptr also performs the coarse level's first smoothing sweep from zero: first_out = b / rowsum.
template <typename T>
__device__ __forceinline__ void restrict_at(const LevelView<T>& C, const OpView<T>& fo, const typename Vec2<T>::type* __restrict__ rf,
                                            typename Vec2<T>::type* bc, typename Vec2<T>::type* first_out, int I, int J) {
    const DevGrid<T>& cg = C.o.g;
    const DevGrid<T>& fg = fo.g;
    int k = cg.idx(I, J);
    uint8_t m = C.o.mask[k];
    T su = T(0), sv = T(0);
    int a0, a1, b0, b1;
    if (!(m & U_IDENTITY)) {
        offsets(true, C.cx, a0, a1);
        offsets(false, C.cy, b0, b1);
        for (int a = a0; a <= a1; ++a)
            for (int b = b0; b <= b1; ++b) {
                int i = ridx(I, a, fg.Nx, fg.px, true, C.cx), j = ridx(J, b, fg.Ny, fg.py, false, C.cy);
                T w = rweight<T>(I, a, cg.Nx, fg.px, true, C.cx) * rweight<T>(J, b, cg.Ny, fg.py, false, C.cy);
                su += w * masked_u(fo, rf, i, j);
            }
    }
    if (!(m & V_IDENTITY)) {
        offsets(false, C.cx, a0, a1);
        offsets(true, C.cy, b0, b1);
        for (int a = a0; a <= a1; ++a)
            for (int b = b0; b <= b1; ++b) {
                int i = ridx(I, a, fg.Nx, fg.px, false, C.cx), j = ridx(J, b, fg.Ny, fg.py, true, C.cy);
                T w = rweight<T>(I, a, cg.Nx, fg.px, false, C.cx) * rweight<T>(J, b, cg.Ny, fg.py, true, C.cy);
                sv += w * masked_v(fo, rf, i, j);
            }
    }
    typename Vec2<T>::type o;
    o.x = su;
    o.y = sv;
    bc[k] = o;
    if (first_out) {
        typename Vec2<T>::type w = C.irs[k], x;
        x.x = su * w.x;
        x.y = sv * w.y;
        first_out[k] = x;
    }
}

// prolongate (:320-327) into one fine point, x_fine += P x_coarse (_prolongate!, :354-360)
template <typename T>
__device__ __forceinline__ typename Vec2<T>::type prolonged(const OpView<T>& fo, const LevelView<T>& C, typename Vec2<T>::type x,
                                                            uint8_t m, const typename Vec2<T>::type* __restrict__ xc, int i, int j) {
    const DevGrid<T>& cg = C.o.g;
    const DevGrid<T>& fg = fo.g;
    int I1, I2, J1, J2;
    T wx1, wx2, wy1, wy2;
    T pu = T(0), pv = T(0);
    if (!(m & U_IDENTITY)) {
        parents<T>(i, cg.Nx, fg.px, true, C.cx, I1, I2, wx1, wx2);
        parents<T>(j, cg.Ny, fg.py, false, C.cy, J1, J2, wy1, wy2);
        pu = wx1 * (wy1 * masked_u(C.o, xc, I1, J1) + wy2 * masked_u(C.o, xc, I1, J2)) +
             wx2 * (wy1 * masked_u(C.o, xc, I2, J1) + wy2 * masked_u(C.o, xc, I2, J2));
    }
    if (!(m & V_IDENTITY)) {
        parents<T>(i, cg.Nx, fg.px, false, C.cx, I1, I2, wx1, wx2);
        parents<T>(j, cg.Ny, fg.py, true, C.cy, J1, J2, wy1, wy2);
        pv = wx1 * (wy1 * masked_v(C.o, xc, I1, J1) + wy2 * masked_v(C.o, xc, I1, J2)) +
             wx2 * (wy1 * masked_v(C.o, xc, I2, J1) + wy2 * masked_v(C.o, xc, I2, J2));
    }
    x.x += pu;
    x.y += pv;
    return x;
}
template <typename T>
__device__ __forceinline__ void prolong_at(const OpView<T>& fo, const LevelView<T>& C, typename Vec2<T>::type* xf,
                                           const typename Vec2<T>::type* __restrict__ xc, int i, int j) {
    int k = fo.g.idx(i, j);
    xf[k] = prolonged(fo, C, xf[k], fo.mask[k], xc, i, j);
}

// line_relax!, :231-253: Thomas algorithm along j for the u line and then the v line of column i.
// `first`: x starts at zero, so q = A x = 0 is not read and x is overwritten by δ.
template <typename T>
__device__ __forceinline__ void line_relax_column(const LevelView<T>& L, typename Vec2<T>::type* x, bool first, int i) {
    const DevGrid<T>& g = L.o.g;
    int Ny = g.Ny;
    for (int comp = 0; comp < 2; ++comp) {
        T cj = 0, tj = 0, dj = 0;
        for (int j = 0; j < Ny; ++j) {
            int k = g.idx(i, j);
            uint8_t m = L.o.mask[k];
            T s = comp == 0 ? x_row_sum(L.o, i, j, m) : y_row_sum(L.o, i, j, m);
            T cj1 = (j == Ny - 1) ? T(0) : (comp == 0 ? x_line_coupling(L.o, i, j + 1) : y_line_coupling(L.o, i, j + 1));
            T mm = s - cj - cj1 + cj * tj;
            T bq = comp == 0 ? (L.b[k].x - (first ? T(0) : L.q[k].x)) : (L.b[k].y - (first ? T(0) : L.q[k].y));
            dj = (bq + cj * dj) / mm;
            tj = -cj1 / mm;
            L.t[k] = tj;
            if (comp == 0) L.q[k].x = dj; else L.q[k].y = dj;
            cj = cj1;
        }
        T delta = 0;
        for (int j = Ny - 1; j >= 0; --j) {
            int k = g.idx(i, j);
            delta = (comp == 0 ? L.q[k].x : L.q[k].y) - L.t[k] * delta;
            if (comp == 0) x[k].x = first ? delta : x[k].x + delta;
            else x[k].y = first ? delta : x[k].y + delta;
        }
    }
}

// ---- grid-wide kernels ---------------------------------------------------------------------------------------
template <typename T>
__global__ void k_smooth_first(LevelView<T> L, const typename Vec2<T>::type* __restrict__ xin, typename Vec2<T>::type* __restrict__ xout,
                               const int* done) {
    NK_BATCH_ENTER(L.o.g, L, xin, xout, done)
    if (stopped(done)) return;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i < L.o.g.Nx && j < L.o.g.Ny) smooth_point_at(L, xin, xout, true, i, j);
}

// One ℓ1-Jacobi sweep x' = x + (b - A x) / rowsum with the column-marching operator apply.  A prescribed row has
// weight 1/rowsum = 0 (k_inverse_row_sum), so the sweep keeps its value whatever q is there, and the identity
// test can share the mask bit of the strain-rate reads.
template <typename T, int R>
__global__ void __launch_bounds__(32 * STRIP_WARPS) k_smooth_point(LevelView<T> L, const typename Vec2<T>::type* __restrict__ xin,
                                                                  typename Vec2<T>::type* __restrict__ xout, const int* done) {
    NK_BATCH_ENTER(L.o.g, L, xin, xout, done)
    if (stopped(done)) return;
    using V2 = typename Vec2<T>::type;
    int i, j0;
    strip_origin<R>(i, j0);
    if (j0 >= L.o.g.Ny) return;   // whole warp
    struct BW { V2 b, w; };
    strip_apply<R, U_INACTIVE, V_INACTIVE>(L.o, xin, i, j0, [&](int k) { return BW{L.b[k], L.irs[k]}; }, [&](int k, V2 q, V2 x, const BW& e) {
        V2 out;
        out.x = x.x + (e.b.x - q.x) * e.w.x;
        out.y = x.y + (e.b.y - q.y) * e.w.y;
        xout[k] = out;
    });
}
template <typename T>
void launch_smooth_point(const LevelView<T>& L, const typename Vec2<T>::type* x_in, typename Vec2<T>::type* x_out, int first,
                         const int* done, cudaStream_t s) {
    if (first) {
        LaunchDims d = dims2d(L.o.g.Nx, L.o.g.Ny);
        k_smooth_first<T><<<d.grid, d.block, 0, s>>>(L, x_in, x_out, done); count_launch();
    } else {
        int rows = strip_rows(L.o.g.Nx, L.o.g.Ny, (int)sizeof(T), STRIP_SMOOTH);
        LaunchDims d = strip_dims(L.o.g.Nx, L.o.g.Ny, rows);
        with_strip_rows(rows, [&](auto r) { k_smooth_point<T, decltype(r)::value><<<d.grid, d.block, 0, s>>>(L, x_in, x_out, done); });
        count_launch();
    }
}

// The first two sweeps from a zero guess in one pass: the operand of the second sweep, x1 = b / rowsum, is formed
// where it is loaded (the same single rounding as the separate first sweep), so x1 is never stored.
template <typename T, int R>
__global__ void __launch_bounds__(32 * STRIP_WARPS) k_smooth_first2(LevelView<T> L, typename Vec2<T>::type* __restrict__ xout,
                                                                   const int* done) {
    NK_BATCH_ENTER(L.o.g, L, xout, done)
    if (stopped(done)) return;
    using V2 = typename Vec2<T>::type;
    int i, j0;
    strip_origin<R>(i, j0);
    if (j0 >= L.o.g.Ny) return;   // whole warp
    const V2* b = L.b;
    const V2* w = L.irs;
    int Nx = L.o.g.Nx, Ny = L.o.g.Ny;
    auto src = [=](int k, int iw, int jw) {
        V2 x;
        x.x = T(0);
        x.y = T(0);
        if (iw < Nx && jw < Ny) {
            V2 bb = b[k], ww = w[k];
            x.x = bb.x * ww.x;
            x.y = bb.y * ww.y;
        }
        return x;
    };
    struct BW { V2 b, w; };
    strip_apply_src<R, U_INACTIVE, V_INACTIVE>(L.o, src, i, j0, [&](int k) { return BW{L.b[k], L.irs[k]}; },
                                               [&](int k, V2 q, V2 x, const BW& e) {
        V2 out;
        out.x = x.x + (e.b.x - q.x) * e.w.x;
        out.y = x.y + (e.b.y - q.y) * e.w.y;
        xout[k] = out;
    });
}
template <typename T>
void launch_smooth_first2(const LevelView<T>& L, typename Vec2<T>::type* x_out, const int* done, cudaStream_t s) {
    int rows = strip_rows(L.o.g.Nx, L.o.g.Ny, (int)sizeof(T), STRIP_SMOOTH);
    LaunchDims d = strip_dims(L.o.g.Nx, L.o.g.Ny, rows);
    with_strip_rows(rows, [&](auto r) { k_smooth_first2<T, decltype(r)::value><<<d.grid, d.block, 0, s>>>(L, x_out, done); });
    count_launch();
}

template <typename T, int R>
__global__ void __launch_bounds__(32 * STRIP_WARPS) k_level_apply(LevelView<T> L, const typename Vec2<T>::type* __restrict__ x,
                                                                 typename Vec2<T>::type* __restrict__ q, int residual, const int* done) {
    NK_BATCH_ENTER(L.o.g, L, x, q, done)
    if (stopped(done)) return;
    using V2 = typename Vec2<T>::type;
    int i, j0;
    strip_origin<R>(i, j0);
    if (j0 >= L.o.g.Ny) return;   // whole warp
    strip_apply<R>(L.o, x, i, j0, [&](int k) { V2 b; b.x = T(0); b.y = T(0); if (residual) b = L.b[k]; return b; },
                   [&](int k, V2 a, V2, const V2& b) {
        if (residual) {
            a.x = b.x - a.x;
            a.y = b.y - a.y;
        }
        q[k] = a;
    });
}
template <typename T>
void launch_level_apply(const LevelView<T>& L, const typename Vec2<T>::type* x, typename Vec2<T>::type* q, int residual,
                        const int* done, cudaStream_t s) {
    int rows = strip_rows(L.o.g.Nx, L.o.g.Ny, (int)sizeof(T), STRIP_RESIDUAL);
    LaunchDims d = strip_dims(L.o.g.Nx, L.o.g.Ny, rows);
    with_strip_rows(rows, [&](auto r) { k_level_apply<T, decltype(r)::value><<<d.grid, d.block, 0, s>>>(L, x, q, residual, done); });
    count_launch();
}

template <typename T>
float time_strip_kernel(const LevelView<T>& L, int kind, int rows, int repeats, cudaStream_t s) {
    LaunchDims d = strip_dims(L.o.g.Nx, L.o.g.Ny, rows);
    auto once = [&] {
        with_strip_rows(rows, [&](auto r) {
            if (kind == STRIP_SMOOTH) k_smooth_point<T, decltype(r)::value><<<d.grid, d.block, 0, s>>>(L, L.x, L.x2, nullptr);
            else k_level_apply<T, decltype(r)::value><<<d.grid, d.block, 0, s>>>(L, L.x, L.q, 1, nullptr);
        });
        count_launch();
    };
    once();   // warm-up
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float ms = -1.f;
    if (cudaEventCreate(&e0) == cudaSuccess && cudaEventCreate(&e1) == cudaSuccess && cudaEventRecord(e0, s) == cudaSuccess) {
        for (int k = 0; k < repeats; ++k) once();
        if (cudaEventRecord(e1, s) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess || cudaGetLastError() != cudaSuccess)
            ms = -1.f;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    return ms < 0.f ? ms : ms / repeats;
}

template <typename T>
__global__ void k_line_relax(LevelView<T> L, typename Vec2<T>::type* x, int first, const int* done) {
    NK_BATCH_ENTER(L.o.g, L, x, done)
    if (stopped(done)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= L.o.g.Nx) return;
    line_relax_column(L, x, first != 0, i);
}
template <typename T>
void launch_line_relax(const LevelView<T>& L, typename Vec2<T>::type* x, int first, const int* done, cudaStream_t s) {
    dim3 nb((L.o.g.Nx + 127) / 128, 1, batch_slots());
    k_line_relax<T><<<nb, 128, 0, s>>>(L, x, first, done); count_launch();
}

// restrict_at for a coarse point away from every edge of a level halved in both directions: its 4 x 4 fine
// footprint (2I-1..2I+2) x (2J-1..2J+2) needs no clamp, wrap or range test and its weights no folding, so the
// pairs and mask bytes are loaded once for both components.  The sums run in restrict_at's order (x offset
// outer, y offset inner) with the same weight products, so the result is bit for bit restrict_at's.
template <typename T>
__device__ __forceinline__ void restrict_interior(const LevelView<T>& C, const OpView<T>& fo, const typename Vec2<T>::type* __restrict__ rf,
                                                  typename Vec2<T>::type* bc, typename Vec2<T>::type* first_out, int I, int J) {
    using V2 = typename Vec2<T>::type;
    const DevGrid<T>& cg = C.o.g;
    const DevGrid<T>& fg = fo.g;
    int k = cg.idx(I, J);
    uint8_t m = C.o.mask[k];
    const T wf[3] = {T(1) / T(2), T(1), T(1) / T(2)};                     // face offsets -1, 0, 1
    const T wc[4] = {T(1) / T(4), T(3) / T(4), T(3) / T(4), T(1) / T(4)}; // centre offsets -1, 0, 1, 2
    T pu[4][3], pv[3][4];   // masked u at [y][x] offsets (-1..2, -1..1), masked v at (-1..1, -1..2)
    int k0 = fg.idx(2 * I - 1, 2 * J - 1);
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int a = 0; a < 4; ++a) {
            int kf = k0 + b * fg.pitch + a;
            uint8_t mf = __ldg(fo.mask + kf);
            V2 r = rf[kf];
            if (a < 3) pu[b][a] = (mf & U_INACTIVE) ? T(0) : r.x;
            if (b < 3) pv[b][a] = (mf & V_INACTIVE) ? T(0) : r.y;
        }
    T su = T(0), sv = T(0);
    if (!(m & U_IDENTITY)) {
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) su += (wf[a] * wc[b]) * pu[b][a];
    }
    if (!(m & V_IDENTITY)) {
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) sv += (wc[a] * wf[b]) * pv[b][a];
    }
    V2 o;
    o.x = su;
    o.y = sv;
    bc[k] = o;
    if (first_out) {
        V2 w = C.irs[k], x;
        x.x = su * w.x;
        x.y = sv * w.y;
        first_out[k] = x;
    }
}

template <typename T>
__global__ void k_restrict(LevelView<T> C, OpView<T> fo, const typename Vec2<T>::type* __restrict__ rf,
                           typename Vec2<T>::type* bc, typename Vec2<T>::type* first_out, const int* done) {
    NK_BATCH_ENTER(C.o.g, C, fo, rf, bc, first_out, done)
    if (stopped(done)) return;
    int I = blockIdx.x * BX + threadIdx.x, J = blockIdx.y * BY + threadIdx.y;
    const DevGrid<T>& cg = C.o.g;
    if (I >= cg.Nx || J >= cg.Ny) return;
    if (C.cx == 2 && C.cy == 2 && I >= 1 && I <= cg.Nx - 2 && J >= 1 && J <= cg.Ny - 2)
        restrict_interior(C, fo, rf, bc, first_out, I, J);
    else
        restrict_at(C, fo, rf, bc, first_out, I, J);
}
template <typename T>
void launch_restrict(const LevelView<T>& coarse, const LevelView<T>& fine, const typename Vec2<T>::type* r_fine,
                     typename Vec2<T>::type* b_coarse, typename Vec2<T>::type* first_out, const int* done, cudaStream_t s) {
    LaunchDims d = dims2d(coarse.o.g.Nx, coarse.o.g.Ny);
    k_restrict<T><<<d.grid, d.block, 0, s>>>(coarse, fine.o, r_fine, b_coarse, first_out, done); count_launch();
}

// prolong_at for a fine point (i, j) in 2..Nx-3 x 2..Ny-3 of a level halved in both directions: its coarse
// parents (i/2 and a neighbour, j/2 and a neighbour) need no clamp, wrap or range test.  Same expression and
// operands as prolonged(), so the result is bit for bit prolong_at's.
template <typename T>
__device__ __forceinline__ void prolong_interior(const OpView<T>& fo, const LevelView<T>& C, typename Vec2<T>::type* xf,
                                                 const typename Vec2<T>::type* __restrict__ xc, int i, int j) {
    const DevGrid<T>& cg = C.o.g;
    int k = fo.g.idx(i, j);
    uint8_t m = fo.mask[k];
    typename Vec2<T>::type x = xf[k];
    int I = i >> 1, J = j >> 1;
    bool ei = (i & 1) == 0, ej = (j & 1) == 0;   // the 1-based index is odd
    auto cu = [&](int a, int b) { int kc = cg.idx(a, b); return (__ldg(C.o.mask + kc) & U_INACTIVE) ? T(0) : xc[kc].x; };
    auto cv = [&](int a, int b) { int kc = cg.idx(a, b); return (__ldg(C.o.mask + kc) & V_INACTIVE) ? T(0) : xc[kc].y; };
    T pu = T(0), pv = T(0);
    if (!(m & U_IDENTITY)) {   // x: face parents (I, I or I + 1); y: centre parents (J, J -+ 1)
        int I2 = ei ? I : I + 1, J2 = ej ? J - 1 : J + 1;
        T wx1 = ei ? T(1) : T(1) / T(2), wx2 = ei ? T(0) : T(1) / T(2), wy1 = T(3) / T(4), wy2 = T(1) / T(4);
        pu = wx1 * (wy1 * cu(I, J) + wy2 * cu(I, J2)) + wx2 * (wy1 * cu(I2, J) + wy2 * cu(I2, J2));
    }
    if (!(m & V_IDENTITY)) {   // x: centre parents (I, I -+ 1); y: face parents (J, J or J + 1)
        int I2 = ei ? I - 1 : I + 1, J2 = ej ? J : J + 1;
        T wx1 = T(3) / T(4), wx2 = T(1) / T(4), wy1 = ej ? T(1) : T(1) / T(2), wy2 = ej ? T(0) : T(1) / T(2);
        pv = wx1 * (wy1 * cv(I, J) + wy2 * cv(I, J2)) + wx2 * (wy1 * cv(I2, J) + wy2 * cv(I2, J2));
    }
    x.x += pu;
    x.y += pv;
    xf[k] = x;
}

template <typename T>
__global__ void k_prolongate(OpView<T> fo, LevelView<T> C, typename Vec2<T>::type* xf, const typename Vec2<T>::type* __restrict__ xc,
                             const int* done) {
    NK_BATCH_ENTER(fo.g, fo, C, xf, xc, done)
    if (stopped(done)) return;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= fo.g.Nx || j >= fo.g.Ny) return;
    if (C.cx == 2 && C.cy == 2 && i >= 2 && i <= fo.g.Nx - 3 && j >= 2 && j <= fo.g.Ny - 3)
        prolong_interior(fo, C, xf, xc, i, j);
    else
        prolong_at(fo, C, xf, xc, i, j);
}
template <typename T>
void launch_prolongate(const LevelView<T>& fine, const LevelView<T>& coarse, typename Vec2<T>::type* x_fine,
                       const typename Vec2<T>::type* x_coarse, const int* done, cudaStream_t s) {
    LaunchDims d = dims2d(fine.o.g.Nx, fine.o.g.Ny);
    k_prolongate<T><<<d.grid, d.block, 0, s>>>(fine.o, coarse, x_fine, x_coarse, done); count_launch();
}

template <typename T>
__global__ void k_zero_vec(DevGrid<T> g, typename Vec2<T>::type* x, const int* done) {
    NK_BATCH_ENTER(g, g, x, done)
    if (stopped(done)) return;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    typename Vec2<T>::type z;
    z.x = T(0);
    z.y = T(0);
    x[g.idx(i, j)] = z;
}
template <typename T>
void launch_zero_vec(const DevGrid<T>& g, typename Vec2<T>::type* x, const int* done, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx + 1, g.Ny + 1);
    k_zero_vec<T><<<d.grid, d.block, 0, s>>>(g, x, done); count_launch();
}

// dst = src over a level's whole pitched plane (halo and padding included), the batched form of a device copy:
// a plain copy in a batched graph would move slot 0 alone.
template <typename T>
__global__ void k_copy_plane(DevGrid<T> g, typename Vec2<T>::type* dst, const typename Vec2<T>::type* __restrict__ src, int n,
                             const int* done) {
    NK_BATCH_ENTER(g, g, dst, src, done)
    if (stopped(done)) return;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) dst[t] = src[t];
}
template <typename T>
void launch_copy_plane(const DevGrid<T>& g, typename Vec2<T>::type* dst, const typename Vec2<T>::type* src, int n, const int* done,
                       cudaStream_t s) {
    dim3 grid((n + 255) / 256, 1, batch_slots());
    k_copy_plane<T><<<grid, 256, 0, s>>>(g, dst, src, n, done); count_launch();
}

// ---- the coarsest level in shared memory ----------------------------------------------------------------------
// The coarsest level takes many sweeps (20 by default) of a grid of about a thousand cells: as separate launches
// each sweep is a few microseconds of latency on the solve's critical path.  For FP32 levels of at most 1024 cells
// one block of 1024 threads runs every sweep on-chip, each thread owning one cell.  Everything that does not
// change between sweeps (shared-memory indices, mask tests, metrics, 2η, η̄Hᶠᶠ times the wall factor, Az β, b,
// 1/rowsum) is computed once into registers; a sweep (1) builds the masked velocities (interior_u / interior_v)
// of the current x on the grid padded by one point (wrapped when periodic, zero outside a Bounded range),
// (2) computes every centre's Δy Txx, Δx Tyy and every corner's shear once (the expressions of the column-marching
// apply), (3) combines them into x' = x + (b - A x) / rowsum and (4) stores x', with block barriers between the
// phases.  (A variant holding several cells per thread, with the constants re-read each sweep, was slower than
// separate launches, in FP64 as well; those levels keep the launches.)
template <typename T>
__global__ void __launch_bounds__(1024, 1)
    k_coarsest_smem_1(LevelView<T> L, int plane, const typename Vec2<T>::type* __restrict__ xin, int sweeps, int from_zero,
                      typename Vec2<T>::type* xout, const int* done) {
    NK_BATCH_ENTER(L.o.g, L, xin, xout, done)
    if (stopped(done)) return;
    using V2 = typename Vec2<T>::type;
    const DevGrid<T>& g = L.o.g;
    const int Nx = g.Nx, Ny = g.Ny, tid = threadIdx.x, nt = blockDim.x;
    const int n = Nx * Ny, ncorner = (Nx + 1) * (Ny + 1), PW = Nx + 2, npad = (Nx + 2) * (Ny + 2);
    extern __shared__ __align__(32) unsigned char smem[];
    V2* x = reinterpret_cast<V2*>(smem);       // plane
    V2* st = x + plane;                        // n
    V2* M = st + n;                            // npad
    T* sh = reinterpret_cast<T*>(M + npad);    // ncorner
    for (int k = tid; k < plane; k += nt) {
        V2 z;
        z.x = T(0);
        z.y = T(0);
        x[k] = xin ? xin[k] : z;
    }
    // padded masked points of this thread: e0 = tid, e1 = tid + nt
    int pk[2];
    uint8_t pf[2];                             // bit 0: u taken, bit 1: v taken
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        int e = tid + a * nt;
        pk[a] = 0;
        pf[a] = 0;
        if (e < npad) {
            int i = e % PW - 1, j = e / PW - 1;
            bool uok = (g.px || (i >= 0 && i <= Nx)) && !g.out_y(j);
            bool vok = !g.out_x(i) && (g.py || (j >= 0 && j <= Ny));
            if (uok || vok) {
                int k = g.idx(g.px ? g.wrap(i, Nx) : i, g.py ? g.wrap(j, Ny) : j);
                uint8_t mk = L.o.mask[k];
                pk[a] = k;
                pf[a] = (uok && !(mk & U_INACTIVE) ? 1 : 0) | (vok && !(mk & V_INACTIVE) ? 2 : 0);
            }
        }
    }
    // the cell c = tid: centre stress constants and the combination constants
    const bool has_cell = tid < n;
    int ci = has_cell ? tid % Nx : 0, cj = has_cell ? tid / Nx : 0;
    int kc = g.idx(ci, cj);
    T c_rdxc = T(0), c_rdyc = T(0), c_dyc = T(0), c_dxc = T(0), c_2eta = T(0), c_dxf = T(0), c_dyf = T(0), azbu = T(0), azbv = T(0);
    V2 bb, ww;
    bb.x = bb.y = ww.x = ww.y = T(0);
    uint8_t c_mask = 0;
    int sw_idx = -1, ss_idx = -1, t01_idx = 0, t10_idx = 0;
    if (has_cell) {
        c_rdxc = g.rdxc[ci]; c_rdyc = g.rdyc[cj]; c_dyc = g.dyc[cj]; c_dxc = g.dxc[ci];
        c_dxf = g.dxf[ci]; c_dyf = g.dyf[cj];
        typename Vec4<T>::type cc = L.o.coef[kc];
        c_2eta = T(2) * cc.x;
        azbu = (c_dxf * c_dyc) * cc.z;
        azbv = (c_dxc * c_dyf) * cc.w;
        bb = L.b[kc];
        ww = L.irs[kc];
        c_mask = L.o.mask[kc];
        if (ci > 0) sw_idx = tid - 1; else if (g.px) sw_idx = cj * Nx + Nx - 1;
        if (cj > 0) ss_idx = tid - Nx; else if (g.py) ss_idx = (Ny - 1) * Nx + ci;
        int jn = (g.py && cj + 1 == Ny) ? 0 : cj + 1, ie = (g.px && ci + 1 == Nx) ? 0 : ci + 1;
        t01_idx = jn * (Nx + 1) + ci;
        t10_idx = cj * (Nx + 1) + ie;
    }
    // corners of this thread: f0 = tid, f1 = tid + nt
    int fm[2][3];                              // padded indices of (i, j), (i, j - 1), (i - 1, j)
    T f_rdyf[2], f_rdxf[2], f_eta[2];
#pragma unroll
    for (int a = 0; a < 2; ++a) {
        int f = tid + a * nt;
        fm[a][0] = fm[a][1] = fm[a][2] = 0;
        f_rdyf[a] = f_rdxf[a] = f_eta[a] = T(0);
        if (f < ncorner) {
            int i = f % (Nx + 1), j = f / (Nx + 1);
            fm[a][0] = (j + 1) * PW + i + 1;
            fm[a][1] = j * PW + i + 1;
            fm[a][2] = (j + 1) * PW + i;
            f_rdyf[a] = g.rdyf[j];
            f_rdxf[a] = g.rdxf[i];
            T eta = L.o.coef[g.ff_idx(i, j)].y;
            f_eta[a] = g.peripheral_ff(i, j) ? eta * L.o.wall_factor : eta;
        }
    }
    __syncthreads();
    for (int sweep = 0; sweep < sweeps; ++sweep) {
        V2 xx = x[kc], nv;
        if (from_zero && sweep == 0) {
            nv.x = bb.x * ww.x;
            nv.y = bb.y * ww.y;
        } else {
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                if (tid + a * nt < npad) {
                    V2 v = x[pk[a]], m;
                    m.x = (pf[a] & 1) ? v.x : T(0);
                    m.y = (pf[a] & 2) ? v.y : T(0);
                    M[tid + a * nt] = m;
                }
            }
            __syncthreads();
            if (has_cell) {
                int p0 = (cj + 1) * PW + ci + 1;
                V2 m0 = M[p0], me = M[p0 + 1], mn = M[p0 + PW];
                T exx = (me.x - m0.x) * c_rdxc;
                T eyy = (mn.y - m0.y) * c_rdyc;
                V2 sv;
                sv.x = c_dyc * (c_2eta * (T(2) * exx + eyy));
                sv.y = c_dxc * (c_2eta * (T(2) * eyy + exx));
                st[tid] = sv;
            }
#pragma unroll
            for (int a = 0; a < 2; ++a) {
                if (tid + a * nt < ncorner) {
                    V2 m0 = M[fm[a][0]], ms = M[fm[a][1]], mw = M[fm[a][2]];
                    T e = (m0.x - ms.x) * f_rdyf[a] + (m0.y - mw.y) * f_rdxf[a];
                    sh[tid + a * nt] = f_eta[a] * e;
                }
            }
            __syncthreads();
            if (has_cell) {
                V2 s0 = st[tid], sw, ss;
                sw.x = sw.y = ss.x = ss.y = T(0);
                if (sw_idx >= 0) sw = st[sw_idx];
                if (ss_idx >= 0) ss = st[ss_idx];
                T t00 = sh[cj * (Nx + 1) + ci], t01 = sh[t01_idx], t10 = sh[t10_idx];
                T divu = (s0.x - sw.x) + (c_dxf * t01 - c_dxf * t00);
                T divv = (s0.y - ss.y) + (c_dyf * t10 - c_dyf * t00);
                V2 q;
                q.x = (c_mask & U_IDENTITY) ? xx.x : azbu * xx.x - divu;
                q.y = (c_mask & V_IDENTITY) ? xx.y : azbv * xx.y - divv;
                nv.x = xx.x + (bb.x - q.x) * ww.x;
                nv.y = xx.y + (bb.y - q.y) * ww.y;
            }
        }
        __syncthreads();
        if (has_cell) x[kc] = nv;
        __syncthreads();
    }
    if (has_cell) xout[kc] = x[kc];
}

// True when the level can run in one block: FP32, at most one cell, one corner beyond the cells and two padded
// points per thread.
template <typename T>
bool coarsest_smem_fits(const LevelView<T>& L, int plane) {
    (void)plane;
    int nx = L.o.g.Nx, ny = L.o.g.Ny;
    return sizeof(T) == 4 && nx * ny <= 1024 && (nx + 2) * (ny + 2) <= 2048 && (nx + 1) * (ny + 1) <= 2048;
}
template <typename T>
void configure_coarsest_smem() {
    if constexpr (sizeof(T) == 4) {
        static bool done = [] {
            int dev = 0, v = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            cudaFuncSetAttribute(k_coarsest_smem_1<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, v);
            return true;
        }();
        (void)done;
    }
}
template <typename T>
void launch_coarsest_smem(const LevelView<T>& L, int plane, const typename Vec2<T>::type* x_in, int sweeps, int from_zero,
                          typename Vec2<T>::type* x_out, const int* done, cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        int nx = L.o.g.Nx, ny = L.o.g.Ny;
        size_t bytes = (size_t)plane * sizeof(typename Vec2<T>::type) + (size_t)nx * ny * sizeof(typename Vec2<T>::type) +
                       (size_t)(nx + 2) * (ny + 2) * sizeof(typename Vec2<T>::type) + (size_t)(nx + 1) * (ny + 1) * sizeof(T);
        k_coarsest_smem_1<T><<<dim3(1, 1, batch_slots()), 1024, bytes, s>>>(L, plane, x_in, sweeps, from_zero, x_out, done);
        count_launch();
    }
}

// ---- fused coarse V-cycle: one thread block runs every remaining level ----------------------------------------
// The coarse levels of a V-cycle are a few thousand cells or less, where a grid-wide launch per sweep costs more
// than the sweep.  One 1024-thread block walks the rest of v_cycle! (:144-163) level by level — smooth, residual,
// restrict, the coarsest sweeps, prolongate, smooth — with a block barrier between phases; all data stays in
// global memory (L1/L2 resident at these sizes).  Level 0 of `C` holds its right-hand side on entry and its
// correction on exit.
template <typename T>
__device__ void block_smooth(const CoarseLevels<T>& C, const LevelView<T>& L, int sweeps, bool first) {
    using V2 = typename Vec2<T>::type;
    const DevGrid<T>& g = L.o.g;
    int n = g.Nx * g.Ny, tid = threadIdx.x, nt = blockDim.x;
    if (sweeps <= 0) {
        if (first)
            for (int c = tid; c < n; c += nt) { V2 z; z.x = T(0); z.y = T(0); L.x[g.idx(c % g.Nx, c / g.Nx)] = z; }
        __syncthreads();
        return;
    }
    if (C.line) {
        for (int k = 0; k < sweeps; ++k) {
            bool f = first && k == 0;
            if (!f) {
                for (int c = tid; c < n; c += nt) apply_or_residual_at(L, (const V2*)L.x, L.q, false, c % g.Nx, c / g.Nx);
                __syncthreads();
            }
            for (int i = tid; i < g.Nx; i += nt) line_relax_column(L, L.x, f, i);
            __syncthreads();
        }
        return;
    }
    const V2* in = L.x;
    if (!first && sweeps % 2 == 1) {
        for (int c = tid; c < n; c += nt) { int k = g.idx(c % g.Nx, c / g.Nx); L.x2[k] = L.x[k]; }
        __syncthreads();
        in = L.x2;
    }
    for (int k = 0; k < sweeps; ++k) {
        V2* out = ((sweeps - 1 - k) % 2 == 0) ? L.x : L.x2;
        bool f = first && k == 0;
        for (int c = tid; c < n; c += nt) smooth_point_at(L, in, out, f, c % g.Nx, c / g.Nx);
        __syncthreads();
        in = out;
    }
}

template <typename T>
constexpr int coarse_threads() { return sizeof(T) == 8 ? 512 : 1024; }   // FP64 needs more registers per thread

template <typename T>
__global__ void __launch_bounds__(sizeof(T) == 8 ? 512 : 1024, 1) k_coarse_vcycle(CoarseLevels<T> C, const int* done) {
    if (stopped(done)) return;
    using V2 = typename Vec2<T>::type;
    int tid = threadIdx.x, nt = blockDim.x;
    int last = C.n - 1;
    for (int l = 0; l < last; ++l) {
        const LevelView<T>& L = C.lv[l];
        const LevelView<T>& N = C.lv[l + 1];
        block_smooth(C, L, C.sweeps, true);
        int n = L.o.g.Nx * L.o.g.Ny;
        for (int c = tid; c < n; c += nt) apply_or_residual_at(L, (const V2*)L.x, L.q, true, c % L.o.g.Nx, c / L.o.g.Nx);
        __syncthreads();
        int m = N.o.g.Nx * N.o.g.Ny;
        for (int c = tid; c < m; c += nt) restrict_at(N, L.o, (const V2*)L.q, N.b, (V2*)nullptr, c % N.o.g.Nx, c / N.o.g.Nx);
        __syncthreads();
    }
    block_smooth(C, C.lv[last], C.coarsest, true);
    for (int l = last - 1; l >= 0; --l) {
        const LevelView<T>& L = C.lv[l];
        const LevelView<T>& N = C.lv[l + 1];
        int n = L.o.g.Nx * L.o.g.Ny;
        for (int c = tid; c < n; c += nt) prolong_at(L.o, N, L.x, (const V2*)N.x, c % L.o.g.Nx, c / L.o.g.Nx);
        __syncthreads();
        block_smooth(C, L, C.sweeps, false);
    }
}
template <typename T>
void launch_coarse_vcycle(const CoarseLevels<T>& C, const int* done, cudaStream_t s) {
    k_coarse_vcycle<T><<<1, coarse_threads<T>(), 0, s>>>(C, done); count_launch();
}

#define NK_INSTANTIATE(T)                                                                                                   \
    template void launch_smooth_point<T>(const LevelView<T>&, const Vec2<T>::type*, Vec2<T>::type*, int, const int*, cudaStream_t); \
    template void launch_smooth_first2<T>(const LevelView<T>&, Vec2<T>::type*, const int*, cudaStream_t); \
    template bool coarsest_smem_fits<T>(const LevelView<T>&, int); \
    template void configure_coarsest_smem<T>(); \
    template void launch_coarsest_smem<T>(const LevelView<T>&, int, const Vec2<T>::type*, int, int, Vec2<T>::type*, const int*, cudaStream_t); \
    template void launch_level_apply<T>(const LevelView<T>&, const Vec2<T>::type*, Vec2<T>::type*, int, const int*, cudaStream_t);  \
    template void launch_line_relax<T>(const LevelView<T>&, Vec2<T>::type*, int, const int*, cudaStream_t);                        \
    template void launch_restrict<T>(const LevelView<T>&, const LevelView<T>&, const Vec2<T>::type*, Vec2<T>::type*, Vec2<T>::type*, \
                                     const int*, cudaStream_t);                                                                     \
    template void launch_prolongate<T>(const LevelView<T>&, const LevelView<T>&, Vec2<T>::type*, const Vec2<T>::type*, const int*, \
                                       cudaStream_t);                                                                               \
    template void launch_zero_vec<T>(const DevGrid<T>&, Vec2<T>::type*, const int*, cudaStream_t);                                 \
    template void launch_copy_plane<T>(const DevGrid<T>&, Vec2<T>::type*, const Vec2<T>::type*, int, const int*, cudaStream_t);    \
    template void launch_coarse_vcycle<T>(const CoarseLevels<T>&, const int*, cudaStream_t);                     \
    template float time_strip_kernel<T>(const LevelView<T>&, int, int, int, cudaStream_t);

NK_INSTANTIATE(double)
NK_INSTANTIATE(float)

}  // namespace nk
