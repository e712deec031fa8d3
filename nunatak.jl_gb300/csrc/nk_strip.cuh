// nk_strip.cuh — column-marching operator apply.
//
// The operator of nk_operator.cuh evaluated by warps that walk down the grid instead of by 2-D tiles in shared
// memory.  Lane l of a warp holds the column i = i_first - 1 + l (32 consecutive faces), so the x neighbours of a
// lane's values are one warp shuffle away; the lane walks R rows j0, j0 + 1, ... keeping the previous
// and the next row in registers, so the y neighbours need no exchange at all.  Per row a lane loads one
// velocity pair with its mask byte and one coefficient record, computes the centre stresses of centre (i, j) and
// the shear of corner (i, j + 1) once, and takes the west centre and the east corner from its neighbour lanes by
// shuffle.  Lanes 0 and 31 only supply those neighbour values: a warp writes the 30 columns of lanes 1..30.
// There is no shared memory and no block barrier.
//
// Each quantity is computed by the same expression as in center_stress / corner_shear / apply_at, in the same
// operand order, so the result equals the per-cell and tiled forms.
#pragma once

#include <type_traits>

#include "nk_operator.cuh"

namespace nk {

constexpr int STRIP_COLS = 30;   // columns written per warp (lanes 1..30)
constexpr int STRIP_WARPS = 4;   // warps per block, stacked in y

// Launch shape of a strip kernel whose warps walk `rows` rows each.
inline LaunchDims strip_dims(int nx, int ny, int rows) {
    LaunchDims d;
    d.block = dim3(32, STRIP_WARPS);
    d.grid = dim3((nx + STRIP_COLS - 1) / STRIP_COLS, (ny + rows * STRIP_WARPS - 1) / (rows * STRIP_WARPS), batch_slots());
    return d;
}

// Rows per warp for an nx x ny grid of `elem_bytes`-byte values (host side; nk_problem.cu).  Long walks
// amortise the two priming rows on large grids; short ones keep enough warps in flight on small grids.
// `kind` names the kernel: the multigrid sweeps and residuals write one value per cell with no reduction, so
// their walk length cannot change a bit of the result and is taken from the autotuner's table when it has an
// entry (nk_problem.cu); the FP64 operator kernels carry block reductions and keep the fixed rule.
enum StripKernel { STRIP_OPERATOR = 0, STRIP_SMOOTH = 1, STRIP_RESIDUAL = 2 };
int strip_rows(int nx, int ny, int elem_bytes, int kind = STRIP_OPERATOR);
constexpr int STRIP_MIN_ROWS = 1;

// Calls f(std::integral_constant<int, R>) for the supported walk lengths R.
template <typename F>
inline void with_strip_rows(int rows, F&& f) {
    switch (rows) {
        case 1: f(std::integral_constant<int, 1>{}); break;
        case 2: f(std::integral_constant<int, 2>{}); break;
        case 4: f(std::integral_constant<int, 4>{}); break;
        default: f(std::integral_constant<int, 8>{}); break;
    }
}

// One row of a lane's column: the velocity pair as stored and its mask byte, plus whether the pair takes part
// in the strain rates as u (interior_u) and as v (interior_v).
template <typename T>
struct StripRow {
    typename Vec2<T>::type raw;
    uint8_t m;
    bool uok, vok;
    __device__ __forceinline__ T mu() const { return (uok && !(m & U_INACTIVE)) ? raw.x : T(0); }
    __device__ __forceinline__ T mv() const { return (vok && !(m & V_INACTIVE)) ? raw.y : T(0); }
};

// The pair at (i, j) as masked_u / masked_v read it; zero outside the ranges those functions read.
// `src(k, iw, jw)` returns the stored pair at pitched index k = idx(iw, jw) (iw, jw wrapped when periodic).
template <typename T, typename Src>
__device__ __forceinline__ StripRow<T> strip_load(const OpView<T>& o, Src&& src, int i, int j, bool col_ok) {
    const DevGrid<T>& g = o.g;
    StripRow<T> r;
    r.raw.x = T(0);
    r.raw.y = T(0);
    r.m = 0;
    r.uok = false;
    r.vok = false;
    if (!col_ok || j > g.Ny) return r;
    r.uok = (g.px || (i >= 0 && i <= g.Nx)) && !g.out_y(j);
    r.vok = !g.out_x(i) && (g.py || (j >= 0 && j <= g.Ny));
    if (!(r.uok || r.vok)) return r;
    int iw = g.px ? g.wrap(i, g.Nx) : i, jw = g.py ? g.wrap(j, g.Ny) : j;
    int k = g.idx(iw, jw);
    r.m = __ldg(o.mask + k);
    r.raw = src(k, iw, jw);
    return r;
}

struct NoExtra {};

// q = A p over the cells of one warp strip.  For every cell (i, j), i < Nx, j < Ny, that the lane owns,
// `extra(k)` is called first (with the loads of the walk, so its global reads are in flight together with them)
// and later `emit(k, q, raw, e)` with k = idx(i, j), q the operator result, raw the stored pair p(i, j) and e what
// extra(k) returned.  Every lane of the warp must call this (shuffles); lanes with nothing to do pass through.
// IU / IV: the mask bits of the identity rows (q = p).  A caller whose own rule already fixes the prescribed rows
// may pass U_INACTIVE / V_INACTIVE, the bits of the strain-rate reads, which then serve both tests.
template <int R, uint8_t IU = U_IDENTITY, uint8_t IV = V_IDENTITY, typename T, typename Src, typename Extra, typename Emit>
__device__ __forceinline__ void strip_apply_general(const OpView<T>& o, Src&& src, int i, int j0, Extra&& extra, Emit&& emit) {
    using V2 = typename Vec2<T>::type;
    using V4 = typename Vec4<T>::type;
    using E = decltype(extra(0));
    const DevGrid<T>& g = o.g;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x;
    const bool col_ok = i <= g.Nx;                       // i >= -1 by construction
    const bool own_col = lane >= 1 && lane <= STRIP_COLS && i < g.Nx;
    T rdxc_i = T(0), dxc_i = T(0), rdxf_i = T(0), dxf_i = T(0);
    int cxi = 0, fxi = 0;
    if (col_ok) {
        rdxc_i = g.rdxc[i];
        dxc_i = g.dxc[i];
        rdxf_i = g.rdxf[i];
        dxf_i = g.dxf[i];
        cxi = g.cx(i);
        fxi = g.fx(i);
    }
    const bool per_ff_x = g.out_x(i) || g.out_x(i - 1);

    // every global read of the walk, issued before any arithmetic
    StripRow<T> row[R + 2];   // rows j0 - 1 .. j0 + R
    V4 rec[R + 1];            // coefficient record of centre (i, j), rows j0 - 1 .. j0 + R - 1
    T cff[R + 1];             // η̄Hᶠᶠ of corner (i, j), rows j0 .. j0 + R
    T rdyc[R + 1], dyc[R + 1], rdyf[R + 1], dyf[R];
    E ex[R];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) row[r] = strip_load(o, src, i, j0 - 1 + r, col_ok);
#pragma unroll
    for (int r = 0; r < R + 1; ++r) {
        int jc = j0 - 1 + r, jf = j0 + r;
        bool okc = col_ok && jc <= g.Ny, okf = col_ok && jf <= g.Ny;
        V4 z;
        z.x = T(0); z.y = T(0); z.z = T(0); z.w = T(0);
        rec[r] = okc ? o.coef[g.idx(cxi, g.cy(jc))] : z;
        rdyc[r] = okc ? g.rdyc[jc] : T(0);
        dyc[r] = okc ? g.dyc[jc] : T(0);
        cff[r] = okf ? o.coef[g.idx(fxi, g.fy(jf))].y : T(0);
        rdyf[r] = okf ? g.rdyf[jf] : T(0);
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
        int j = j0 + r;
        dyf[r] = (col_ok && j <= g.Ny) ? g.dyf[j] : T(0);
        if (own_col && j < g.Ny) ex[r] = extra(g.idx(i, j));
    }

    // centre (i, j) from row j (index a of row[]) and row j + 1: Δy Txx, Δx Tyy; c indexes rec/rdyc/dyc
    auto centre = [&](int a, int c, T& sxx, T& syy) {
        T mu = row[a].mu(), mv = row[a].mv(), mvn = row[a + 1].mv();
        T mue = __shfl_down_sync(full, mu, 1);
        T exx = (mue - mu) * rdxc_i;
        T eyy = (mvn - mv) * rdyc[c];
        T eta = rec[c].x;
        sxx = dyc[c] * (T(2) * eta * (T(2) * exx + eyy));
        syy = dxc_i * (T(2) * eta * (T(2) * eyy + exx));
    };
    // corner (i, j) from rows j - 1 (index a - 1) and j (index a): 2 η̄Hᶠᶠ ε̇xy; c indexes cff/rdyf, j the row
    auto corner = [&](int a, int c, int j) -> T {
        T mu = row[a].mu(), mus = row[a - 1].mu(), mv = row[a].mv();
        T mvw = __shfl_up_sync(full, mv, 1);
        T dudy = (mu - mus) * rdyf[c];
        T dvdx = (mv - mvw) * rdxf_i;
        // 2 η̄Hᶠᶠ ε̇xy with ε̇xy = (dudy + dvdx) / 2 (× the wall factor), written as η̄Hᶠᶠ (dudy + dvdx): the
        // halving and doubling are exact, so this drops two operations and changes only how the compiler may
        // contract the sum into a multiply-add (last-bit differences)
        T e = dudy + dvdx;
        if (per_ff_x || g.out_y(j) || g.out_y(j - 1)) e = o.wall_factor * e;
        return cff[c] * e;
    };

    T sxx_s, syy_s;
    centre(0, 0, sxx_s, syy_s);    // centre (i, j0 - 1)
    T t_c = corner(1, 0, j0);      // corner (i, j0)
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = j0 + r;
        T sxx, syy;
        centre(r + 1, r + 1, sxx, syy);          // centre (i, j)
        T t_n = corner(r + 2, r + 1, j + 1);     // corner (i, j + 1)
        T sxx_w = __shfl_up_sync(full, sxx, 1);
        T t_e = __shfl_down_sync(full, t_c, 1);
        if (own_col && j < g.Ny) {
            const V4& c = rec[r + 1];             // the record of (i, j) itself: cx(i) = i, cy(j) = j here
            const V2& x = row[r + 1].raw;
            T divu = (sxx - sxx_w) + (dxf_i * t_n - dxf_i * t_c);
            T divv = (syy - syy_s) + (dyf[r] * t_e - dyf[r] * t_c);
            V2 q;
            q.x = (row[r + 1].m & IU) ? x.x : (dxf_i * dyc[r + 1]) * c.z * x.x - divu;
            q.y = (row[r + 1].m & IV) ? x.y : (dxc_i * dyf[r]) * c.w * x.y - divv;
            emit(g.idx(i, j), q, x, ex[r]);
        }
        syy_s = syy;
        t_c = t_n;
    }
}

// The same walk for a warp whose 32 columns and R + 2 rows lie strictly inside the grid (columns 1 .. Nx - 2, rows
// 1 .. Ny - 2): every index is its own stored index (no wrap, no clamp), every velocity takes part in the strain rates
// (only the mask byte decides), no corner is a wall corner, and the corner record of row j is the centre record of
// row j, so it is not loaded twice.  The arithmetic is the general walk's, expression for expression, so both give
// the same bits.
template <int R, uint8_t IU = U_IDENTITY, uint8_t IV = V_IDENTITY, typename T, typename Src, typename Extra, typename Emit>
__device__ __forceinline__ void strip_apply_interior(const OpView<T>& o, Src&& src, int i, int j0, Extra&& extra, Emit&& emit) {
    using V2 = typename Vec2<T>::type;
    using V4 = typename Vec4<T>::type;
    using E = decltype(extra(0));
    const DevGrid<T>& g = o.g;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x;
    const bool own_col = lane >= 1 && lane <= STRIP_COLS;
    const T rdxc_i = g.rdxc[i], dxc_i = g.dxc[i], rdxf_i = g.rdxf[i], dxf_i = g.dxf[i];

    V2 raw[R + 2];            // rows j0 - 1 .. j0 + R
    uint8_t msk[R + 2];
    V4 rec[R + 1];            // centre (i, j), rows j0 - 1 .. j0 + R - 1
    T cffR;                   // η̄Hᶠᶠ of corner (i, j0 + R); the others are rec[r + 1].y
    T rdyc[R + 1], dyc[R + 1], rdyf[R + 1], dyf[R];
    E ex[R];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) {
        int k = g.idx(i, j0 - 1 + r);
        msk[r] = __ldg(o.mask + k);
        raw[r] = src(k, i, j0 - 1 + r);
    }
#pragma unroll
    for (int r = 0; r < R + 1; ++r) {
        int jc = j0 - 1 + r;
        rec[r] = o.coef[g.idx(i, jc)];
        rdyc[r] = g.rdyc[jc];
        dyc[r] = g.dyc[jc];
        rdyf[r] = g.rdyf[jc + 1];
    }
    cffR = o.coef[g.idx(i, j0 + R)].y;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        dyf[r] = g.dyf[j0 + r];
        if (own_col) ex[r] = extra(g.idx(i, j0 + r));
    }
    auto mu = [&](int a) { return (msk[a] & U_INACTIVE) ? T(0) : raw[a].x; };
    auto mv = [&](int a) { return (msk[a] & V_INACTIVE) ? T(0) : raw[a].y; };
    auto cff = [&](int c) { return c < R ? rec[c + 1].y : cffR; };

    auto centre = [&](int a, int c, T& sxx, T& syy) {
        T u0 = mu(a), v0 = mv(a), vn = mv(a + 1);
        T ue = __shfl_down_sync(full, u0, 1);
        T exx = (ue - u0) * rdxc_i;
        T eyy = (vn - v0) * rdyc[c];
        T eta = rec[c].x;
        sxx = dyc[c] * (T(2) * eta * (T(2) * exx + eyy));
        syy = dxc_i * (T(2) * eta * (T(2) * eyy + exx));
    };
    auto corner = [&](int a, int c) -> T {
        T u0 = mu(a), us = mu(a - 1), v0 = mv(a);
        T vw = __shfl_up_sync(full, v0, 1);
        T dudy = (u0 - us) * rdyf[c];
        T dvdx = (v0 - vw) * rdxf_i;
        T e = dudy + dvdx;
        return cff(c) * e;
    };

    T sxx_s, syy_s;
    centre(0, 0, sxx_s, syy_s);
    T t_c = corner(1, 0);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        T sxx, syy;
        centre(r + 1, r + 1, sxx, syy);
        T t_n = corner(r + 2, r + 1);
        T sxx_w = __shfl_up_sync(full, sxx, 1);
        T t_e = __shfl_down_sync(full, t_c, 1);
        if (own_col) {
            const V4& c = rec[r + 1];
            const V2& x = raw[r + 1];
            T divu = (sxx - sxx_w) + (dxf_i * t_n - dxf_i * t_c);
            T divv = (syy - syy_s) + (dyf[r] * t_e - dyf[r] * t_c);
            V2 q;
            q.x = (msk[r + 1] & IU) ? x.x : (dxf_i * dyc[r + 1]) * c.z * x.x - divu;
            q.y = (msk[r + 1] & IV) ? x.y : (dxc_i * dyf[r]) * c.w * x.y - divv;
            emit(g.idx(i, j0 + r), q, x, ex[r]);
        }
        syy_s = syy;
        t_c = t_n;
    }
}

// The interior walk on a regular square grid (every spacing h, DevGrid::h != 0): with Δx = Δy = h the metric factors
// of the stencil cancel, Δy Txx = 2η̄H (2 Δu + Δv), Δx Tyy = 2η̄H (2 Δv + Δu), Δx η̄Hᶠᶠ (∂u/∂y + ∂v/∂x) =
// η̄Hᶠᶠ (Δᵧu + Δₓv) and Az β = h² β, with Δ the differences of neighbouring velocities.  The same operator in the same
// sums, with the products by h and 1/h left out: results differ from the general walk in the last bits only.  No
// metric is loaded.
template <int R, uint8_t IU = U_IDENTITY, uint8_t IV = V_IDENTITY, typename T, typename Src, typename Extra, typename Emit>
__device__ __forceinline__ void strip_apply_uniform(const OpView<T>& o, Src&& src, int i, int j0, Extra&& extra, Emit&& emit) {
    using V2 = typename Vec2<T>::type;
    using V4 = typename Vec4<T>::type;
    using E = decltype(extra(0));
    const DevGrid<T>& g = o.g;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x;
    const bool own_col = lane >= 1 && lane <= STRIP_COLS;
    const T h2 = g.h * g.h;

    V2 raw[R + 2];            // rows j0 - 1 .. j0 + R
    uint8_t msk[R + 2];
    V4 rec[R + 1];            // centre (i, j), rows j0 - 1 .. j0 + R - 1
    T cffR;                   // η̄Hᶠᶠ of corner (i, j0 + R); the others are rec[r + 1].y
    E ex[R];
#pragma unroll
    for (int r = 0; r < R + 2; ++r) {
        int k = g.idx(i, j0 - 1 + r);
        msk[r] = __ldg(o.mask + k);
        raw[r] = src(k, i, j0 - 1 + r);
    }
#pragma unroll
    for (int r = 0; r < R + 1; ++r) rec[r] = o.coef[g.idx(i, j0 - 1 + r)];
    cffR = o.coef[g.idx(i, j0 + R)].y;
#pragma unroll
    for (int r = 0; r < R; ++r)
        if (own_col) ex[r] = extra(g.idx(i, j0 + r));
    auto mu = [&](int a) { return (msk[a] & U_INACTIVE) ? T(0) : raw[a].x; };
    auto mv = [&](int a) { return (msk[a] & V_INACTIVE) ? T(0) : raw[a].y; };
    auto cff = [&](int c) { return c < R ? rec[c + 1].y : cffR; };

    auto centre = [&](int a, int c, T& sxx, T& syy) {
        T u0 = mu(a), v0 = mv(a), vn = mv(a + 1);
        T ue = __shfl_down_sync(full, u0, 1);
        T du = ue - u0, dv = vn - v0;
        T e2 = T(2) * rec[c].x;
        sxx = e2 * (T(2) * du + dv);
        syy = e2 * (T(2) * dv + du);
    };
    auto corner = [&](int a, int c) -> T {   // Δx × the corner shear (= Δy × it)
        T u0 = mu(a), us = mu(a - 1), v0 = mv(a);
        T vw = __shfl_up_sync(full, v0, 1);
        return cff(c) * ((u0 - us) + (v0 - vw));
    };

    T sxx_s, syy_s;
    centre(0, 0, sxx_s, syy_s);
    T t_c = corner(1, 0);
#pragma unroll
    for (int r = 0; r < R; ++r) {
        T sxx, syy;
        centre(r + 1, r + 1, sxx, syy);
        T t_n = corner(r + 2, r + 1);
        T sxx_w = __shfl_up_sync(full, sxx, 1);
        T t_e = __shfl_down_sync(full, t_c, 1);
        if (own_col) {
            const V4& c = rec[r + 1];
            const V2& x = raw[r + 1];
            T divu = (sxx - sxx_w) + (t_n - t_c);
            T divv = (syy - syy_s) + (t_e - t_c);
            V2 q;
            q.x = (msk[r + 1] & IU) ? x.x : h2 * c.z * x.x - divu;
            q.y = (msk[r + 1] & IV) ? x.y : h2 * c.w * x.y - divv;
            emit(g.idx(i, j0 + r), q, x, ex[r]);
        }
        syy_s = syy;
        t_c = t_n;
    }
}

// The walk of the calling warp: the interior form when all its columns and rows are strictly inside the grid
// (warp-uniform test; its regular-square-grid form when the level is one), the general one otherwise.
template <int R, uint8_t IU = U_IDENTITY, uint8_t IV = V_IDENTITY, typename T, typename Src, typename Extra, typename Emit>
__device__ __forceinline__ void strip_apply_src(const OpView<T>& o, Src&& src, int i, int j0, Extra&& extra, Emit&& emit) {
    const int i_first = i - (int)threadIdx.x;
    const bool interior = i_first >= 1 && i_first + 31 <= o.g.Nx - 2 && j0 - 1 >= 1 && j0 + R <= o.g.Ny - 2;
    if (interior && o.g.h != decltype(o.g.h)(0)) strip_apply_uniform<R, IU, IV>(o, src, i, j0, extra, emit);
    else if (interior) strip_apply_interior<R, IU, IV>(o, src, i, j0, extra, emit);
    else strip_apply_general<R, IU, IV>(o, src, i, j0, extra, emit);
}

// strip_apply_src with the operand read from an array.
template <int R, uint8_t IU = U_IDENTITY, uint8_t IV = V_IDENTITY, typename T, typename Extra, typename Emit>
__device__ __forceinline__ void strip_apply(const OpView<T>& o, const typename Vec2<T>::type* __restrict__ p, int i, int j0,
                                            Extra&& extra, Emit&& emit) {
    strip_apply_src<R, IU, IV>(o, [p](int k, int, int) { return p[k]; }, i, j0, extra, emit);
}

// Column and first row of the calling thread in a strip launch of R rows per warp (strip_dims).
template <int R>
__device__ __forceinline__ void strip_origin(int& i, int& j0) {
    i = blockIdx.x * STRIP_COLS - 1 + (int)threadIdx.x;
    j0 = (blockIdx.y * STRIP_WARPS + (int)threadIdx.y) * R;
}

}  // namespace nk
