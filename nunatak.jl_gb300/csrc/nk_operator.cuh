// nk_operator.cuh — device functions of the matrix-free SSA / DIVA operator on the C grid.
//
// Restates src/StressBalances/ssa_operator.jl:47-89 and strain_rates.jl:1-32 (operator, strain rates, wall handling),
// src/StressBalances/diagonal_preconditioner.jl:20-44 (operator diagonal) and
// src/StressBalances/multigrid_preconditioner.jl:195-227 (ℓ1 row sums, line couplings), with the
// metric divisions replaced by multiplications with precomputed reciprocals.
#pragma once

#include "nk_internal.cuh"

namespace nk {

template <typename T>
struct OpView {
    DevGrid<T> g;
    const typename Vec4<T>::type* coef;   // (eta_H, eta_H_ff, beta_u, beta_v) per (i, j)
    const uint8_t* mask;                  // U/V_INACTIVE, _WALL, _DIRICHLET bits per (i, j)
    T wall_factor;                        // wall_shear_factor: 0 free slip, 2 no slip (strain_rates.jl:11-12)
};
template <typename T>
__device__ __forceinline__ void rebase(OpView<T>& o, long long d) {
    rebase(o.g, d);
    shift_ptr(o.coef, d);
    shift_ptr(o.mask, d);
}

// interior_u / interior_v (strain_rates.jl:5-6) with the operator's mask (walls and ice-free points); a prescribed
// face passes its value (U_DIRICHLET / V_DIRICHLET).
template <typename T, typename V2>
__device__ __forceinline__ T masked_u(const OpView<T>& o, const V2* __restrict__ p, int i, int j) {
    const DevGrid<T>& g = o.g;
    if ((!g.px && (i < 0 || i > g.Nx)) || g.out_y(j)) return T(0);
    int k = g.idx(g.px ? g.wrap(i, g.Nx) : i, g.py ? g.wrap(j, g.Ny) : j);
    return (__ldg(o.mask + k) & U_INACTIVE) ? T(0) : p[k].x;
}
template <typename T, typename V2>
__device__ __forceinline__ T masked_v(const OpView<T>& o, const V2* __restrict__ p, int i, int j) {
    const DevGrid<T>& g = o.g;
    if (g.out_x(i) || (!g.py && (j < 0 || j > g.Ny))) return T(0);
    int k = g.idx(g.px ? g.wrap(i, g.Nx) : i, g.py ? g.wrap(j, g.Ny) : j);
    return (__ldg(o.mask + k) & V_INACTIVE) ? T(0) : p[k].y;
}

// Δy Txx and Δx Tyy at centre (i, j): normal_stress_xx/yy times the face length (ssa_operator.jl:60-65).
template <typename T, typename V2>
__device__ __forceinline__ void center_stress(const OpView<T>& o, const V2* __restrict__ p, int i, int j, T& sxx, T& syy) {
    const DevGrid<T>& g = o.g;
    T exx = (masked_u(o, p, i + 1, j) - masked_u(o, p, i, j)) * g.rdxc[i];
    T eyy = (masked_v(o, p, i, j + 1) - masked_v(o, p, i, j)) * g.rdyc[j];
    T eta = o.coef[g.c_idx(i, j)].x;
    sxx = g.dyc[j] * (T(2) * eta * (T(2) * exx + eyy));
    syy = g.dxc[i] * (T(2) * eta * (T(2) * eyy + exx));
}

// shear_stress at corner (i, j) = 2 η̄Hᶠᶠ ε̇xy, ε̇xy scaled by the wall factor on wall corners (ssa_operator.jl:62, strain_rates.jl:14-17).
template <typename T, typename V2>
__device__ __forceinline__ T corner_shear(const OpView<T>& o, const V2* __restrict__ p, int i, int j) {
    const DevGrid<T>& g = o.g;
    T dudy = (masked_u(o, p, i, j) - masked_u(o, p, i, j - 1)) * g.rdyf[j];
    T dvdx = (masked_v(o, p, i, j) - masked_v(o, p, i - 1, j)) * g.rdxf[i];
    T e = (dudy + dvdx) / T(2);
    if (g.peripheral_ff(i, j)) e = o.wall_factor * e;
    return T(2) * o.coef[g.ff_idx(i, j)].y * e;
}

// q = A p at (i, j) for both components (x_stress_balance / y_stress_balance, ssa_operator.jl:69-89).
template <typename T, typename V2>
__device__ __forceinline__ V2 apply_at(const OpView<T>& o, const V2* __restrict__ p, int i, int j) {
    const DevGrid<T>& g = o.g;
    int k = g.idx(i, j);
    V2 pc = p[k];
    uint8_t m = __ldg(o.mask + k);
    auto c = o.coef[k];
    T sxx0, syy0, sxxw, syyw, sxxs, syys;
    center_stress(o, p, i, j, sxx0, syy0);
    center_stress(o, p, i - 1, j, sxxw, syyw);
    center_stress(o, p, i, j - 1, sxxs, syys);
    T t00 = corner_shear(o, p, i, j);
    T t01 = corner_shear(o, p, i, j + 1);
    T t10 = corner_shear(o, p, i + 1, j);
    V2 q;
    T divu = (sxx0 - sxxw) + (g.dxf[i] * t01 - g.dxf[i] * t00);
    T divv = (syy0 - syys) + (g.dyf[j] * t10 - g.dyf[j] * t00);
    q.x = (m & U_IDENTITY) ? pc.x : g.Az_fc(i, j) * c.z * pc.x - divu;
    q.y = (m & V_IDENTITY) ? pc.y : g.Az_cf(i, j) * c.w * pc.y - divv;
    return q;
}

// ---- diagonal and ℓ1 row sums ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T eta_c(const OpView<T>& o, int i, int j) { return o.coef[o.g.c_idx(i, j)].x; }
template <typename T>
__device__ __forceinline__ T eta_ff(const OpView<T>& o, int i, int j) { return o.coef[o.g.ff_idx(i, j)].y; }
template <typename T>
__device__ __forceinline__ T corner_factor(const OpView<T>& o, int i, int j) { return o.g.peripheral_ff(i, j) ? o.wall_factor : T(1); }
template <typename T>
__device__ __forceinline__ T x_normal_diagonal(const OpView<T>& o, int i, int j) { return T(4) * o.g.dyc[j] * eta_c(o, i, j) * o.g.rdxc[i]; }
template <typename T>
__device__ __forceinline__ T y_normal_diagonal(const OpView<T>& o, int i, int j) { return T(4) * o.g.dxc[i] * eta_c(o, i, j) * o.g.rdyc[j]; }
template <typename T>
__device__ __forceinline__ T x_shear_diagonal(const OpView<T>& o, int i, int j) { return corner_factor(o, i, j) * o.g.dxf[i] * eta_ff(o, i, j) * o.g.rdyf[j]; }
template <typename T>
__device__ __forceinline__ T y_shear_diagonal(const OpView<T>& o, int i, int j) { return corner_factor(o, i, j) * o.g.dyf[j] * eta_ff(o, i, j) * o.g.rdxf[i]; }

// x_diagonal / y_diagonal (diagonal_preconditioner.jl:32-44); unit where inactive or zero.
template <typename T>
__device__ __forceinline__ T x_diagonal(const OpView<T>& o, int i, int j, uint8_t m) {
    T d = o.g.Az_fc(i, j) * o.coef[o.g.idx(i, j)].z + x_normal_diagonal(o, i, j) + x_normal_diagonal(o, i - 1, j) +
          x_shear_diagonal(o, i, j) + x_shear_diagonal(o, i, j + 1);
    return ((m & U_IDENTITY) || d == T(0)) ? T(1) : d;
}
template <typename T>
__device__ __forceinline__ T y_diagonal(const OpView<T>& o, int i, int j, uint8_t m) {
    T d = o.g.Az_cf(i, j) * o.coef[o.g.idx(i, j)].w + y_normal_diagonal(o, i, j) + y_normal_diagonal(o, i, j - 1) +
          y_shear_diagonal(o, i, j) + y_shear_diagonal(o, i + 1, j);
    return ((m & V_IDENTITY) || d == T(0)) ? T(1) : d;
}

// x_absolute_row_sum / y_absolute_row_sum (multigrid_preconditioner.jl:195-211).
template <typename T>
__device__ __forceinline__ T x_row_sum(const OpView<T>& o, int i, int j, uint8_t m) {
    T s = o.g.Az_fc(i, j) * o.coef[o.g.idx(i, j)].z +
          T(2) * (x_normal_diagonal(o, i, j) + x_normal_diagonal(o, i - 1, j)) +
          T(4) * (eta_c(o, i, j) + eta_c(o, i - 1, j)) +
          T(2) * (x_shear_diagonal(o, i, j) + x_shear_diagonal(o, i, j + 1)) +
          T(2) * (corner_factor(o, i, j) * eta_ff(o, i, j) + corner_factor(o, i, j + 1) * eta_ff(o, i, j + 1));
    return ((m & U_IDENTITY) || s == T(0)) ? T(1) : s;
}
template <typename T>
__device__ __forceinline__ T y_row_sum(const OpView<T>& o, int i, int j, uint8_t m) {
    T s = o.g.Az_cf(i, j) * o.coef[o.g.idx(i, j)].w +
          T(2) * (y_normal_diagonal(o, i, j) + y_normal_diagonal(o, i, j - 1)) +
          T(4) * (eta_c(o, i, j) + eta_c(o, i, j - 1)) +
          T(2) * (y_shear_diagonal(o, i, j) + y_shear_diagonal(o, i + 1, j)) +
          T(2) * (corner_factor(o, i, j) * eta_ff(o, i, j) + corner_factor(o, i + 1, j) * eta_ff(o, i + 1, j));
    return ((m & V_IDENTITY) || s == T(0)) ? T(1) : s;
}

// Operator mask inactive test of a face (peripheral or ice free) outside the stored range.
template <typename T>
__device__ __forceinline__ bool u_inactive(const OpView<T>& o, int i, int j) {
    const DevGrid<T>& g = o.g;
    if ((!g.px && (i < 0 || i > g.Nx)) || g.out_y(j)) return true;
    return __ldg(o.mask + g.idx(g.px ? g.wrap(i, g.Nx) : i, g.py ? g.wrap(j, g.Ny) : j)) & U_IDENTITY;
}
template <typename T>
__device__ __forceinline__ bool v_inactive(const OpView<T>& o, int i, int j) {
    const DevGrid<T>& g = o.g;
    if (g.out_x(i) || (!g.py && (j < 0 || j > g.Ny))) return true;
    return __ldg(o.mask + g.idx(g.px ? g.wrap(i, g.Nx) : i, g.py ? g.wrap(j, g.Ny) : j)) & V_IDENTITY;
}

// y-line couplings of the line smoother (multigrid_preconditioner.jl:223-227).
template <typename T>
__device__ __forceinline__ T x_line_coupling(const OpView<T>& o, int i, int j) {
    return (u_inactive(o, i, j - 1) || u_inactive(o, i, j)) ? T(0) : x_shear_diagonal(o, i, j);
}
template <typename T>
__device__ __forceinline__ T y_line_coupling(const OpView<T>& o, int i, int j) {
    return (v_inactive(o, i, j - 1) || v_inactive(o, i, j)) ? T(0) : y_normal_diagonal(o, i, j - 1);
}

}  // namespace nk

namespace nk {

// ---- tiled operator apply ------------------------------------------------------------------------------------
// One BX x BY thread block computes q = A p for its BX x BY cells in three phases:
//   1. the masked velocities (interior_u / interior_v) of the tile and a one-cell halo into shared memory;
//   2. every centre stress Δy Txx, Δx Tyy and corner stress Txy the tile needs, once each, into shared memory
//      (the per-cell form recomputes each of them two to three times);
//   3. the divergence of the stresses plus the drag term for the thread's own cell.
// Every thread of the block must call tiled_apply (it synchronises the block); `inside` tells whether the
// thread's cell exists.
template <typename T>
struct ApplyTile {
    typename Vec2<T>::type pm[BY + 2][BX + 2];   // masked p at (i0 - 1 + a, j0 - 1 + b) -> [b][a]
    T sxx[BY + 1][BX + 1];                        // Δy Txx at centre (i0 - 1 + a, j0 - 1 + b)
    T syy[BY + 1][BX + 1];                        // Δx Tyy at the same centres
    T txy[BY + 1][BX + 1];                        // Txy at corner (i0 + a, j0 + b)
};

template <typename T, typename V2>
__device__ __forceinline__ V2 tiled_apply(const OpView<T>& o, const V2* __restrict__ p, ApplyTile<T>& sm, int i0, int j0,
                                          int i, int j, bool inside) {
    const DevGrid<T>& g = o.g;
    int tid = threadIdx.y * BX + threadIdx.x;
    for (int t = tid; t < (BX + 2) * (BY + 2); t += BX * BY) {
        int a = t % (BX + 2), b = t / (BX + 2);
        int ii = i0 - 1 + a, jj = j0 - 1 + b;
        V2 m;
        m.x = T(0);
        m.y = T(0);
        if (ii <= g.Nx && jj <= g.Ny) {   // beyond index N nothing of the tile's cells is read (and wrap() covers one period)
            m.x = masked_u(o, p, ii, jj);
            m.y = masked_v(o, p, ii, jj);
        }
        sm.pm[b][a] = m;
    }
    __syncthreads();
    for (int t = tid; t < (BX + 1) * (BY + 1); t += BX * BY) {
        int a = t % (BX + 1), b = t / (BX + 1);
        int ci = i0 - 1 + a, cj = j0 - 1 + b;   // centre
        if (ci < g.Nx && cj < g.Ny) {
            T exx = (sm.pm[b][a + 1].x - sm.pm[b][a].x) * g.rdxc[ci];
            T eyy = (sm.pm[b + 1][a].y - sm.pm[b][a].y) * g.rdyc[cj];
            T eta = o.coef[g.c_idx(ci, cj)].x;
            sm.sxx[b][a] = g.dyc[cj] * (T(2) * eta * (T(2) * exx + eyy));
            sm.syy[b][a] = g.dxc[ci] * (T(2) * eta * (T(2) * eyy + exx));
        }
        int fi = i0 + a, fj = j0 + b;           // corner
        if (fi <= g.Nx && fj <= g.Ny) {
            T dudy = (sm.pm[b + 1][a + 1].x - sm.pm[b][a + 1].x) * g.rdyf[fj];
            T dvdx = (sm.pm[b + 1][a + 1].y - sm.pm[b + 1][a].y) * g.rdxf[fi];
            T e = (dudy + dvdx) / T(2);
            if (g.peripheral_ff(fi, fj)) e = o.wall_factor * e;
            sm.txy[b][a] = T(2) * o.coef[g.ff_idx(fi, fj)].y * e;
        }
    }
    __syncthreads();
    V2 q;
    q.x = T(0);
    q.y = T(0);
    if (!inside) return q;
    int tx = threadIdx.x, ty = threadIdx.y;
    int k = g.idx(i, j);
    V2 pc = p[k];
    uint8_t m = __ldg(o.mask + k);
    auto c = o.coef[k];
    T divu = (sm.sxx[ty + 1][tx + 1] - sm.sxx[ty + 1][tx]) + (g.dxf[i] * sm.txy[ty + 1][tx] - g.dxf[i] * sm.txy[ty][tx]);
    T divv = (sm.syy[ty + 1][tx + 1] - sm.syy[ty][tx + 1]) + (g.dyf[j] * sm.txy[ty][tx + 1] - g.dyf[j] * sm.txy[ty][tx]);
    q.x = (m & U_IDENTITY) ? pc.x : g.Az_fc(i, j) * c.z * pc.x - divu;
    q.y = (m & V_IDENTITY) ? pc.y : g.Az_cf(i, j) * c.w * pc.y - divv;
    return q;
}

}  // namespace nk
