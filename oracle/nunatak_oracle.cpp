// nunatak_oracle.cpp — TEST INFRASTRUCTURE ONLY.
//
// A plain FP64 CPU restatement of Nunatak.jl's velocity solve (Picard iteration around preconditioned
// conjugate gradients for the SSA / DIVA stress balance on the C grid).  It is the checker of the GPU
// library: only the tests, the smoke check and the CPU-baseline leg of the benchmark load it.  It is
// never linked into, or called by, libnunatak_gb300.so.
//
// Every function names the reference file:line it restates.  The reference runs on Oceananigans fields
// with halos; this file keeps that representation (fields with halo cells, fill_halo_regions! with
// periodic wrap and zero-gradient copies for cell-centred data in Bounded directions) so that the
// index semantics are the reference's, not the GPU library's clamped / wrapped indexing.
//
// Floating-point expressions keep the reference's evaluation order (left-associative sums and
// products as written in the Julia source).  Build with -ffp-contract=off so that no multiply-add is
// fused and the results are the same on x86-64 and aarch64.
//
// Oceananigans conventions restated here (Oceananigans is not vendored in the reference):
//   face i is the west face of centre i; Bounded faces run 1..N+1, Periodic faces 1..N;
//   δxᶠ f(i) = f(i) - f(i-1), δxᶜ f(i) = f(i+1) - f(i); ℑxᶠ f(i) = (f(i-1) + f(i)) / 2,
//   ℑxᶜ f(i) = (f(i) + f(i+1)) / 2; two-dimensional interpolations interpolate in x, then in y;
//   Δxᶜ(i) = xᶠ(i+1) - xᶠ(i) (cell width), Δxᶠ(i) = xᶜ(i) - xᶜ(i-1) (centre spacing); Az = Δx Δy at
//   the location; regular grids use the single spacing L/N for both;
//   a cell is inactive outside 1..N in a Bounded direction; a Face point is peripheral when either
//   neighbouring cell is inactive, a Face-Face corner when any of its four cells is.
#include "../include/nunatak_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

enum Loc { CENTER = 0, FACE = 1 };

// ------------------------------------------------------------------------------------------------
// Grid: one axis of a RectilinearGrid (Oceananigans generate_coordinate), with halo nodes.
// ------------------------------------------------------------------------------------------------
struct Axis {
    int N = 0, H = 0;
    bool periodic = false;
    bool regular = true;
    double delta = 0;
    int lo = 0;                        // lowest stored index (1 - H - 1)
    std::vector<double> F, C, dC, dF;  // faces, centres, cell widths Δᶜ, centre spacings Δᶠ

    int at(int i) const { return i - lo; }
    double face(int i) const { return F[at(i)]; }
    double center(int i) const { return C[at(i)]; }
    double dc(int i) const { return regular ? delta : dC[at(i)]; }
    double df(int i) const { return regular ? delta : dF[at(i)]; }

    void build_regular(int n, int h, bool per, double x0, double L) {
        N = n; H = h; periodic = per; regular = true; delta = L / n;
        lo = -H - 1;
        int count = N + 2 * H + 4;
        F.assign(count, 0); C.assign(count, 0); dC.assign(count, delta); dF.assign(count, delta);
        for (int i = lo; i < lo + count; ++i) {
            F[at(i)] = x0 + ((i - 1) * L) / N;
            C[at(i)] = x0 + ((i - 1) * L) / N + delta / 2;
        }
    }

    // Vector of N+1 interior faces: halo faces extend the edge spacing (Bounded) or wrap (Periodic).
    void build_faces(int n, int h, bool per, const double* faces) {
        N = n; H = h; periodic = per; regular = false; delta = 0;
        lo = -H - 1;
        int count = N + 2 * H + 4;
        F.assign(count, 0); C.assign(count, 0); dC.assign(count, 0); dF.assign(count, 0);
        for (int i = 1; i <= N + 1; ++i) F[at(i)] = faces[i - 1];
        if (per) {
            double L = faces[N] - faces[0];
            for (int m = 1; at(1 - m) >= 0; ++m) F[at(1 - m)] = F[at(N + 1 - m)] - L;
            for (int m = 1; at(N + 1 + m) < count; ++m) F[at(N + 1 + m)] = F[at(1 + m)] + L;
        } else {
            double dm = faces[1] - faces[0], dp = faces[N] - faces[N - 1];
            for (int m = 1; at(1 - m) >= 0; ++m) F[at(1 - m)] = faces[0] - m * dm;
            for (int m = 1; at(N + 1 + m) < count; ++m) F[at(N + 1 + m)] = faces[N] + m * dp;
        }
        for (int i = lo; i < lo + count - 1; ++i) {
            C[at(i)] = (F[at(i + 1)] + F[at(i)]) / 2;
            dC[at(i)] = F[at(i + 1)] - F[at(i)];
        }
        for (int i = lo + 1; i < lo + count - 1; ++i) dF[at(i)] = C[at(i)] - C[at(i - 1)];
    }

    // Number of interior points of a field located at `loc` along this axis.
    int size(Loc loc) const { return (loc == FACE && !periodic) ? N + 1 : N; }
    bool inactive_cell(int i) const { return !periodic && (i < 1 || i > N); }
};

struct Field;

struct Grid {
    Axis x, y;
    // Prescribed velocities (the extension for an inflow; the reference has no velocity boundary condition):
    // u_D at Face-Center, v_D at Center-Face, NaN where free.  Null on the coarse multigrid levels.
    const Field* pu = nullptr;
    const Field* pv = nullptr;
    int Nx() const { return x.N; }
    int Ny() const { return y.N; }
    bool inactive_cell(int i, int j) const { return x.inactive_cell(i) || y.inactive_cell(j); }
    // peripheral_node(i, j, k, grid, Face, Center, Center) and friends (Oceananigans Grids/inactive_node.jl)
    bool peripheral_fc(int i, int j) const { return inactive_cell(i, j) || inactive_cell(i - 1, j); }
    bool peripheral_cf(int i, int j) const { return inactive_cell(i, j) || inactive_cell(i, j - 1); }
    bool peripheral_ff(int i, int j) const {
        return inactive_cell(i, j) || inactive_cell(i - 1, j) || inactive_cell(i, j - 1) || inactive_cell(i - 1, j - 1);
    }
    // Metrics (Oceananigans Operators/spacings_and_areas_and_volumes.jl on a RectilinearGrid).
    double dx_c(int i) const { return x.dc(i); }   // Δxᶜᶜᶜ, Δxᶜᶠᶜ
    double dx_f(int i) const { return x.df(i); }   // Δxᶠᶜᶜ, Δxᶠᶠᶜ
    double dy_c(int j) const { return y.dc(j); }   // Δyᶜᶜᶜ, Δyᶠᶜᶜ
    double dy_f(int j) const { return y.df(j); }   // Δyᶜᶠᶜ, Δyᶠᶠᶜ
    double Az_ccc(int i, int j) const { return dx_c(i) * dy_c(j); }
    double Az_fcc(int i, int j) const { return dx_f(i) * dy_c(j); }
    double Az_cfc(int i, int j) const { return dx_c(i) * dy_f(j); }
};

// ------------------------------------------------------------------------------------------------
// Field: two-dimensional Oceananigans Field at (lx, ly) with halos.
// ------------------------------------------------------------------------------------------------
struct Field {
    Loc lx = CENTER, ly = CENTER;
    const Grid* g = nullptr;
    int ox = 0, oy = 0, sx = 0, sy = 0;
    std::vector<double> d;
    Field() = default;
    Field(const Grid* grid, Loc lx_, Loc ly_) { init(grid, lx_, ly_); }
    void init(const Grid* grid, Loc lx_, Loc ly_) {
        g = grid; lx = lx_; ly = ly_;
        ox = grid->x.H + 2; oy = grid->y.H + 2;
        sx = grid->x.N + 2 * grid->x.H + 5; sy = grid->y.N + 2 * grid->y.H + 5;
        d.assign((size_t)sx * sy, 0.0);
    }
    double& operator()(int i, int j) { return d[(size_t)(j + oy) * sx + (i + ox)]; }
    double operator()(int i, int j) const { return d[(size_t)(j + oy) * sx + (i + ox)]; }
    int nx() const { return g->x.size(lx); }
    int ny() const { return g->y.size(ly); }
    void zero() { std::fill(d.begin(), d.end(), 0.0); }
};

// fill_halo_regions! with default boundary conditions: Periodic wraps; in a Bounded direction a
// Center location copies the edge value (zero flux), a Face location is left as it is (its boundary
// values are interior points and its halo is never read unmasked by the velocity solve).
static void fill_halo(Field& f) {
    const Grid& g = *f.g;
    int Hx = g.x.H + 1, Hy = g.y.H + 1;
    int Nx = g.x.N, Ny = g.y.N;
    int nyi = f.ny();
    for (int j = 1; j <= nyi; ++j) {
        if (g.x.periodic) {
            for (int m = 1; m <= Hx; ++m) { f(1 - m, j) = f(Nx + 1 - m, j); f(Nx + m, j) = f(m, j); }
        } else if (f.lx == CENTER) {
            for (int m = 1; m <= Hx; ++m) { f(1 - m, j) = f(1, j); f(Nx + m, j) = f(Nx, j); }
        }
    }
    for (int i = -Hx; i <= Nx + 1 + Hx - 1; ++i) {
        if (g.y.periodic) {
            for (int m = 1; m <= Hy; ++m) { f(i, 1 - m) = f(i, Ny + 1 - m); f(i, Ny + m) = f(i, m); }
        } else if (f.ly == CENTER) {
            for (int m = 1; m <= Hy; ++m) { f(i, 1 - m) = f(i, 1); f(i, Ny + m) = f(i, Ny); }
        }
    }
}

// Field on the sigma grid: Nσ horizontal layers (Center in z).
struct SigmaField {
    std::vector<Field> k;
    void init(const Grid* g, Loc lx, Loc ly, int Ns) { k.assign(Ns, Field(g, lx, ly)); }
};

struct VelocityVector {        // src/Solvers/velocity_vector.jl:10-33
    Field u, v;
    void init(const Grid* g) { u.init(g, FACE, CENTER); v.init(g, CENTER, FACE); }
};

static void fill_halo(VelocityVector& x) { fill_halo(x.u); fill_halo(x.v); }

template <class F>
static void for_xy(int Nx, int Ny, F&& f) {   // launch!(arch, grid, :xyz, ...) over 1..Nx x 1..Ny
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= Ny; ++j)
        for (int i = 1; i <= Nx; ++i) f(i, j);
}

// ------------------------------------------------------------------------------------------------
// Masks and strain rates, src/StressBalances/strain_rates.jl:1-32 and
// src/Models/smooth_ice_mask.jl:72-75.  `eta` is η̄H (operator) or nullptr (`nothing`).
// ------------------------------------------------------------------------------------------------
static inline bool ice_free_fc(int i, int j, const Field* mu) { return mu && ((*mu)(i - 1, j) + (*mu)(i, j)) == 0.0; }   // smooth_ice_mask.jl:72
static inline bool ice_free_cf(int i, int j, const Field* mu) { return mu && ((*mu)(i, j - 1) + (*mu)(i, j)) == 0.0; }   // smooth_ice_mask.jl:73
// A prescribed face: one of the solved rows (i, j in 1..Nx x 1..Ny, wrapped when periodic: the west / south
// boundary faces and the interior faces) whose prescribed value is finite.  Its row is an identity row
// (inactive) and its value still enters the strain rates (interior_u / interior_v pass it).
static inline bool prescribed(const Grid& g, const Field* d, int i, int j) {
    if (!d || (!g.x.periodic && (i < 1 || i > g.Nx())) || (!g.y.periodic && (j < 1 || j > g.Ny()))) return false;
    return !std::isnan((*d)(i, j));   // periodic halos hold the wrapped values
}
static inline bool prescribed_fc(const Grid& g, int i, int j) { return prescribed(g, g.pu, i, j); }
static inline bool prescribed_cf(const Grid& g, int i, int j) { return prescribed(g, g.pv, i, j); }
static inline bool inactive_fc(const Grid& g, int i, int j, const Field* eta) {   // strain_rates.jl:2 (+ prescribed)
    return g.peripheral_fc(i, j) || ice_free_fc(i, j, eta) || prescribed_fc(g, i, j);
}
static inline bool inactive_cf(const Grid& g, int i, int j, const Field* eta) {   // strain_rates.jl:3 (+ prescribed)
    return g.peripheral_cf(i, j) || ice_free_cf(i, j, eta) || prescribed_cf(g, i, j);
}
static inline double interior_u(const Grid& g, int i, int j, const Field& u, const Field* eta) {   // strain_rates.jl:5
    return (inactive_fc(g, i, j, eta) && !prescribed_fc(g, i, j)) ? 0.0 : u(i, j);
}
static inline double interior_v(const Grid& g, int i, int j, const Field& v, const Field* eta) {   // strain_rates.jl:6
    return (inactive_cf(g, i, j, eta) && !prescribed_cf(g, i, j)) ? 0.0 : v(i, j);
}

static inline double strain_rate_xx(const Grid& g, int i, int j, const Field& u, const Field* eta) {   // strain_rates.jl:8
    return (interior_u(g, i + 1, j, u, eta) - interior_u(g, i, j, u, eta)) / g.dx_c(i);
}
static inline double strain_rate_yy(const Grid& g, int i, int j, const Field& v, const Field* eta) {   // strain_rates.jl:9
    return (interior_v(g, i, j + 1, v, eta) - interior_v(g, i, j, v, eta)) / g.dy_c(j);
}
static inline double wall_shear_factor(int walls) { return walls == NK_NO_SLIP ? 2.0 : 0.0; }         // strain_rates.jl:11-12
static inline double strain_rate_xy(const Grid& g, int i, int j, const Field& u, const Field& v, int walls, const Field* eta) {  // strain_rates.jl:14-17
    double dudy = (interior_u(g, i, j, u, eta) - interior_u(g, i, j - 1, u, eta)) / g.dy_f(j);
    double dvdx = (interior_v(g, i, j, v, eta) - interior_v(g, i - 1, j, v, eta)) / g.dx_f(i);
    double e = (dudy + dvdx) / 2;
    return g.peripheral_ff(i, j) ? wall_shear_factor(walls) * e : e;
}
static inline double strain_rate_xy2(const Grid& g, int i, int j, const Field& u, const Field& v, int walls) {  // strain_rates.jl:19
    double e = strain_rate_xy(g, i, j, u, v, walls, nullptr);
    return e * e;
}
// effective_strain_rate², strain_rates.jl:27-32; ℑxyᶜᶜᵃ = ℑyᵃᶜᵃ(ℑxᶜᵃᵃ(·))
static inline double effective_strain_rate2(const Grid& g, int i, int j, const Field& u, const Field& v, int walls) {
    double exx = strain_rate_xx(g, i, j, u, nullptr);
    double eyy = strain_rate_yy(g, i, j, v, nullptr);
    double a = (strain_rate_xy2(g, i, j, u, v, walls) + strain_rate_xy2(g, i + 1, j, u, v, walls)) / 2;
    double b = (strain_rate_xy2(g, i, j + 1, u, v, walls) + strain_rate_xy2(g, i + 1, j + 1, u, v, walls)) / 2;
    double exy2 = (a + b) / 2;
    return exx * exx + eyy * eyy + exx * eyy + exy2;
}

// ------------------------------------------------------------------------------------------------
// SSA operator, src/StressBalances/ssa_operator.jl:47-89.
// ------------------------------------------------------------------------------------------------
struct Coefficients {   // the (η̄H, η̄Hᶠᶠ, βᵘ, βᵛ) prefix of the coefficient tuple
    Field* etaH; Field* etaHff; Field* bu; Field* bv;
};

static inline double normal_stress_xx(const Grid& g, int i, int j, const Field& u, const Field& v, const Field& eta) {  // :60
    return 2 * eta(i, j) * (2 * strain_rate_xx(g, i, j, u, &eta) + strain_rate_yy(g, i, j, v, &eta));
}
static inline double normal_stress_yy(const Grid& g, int i, int j, const Field& u, const Field& v, const Field& eta) {  // :61
    return 2 * eta(i, j) * (2 * strain_rate_yy(g, i, j, v, &eta) + strain_rate_xx(g, i, j, u, &eta));
}
static inline double shear_stress(const Grid& g, int i, int j, const Field& u, const Field& v, const Field& etaff, int walls, const Field& eta) {  // :62
    return 2 * etaff(i, j) * strain_rate_xy(g, i, j, u, v, walls, &eta);
}
// The halos of p, η̄H and η̄Hᶠᶠ must be filled.  ssa_operator.jl:47-89 evaluates every stress of a row from the
// masked velocities (interior_u / interior_v with η̄H).  Here the masked velocities are taken once per point and
// each stress once per centre or corner, by the same expressions on the same values, and the rows read them: the
// results (and bits) are those of the per-row evaluation.  Txx at centres 0..Nx x 1..Ny, Tyy at 1..Nx x 0..Ny,
// Txy at corners 1..Nx+1 x 1..Ny+1; the masked velocities at the points those read.
static void ssa_operator(const Grid& g, VelocityVector& q, const VelocityVector& p, const Coefficients& c, int walls) {  // :47-52, :81-89
    const int Nx = g.Nx(), Ny = g.Ny(), sx = Nx + 3;
    const size_t n = (size_t)sx * (Ny + 3);
    static thread_local std::vector<double> scratch;   // grown once, so repeated applies touch no new pages
    if (scratch.size() < 5 * n) scratch.resize(5 * n);
    double *mu = scratch.data(), *mv = mu + n, *txx = mv + n, *tyy = txx + n, *txy = tyy + n;
    auto at = [sx](int i, int j) { return (size_t)(j + 1) * sx + (i + 1); };   // i, j from -1
    const Field &eta = *c.etaH, &ff = *c.etaHff;
#pragma omp parallel for schedule(static)
    for (int j = -1; j <= Ny + 1; ++j)
        for (int i = -1; i <= Nx + 1; ++i) {
            mu[at(i, j)] = interior_u(g, i, j, p.u, &eta);
            mv[at(i, j)] = interior_v(g, i, j, p.v, &eta);
        }
    const double wf = wall_shear_factor(walls);
#pragma omp parallel for schedule(static)
    for (int j = 0; j <= Ny + 1; ++j)
        for (int i = 0; i <= Nx + 1; ++i) {
            if (i <= Nx && j <= Ny) {
                double exx = (mu[at(i + 1, j)] - mu[at(i, j)]) / g.dx_c(i);   // strain_rate_xx
                double eyy = (mv[at(i, j + 1)] - mv[at(i, j)]) / g.dy_c(j);   // strain_rate_yy
                txx[at(i, j)] = 2 * eta(i, j) * (2 * exx + eyy);               // normal_stress_xx, :60
                tyy[at(i, j)] = 2 * eta(i, j) * (2 * eyy + exx);               // normal_stress_yy, :61
            }
            if (i >= 1 && j >= 1) {                                            // shear_stress, :62; strain_rate_xy
                double dudy = (mu[at(i, j)] - mu[at(i, j - 1)]) / g.dy_f(j);
                double dvdx = (mv[at(i, j)] - mv[at(i - 1, j)]) / g.dx_f(i);
                double e = (dudy + dvdx) / 2;
                txy[at(i, j)] = 2 * ff(i, j) * (g.peripheral_ff(i, j) ? wf * e : e);
            }
        }
    for_xy(Nx, Ny, [&](int i, int j) {
        bool wu = inactive_fc(g, i, j, c.etaH), wv = inactive_cf(g, i, j, c.etaH);
        if (wu) {
            q.u(i, j) = p.u(i, j);
        } else {   // x_stress_balance, :69-73
            double div = (g.dy_c(j) * txx[at(i, j)] - g.dy_c(j) * txx[at(i - 1, j)]) +
                         (g.dx_f(i) * txy[at(i, j + 1)] - g.dx_f(i) * txy[at(i, j)]);
            q.u(i, j) = g.Az_fcc(i, j) * (*c.bu)(i, j) * p.u(i, j) - div;
        }
        if (wv) {
            q.v(i, j) = p.v(i, j);
        } else {   // y_stress_balance, :75-79
            double div = (g.dx_c(i) * tyy[at(i, j)] - g.dx_c(i) * tyy[at(i, j - 1)]) +
                         (g.dy_f(j) * txy[at(i + 1, j)] - g.dy_f(j) * txy[at(i, j)]);
            q.v(i, j) = g.Az_cfc(i, j) * (*c.bv)(i, j) * p.v(i, j) - div;
        }
    });
}

// ------------------------------------------------------------------------------------------------
// Diagonal preconditioner, src/StressBalances/diagonal_preconditioner.jl:9-54.
// ------------------------------------------------------------------------------------------------
static inline double x_normal_diagonal(const Grid& g, int i, int j, const Field& eta) { return 4 * g.dy_c(j) * eta(i, j) / g.dx_c(i); }  // :20
static inline double y_normal_diagonal(const Grid& g, int i, int j, const Field& eta) { return 4 * g.dx_c(i) * eta(i, j) / g.dy_c(j); }  // :21
static inline double corner_shear_factor(const Grid& g, int i, int j, int walls) { return g.peripheral_ff(i, j) ? wall_shear_factor(walls) : 1.0; }  // :25
static inline double x_shear_diagonal(const Grid& g, int i, int j, const Field& ff, int walls) {   // :27-28
    return corner_shear_factor(g, i, j, walls) * g.dx_f(i) * ff(i, j) / g.dy_f(j);
}
static inline double y_shear_diagonal(const Grid& g, int i, int j, const Field& ff, int walls) {   // :29-30
    return corner_shear_factor(g, i, j, walls) * g.dy_f(j) * ff(i, j) / g.dx_f(i);
}
static inline double x_diagonal(const Grid& g, int i, int j, const Coefficients& c, int walls) {   // :32-37
    double d = g.Az_fcc(i, j) * (*c.bu)(i, j) + x_normal_diagonal(g, i, j, *c.etaH) + x_normal_diagonal(g, i - 1, j, *c.etaH) +
               x_shear_diagonal(g, i, j, *c.etaHff, walls) + x_shear_diagonal(g, i, j + 1, *c.etaHff, walls);
    return (inactive_fc(g, i, j, c.etaH) || d == 0.0) ? 1.0 : d;
}
static inline double y_diagonal(const Grid& g, int i, int j, const Coefficients& c, int walls) {   // :39-44
    double d = g.Az_cfc(i, j) * (*c.bv)(i, j) + y_normal_diagonal(g, i, j, *c.etaH) + y_normal_diagonal(g, i, j - 1, *c.etaH) +
               y_shear_diagonal(g, i, j, *c.etaHff, walls) + y_shear_diagonal(g, i + 1, j, *c.etaHff, walls);
    return (inactive_cf(g, i, j, c.etaH) || d == 0.0) ? 1.0 : d;
}

// ------------------------------------------------------------------------------------------------
// Vector operations, src/Solvers/velocity_vector.jl:48-141.  All act on the Nx x Ny range.
// ------------------------------------------------------------------------------------------------
static void linear_combination(const Grid& g, VelocityVector& z, double a, const VelocityVector& x, double b, const VelocityVector& y) {  // :48-62
    for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
        z.u(i, j) = a * x.u(i, j) + b * y.u(i, j);
        z.v(i, j) = a * x.v(i, j) + b * y.v(i, j);
    });
}
static void copyto(const Grid& g, VelocityVector& x, const VelocityVector& y) { linear_combination(g, x, 1.0, y, 0.0, y); }  // :69
static void axpy(const Grid& g, double a, const VelocityVector& y, VelocityVector& x) { linear_combination(g, x, 1.0, x, a, y); }  // :82
static void xpby(const Grid& g, const VelocityVector& y, double b, VelocityVector& x) { linear_combination(g, x, 1.0, y, b, x); }  // :89
static void subtract(const Grid& g, VelocityVector& r, const VelocityVector& b, const VelocityVector& q) { linear_combination(g, r, 1.0, b, -1.0, q); }  // :96
static void fill_interior(VelocityVector& x, double value) {   // :71-75 (interior includes wall faces)
    for (int j = 1; j <= x.u.ny(); ++j) for (int i = 1; i <= x.u.nx(); ++i) x.u(i, j) = value;
    for (int j = 1; j <= x.v.ny(); ++j) for (int i = 1; i <= x.v.nx(); ++i) x.v(i, j) = value;
}

// Dot product over the Nx x Ny range of each component, vector_dot! :125-133.  Rows are summed in
// order of increasing i, then rows in order of increasing j, so the result does not depend on the
// thread count.  (Julia's pairwise `sum` over the parent array differs only in rounding.)
static double component_dot(const Grid& g, const Field& x, const Field& y) {
    int Nx = g.Nx(), Ny = g.Ny();
    std::vector<double> rows(Ny + 1, 0.0);
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= Ny; ++j) {
        double s = 0;
        for (int i = 1; i <= Nx; ++i) s += x(i, j) * y(i, j);
        rows[j] = s;
    }
    double s = 0;
    for (int j = 1; j <= Ny; ++j) s += rows[j];
    return s;
}
static double vector_dot(const Grid& g, const VelocityVector& x, const VelocityVector& y) {
    return component_dot(g, x.u, y.u) + component_dot(g, x.v, y.v);
}

// ------------------------------------------------------------------------------------------------
// Multigrid, src/StressBalances/multigrid_preconditioner.jl.
// ------------------------------------------------------------------------------------------------
enum Coarsening { UNCHANGED = 1, HALVED = 2 };

static Coarsening coarsening(int N, int H, int minimum) {   // :86
    return ((N % 2 == 0) && (N / 2 >= std::max(minimum, H))) ? HALVED : UNCHANGED;
}

struct Level {   // :98-107
    std::unique_ptr<Grid> grid;
    Coarsening cx, cy;
    Field etaH, etaHff, bu, bv, scratch;
    VelocityVector x, b, q;
    std::vector<double> line_t;   // unused: the line solver keeps t in `scratch`
};

static std::unique_ptr<Grid> coarsened_grid(const Grid& g, Coarsening cx, Coarsening cy) {   // :111-120
    auto c = std::make_unique<Grid>();
    int fx = cx, fy = cy;
    std::vector<double> xf, yf;
    for (int i = 1; i <= g.x.N + 1; i += fx) xf.push_back(g.x.face(i));
    for (int j = 1; j <= g.y.N + 1; j += fy) yf.push_back(g.y.face(j));
    c->x.build_faces(g.x.N / fx, g.x.H, g.x.periodic, xf.data());
    c->y.build_faces(g.y.N / fy, g.y.H, g.y.periodic, yf.data());
    return c;
}

static void coarse_levels(const Grid& g, int minimum, std::vector<std::unique_ptr<Level>>& out) {   // :88-109
    Coarsening cx = coarsening(g.x.N, g.x.H, minimum), cy = coarsening(g.y.N, g.y.H, minimum);
    if (cx == UNCHANGED && cy == UNCHANGED) return;
    auto L = std::make_unique<Level>();
    L->grid = coarsened_grid(g, cx, cy);
    L->cx = cx; L->cy = cy;
    const Grid* cg = L->grid.get();
    L->etaH.init(cg, CENTER, CENTER); L->etaHff.init(cg, FACE, FACE);
    L->bu.init(cg, FACE, CENTER); L->bv.init(cg, CENTER, FACE);
    L->scratch.init(cg, CENTER, CENTER);
    L->x.init(cg); L->b.init(cg); L->q.init(cg);
    const Grid& next = *cg;
    out.push_back(std::move(L));
    coarse_levels(next, minimum, out);
}

// restriction_offsets / restriction_index / restriction_weight, :264-283
static inline void restriction_offsets(Loc l, Coarsening c, int& a0, int& a1) {
    if (c == UNCHANGED) { a0 = 0; a1 = 0; } else if (l == FACE) { a0 = -1; a1 = 1; } else { a0 = -1; a1 = 2; }
}
static inline int mod1(int x, int N) { int r = (x - 1) % N; if (r < 0) r += N; return r + 1; }
static inline int restriction_index(int I, int a, int N, bool periodic, Loc l, Coarsening c) {
    if (c == UNCHANGED) return I;
    if (periodic) return mod1(2 * I - 1 + a, N);
    if (l == FACE) return std::max(2 * I - 1 + a, 1);
    return std::min(std::max(2 * I - 1 + a, 1), N);
}
static inline double restriction_weight(int I, int a, int Nc, bool periodic, Loc l, Coarsening c) {
    if (c == UNCHANGED) return 1.0;
    if (l == FACE) {
        double w = (a == 0) ? 1.0 : 1.0 / 2;
        if (!periodic && 2 * I - 1 + a < 1) return 0.0;
        return w;
    }
    double w = (a == 0 || a == 1) ? 3.0 / 4 : 1.0 / 4;
    if (periodic) return w;
    bool outside = (I == 1 && a == -1) || (I == Nc && a == 2);
    bool folded = (I == 1 && a == 0) || (I == Nc && a == 1);
    w = w + (folded ? 1.0 / 4 : 0.0);
    return outside ? 0.0 : w;
}
// parents, :286-305
static inline void parents(int i, int Nc, bool periodic, Loc l, Coarsening c, int& I1, int& I2, double& w1, double& w2) {
    if (c == UNCHANGED) { I1 = i; I2 = i; w1 = 1.0; w2 = 0.0; return; }
    int I = (i + 1) / 2;
    bool odd = (i % 2) != 0;
    if (l == FACE) {
        int up = periodic ? mod1(I + 1, Nc) : I + 1;
        I1 = I; I2 = odd ? I : up; w1 = odd ? 1.0 : 1.0 / 2; w2 = odd ? 0.0 : 1.0 / 2;
    } else {
        int Ip = odd ? I - 1 : I + 1;
        I1 = I; I2 = periodic ? mod1(Ip, Nc) : std::min(std::max(Ip, 1), Nc); w1 = 3.0 / 4; w2 = 1.0 / 4;
    }
}

// restrict(I, J, k, ℓx, ℓy, cx, cy, coarse_grid, fine_grid, ϕ, args...), :307-318
template <class Phi>
static double restrict_point(int I, int J, Loc lx, Loc ly, Coarsening cx, Coarsening cy, const Grid& coarse, const Grid& fine, Phi&& phi) {
    int a0, a1, b0, b1;
    restriction_offsets(lx, cx, a0, a1);
    restriction_offsets(ly, cy, b0, b1);
    double s = 0;
    for (int a = a0; a <= a1; ++a)
        for (int b = b0; b <= b1; ++b) {
            int i = restriction_index(I, a, fine.x.N, fine.x.periodic, lx, cx);
            int j = restriction_index(J, b, fine.y.N, fine.y.periodic, ly, cy);
            double w = restriction_weight(I, a, coarse.x.N, fine.x.periodic, lx, cx) * restriction_weight(J, b, coarse.y.N, fine.y.periodic, ly, cy);
            s += w * phi(i, j);
        }
    return s;
}
// prolongate(i, j, k, ℓx, ℓy, cx, cy, fine_grid, coarse_grid, ϕ, args...), :320-327
template <class Phi>
static double prolongate_point(int i, int j, Loc lx, Loc ly, Coarsening cx, Coarsening cy, const Grid& fine, const Grid& coarse, Phi&& phi) {
    int I1, I2, J1, J2; double wx1, wx2, wy1, wy2;
    parents(i, coarse.x.N, fine.x.periodic, lx, cx, I1, I2, wx1, wx2);
    parents(j, coarse.y.N, fine.y.periodic, ly, cy, J1, J2, wy1, wy2);
    return wx1 * (wy1 * phi(I1, J1) + wy2 * phi(I1, J2)) + wx2 * (wy1 * phi(I2, J1) + wy2 * phi(I2, J2));
}

// ℑxyᶠᶠᵃ(η̄H) over size(η̄Hᶠᶠ), _interpolate_to_corners!, src/StressBalances/stress_balance_coefficients.jl:26-29
static void interpolate_to_corners(const Grid& g, Field& ff, const Field& eta) {
    int nx = ff.nx(), ny = ff.ny();
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ny; ++j)
        for (int i = 1; i <= nx; ++i) {
            double lo = (eta(i - 1, j - 1) + eta(i, j - 1)) / 2;
            double hi = (eta(i - 1, j) + eta(i, j)) / 2;
            ff(i, j) = (lo + hi) / 2;
        }
    (void)g;
}

// _coarsen_coefficients!, :331-344, and coarsen_coefficients!, :130-141
static void coarsen_coefficients(std::vector<std::unique_ptr<Level>>& levels, size_t l, const Field& eta, const Field& bu, const Field& bv) {
    if (l >= levels.size()) return;
    Level& L = *levels[l];
    const Grid& cg = *L.grid;
    const Grid& fg = *eta.g;
    int fx = L.cx, fy = L.cy;
    for_xy(cg.Nx(), cg.Ny(), [&](int I, int J) {
        int i = fx * (I - 1) + 1, j = fy * (J - 1) + 1;
        double S = 0;
        for (int a = 0; a <= fx - 1; ++a)
            for (int b = 0; b <= fy - 1; ++b) S += fg.Az_ccc(i + a, j + b) * eta(i + a, j + b);
        L.etaH(I, J) = S / cg.Az_ccc(I, J);
        L.bu(I, J) = restrict_point(I, J, FACE, CENTER, L.cx, L.cy, cg, fg, [&](int ii, int jj) { return fg.Az_fcc(ii, jj) * bu(ii, jj); }) / cg.Az_fcc(I, J);
        L.bv(I, J) = restrict_point(I, J, CENTER, FACE, L.cx, L.cy, cg, fg, [&](int ii, int jj) { return fg.Az_cfc(ii, jj) * bv(ii, jj); }) / cg.Az_cfc(I, J);
    });
    fill_halo(L.etaH);
    interpolate_to_corners(cg, L.etaHff, L.etaH);
    fill_halo(L.etaHff);
    fill_halo(L.bu); fill_halo(L.bv);
    coarsen_coefficients(levels, l + 1, L.etaH, L.bu, L.bv);
}

// _restrict!, :346-352
static void restrict_vector(const Grid& cg, const Grid& fg, Level& L, VelocityVector& coarse, const VelocityVector& fine, const Field& coarse_eta, const Field& fine_eta) {
    for_xy(cg.Nx(), cg.Ny(), [&](int I, int J) {
        coarse.u(I, J) = inactive_fc(cg, I, J, &coarse_eta) ? 0.0 :
            restrict_point(I, J, FACE, CENTER, L.cx, L.cy, cg, fg, [&](int i, int j) { return interior_u(fg, i, j, fine.u, &fine_eta); });
        coarse.v(I, J) = inactive_cf(cg, I, J, &coarse_eta) ? 0.0 :
            restrict_point(I, J, CENTER, FACE, L.cx, L.cy, cg, fg, [&](int i, int j) { return interior_v(fg, i, j, fine.v, &fine_eta); });
    });
}
// _prolongate!, :354-360
static void prolongate_vector(const Grid& fg, const Grid& cg, Level& L, VelocityVector& fine, const VelocityVector& coarse, const Field& fine_eta, const Field& coarse_eta) {
    for_xy(fg.Nx(), fg.Ny(), [&](int i, int j) {
        fine.u(i, j) += inactive_fc(fg, i, j, &fine_eta) ? 0.0 :
            prolongate_point(i, j, FACE, CENTER, L.cx, L.cy, fg, cg, [&](int I, int J) { return interior_u(cg, I, J, coarse.u, &coarse_eta); });
        fine.v(i, j) += inactive_cf(fg, i, j, &fine_eta) ? 0.0 :
            prolongate_point(i, j, CENTER, FACE, L.cx, L.cy, fg, cg, [&](int I, int J) { return interior_v(cg, I, J, coarse.v, &coarse_eta); });
    });
}

// ℓ1-Jacobi row sums, :195-211
static inline double x_absolute_row_sum(const Grid& g, int i, int j, const Coefficients& c, int walls) {
    const Field& eta = *c.etaH; const Field& ff = *c.etaHff;
    double s = g.Az_fcc(i, j) * (*c.bu)(i, j) +
               2 * (x_normal_diagonal(g, i, j, eta) + x_normal_diagonal(g, i - 1, j, eta)) +
               4 * (eta(i, j) + eta(i - 1, j)) +
               2 * (x_shear_diagonal(g, i, j, ff, walls) + x_shear_diagonal(g, i, j + 1, ff, walls)) +
               2 * (corner_shear_factor(g, i, j, walls) * ff(i, j) + corner_shear_factor(g, i, j + 1, walls) * ff(i, j + 1));
    return (inactive_fc(g, i, j, &eta) || s == 0.0) ? 1.0 : s;
}
static inline double y_absolute_row_sum(const Grid& g, int i, int j, const Coefficients& c, int walls) {
    const Field& eta = *c.etaH; const Field& ff = *c.etaHff;
    double s = g.Az_cfc(i, j) * (*c.bv)(i, j) +
               2 * (y_normal_diagonal(g, i, j, eta) + y_normal_diagonal(g, i, j - 1, eta)) +
               4 * (eta(i, j) + eta(i, j - 1)) +
               2 * (y_shear_diagonal(g, i, j, ff, walls) + y_shear_diagonal(g, i + 1, j, ff, walls)) +
               2 * (corner_shear_factor(g, i, j, walls) * ff(i, j) + corner_shear_factor(g, i + 1, j, walls) * ff(i + 1, j));
    return (inactive_cf(g, i, j, &eta) || s == 0.0) ? 1.0 : s;
}
// y-line couplings, :223-227
static inline double x_line_coupling(const Grid& g, int i, int j, const Coefficients& c, int walls) {
    return (inactive_fc(g, i, j - 1, c.etaH) || inactive_fc(g, i, j, c.etaH)) ? 0.0 : x_shear_diagonal(g, i, j, *c.etaHff, walls);
}
static inline double y_line_coupling(const Grid& g, int i, int j, const Coefficients& c, int walls) {
    return (inactive_cf(g, i, j - 1, c.etaH) || inactive_cf(g, i, j, c.etaH)) ? 0.0 : y_normal_diagonal(g, i, j - 1, *c.etaH);
}

// line_relax!, :231-253 (Thomas algorithm along j with M = tridiagonal block + absolute couplings)
template <class RowSum, class Coupling>
static void line_relax(const Grid& g, Field& x, const Field& b, Field& q, Field& t, int i, RowSum&& row_sum, Coupling&& coupling) {
    int Ny = g.Ny();
    double cj = 0, tj = 0, dj = 0;
    for (int j = 1; j <= Ny; ++j) {
        double s = row_sum(i, j);
        double cj1 = (j == Ny) ? 0.0 : coupling(i, j + 1);
        double m = s - cj - cj1 + cj * tj;
        dj = (b(i, j) - q(i, j) + cj * dj) / m;
        tj = -cj1 / m;
        t(i, j) = tj;
        q(i, j) = dj;
        cj = cj1;
    }
    double delta = 0;
    for (int j = Ny; j >= 1; --j) {
        delta = q(i, j) - t(i, j) * delta;
        x(i, j) += delta;
    }
}

// smooth!, :165-180 and _smooth! / _line_smooth!, :213-219, :255-259
static void smooth(const Grid& g, VelocityVector& x, const VelocityVector& b, VelocityVector& q, Field& t, const Coefficients& c,
                   int walls, int smoother, int sweeps) {
    // the ℓ1 row sums depend on the coefficients only: evaluated once for all sweeps, by the same functions
    static thread_local std::vector<double> sums;
    const int sx = g.Nx() + 1;
    const size_t n = (size_t)sx * (g.Ny() + 1);
    double *rsu = nullptr, *rsv = nullptr;
    if (smoother == NK_SMOOTHER_POINT_JACOBI) {
        if (sums.size() < 2 * n) sums.resize(2 * n);
        rsu = sums.data();
        rsv = rsu + n;
        for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
            rsu[(size_t)j * sx + i] = x_absolute_row_sum(g, i, j, c, walls);
            rsv[(size_t)j * sx + i] = y_absolute_row_sum(g, i, j, c, walls);
        });
    }
    for (int s = 0; s < sweeps; ++s) {
        fill_halo(x);
        ssa_operator(g, q, x, c, walls);
        if (smoother == NK_SMOOTHER_POINT_JACOBI) {
            for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
                x.u(i, j) += (b.u(i, j) - q.u(i, j)) / rsu[(size_t)j * sx + i];
                x.v(i, j) += (b.v(i, j) - q.v(i, j)) / rsv[(size_t)j * sx + i];
            });
        } else {
#pragma omp parallel for schedule(static)
            for (int i = 1; i <= g.Nx(); ++i) {
                line_relax(g, x.u, b.u, q.u, t, i, [&](int ii, int jj) { return x_absolute_row_sum(g, ii, jj, c, walls); },
                           [&](int ii, int jj) { return x_line_coupling(g, ii, jj, c, walls); });
                line_relax(g, x.v, b.v, q.v, t, i, [&](int ii, int jj) { return y_absolute_row_sum(g, ii, jj, c, walls); },
                           [&](int ii, int jj) { return y_line_coupling(g, ii, jj, c, walls); });
            }
        }
    }
}

struct Multigrid {   // StressBalanceMultigridPreconditioner, :18-62
    std::vector<std::unique_ptr<Level>> levels;
    VelocityVector residual;
    Field scratch;
    int smoother = NK_SMOOTHER_POINT_JACOBI, sweeps = 2, coarsest = 20;
};

// v_cycle!, :144-163
static void v_cycle(const Grid& g, VelocityVector& x, const VelocityVector& b, VelocityVector& q, Field& t, const Coefficients& c,
                    Multigrid& P, size_t l, int walls) {
    if (l >= P.levels.size()) {
        fill_interior(x, 0.0);
        smooth(g, x, b, q, t, c, walls, P.smoother, P.coarsest);
        return;
    }
    Level& C = *P.levels[l];
    fill_interior(x, 0.0);
    smooth(g, x, b, q, t, c, walls, P.smoother, P.sweeps);
    fill_halo(x);
    ssa_operator(g, q, x, c, walls);
    subtract(g, q, b, q);
    fill_halo(q);
    restrict_vector(*C.grid, g, C, C.b, q, C.etaH, *c.etaH);
    Coefficients cc{&C.etaH, &C.etaHff, &C.bu, &C.bv};
    v_cycle(*C.grid, C.x, C.b, C.q, C.scratch, cc, P, l + 1, walls);
    fill_halo(C.x);
    prolongate_vector(g, *C.grid, C, x, C.x, *c.etaH, C.etaH);
    smooth(g, x, b, q, t, c, walls, P.smoother, P.sweeps);
}

// ------------------------------------------------------------------------------------------------
// Rheology, friction, column integrals, DIVA.
// ------------------------------------------------------------------------------------------------
struct Sigma {   // SigmaGrid column: faces ζ_0..ζ_Nσ (src/Grids/sigma_grid.jl:20-22)
    int N = 1;
    std::vector<double> faces;
    double zf(int k) const { return faces[k - 1]; }                       // znode(k, Face), k = 1..N+1
    double zc(int k) const { return (faces[k - 1] + faces[k]) / 2; }      // znode(k, Center)
};

// Exact integral of (1 - ζ)^p, src/StressBalances/column_integrals.jl:1-2
static inline double ipow(double x, int n) { double r = x; for (int m = 1; m < n; ++m) r *= x; return r; }
static inline double power_integral(double zm, double zp, int p) { return (ipow(1 - zm, p + 1) - ipow(1 - zp, p + 1)) / (p + 1); }
static inline double layer_weight(const Sigma& s, int k, int p) { return power_integral(s.zf(k), s.zf(k + 1), p); }   // :4-6
static inline double profile_weight(const Sigma& s, int kp, int k, int p) {   // :8-14
    double zm = s.zf(kp);
    double zp = (kp == k) ? s.zc(k) : s.zf(kp + 1);
    return power_integral(zm, zp, p);
}
static inline double layer_thickness(const Sigma& s, int k) { return s.zf(k + 1) - s.zf(k); }   // :44-45

struct Physics {
    int walls = NK_FREE_SLIP;
    double n = 3, eps0 = 1e-13;
    int friction = NK_FRICTION_NONE;
    double m = 1.0 / 3, alpha2 = 0.5, u0 = 1e-8;
    double rho_i = 918, rho_w = 1028, g = 9.81;
};

static inline double basal_drag(double U, double C, double N, const Physics& ph) {   // frictions.jl:83-89
    if (ph.friction == NK_WEERTMAN) return C * std::pow(U, ph.m - 1);
    double tc = ph.alpha2 * N;
    return C * std::pow(U, ph.m - 1) * tc / std::pow(std::pow(C, 1 / ph.m) * U + std::pow(tc, 1 / ph.m), ph.m);
}

// compute_basal_drag!, frictions.jl:127-160.  N may be nullptr (`nothing`).
static void compute_basal_drag(const Grid& g, Field& bu, Field& bv, const Physics& ph, const Field& u, const Field& v,
                               const Field& phu, const Field& phv, const Field* N, const Field& C) {
    if (ph.friction == NK_FRICTION_NONE) return;
    double u02 = ph.u0 * ph.u0;
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= bu.ny(); ++j)
        for (int i = 1; i <= bu.nx(); ++i) {
            double vf = ((v(i - 1, j) + v(i, j)) / 2 + (v(i - 1, j + 1) + v(i, j + 1)) / 2) / 2;   // ℑxyᶠᶜᵃ(v)
            double U = std::sqrt(u(i, j) * u(i, j) + vf * vf + u02);
            double Cf = (C(i - 1, j) + C(i, j)) / 2;
            double Nf = N ? ((*N)(i - 1, j) + (*N)(i, j)) / 2 : 0.0;
            double b = phu(i, j) * basal_drag(U, Cf, Nf, ph);
            bu(i, j) = g.peripheral_fc(i, j) ? 0.0 : b;
        }
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= bv.ny(); ++j)
        for (int i = 1; i <= bv.nx(); ++i) {
            double uf = ((u(i, j - 1) + u(i + 1, j - 1)) / 2 + (u(i, j) + u(i + 1, j)) / 2) / 2;   // ℑxyᶜᶠᵃ(u)
            double U = std::sqrt(v(i, j) * v(i, j) + uf * uf + u02);
            double Cf = (C(i, j - 1) + C(i, j)) / 2;
            double Nf = N ? ((*N)(i, j - 1) + (*N)(i, j)) / 2 : 0.0;
            double b = phv(i, j) * basal_drag(U, Cf, Nf, ph);
            bv(i, j) = g.peripheral_cf(i, j) ? 0.0 : b;
        }
}

// Glen viscosity, src/Rheologies/glen_flow_law.jl:97-111 (membrane) and :122-143 (DIVA vertical shear).
// A is 2-D (A2) or on the sigma grid (A3); bbu/bbv/ub/vb non-null selects the DIVA form.
static void compute_viscosity(const Grid& g, const Sigma& sg, SigmaField& eta_s, const Physics& ph, const Field& u, const Field& v,
                              const Field* A2, const SigmaField* A3,
                              const Field* bbu, const Field* bbv, const Field* ub, const Field* vb) {
    double n = ph.n;
    double e0 = ph.eps0;
    for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
        double e2 = effective_strain_rate2(g, i, j, u, v, ph.walls);
        for (int k = 1; k <= sg.N; ++k) {
            double A = A3 ? A3->k[k - 1](i, j) : (*A2)(i, j);
            double ee;
            if (bbu) {
                double zeta = sg.zc(k);
                double em = eta_s.k[k - 1](i, j);
                em = (em == 0.0) ? std::numeric_limits<double>::infinity() : em;
                double tx = ((*bbu)(i, j) * (*ub)(i, j) + (*bbu)(i + 1, j) * (*ub)(i + 1, j)) / 2;   // ℑxᶜᵃᵃ(βᵇᵘ uᵇ)
                double ty = ((*bbv)(i, j) * (*vb)(i, j) + (*bbv)(i, j + 1) * (*vb)(i, j + 1)) / 2;   // ℑyᵃᶜᵃ(βᵇᵛ vᵇ)
                double exz = tx * (1 - zeta) / (2 * em);
                double eyz = ty * (1 - zeta) / (2 * em);
                ee = e2 + exz * exz + eyz * eyz + e0 * e0;
            } else {
                ee = e2 + e0 * e0;
            }
            eta_s.k[k - 1](i, j) = std::pow(A, -1 / n) * std::pow(ee, (1 - n) / (2 * n)) / 2;
        }
    });
}

// compute_column_integrals!, src/StressBalances/column_integrals.jl:54-72.  mu may be nullptr.
static void compute_column_integrals(const Grid& g, const Sigma& sg, Field& etaH, Field& F2, const SigmaField& eta_s,
                                     const Field& H, const Field* mu) {
    for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
        double e = 0, F = 0;
        for (int k = 1; k <= sg.N; ++k) {
            e += eta_s.k[k - 1](i, j) * layer_thickness(sg, k);
            F += (1 / eta_s.k[k - 1](i, j)) * layer_weight(sg, k, 2);
        }
        double m = mu ? (*mu)(i, j) : 1.0;
        etaH(i, j) = mu ? e * H(i, j) * m : e * H(i, j);
        F2(i, j) = F * H(i, j);
    });
}

// DIVA, src/StressBalances/diva.jl:1-51
static void compute_basal_velocities(const Grid& g, Field& ub, Field& vb, const Field& u, const Field& v, const Field& bbu, const Field& bbv, const Field& F2) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= ub.ny(); ++j)
        for (int i = 1; i <= ub.nx(); ++i) ub(i, j) = u(i, j) / (1 + bbu(i, j) * ((F2(i - 1, j) + F2(i, j)) / 2));
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= vb.ny(); ++j)
        for (int i = 1; i <= vb.nx(); ++i) vb(i, j) = v(i, j) / (1 + bbv(i, j) * ((F2(i, j - 1) + F2(i, j)) / 2));
    (void)g;
}
static void compute_effective_drag(Field& bu, Field& bv, const Field& bbu, const Field& bbv, const Field& F2) {
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= bu.ny(); ++j)
        for (int i = 1; i <= bu.nx(); ++i) bu(i, j) = bbu(i, j) / (1 + bbu(i, j) * ((F2(i - 1, j) + F2(i, j)) / 2));
#pragma omp parallel for schedule(static)
    for (int j = 1; j <= bv.ny(); ++j)
        for (int i = 1; i <= bv.nx(); ++i) bv(i, j) = bbv(i, j) / (1 + bbv(i, j) * ((F2(i, j - 1) + F2(i, j)) / 2));
}

// ------------------------------------------------------------------------------------------------
// Geometry and driving stress.
// ------------------------------------------------------------------------------------------------
static inline double nonzero(double x) { return x == 0.0 ? 1.0 : x; }   // subgrid_grounded_fraction.jl:51
static inline double segment_grounded_fraction(double f1, double f2) {   // :34-38
    double fp = std::max(f1, 0.0) + std::max(f2, 0.0);
    double S = std::abs(f1) + std::abs(f2);
    return S == 0.0 ? 1.0 : fp / nonzero(S);
}
static inline double triangle_grounded_fraction(double f1, double f2, double f3) {   // :41-49
    double a = std::min(std::min(f1, f2), f3);
    double c = std::max(std::max(f1, f2), f3);
    double b = f1 + f2 + f3 - a - c;
    double one_grounded = c * c / nonzero((c - a) * (c - b));
    double one_floating = 1.0 - a * a / nonzero((b - a) * (c - a));
    double phi = b > 0 ? one_floating : one_grounded;
    return a >= 0 ? 1.0 : (c <= 0 ? 0.0 : phi);
}

struct Problem;

}  // namespace oracle

// ==================================================================================================
// Problem object and the C entry points (same shape as the library's nk_* functions).
// ==================================================================================================
namespace oracle {

struct Problem {
    Grid grid;
    Sigma sigma;
    Physics ph;
    nk_physics_desc pdesc{};
    nk_solver_desc sdesc{};
    int stress_balance = NK_SSA;
    int rate_layout = NK_RATE_FACTOR_2D;
    bool use_mask = true, use_N = true;
    int grounding = 1, gl_stress = 0;
    double mask_min = 1, mask_trans = 1;

    VelocityVector x, tau;
    VelocityVector ud;            // prescribed velocities, NaN where free (grid.pu / grid.pv once set)
    Field H, bed, s, mu, phi, phu, phv, N, C, A2, etaH, etaHff, bu, bv, F2, bbu, bbv, ub, vb;
    SigmaField A3, eta_s, T, us, vs;
    SigmaField E, omega;          // enthalpy and water fraction (nko_compute_thermal_diagnostics)
    // energy step (nko_step_enthalpy): basal water Hw, grounded melt mᵍ (gmelt), geothermal flux G, surface and ocean
    // temperatures, basal melt rate m, thickness of the previous energy step Hⁿ, strain heating Φ
    Field Hw, gmelt, G, Ts, To, melt, Hn, sb;   // sb: the temperate fraction sᵇ of the basal layer (output)
    Field smb, clipped;           // thickness step (nko_step_thickness): surface mass balance, clipped thickness
    Field H_step0;                // the thickness at the start of the current step (its stages start from it)
    // thickness advection (nko_set_thickness_advection); the reference's default for the SSA and the DIVA is
    // WENO(order = 5, bounds = (0, 1e5)) (default_thickness_advection, src/Models/ice_sheet_model.jl:123)
    nk_advection_desc advection{NK_ADVECTION_WENO, 5, 1, 0, 0.0, 1e5};
    Field theta;                  // the bounds-preserving limiter of each cell (and of the first halo layer)
    // PartialCellFront (nko_set_front): the front thickness Hʳ, the calved thickness, MaximumExtentCalving's extent and
    // the overflow / retreat scratch; the ice mask μ is then the prognostic 0/1 flag of full cells
    nk_front_desc front{0, 4, NK_CALVING_NONE, 0, 0.0, 0.0, 0.0, 0.0, 0.0};
    Field Hr, calved, extent, O;
    // TillEffectivePressure (nko_set_till): N from the basal water Hw, and drain_till in the energy step
    nk_till_desc till{0, 0, 1000.0, 0.02, 0.69, 0.12, 2.0, 0.0};
    Field qg;                     // basal heat flux qᵍ = φ G + τᵇ⋅uᵇ of the last energy step (output)
    SigmaField Phi;

    // CG workspace (VelocityConjugateGradientSolver, conjugate_gradient.jl:52-102) and Picard x⁻
    VelocityVector r, z, p, q, w, xprev;
    Field eta_prev;               // η̄H of the previous Picard iteration (NK_VISCOSITY_CONVERGENCE)
    Multigrid mg;
    VelocityVector diag;          // the operator diagonal of the current coefficients (diagonal preconditioner)
    bool mg_ready = false;
};

static Coefficients coeffs(Problem& P) { return Coefficients{&P.etaH, &P.etaHff, &P.bu, &P.bv}; }

// x = val on the prescribed faces (the identity rows' values), halos refilled.
static void impose_prescribed(Problem& P, VelocityVector& x, const VelocityVector& val) {
    const Grid& g = P.grid;
    if (!g.pu) return;
    for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
        if (prescribed_fc(g, i, j)) x.u(i, j) = val.u(i, j);
        if (prescribed_cf(g, i, j)) x.v(i, j) = val.v(i, j);
    });
    fill_halo(x);
}

// conjugate_gradient.jl:36; multigrid_preconditioner.jl:128.  The diagonal preconditioner recomputes the operator
// diagonal from the coefficients at every application (diagonal_preconditioner.jl:11-18); the coefficients are
// fixed during a solve, so it is taken here once per solve, by the same functions, and divided by as before.
static void update_preconditioner(Problem& P) {
    if (P.sdesc.preconditioner == NK_PRECONDITIONER_MULTIGRID) coarsen_coefficients(P.mg.levels, 0, P.etaH, P.bu, P.bv);
    if (P.sdesc.preconditioner == NK_PRECONDITIONER_DIAGONAL) {
        const Grid& g = P.grid;
        Coefficients c{&P.etaH, &P.etaHff, &P.bu, &P.bv};
        if (!P.diag.u.g) P.diag.init(&g);
        int nux = P.diag.u.nx(), nuy = P.diag.u.ny(), nvx = P.diag.v.nx(), nvy = P.diag.v.ny();
#pragma omp parallel for schedule(static)
        for (int j = 1; j <= nuy; ++j) for (int i = 1; i <= nux; ++i) P.diag.u(i, j) = x_diagonal(g, i, j, c, P.ph.walls);
#pragma omp parallel for schedule(static)
        for (int j = 1; j <= nvy; ++j) for (int i = 1; i <= nvx; ++i) P.diag.v(i, j) = y_diagonal(g, i, j, c, P.ph.walls);
    }
}

static void precondition(Problem& P, VelocityVector& z, VelocityVector& r) {
    Coefficients c = coeffs(P);
    switch (P.sdesc.preconditioner) {
        case NK_PRECONDITIONER_NONE: copyto(P.grid, z, r); break;                        // conjugate_gradient.jl:33
        case NK_PRECONDITIONER_DIAGONAL: {   // z = r / diag, diagonal_preconditioner.jl:11-18, 46-54
            int nux = z.u.nx(), nuy = z.u.ny(), nvx = z.v.nx(), nvy = z.v.ny();
#pragma omp parallel for schedule(static)
            for (int j = 1; j <= nuy; ++j) for (int i = 1; i <= nux; ++i) z.u(i, j) = r.u(i, j) / P.diag.u(i, j);
#pragma omp parallel for schedule(static)
            for (int j = 1; j <= nvy; ++j) for (int i = 1; i <= nvx; ++i) z.v(i, j) = r.v(i, j) / P.diag.v(i, j);
            break;
        }
        default: v_cycle(P.grid, z, r, P.mg.residual, P.mg.scratch, c, P.mg, 0, P.ph.walls); break;  // multigrid :122-126
    }
}

// conjugate_gradient!, conjugate_gradient.jl:158-223.  Returns the iteration count.
static int conjugate_gradient(Problem& P, VelocityVector& x, const VelocityVector& b, nk_solve_stats* st, int* status) {
    const Grid& g = P.grid;
    Coefficients c = coeffs(P);
    VelocityVector &r = P.r, &z = P.z, &p = P.p, &q = P.q;
    fill_halo(x);
    ssa_operator(g, q, x, c, P.ph.walls);
    subtract(g, r, b, q);
    update_preconditioner(P);
    precondition(P, z, r);
    copyto(g, p, z);
    double rho = vector_dot(g, r, z);

    auto step = [&](double rho_) {   // conjugate_gradient_step!, :343-364
        fill_halo(p);
        ssa_operator(g, q, p, c, P.ph.walls);
        double pq = vector_dot(g, p, q);
        double alpha = pq == 0.0 ? 0.0 : rho_ / pq;
        axpy(g, alpha, p, x);
        axpy(g, -alpha, q, r);
        precondition(P, z, r);
        double rho1 = vector_dot(g, r, z);
        double beta = rho_ == 0.0 ? 0.0 : rho1 / rho_;
        xpby(g, z, beta, p);
        return rho1;
    };

    const nk_iteration_control& ctl = P.sdesc.linear;
    int it = 0;
    double r0 = std::sqrt(vector_dot(g, r, r));
    double rn = r0;
    if (ctl.kind == NK_FIXED_ITERATIONS) {   // :178-183
        for (int k = 0; k < ctl.iterations; ++k) rho = step(rho);
        it = ctl.iterations;
        rn = std::sqrt(vector_dot(g, r, r));
    } else {                                  // :185-200
        double tol = std::max(ctl.reltol * r0, ctl.abstol);
        while (rn > tol && it < ctl.maxiter) {
            rho = step(rho);
            rn = std::sqrt(vector_dot(g, r, r));
            ++it;
        }
        if (rn > tol && *status == NK_OK) *status = NK_NOT_CONVERGED;
    }
    if (!std::isfinite(rn)) *status = NK_NONFINITE;
    if (st) { st->residual_norm = rn; st->initial_residual_norm = r0; st->linear_iterations_last = it; st->linear_iterations_total += it; }
    return it;
}

static const Field* mu_or_null(Problem& P) { return P.use_mask ? &P.mu : nullptr; }

// update_stress_balance_coefficients!, stress_balance_coefficients.jl:10-20
static void update_ssa(Problem& P) {
    const Grid& g = P.grid;
    fill_halo(P.x);
    compute_viscosity(g, P.sigma, P.eta_s, P.ph, P.x.u, P.x.v, P.rate_layout == NK_RATE_FACTOR_2D ? &P.A2 : nullptr,
                      P.rate_layout == NK_RATE_FACTOR_SIGMA ? &P.A3 : nullptr, nullptr, nullptr, nullptr, nullptr);
    compute_column_integrals(g, P.sigma, P.etaH, P.F2, P.eta_s, P.H, mu_or_null(P));
    fill_halo(P.etaH);
    interpolate_to_corners(g, P.etaHff, P.etaH);
    fill_halo(P.etaHff);
    compute_basal_drag(g, P.bu, P.bv, P.ph, P.x.u, P.x.v, P.phu, P.phv, P.use_N ? &P.N : nullptr, P.C);
    fill_halo(P.bu); fill_halo(P.bv);
}

// update_diva_coefficients!, diva.jl:61-75
static void update_diva(Problem& P) {
    const Grid& g = P.grid;
    fill_halo(P.x);
    compute_basal_velocities(g, P.ub, P.vb, P.x.u, P.x.v, P.bbu, P.bbv, P.F2);
    fill_halo(P.ub); fill_halo(P.vb);
    compute_basal_drag(g, P.bbu, P.bbv, P.ph, P.ub, P.vb, P.phu, P.phv, P.use_N ? &P.N : nullptr, P.C);
    fill_halo(P.bbu); fill_halo(P.bbv);
    compute_viscosity(g, P.sigma, P.eta_s, P.ph, P.x.u, P.x.v, P.rate_layout == NK_RATE_FACTOR_2D ? &P.A2 : nullptr,
                      P.rate_layout == NK_RATE_FACTOR_SIGMA ? &P.A3 : nullptr, &P.bbu, &P.bbv, &P.ub, &P.vb);
    compute_column_integrals(g, P.sigma, P.etaH, P.F2, P.eta_s, P.H, mu_or_null(P));
    fill_halo(P.etaH); fill_halo(P.F2);
    interpolate_to_corners(g, P.etaHff, P.etaH);
    fill_halo(P.etaHff);
    compute_effective_drag(P.bu, P.bv, P.bbu, P.bbv, P.F2);
    fill_halo(P.bu); fill_halo(P.bv);
}

static void update_coefficients(Problem& P) { if (P.stress_balance == NK_DIVA) update_diva(P); else update_ssa(P); }

// picard_solve!, picard.jl:63-90
static void picard_solve(Problem& P, nk_solve_stats* st) {
    const Grid& g = P.grid;
    int status = NK_OK;
    impose_prescribed(P, P.x, P.ud);   // the identity rows start solved
    const nk_iteration_control& ctl = P.sdesc.picard;
    int it = 0;
    if (st) { std::memset(st, 0, sizeof(*st)); }
    if (ctl.kind == NK_FIXED_ITERATIONS) {
        for (int k = 0; k < ctl.iterations; ++k) { update_coefficients(P); conjugate_gradient(P, P.x, P.tau, st, &status); }
        it = ctl.iterations;
    } else {
        double D = std::numeric_limits<double>::infinity(), X = 0;
        while (D > std::max(ctl.reltol * X, ctl.abstol) && it < ctl.maxiter) {
            copyto(g, P.xprev, P.x);
            update_coefficients(P);
            conjugate_gradient(P, P.x, P.tau, st, &status);
            if (ctl.kind == NK_VISCOSITY_CONVERGENCE) {   // the extension: change of η̄H between coefficient updates
                double dd = 0, ee = 0;
                for (int j = 1; j <= g.Ny(); ++j)
                    for (int i = 1; i <= g.Nx(); ++i) {
                        double e = P.etaH(i, j), d = e - P.eta_prev(i, j);
                        dd += d * d;
                        ee += e * e;
                        P.eta_prev(i, j) = e;
                    }
                D = it == 0 ? std::numeric_limits<double>::infinity() : std::sqrt(dd);
                X = std::sqrt(ee);
            } else {
                axpy(g, -1.0, P.x, P.xprev);
                D = std::sqrt(vector_dot(g, P.xprev, P.xprev));
                X = std::sqrt(vector_dot(g, P.x, P.x));
            }
            ++it;
        }
        if (D > std::max(ctl.reltol * X, ctl.abstol) && status == NK_OK) status = NK_NOT_CONVERGED;
        if (st) { st->picard_change = D; st->picard_norm = X; }
        if ((ctl.kind == NK_VISCOSITY_CONVERGENCE ? (std::isnan(D) || !std::isfinite(X)) : !std::isfinite(D)) && it > 0) status = NK_NONFINITE;
    }
    fill_halo(P.x);
    if (st) { st->picard_iterations = it; st->status = status; }
}

// update_geometry!, ice_sheet_model_methods.jl:103-111, and compute_driving_stress!, driving_stress.jl:43-125.
static void compute_geometry(Problem& P) {
    const Grid& g = P.grid;
    double rw_ri = P.ph.rho_w / P.ph.rho_i, ri_rw = P.ph.rho_i / P.ph.rho_w;
    int Nx = g.Nx(), Ny = g.Ny();
    // compute_surface_elevation!, subgrid_grounded_fraction.jl:211-232
    for_xy(Nx, Ny, [&](int i, int j) {
        P.s(i, j) = P.grounding ? std::max(P.bed(i, j) + P.H(i, j), (1 - ri_rw) * P.H(i, j)) : P.bed(i, j) + P.H(i, j);
    });
    // compute_grounded_fractions!, :234-264
    auto f = [&](int i, int j) { return P.H(i, j) + rw_ri * P.bed(i, j); };
    if (P.grounding) {
        for_xy(Nx, Ny, [&](int i, int j) {
            double fc = f(i, j);
            double fe = (fc + f(i + 1, j)) / 2, fw = (fc + f(i - 1, j)) / 2, fn = (fc + f(i, j + 1)) / 2, fs = (fc + f(i, j - 1)) / 2;
            double fne = (fc + f(i + 1, j) + f(i, j + 1) + f(i + 1, j + 1)) / 4;
            double fnw = (fc + f(i - 1, j) + f(i, j + 1) + f(i - 1, j + 1)) / 4;
            double fse = (fc + f(i + 1, j) + f(i, j - 1) + f(i + 1, j - 1)) / 4;
            double fsw = (fc + f(i - 1, j) + f(i, j - 1) + f(i - 1, j - 1)) / 4;
            double phi = triangle_grounded_fraction(fc, fe, fne) + triangle_grounded_fraction(fc, fn, fne) +
                         triangle_grounded_fraction(fc, fn, fnw) + triangle_grounded_fraction(fc, fw, fnw) +
                         triangle_grounded_fraction(fc, fw, fsw) + triangle_grounded_fraction(fc, fs, fsw) +
                         triangle_grounded_fraction(fc, fs, fse) + triangle_grounded_fraction(fc, fe, fse);
            P.phi(i, j) = phi / 8;
        });
        for (int j = 1; j <= P.phu.ny(); ++j) for (int i = 1; i <= P.phu.nx(); ++i) P.phu(i, j) = segment_grounded_fraction(f(i - 1, j), f(i, j));
        for (int j = 1; j <= P.phv.ny(); ++j) for (int i = 1; i <= P.phv.nx(); ++i) P.phv(i, j) = segment_grounded_fraction(f(i, j - 1), f(i, j));
    } else {
        for (int j = 1; j <= Ny; ++j) for (int i = 1; i <= Nx; ++i) P.phi(i, j) = 1;
        for (int j = 1; j <= P.phu.ny(); ++j) for (int i = 1; i <= P.phu.nx(); ++i) P.phu(i, j) = 1;
        for (int j = 1; j <= P.phv.ny(); ++j) for (int i = 1; i <= P.phv.nx(); ++i) P.phv(i, j) = 1;
    }
    // compute_effective_pressure!, subgrid_grounded_fraction.jl:168-183: the ocean-connected law, or with a till
    // effective_pressure of TillEffectivePressure (till_effective_pressure.jl:63-70) capped by it
    double rig = P.ph.rho_i * P.ph.g, rwg = P.ph.rho_w * P.ph.g;
    const nk_till_desc& till = P.till;
    for_xy(Nx, Ny, [&](int i, int j) {
        double P0 = rig * P.H(i, j);
        double No = std::max(P0 + rwg * std::min(P.bed(i, j), 0.0), 0.0);
        if (till.enabled) {
            double N0 = till.reference_effective_pressure, delta = till.overburden_fraction;
            double s = std::min(std::max(P.Hw(i, j) / till.maximum_water_thickness, 0.0), 1.0);
            double Pt = P0 > 0 ? P0 : N0 / delta;
            double Nt = N0 * std::pow(delta * Pt / N0, s) * std::pow(10.0, till.reference_void_ratio / till.compressibility * (1 - s));
            P.N(i, j) = std::min(Nt, No);
        } else {
            P.N(i, j) = No;
        }
    });
    // compute_ice_mask!, smooth_ice_mask.jl:50-69; a PartialCellFront's flag is prognostic (partial_cell_front.jl:95)
    if (!P.front.enabled)
        for_xy(Nx, Ny, [&](int i, int j) {
            double t = std::min(std::max((P.H(i, j) - P.mask_min) / P.mask_trans, 0.0), 1.0);
            P.mu(i, j) = t * t * (3 - 2 * t);
        });
    fill_halo(P.s); fill_halo(P.N); fill_halo(P.mu); fill_halo(P.phi); fill_halo(P.phu); fill_halo(P.phv);

    // compute_driving_stress!, driving_stress.jl:43-125
    const Field* mu = mu_or_null(P);
    double ri = P.ph.rho_i, rw = P.ph.rho_w, gg = P.ph.g;
    auto front_force = [&](int i, int j) {   // :56-60
        double Hi = P.H(i, j);
        double D = std::min(std::max(Hi - P.s(i, j), 0.0), Hi);
        return gg * (ri * Hi * Hi - rw * D * D) / 2;
    };
    auto gl_stress = [&](double H1, double H2, double s1, double s2, double b1, double b2, bool& straddles) {   // :84-92
        double f1 = H1 + rw / ri * b1, f2 = H2 + rw / ri * b2;
        straddles = ((f1 > 0) != (f2 > 0)) && (H1 > 0) && (H2 > 0);
        double theta = f1 / (straddles ? f1 - f2 : 1.0);
        double Hg = H1 + theta * (H2 - H1);
        double sg = (1 - ri / rw) * Hg;
        return -ri * gg * ((H1 + Hg) * (sg - s1) + (Hg + H2) * (s2 - sg)) / 2;
    };
    for (int j = 1; j <= P.tau.u.ny(); ++j)
        for (int i = 1; i <= P.tau.u.nx(); ++i) {   // _compute_x_driving_stress!, :109-116
            bool wall = inactive_fc(g, i, j, mu);
            bool front = false; double tf = 0;
            if (mu) {
                bool w = (*mu)(i - 1, j) > 0 && !((*mu)(i, j) > 0), e = !((*mu)(i - 1, j) > 0) && (*mu)(i, j) > 0;
                double F = (w ? front_force(i - 1, j) : 0.0) - (e ? front_force(i, j) : 0.0);
                front = w || e; tf = g.dy_c(j) * F;
            }
            bool straddles = false; double tg = 0;
            if (P.gl_stress) {
                tg = g.dy_c(j) * gl_stress(P.H(i - 1, j), P.H(i, j), P.s(i - 1, j), P.s(i, j), P.bed(i - 1, j), P.bed(i, j), straddles);
            }
            double t = -g.Az_fcc(i, j) * ri * gg * ((P.H(i - 1, j) + P.H(i, j)) / 2) * ((P.s(i, j) - P.s(i - 1, j)) / g.dx_f(i));
            P.tau.u(i, j) = wall ? 0.0 : (front ? tf : (straddles ? tg : t));
            if (prescribed_fc(g, i, j)) P.tau.u(i, j) = P.ud.u(i, j);   // the identity row's right-hand side
        }
    for (int j = 1; j <= P.tau.v.ny(); ++j)
        for (int i = 1; i <= P.tau.v.nx(); ++i) {   // _compute_y_driving_stress!, :118-125
            bool wall = inactive_cf(g, i, j, mu);
            bool front = false; double tf = 0;
            if (mu) {
                bool s_ = (*mu)(i, j - 1) > 0 && !((*mu)(i, j) > 0), n_ = !((*mu)(i, j - 1) > 0) && (*mu)(i, j) > 0;
                double F = (s_ ? front_force(i, j - 1) : 0.0) - (n_ ? front_force(i, j) : 0.0);
                front = s_ || n_; tf = g.dx_c(i) * F;
            }
            bool straddles = false; double tg = 0;
            if (P.gl_stress) {
                tg = g.dx_c(i) * gl_stress(P.H(i, j - 1), P.H(i, j), P.s(i, j - 1), P.s(i, j), P.bed(i, j - 1), P.bed(i, j), straddles);
            }
            double t = -g.Az_cfc(i, j) * ri * gg * ((P.H(i, j - 1) + P.H(i, j)) / 2) * ((P.s(i, j) - P.s(i, j - 1)) / g.dy_f(j));
            P.tau.v(i, j) = wall ? 0.0 : (front ? tf : (straddles ? tg : t));
            if (prescribed_cf(g, i, j)) P.tau.v(i, j) = P.ud.v(i, j);
        }
}

// compute_velocity_profile! (DIVA, diva.jl:89-109) / extend_depth_average! (SSA, ice_sheet_model_methods.jl:167-180)
static void velocity_profile(Problem& P) {
    const Grid& g = P.grid;
    fill_halo(P.x);
    if (P.stress_balance == NK_SSA) {
        for (int j = 1; j <= P.ub.ny(); ++j) for (int i = 1; i <= P.ub.nx(); ++i) P.ub(i, j) = P.x.u(i, j);
        for (int j = 1; j <= P.vb.ny(); ++j) for (int i = 1; i <= P.vb.nx(); ++i) P.vb(i, j) = P.x.v(i, j);
        for (int k = 0; k < P.sigma.N; ++k) {
            for (int j = 1; j <= P.ub.ny(); ++j) for (int i = 1; i <= P.ub.nx(); ++i) P.us.k[k](i, j) = P.x.u(i, j);
            for (int j = 1; j <= P.vb.ny(); ++j) for (int i = 1; i <= P.vb.nx(); ++i) P.vs.k[k](i, j) = P.x.v(i, j);
        }
        return;
    }
    for (auto& f : P.eta_s.k) fill_halo(f);
    compute_basal_velocities(g, P.ub, P.vb, P.x.u, P.x.v, P.bbu, P.bbv, P.F2);
    const Sigma& sg = P.sigma;
    auto shear_integral = [&](int i, int j, int k) {   // column_integrals.jl:42
        double I = 0;
        for (int kp = 1; kp <= k; ++kp) I += (1 / P.eta_s.k[kp - 1](i, j)) * profile_weight(sg, kp, k, 1);
        return I * P.H(i, j);
    };
    for (int k = 1; k <= sg.N; ++k) {
        for (int j = 1; j <= P.ub.ny(); ++j)
            for (int i = 1; i <= P.ub.nx(); ++i) {
                double F1 = (shear_integral(i - 1, j, k) + shear_integral(i, j, k)) / 2;
                P.us.k[k - 1](i, j) = P.ub(i, j) * (1 + P.bbu(i, j) * F1);
            }
        for (int j = 1; j <= P.vb.ny(); ++j)
            for (int i = 1; i <= P.vb.nx(); ++i) {
                double F1 = (shear_integral(i, j - 1, k) + shear_integral(i, j, k)) / 2;
                P.vs.k[k - 1](i, j) = P.vb(i, j) * (1 + P.bbv(i, j) * F1);
            }
    }
}

// ------------------------------------------------------------------------------------------------
// Fixed-point adjoint of a converged SSA picard_solve! (the reverse rule of ext/NunatakEnzymeExt.jl:159-240,
// with picard_coefficient_step! :142-146 and picard_step_adjoint! :148-157).  One Picard step maps x to
// A(c(x))⁻¹ b.  At its fixed point x* the adjoint λ solves λ = A⁻ᵀ (x̄ + ȳ(λ)), ȳ = -(∂[A(c(x)) x*]/∂x)ᵀ λ,
// iterated from λ = 0 with the problem's CG warm-started from the previous λ until
// ‖λ⁺ - λ‖ ≤ max(reltol ‖λ⁺‖, abstol).  Then b̄ = λ and p̄ = -(∂[A(c(p)) x*]/∂p)ᵀ λ for p = log C, log A.
//
// The transposes below are written as reverse-mode sweeps over the forward functions of this file, in their
// representation: every forward read of an input accumulates the adjoint into that input, reads of halo cells
// included, and fill_halo_adjoint then returns each halo cell's adjoint to the cell fill_halo copied it from.
// G fields hold λ-signed sensitivities ∂(λᵀ q)/∂(·) with q = A(c) x* over the operator's active rows.
// ------------------------------------------------------------------------------------------------

// The transpose of fill_halo: the assignments run backwards, each adding the target's adjoint to its source and
// clearing the target.  Halo cells that fill_halo leaves alone (Face locations in a Bounded direction) hold
// constants, so their adjoints are dropped.
static void fill_halo_adjoint(Field& f) {
    const Grid& g = *f.g;
    int Hx = g.x.H + 1, Hy = g.y.H + 1;
    int Nx = g.x.N, Ny = g.y.N;
    int nxi = f.nx(), nyi = f.ny();
    for (int i = Nx + 1 + Hx - 1; i >= -Hx; --i) {
        if (g.y.periodic) {
            for (int m = Hy; m >= 1; --m) {
                f(i, m) += f(i, Ny + m); f(i, Ny + m) = 0;
                f(i, Ny + 1 - m) += f(i, 1 - m); f(i, 1 - m) = 0;
            }
        } else if (f.ly == CENTER) {
            for (int m = Hy; m >= 1; --m) {
                f(i, Ny) += f(i, Ny + m); f(i, Ny + m) = 0;
                f(i, 1) += f(i, 1 - m); f(i, 1 - m) = 0;
            }
        }
    }
    for (int j = nyi; j >= 1; --j) {
        if (g.x.periodic) {
            for (int m = Hx; m >= 1; --m) {
                f(m, j) += f(Nx + m, j); f(Nx + m, j) = 0;
                f(Nx + 1 - m, j) += f(1 - m, j); f(1 - m, j) = 0;
            }
        } else if (f.lx == CENTER) {
            for (int m = Hx; m >= 1; --m) {
                f(Nx, j) += f(Nx + m, j); f(Nx + m, j) = 0;
                f(1, j) += f(1 - m, j); f(1 - m, j) = 0;
            }
        }
    }
    // what is left outside the interior sits on cells that are never copied into: constants
    for (int j = -(g.y.H + 2); j < f.sy - (g.y.H + 2); ++j)
        for (int i = -(g.x.H + 2); i < f.sx - (g.x.H + 2); ++i)
            if (i < 1 || i > nxi || j < 1 || j > nyi) f(i, j) = 0;
}

// basal_drag and its derivatives with respect to the speed U and the face coefficient C (frictions.jl:83-89):
// Weertman β = C U^(m-1); regularised Coulomb β = C U^(m-1) τc / (C^(1/m) U + τc^(1/m))^m, τc = α² N.
static void basal_drag_and_derivatives(double U, double C, double N, const Physics& ph, double& b, double& dU, double& dC) {
    b = basal_drag(U, C, N, ph);
    if (ph.friction == NK_WEERTMAN) {
        dU = (ph.m - 1) * b / U;
        dC = std::pow(U, ph.m - 1);
        return;
    }
    if (b == 0.0) { dU = 0.0; dC = 0.0; return; }
    double cm = std::pow(C, 1 / ph.m), den = cm * U + std::pow(ph.alpha2 * N, 1 / ph.m);
    dU = b * ((ph.m - 1) / U - ph.m * cm / den);
    dC = b * (1 / C - cm * U / (C * den));
}

struct AdjointSweep {   // the G fields of one reverse sweep
    VelocityVector x;             // ∂(λᵀq)/∂x through the coefficients (x* frozen in the product)
    Field eta, ff, bu, bv, C;     // ∂(λᵀq)/∂η̄H, ∂/∂η̄Hᶠᶠ, ∂/∂βᵘ, ∂/∂βᵛ, ∂/∂C
    SigmaField logA;              // ∂(λᵀq)/∂log A per layer
    void init(const Grid* g, int Ns) {
        x.init(g);
        eta.init(g, CENTER, CENTER); ff.init(g, FACE, FACE); bu.init(g, FACE, CENTER); bv.init(g, CENTER, FACE);
        C.init(g, CENTER, CENTER);
        logA.init(g, CENTER, CENTER, Ns);
    }
    void zero() {
        x.u.zero(); x.v.zero(); eta.zero(); ff.zero(); bu.zero(); bv.zero(); C.zero();
        for (auto& f : logA.k) f.zero();
    }
};

// The operator part of a reverse sweep: ∂(λᵀq)/∂η̄H, ∂/∂η̄Hᶠᶠ (after fill_halo(η̄Hᶠᶠ) and _interpolate_to_corners!
// are reversed, both land on G.eta, halos returned), ∂/∂βᵘ and ∂/∂βᵛ for q = A(c) x* (ssa_operator.jl:60-89).
static void operator_sweep(Problem& P, const VelocityVector& lam, AdjointSweep& G) {
    const Grid& g = P.grid;
    const Physics& ph = P.ph;
    const VelocityVector& xs = P.x;
    const Field& eta = P.etaH;
    G.zero();
    // operator: q_u = Az βᵘ u - [Δy Txx(i) - Δy Txx(i-1) + Δx Txy(i, j+1) - Δx Txy(i, j)] on the active rows
    for (int j = 1; j <= g.Ny(); ++j)
        for (int i = 1; i <= g.Nx(); ++i) {
            if (!inactive_fc(g, i, j, &eta)) {
                double l = lam.u(i, j);
                G.eta(i, j) += -g.dy_c(j) * l * 2 * (2 * strain_rate_xx(g, i, j, xs.u, &eta) + strain_rate_yy(g, i, j, xs.v, &eta));
                G.eta(i - 1, j) += g.dy_c(j) * l * 2 * (2 * strain_rate_xx(g, i - 1, j, xs.u, &eta) + strain_rate_yy(g, i - 1, j, xs.v, &eta));
                G.ff(i, j + 1) += -g.dx_f(i) * l * 2 * strain_rate_xy(g, i, j + 1, xs.u, xs.v, ph.walls, &eta);
                G.ff(i, j) += g.dx_f(i) * l * 2 * strain_rate_xy(g, i, j, xs.u, xs.v, ph.walls, &eta);
                G.bu(i, j) += l * g.Az_fcc(i, j) * xs.u(i, j);
            }
            if (!inactive_cf(g, i, j, &eta)) {
                double l = lam.v(i, j);
                G.eta(i, j) += -g.dx_c(i) * l * 2 * (2 * strain_rate_yy(g, i, j, xs.v, &eta) + strain_rate_xx(g, i, j, xs.u, &eta));
                G.eta(i, j - 1) += g.dx_c(i) * l * 2 * (2 * strain_rate_yy(g, i, j - 1, xs.v, &eta) + strain_rate_xx(g, i, j - 1, xs.u, &eta));
                G.ff(i + 1, j) += -g.dy_f(j) * l * 2 * strain_rate_xy(g, i + 1, j, xs.u, xs.v, ph.walls, &eta);
                G.ff(i, j) += g.dy_f(j) * l * 2 * strain_rate_xy(g, i, j, xs.u, xs.v, ph.walls, &eta);
                G.bv(i, j) += l * g.Az_cfc(i, j) * xs.v(i, j);
            }
        }
    fill_halo_adjoint(G.ff);
    for (int j = 1; j <= G.ff.ny(); ++j)          // ff = ((η(i-1,j-1) + η(i,j-1)) / 2 + (η(i-1,j) + η(i,j)) / 2) / 2
        for (int i = 1; i <= G.ff.nx(); ++i) {
            double w = G.ff(i, j) / 4;
            G.eta(i - 1, j - 1) += w; G.eta(i, j - 1) += w; G.eta(i - 1, j) += w; G.eta(i, j) += w;
        }
    fill_halo_adjoint(G.eta);
}

// Reverse of the wall-masked membrane strain rate S(i, j) = ε̇xx² + ε̇yy² + ε̇xx ε̇yy + ℑxyᶜᶜ(ε̇xy²) of the viscosity
// (strain_rates.jl:27-32 with η̄H absent) for the adjoint gS of S: accumulates into gx (halos included).
static void strain_rate2_adjoint(const Grid& g, const VelocityVector& xs, int walls, int i, int j, double gS, VelocityVector& gx) {
    double exx = strain_rate_xx(g, i, j, xs.u, nullptr), eyy = strain_rate_yy(g, i, j, xs.v, nullptr);
    double gxx = gS * (2 * exx + eyy), gyy = gS * (2 * eyy + exx);
    if (!inactive_fc(g, i + 1, j, nullptr)) gx.u(i + 1, j) += gxx / g.dx_c(i);
    if (!inactive_fc(g, i, j, nullptr)) gx.u(i, j) -= gxx / g.dx_c(i);
    if (!inactive_cf(g, i, j + 1, nullptr)) gx.v(i, j + 1) += gyy / g.dy_c(j);
    if (!inactive_cf(g, i, j, nullptr)) gx.v(i, j) -= gyy / g.dy_c(j);
    for (int b = j; b <= j + 1; ++b)          // ((e²(i,j) + e²(i+1,j)) / 2 + (e²(i,j+1) + e²(i+1,j+1)) / 2) / 2
        for (int a = i; a <= i + 1; ++a) {
            double e = strain_rate_xy(g, a, b, xs.u, xs.v, walls, nullptr);
            double ge_raw = gS / 4 * 2 * e * (g.peripheral_ff(a, b) ? wall_shear_factor(walls) : 1.0);
            double gdudy = ge_raw / 2, gdvdx = ge_raw / 2;
            if (!inactive_fc(g, a, b, nullptr)) gx.u(a, b) += gdudy / g.dy_f(b);
            if (!inactive_fc(g, a, b - 1, nullptr)) gx.u(a, b - 1) -= gdudy / g.dy_f(b);
            if (!inactive_cf(g, a, b, nullptr)) gx.v(a, b) += gdvdx / g.dx_f(a);
            if (!inactive_cf(g, a - 1, b, nullptr)) gx.v(a - 1, b) -= gdvdx / g.dx_f(a);
        }
}

// Reverse of compute_basal_drag! (frictions.jl:127-160) read on the velocity pair (u, v) for the drag adjoints
// gbu, gbv: βᵘ = φᵘ β(U, C̄, N̄), U = √(u² + ℑxy(v)² + u₀²), C̄ and N̄ face means, zero on peripheral faces.
// Accumulates into gx and gC (halos included).
static void basal_drag_adjoint(Problem& P, const VelocityVector& xs, const Field& gbu, const Field& gbv, VelocityVector& gx, Field& gC) {
    const Grid& g = P.grid;
    const Physics& ph = P.ph;
    if (ph.friction == NK_FRICTION_NONE) return;
    double u02 = ph.u0 * ph.u0;
    const Field* N = P.use_N ? &P.N : nullptr;
    for (int j = 1; j <= gbu.ny(); ++j)
        for (int i = 1; i <= gbu.nx(); ++i) {
            if (g.peripheral_fc(i, j) || gbu(i, j) == 0.0) continue;
            double vf = ((xs.v(i - 1, j) + xs.v(i, j)) / 2 + (xs.v(i - 1, j + 1) + xs.v(i, j + 1)) / 2) / 2;
            double U = std::sqrt(xs.u(i, j) * xs.u(i, j) + vf * vf + u02);
            double Cf = (P.C(i - 1, j) + P.C(i, j)) / 2, Nf = N ? ((*N)(i - 1, j) + (*N)(i, j)) / 2 : 0.0;
            double b, dU, dC;
            basal_drag_and_derivatives(U, Cf, Nf, ph, b, dU, dC);
            double gb = gbu(i, j) * P.phu(i, j);
            double gU = gb * dU;
            gx.u(i, j) += gU * xs.u(i, j) / U;
            double gv = gU * vf / U / 4;
            gx.v(i - 1, j) += gv; gx.v(i, j) += gv; gx.v(i - 1, j + 1) += gv; gx.v(i, j + 1) += gv;
            gC(i - 1, j) += gb * dC / 2; gC(i, j) += gb * dC / 2;
        }
    for (int j = 1; j <= gbv.ny(); ++j)
        for (int i = 1; i <= gbv.nx(); ++i) {
            if (g.peripheral_cf(i, j) || gbv(i, j) == 0.0) continue;
            double uf = ((xs.u(i, j - 1) + xs.u(i + 1, j - 1)) / 2 + (xs.u(i, j) + xs.u(i + 1, j)) / 2) / 2;
            double U = std::sqrt(xs.v(i, j) * xs.v(i, j) + uf * uf + u02);
            double Cf = (P.C(i, j - 1) + P.C(i, j)) / 2, Nf = N ? ((*N)(i, j - 1) + (*N)(i, j)) / 2 : 0.0;
            double b, dU, dC;
            basal_drag_and_derivatives(U, Cf, Nf, ph, b, dU, dC);
            double gb = gbv(i, j) * P.phv(i, j);
            double gU = gb * dU;
            gx.v(i, j) += gU * xs.v(i, j) / U;
            double gu = gU * uf / U / 4;
            gx.u(i, j - 1) += gu; gx.u(i + 1, j - 1) += gu; gx.u(i, j) += gu; gx.u(i + 1, j) += gu;
            gC(i, j - 1) += gb * dC / 2; gC(i, j) += gb * dC / 2;
        }
}

// One reverse sweep of the SSA step q = A(c(x)) x* for the seed λ (halos of λ filled): the operator, then
// compute_column_integrals! and compute_viscosity! (membrane, wall-masked strain rates) and
// compute_basal_drag!, in reverse order.  λ-signed: G.x = ∂(λᵀq)/∂x.
// eta_bar: ∂J/∂η̄H per centre from outside the solve (a true adjoint; NULL: none), the shadow of the overwritten
// coefficient that the reverse rule adds in every pass (ext/NunatakEnzymeExt.jl:204-214).
static void adjoint_sweep(Problem& P, const VelocityVector& lam, AdjointSweep& G, const Field* eta_bar = nullptr) {
    const Grid& g = P.grid;
    const Physics& ph = P.ph;
    const VelocityVector& xs = P.x;
    operator_sweep(P, lam, G);
    if (eta_bar)   // G.eta is λ-signed: minus the true adjoint
        for (int j = 1; j <= g.Ny(); ++j) for (int i = 1; i <= g.Nx(); ++i) G.eta(i, j) -= (*eta_bar)(i, j);
    // column integrals and viscosity: η̄H = μ H Σₖ ηₖ Δζₖ, ηₖ = ½ Aₖ^(-1/n) S^((1-n)/2n), S = ε̇ₑ² + ε̇₀²
    double n = ph.n, p = (1 - n) / (2 * n);
    for (int j = 1; j <= g.Ny(); ++j)
        for (int i = 1; i <= g.Nx(); ++i) {
            double ge = G.eta(i, j) * P.H(i, j) * (P.use_mask ? P.mu(i, j) : 1.0);
            if (ge == 0.0) continue;
            double S = effective_strain_rate2(g, i, j, xs.u, xs.v, ph.walls) + ph.eps0 * ph.eps0;
            double gS = 0;
            for (int k = 1; k <= P.sigma.N; ++k) {
                double ek = P.eta_s.k[k - 1](i, j);
                double gk = ge * layer_thickness(P.sigma, k);
                gS += gk * ek * p / S;
                G.logA.k[k - 1](i, j) = gk * (-ek / n);
            }
            strain_rate2_adjoint(g, xs, ph.walls, i, j, gS, G.x);
        }
    basal_drag_adjoint(P, xs, G.bu, G.bv, G.x, G.C);
    fill_halo_adjoint(G.x.u);
    fill_halo_adjoint(G.x.v);
    fill_halo_adjoint(G.C);
}

// ---- DIVA: the reverse of one update_diva_coefficients! step (diva.jl:61-75) at the fixed point ----------------
// The step reads x and the lagged state s⁻ = (βᵇ⁻, F₂⁻, ησ⁻) and writes uᵇ = x / (1 + βᵇ⁻ ℑF₂⁻), βᵇ = φ drag(uᵇ),
// ησ (Glen with the lagged vertical shear), η̄H, F₂, the corners and β = βᵇ / (1 + βᵇ ℑF₂); its state outputs are
// (βᵇ, F₂, ησ).  At the fixed point the lagged and new state coincide, so the problem's arrays after the last
// update serve both.  The reference's rule sweeps the adjoint σ of the state along with λ
// (ext/NunatakEnzymeExt.jl:204-214).  True adjoints here (q̄ = -λ): the operator's λ-signed sensitivities are
// negated.
struct DivaState {   // adjoints of (βᵇᵘ, βᵇᵛ, F₂, ησ), halos included
    Field bbu, bbv, F2;
    SigmaField eta;
    void init(const Grid* g, int Ns) {
        bbu.init(g, FACE, CENTER); bbv.init(g, CENTER, FACE); F2.init(g, CENTER, CENTER);
        eta.init(g, CENTER, CENTER, Ns);
    }
    void zero() { bbu.zero(); bbv.zero(); F2.zero(); for (auto& f : eta.k) f.zero(); }
};

// One reverse sweep: seeds λ (halos filled) and the state outputs' adjoints sin; returns ȳ in G.x, C̄ in G.C,
// ∂J/∂log A in G.logA (all true adjoints) and the adjoints of the lagged state inputs in sout.
static void diva_sweep(Problem& P, const VelocityVector& lam, const DivaState& sin, DivaState& sout, AdjointSweep& G) {
    const Grid& g = P.grid;
    const Physics& ph = P.ph;
    const VelocityVector& xs = P.x;
    operator_sweep(P, lam, G);
    sout.zero();
    Field bbub = sin.bbu, bbvb = sin.bbv, F2b = sin.F2;
    VelocityVector ubb;
    ubb.init(&g);
    // β = βᵇ / (1 + βᵇ ℑF₂) over size(β); β̄ = -G.bu
    for (int j = 1; j <= P.bu.ny(); ++j)
        for (int i = 1; i <= P.bu.nx(); ++i) {
            double b = P.bbu(i, j), m = (P.F2(i - 1, j) + P.F2(i, j)) / 2, den = 1 + b * m;
            double gb = -G.bu(i, j);
            bbub(i, j) += gb / (den * den);
            double dm = gb * (-b * b / (den * den));
            F2b(i - 1, j) += dm / 2; F2b(i, j) += dm / 2;
        }
    for (int j = 1; j <= P.bv.ny(); ++j)
        for (int i = 1; i <= P.bv.nx(); ++i) {
            double b = P.bbv(i, j), m = (P.F2(i, j - 1) + P.F2(i, j)) / 2, den = 1 + b * m;
            double gb = -G.bv(i, j);
            bbvb(i, j) += gb / (den * den);
            double dm = gb * (-b * b / (den * den));
            F2b(i, j - 1) += dm / 2; F2b(i, j) += dm / 2;
        }
    fill_halo_adjoint(F2b);
    // column integrals and the Glen law with the lagged shear: η̄H = μ H Σ ησₖ Δζₖ, F₂ = H Σ w₂ₖ / ησₖ,
    // ησₖ = ½ Aₖ^(-1/n) eeₖ^((1-n)/2n), eeₖ = ε̇ₑ²(x) + (τx aₖ)² + (τy aₖ)² + ε̇₀², aₖ = (1 - ζₖ) / 2ησ⁻ₖ,
    // τx = ℑxᶜ(βᵇᵘ uᵇ), τy = ℑyᶜ(βᵇᵛ vᵇ)
    double n = ph.n, p = (1 - n) / (2 * n);
    for (int j = 1; j <= g.Ny(); ++j)
        for (int i = 1; i <= g.Nx(); ++i) {
            double H = P.H(i, j);
            double eb = -G.eta(i, j) * H * (P.use_mask ? P.mu(i, j) : 1.0);
            double fb = F2b(i, j) * H;
            double tx = (P.bbu(i, j) * P.ub(i, j) + P.bbu(i + 1, j) * P.ub(i + 1, j)) / 2;
            double ty = (P.bbv(i, j) * P.vb(i, j) + P.bbv(i, j + 1) * P.vb(i, j + 1)) / 2;
            double e2 = effective_strain_rate2(g, i, j, xs.u, xs.v, ph.walls);
            double gS = 0, txb = 0, tyb = 0;
            for (int k = 1; k <= P.sigma.N; ++k) {
                double eta = P.eta_s.k[k - 1](i, j);
                double em = eta == 0.0 ? std::numeric_limits<double>::infinity() : eta;
                double zeta = P.sigma.zc(k);
                double exz = tx * (1 - zeta) / (2 * em), eyz = ty * (1 - zeta) / (2 * em);
                double ee = e2 + exz * exz + eyz * eyz + ph.eps0 * ph.eps0;
                double etab = sin.eta.k[k - 1](i, j) + eb * layer_thickness(P.sigma, k) + fb * (-layer_weight(P.sigma, k, 2) / (eta * eta));
                double eeb = etab * eta * p / ee;
                gS += eeb;
                double exzb = eeb * 2 * exz, eyzb = eeb * 2 * eyz;
                txb += exzb * (1 - zeta) / (2 * em);
                tyb += eyzb * (1 - zeta) / (2 * em);
                sout.eta.k[k - 1](i, j) = eta == 0.0 ? 0.0 : -(exzb * exz + eyzb * eyz) / em;
                G.logA.k[k - 1](i, j) = etab * (-eta / n);
            }
            strain_rate2_adjoint(g, xs, ph.walls, i, j, gS, G.x);
            bbub(i, j) += txb * P.ub(i, j) / 2; ubb.u(i, j) += txb * P.bbu(i, j) / 2;
            bbub(i + 1, j) += txb * P.ub(i + 1, j) / 2; ubb.u(i + 1, j) += txb * P.bbu(i + 1, j) / 2;
            bbvb(i, j) += tyb * P.vb(i, j) / 2; ubb.v(i, j) += tyb * P.bbv(i, j) / 2;
            bbvb(i, j + 1) += tyb * P.vb(i, j + 1) / 2; ubb.v(i, j + 1) += tyb * P.bbv(i, j + 1) / 2;
        }
    // βᵇ = φ drag(uᵇ): the drag reads the basal velocities
    fill_halo_adjoint(bbub);
    fill_halo_adjoint(bbvb);
    VelocityVector ubs;
    ubs.init(&g);
    ubs.u = P.ub;
    ubs.v = P.vb;
    basal_drag_adjoint(P, ubs, bbub, bbvb, ubb, G.C);
    fill_halo_adjoint(ubb.u);
    fill_halo_adjoint(ubb.v);
    // uᵇ = x / (1 + βᵇ⁻ ℑF₂⁻) over size(uᵇ)
    for (int j = 1; j <= P.ub.ny(); ++j)
        for (int i = 1; i <= P.ub.nx(); ++i) {
            double m = (P.F2(i - 1, j) + P.F2(i, j)) / 2, den = 1 + P.bbu(i, j) * m;
            double gub = ubb.u(i, j);
            G.x.u(i, j) += gub / den;
            double d = gub * (-P.ub(i, j) / den);
            sout.bbu(i, j) += d * m;
            sout.F2(i - 1, j) += d * P.bbu(i, j) / 2; sout.F2(i, j) += d * P.bbu(i, j) / 2;
        }
    for (int j = 1; j <= P.vb.ny(); ++j)
        for (int i = 1; i <= P.vb.nx(); ++i) {
            double m = (P.F2(i, j - 1) + P.F2(i, j)) / 2, den = 1 + P.bbv(i, j) * m;
            double gvb = ubb.v(i, j);
            G.x.v(i, j) += gvb / den;
            double d = gvb * (-P.vb(i, j) / den);
            sout.bbv(i, j) += d * m;
            sout.F2(i, j - 1) += d * P.bbv(i, j) / 2; sout.F2(i, j) += d * P.bbv(i, j) / 2;
        }
    fill_halo_adjoint(G.x.u);
    fill_halo_adjoint(G.x.v);
    fill_halo_adjoint(G.C);
}

// nk_picard_adjoint.  xbar (interior layout of u, v) = ∂J/∂x*; lam receives λ = ∂J/∂τ, gradC ∂J/∂log C per
// cell, gradA ∂J/∂log A in the rate factor's layout (2-D: summed over the layers that share it).  The SSA sweep is
// λ-signed (ȳ = -G.x), the DIVA sweep true (ȳ = G.x) and carries the lagged-state adjoint σ.
// sig_final (DIVA): the adjoint σ of the lagged state's outputs seeded into the final pass (the reverse rule's s̄ + sweep).
static int picard_adjoint(Problem& P, const VelocityVector& xbar, const nk_iteration_control& ctl, VelocityVector& lam,
                          Field& gradC, SigmaField& gradA, nk_solve_stats* st, const Field* eta_bar = nullptr,
                          DivaState* sig_final = nullptr) {
    const Grid& g = P.grid;
    const bool diva = P.stress_balance == NK_DIVA;
    const double sign = diva ? 1.0 : -1.0;
    fill_halo(P.x);
    update_coefficients(P);                   // c(x*)
    AdjointSweep G;
    G.init(&g, P.sigma.N);
    DivaState sig, sig_next;
    if (diva) { sig.init(&g, P.sigma.N); sig_next.init(&g, P.sigma.N); }
    auto sweep = [&] {
        fill_halo(lam);
        if (diva) {
            diva_sweep(P, lam, sig, sig_next, G);
            std::swap(sig, sig_next);
        } else {
            adjoint_sweep(P, lam, G, eta_bar);
        }
    };
    VelocityVector r, next;
    r.init(&g); next.init(&g);
    lam.init(&g);
    bool fixed = ctl.kind == NK_FIXED_ITERATIONS;
    int limit = fixed ? ctl.iterations : ctl.maxiter;
    int it = 0, status = NK_OK;
    double D = std::numeric_limits<double>::infinity(), M = 0.0;
    std::memset(st, 0, sizeof(*st));
    while (it < limit && (fixed || D > std::max(ctl.reltol * M, ctl.abstol))) {
        sweep();
        for (int j = 1; j <= r.u.ny(); ++j) for (int i = 1; i <= r.u.nx(); ++i) r.u(i, j) = xbar.u(i, j) + sign * G.x.u(i, j);
        for (int j = 1; j <= r.v.ny(); ++j) for (int i = 1; i <= r.v.nx(); ++i) r.v(i, j) = xbar.v(i, j) + sign * G.x.v(i, j);
        fill_halo(r);
        for (int j = 1; j <= lam.u.ny(); ++j) for (int i = 1; i <= lam.u.nx(); ++i) next.u(i, j) = lam.u(i, j);
        for (int j = 1; j <= lam.v.ny(); ++j) for (int i = 1; i <= lam.v.nx(); ++i) next.v(i, j) = lam.v(i, j);
        int cg_status = NK_OK;
        conjugate_gradient(P, next, r, st, &cg_status);   // next = A⁻ᵀ r from the previous λ (A is symmetric)
        if (cg_status == NK_NONFINITE) status = NK_NONFINITE;
        VelocityVector& d = r;                              // r is free again: Δ = ‖next - λ‖
        linear_combination(g, d, 1.0, next, -1.0, lam);
        D = std::sqrt(vector_dot(g, d, d));
        M = std::sqrt(vector_dot(g, next, next));
        for (int j = 1; j <= lam.u.ny(); ++j) for (int i = 1; i <= lam.u.nx(); ++i) lam.u(i, j) = next.u(i, j);
        for (int j = 1; j <= lam.v.ny(); ++j) for (int i = 1; i <= lam.v.nx(); ++i) lam.v(i, j) = next.v(i, j);
        ++it;
        if (!std::isfinite(D) || status == NK_NONFINITE) break;
    }
    if (diva && sig_final) *sig_final = sig;
    sweep();
    gradC.init(&g, CENTER, CENTER);
    for (int j = 1; j <= g.Ny(); ++j) for (int i = 1; i <= g.Nx(); ++i) gradC(i, j) = sign * P.C(i, j) * G.C(i, j);
    int planes = P.rate_layout == NK_RATE_FACTOR_SIGMA ? P.sigma.N : 1;
    gradA.init(&g, CENTER, CENTER, planes);
    for (int j = 1; j <= g.Ny(); ++j)
        for (int i = 1; i <= g.Nx(); ++i)
            for (int k = 1; k <= P.sigma.N; ++k) gradA.k[planes == 1 ? 0 : k - 1](i, j) += sign * G.logA.k[k - 1](i, j);
    st->picard_iterations = it;
    st->picard_change = D;
    st->picard_norm = M;
    // the reverse rule's warning (ext/NunatakEnzymeExt.jl:222): the stopping test unmet when maxiter ended it
    st->status = (!std::isfinite(D) || status == NK_NONFINITE) ? NK_NONFINITE
               : (!fixed && !(D <= std::max(ctl.reltol * M, ctl.abstol))) ? NK_NOT_CONVERGED : NK_OK;
    return st->status;
}

// ------------------------------------------------------------------------------------------------
// One energy step of EnthalpyThermodynamics (TEST INFRASTRUCTURE: no library counterpart yet).
// step_thermodynamics! / advance_enthalpy!, src/Thermodynamics/column_energy_solve.jl:26-78: the strain heating of
// the current velocities (strain_heating.jl:7-56), the layer volume fluxes (layer_transport.jl:34-44), the basal
// state (column_energy_solve.jl:127-146), one implicit tridiagonal system per column (:148-221), solved by the
// Thomas algorithm (Oceananigans' BatchedTridiagonalSolver in z: row k reads a[k-1] E[k-1] + b[k] E[k] +
// c[k] E[k+1] = f[k]), the basal water and drainage (:223-259), then the thermal diagnostics (:112-117).
// prm: the EnthalpyThermodynamics constants in the order of struct EnergyParams.
// ------------------------------------------------------------------------------------------------
struct EnergyParams {
    double k, c, L, beta, T0, Tr;              // conductivity, heat capacity, latent heat, Clausius-Clapeyron, melting, reference
    double temperate_ratio, blend, water_blend, min_thickness, drainage_fraction, max_drainage_rate;
    int coupled;                               // grounded_melt_coupling
};

static inline double unit_ramp(double x, double w) { return std::min(std::max(x / w, 0.0), 1.0); }   // enthalpy_conversions.jl:69

static void step_enthalpy(Problem& P, const EnergyParams& q, double dt) {
    const Grid& g = P.grid;
    const Sigma& sg = P.sigma;
    const int Ns = sg.N, Nx = g.Nx(), Ny = g.Ny();
    const double rho = P.ph.rho_i, ga = P.ph.g;
    const bool diva = P.stress_balance == NK_DIVA;
    const Field& bu = diva ? P.bbu : P.bu;   // basal_drag(::SSA) = (βᵘ, βᵛ), (::DIVA) = (βᵇᵘ, βᵇᵛ), column_energy_solve.jl:18-20
    const Field& bv = diva ? P.bbv : P.bv;
    auto Tpm = [&](double p) { return q.T0 - q.beta * p; };                                   // :6
    auto Epm = [&](double p) { return q.c * (Tpm(p) - q.Tr); };                               // :13
    auto enthalpy = [&](double T, double w, double p) { return q.c * (std::min(T, Tpm(p)) - q.Tr) + w * q.L; };   // :49-52
    auto water_fraction = [&](double E, double p) { return std::max(0.0, E - Epm(p)) / q.L; };   // :42
    auto thickness = [&](double H) { return std::max(H, q.min_thickness); };                 // column_thickness, :56
    auto layer_pressure = [&](int i, int j, int k) { return rho * ga * P.H(i, j) * (1 - sg.zc(k)); };   // :61-64
    auto diffusivity = [&](int i, int j, int k) {                                             // layer_diffusivity, :72-78
        double w = unit_ramp(P.E.k[k - 1](i, j) - Epm(layer_pressure(i, j, k)) + q.blend, q.blend);
        return q.k / q.c * (1 - w + w * q.temperate_ratio);
    };
    auto grounded_part = [&](int i, int j) { return P.grounding ? P.phi(i, j) : 1.0; };        // :118-119
    for (int k = 0; k < Ns; ++k) fill_halo(P.E.k[k]);
    for (Field* f : {&P.Hw, &P.gmelt, &P.G, &P.Ts, &P.To, &P.melt, &P.Hn}) fill_halo(*f);
    // fill_halo_regions!((basal_drag(...)..., uᵇ, vᵇ)) and ((uσ, vσ)), column_energy_solve.jl:28-29
    for (Field* f : {&P.ub, &P.vb, diva ? &P.bbu : &P.bu, diva ? &P.bbv : &P.bv}) fill_halo(*f);

    // strain heating Φ = 4 η ε̇ₑ² (membrane, without ε̇₀), plus τᵇ² w₂ₖ / Δζₖ / η for DIVA (strain_heating.jl:43-56)
    fill_halo(P.x);
    for_xy(Nx, Ny, [&](int i, int j) {
        double e2 = effective_strain_rate2(g, i, j, P.x.u, P.x.v, P.ph.walls);
        double tb2 = 0;
        if (diva) {
            auto sq = [](double a) { return a * a; };
            tb2 = (sq(P.bbu(i, j) * P.ub(i, j)) + sq(P.bbu(i + 1, j) * P.ub(i + 1, j))) / 2 +
                  (sq(P.bbv(i, j) * P.vb(i, j)) + sq(P.bbv(i, j + 1) * P.vb(i, j + 1))) / 2;
        }
        for (int k = 1; k <= Ns; ++k) {
            double eta = P.eta_s.k[k - 1](i, j);
            double phi = 4 * eta * e2;
            if (diva) phi += tb2 * layer_weight(sg, k, 2) / layer_thickness(sg, k) / (eta == 0.0 ? std::numeric_limits<double>::infinity() : eta);
            P.Phi.k[k - 1](i, j) = phi;
        }
    });

    // layer volume fluxes W (faces 1..Nσ+1 of each column), layer_transport.jl:8-44
    auto layer_u = [&](int i, int j, int k) { return g.peripheral_fc(i, j) ? 0.0 : P.us.k[k - 1](i, j); };
    auto layer_v = [&](int i, int j, int k) { return g.peripheral_cf(i, j) ? 0.0 : P.vs.k[k - 1](i, j); };
    auto upwind = [](double u, double cm, double cp) { return u > 0 ? cm : cp; };
    auto xvol = [&](int i, int j, int k) { double u = layer_u(i, j, k); return g.dy_c(j) * u * upwind(u, P.Hn(i - 1, j), P.Hn(i, j)); };
    auto yvol = [&](int i, int j, int k) { double v = layer_v(i, j, k); return g.dx_c(i) * v * upwind(v, P.Hn(i, j - 1), P.Hn(i, j)); };
    auto xenth = [&](int i, int j, int k) { return xvol(i, j, k) * upwind(P.us.k[k - 1](i, j), P.E.k[k - 1](i - 1, j), P.E.k[k - 1](i, j)); };
    auto yenth = [&](int i, int j, int k) { return yvol(i, j, k) * upwind(P.vs.k[k - 1](i, j), P.E.k[k - 1](i, j - 1), P.E.k[k - 1](i, j)); };
    for (int k = 1; k <= Ns; ++k) { fill_halo(P.us.k[k - 1]); fill_halo(P.vs.k[k - 1]); }

    std::vector<double> W((size_t)(Ns + 1) * Nx * Ny), rb((size_t)Nx * Ny), sb(rb.size()), Db(rb.size()), qg(rb.size());
    auto col = [&](int i, int j) { return (size_t)(j - 1) * Nx + (i - 1); };
    for_xy(Nx, Ny, [&](int i, int j) {
        double* w = &W[col(i, j) * (Ns + 1)];
        double dHdt = (thickness(P.H(i, j)) - thickness(P.Hn(i, j))) / dt;
        double m = P.grounding ? (1 - P.phi(i, j)) * P.melt(i, j) : P.melt(i, j);   // basal_melt, time_stepping.jl:51-52
        w[0] = -m - (q.coupled ? P.gmelt(i, j) : 0.0);
        for (int k = 1; k <= Ns; ++k) {
            double div = (xvol(i + 1, j, k) - xvol(i, j, k) + yvol(i, j + 1, k) - yvol(i, j, k)) / g.Az_ccc(i, j);
            w[k] = w[k - 1] - layer_thickness(sg, k) * (dHdt + div);
        }
        // basal state, column_energy_solve.jl:127-146
        double Ht = thickness(P.H(i, j));
        double D = diffusivity(i, j, 1) / (Ht * sg.zc(1));
        double F = (bu(i, j) * P.ub(i, j) * P.ub(i, j) + bu(i + 1, j) * P.ub(i + 1, j) * P.ub(i + 1, j) +
                    bv(i, j) * P.vb(i, j) * P.vb(i, j) + bv(i, j + 1) * P.vb(i, j + 1) * P.vb(i, j + 1)) / 2;
        double Epm_b = Epm(rho * ga * P.H(i, j));
        double Eb = P.E.k[0](i, j) + (P.G(i, j) + F) / D;
        double r = std::max(unit_ramp(Eb - Epm_b, q.blend), unit_ramp(P.Hw(i, j), q.water_blend));
        double E1pm = Epm(layer_pressure(i, j, 1));
        Db[col(i, j)] = D;
        rb[col(i, j)] = r;
        sb[col(i, j)] = unit_ramp(P.E.k[0](i, j) - E1pm + q.blend, q.blend);
        P.sb(i, j) = sb[col(i, j)];
        qg[col(i, j)] = grounded_part(i, j) * P.G(i, j) + F;
        P.qg(i, j) = qg[col(i, j)];
    });

    // the column systems (from the old E), then the Thomas solve into E
    std::vector<double> a((size_t)Ns * Nx * Ny), b(a.size()), cc(a.size()), f(a.size());
    for_xy(Nx, Ny, [&](int i, int j) {
        size_t o = col(i, j) * Ns;
        const double* w = &W[col(i, j) * (Ns + 1)];
        double Ht = thickness(P.H(i, j)), Hnt = thickness(P.Hn(i, j));
        bool mu = P.H(i, j) > q.min_thickness;                                   // column_has_ice, :58
        double Es = enthalpy(P.Ts(i, j), 0.0, 0.0);                              // surface_enthalpy, :54
        double phi = grounded_part(i, j), r = rb[col(i, j)];
        double chi = phi * r * (1 - sb[col(i, j)]);
        double pb = rho * ga * P.H(i, j);
        double Epm_b = Epm(pb), Eo = enthalpy(P.To(i, j), 0.0, pb);
        double Fb = rho * w[0];
        double Lam = Db[col(i, j)] * (chi + 1 - phi) + std::max(-Fb, 0.0);
        double S = (1 - r) * qg[col(i, j)] + Db[col(i, j)] * (chi * Epm_b + (1 - phi) * Eo) + std::max(Fb, 0.0) * Epm_b;
        double Fs = rho * w[Ns];
        double Ks = diffusivity(i, j, Ns) / (Ht * (1 - sg.zc(Ns)));             // surface_conductance, :160-165
        double Ds = Ks + std::max(Fs, 0.0), Ss = (Ks + std::max(-Fs, 0.0)) * Es;
        auto couplings = [&](int kf, double& lower, double& upper) {            // face_couplings, :169-177, interior face kf
            double zf = sg.zf(kf), zm = sg.zc(kf - 1), zp = sg.zc(kf);
            double theta = (zf - zm) / (zp - zm);
            double Fk = rho * w[kf - 1];
            double cond = 1 / (Ht * ((zf - zm) / diffusivity(i, j, kf - 1) + (zp - zf) / diffusivity(i, j, kf)));   // face_conductance
            double Dk = std::max(cond, std::max(std::max(Fk, 0.0) * theta, std::max(-Fk, 0.0) * (1 - theta)));
            lower = -Fk * (1 - theta) - Dk;
            upper = Fk * theta - Dk;
        };
        for (int k = 1; k <= Ns; ++k) {
            double dz = layer_thickness(sg, k);
            double lower_m = 0, upper_m = 0, lower_p = 0, upper_p = 0;
            if (k > 1) couplings(k, lower_m, upper_m);
            if (k < Ns) couplings(k + 1, lower_p, upper_p);
            double diag_m = k == 1 ? Lam : -upper_m;
            double diag_p = k == Ns ? Ds : -lower_p;
            double forcing = (k == 1 ? S : 0.0) + (k == Ns ? Ss : 0.0);
            double transport = rho * dz * ((xenth(i + 1, j, k) - xenth(i, j, k) + yenth(i, j + 1, k) - yenth(i, j, k)) / g.Az_ccc(i, j));
            a[o + k - 1] = mu ? lower_p : 0.0;
            cc[o + k - 1] = mu ? upper_p : 0.0;
            b[o + k - 1] = mu ? rho * Ht * dz / dt + diag_m + diag_p : 1.0;
            f[o + k - 1] = mu ? rho * Hnt * dz * P.E.k[k - 1](i, j) / dt - transport + Ht * dz * P.Phi.k[k - 1](i, j) + forcing : Es;
        }
    });
    for_xy(Nx, Ny, [&](int i, int j) {                                          // Thomas algorithm, top-down then back
        size_t o = col(i, j) * Ns;
        std::vector<double> t(Ns + 1, 0.0), e(Ns + 1, 0.0);
        double beta_ = b[o];
        e[1] = f[o] / beta_;
        for (int k = 2; k <= Ns; ++k) {
            t[k] = cc[o + k - 2] / beta_;
            beta_ = b[o + k - 1] - a[o + k - 2] * t[k];
            e[k] = (f[o + k - 1] - a[o + k - 2] * e[k - 1]) / beta_;
        }
        for (int k = Ns - 1; k >= 1; --k) e[k] -= t[k + 1] * e[k + 1];
        for (int k = 1; k <= Ns; ++k) P.E.k[k - 1](i, j) = e[k];
    });

    // basal water and drainage, column_energy_solve.jl:223-259 (no till: drain_till leaves Hw)
    for_xy(Nx, Ny, [&](int i, int j) {
        double Ht = thickness(P.H(i, j));
        bool mu = P.H(i, j) > q.min_thickness;
        double Epm_b = Epm(rho * ga * P.H(i, j));
        double qb = Db[col(i, j)] * (Epm_b - P.E.k[0](i, j));
        double m = rb[col(i, j)] * (qg[col(i, j)] - grounded_part(i, j) * (1 - sb[col(i, j)]) * qb) / (rho * q.L);
        double drained = 0;
        for (int k = 1; k <= Ns; ++k) {
            double w = water_fraction(P.E.k[k - 1](i, j), layer_pressure(i, j, k));
            double x = w / q.drainage_fraction;                                   // drainage_rate, :212-216
            double rate = q.max_drainage_rate * (std::min(std::max(x - 1, 0.0), 1.0) / 10 + 9 * std::min(std::max(x - 2, 0.0), 1.0) / 10);
            double dw = std::min(dt * rate, std::max(w - q.drainage_fraction, 0.0));
            dw = mu ? dw : 0.0;
            P.E.k[k - 1](i, j) -= q.L * dw;
            drained += Ht * layer_thickness(sg, k) * dw;
        }
        double Hstar = P.Hw(i, j) + dt * (mu ? m : 0.0) + drained;
        double Hplus = std::max(0.0, Hstar);
        double missing = Hplus - Hstar;
        P.gmelt(i, j) = (Hplus - P.Hw(i, j)) / dt;
        // drain_till, till_effective_pressure.jl:76-77: the till drains and holds at most its maximum water
        P.Hw(i, j) = P.till.enabled ? std::min(std::max(Hplus - dt * P.till.drainage_rate, 0.0), P.till.maximum_water_thickness) : Hplus;
        P.E.k[0](i, j) -= q.L * missing / (Ht * layer_thickness(sg, 1));
    });

    // thermal diagnostics (T and the water fraction), and Hⁿ = H
    for (int k = 1; k <= Ns; ++k)
        for_xy(Nx, Ny, [&](int i, int j) {
            double p = layer_pressure(i, j, k), E = P.E.k[k - 1](i, j);
            P.T.k[k - 1](i, j) = std::min(Tpm(p), q.Tr + E / q.c);
            P.omega.k[k - 1](i, j) = water_fraction(E, p);
        });
    for_xy(Nx, Ny, [&](int i, int j) { P.Hn(i, j) = P.H(i, j); });
    for (int k = 0; k < Ns; ++k) { fill_halo(P.E.k[k]); fill_halo(P.T.k[k]); fill_halo(P.omega.k[k]); }
    for (Field* f : {&P.Hw, &P.gmelt, &P.Hn}) fill_halo(*f);
}

// ------------------------------------------------------------------------------------------------
// Thickness advection (the face thickness that u H carries through a face).  The reference takes it from
// Oceananigans 0.117's UpwindBiased and WENO schemes (src/Models/time_stepping.jl:59-63 through div_Uc), which are
// not vendored; this restates their published algorithms.  s(m), m = -2..2, is the thickness m cells away from the
// upwind cell s(0) of the face, m > 0 towards the face and beyond (downwind).  Stored as s[m + 2].
// ------------------------------------------------------------------------------------------------
// UpwindBiased(order = 3): the third-order upwind-biased interpolation.
static double upwind3_face(const double* s) { return (-s[1] + 5 * s[2] + 2 * s[3]) / 6; }

// WENO(order = 5): the three third-order candidates on the stencils (-2..0), (-1..1), (0..2), their Jiang-Shu
// smoothness indicators β and the WENO-Z weights α_k = d_k (1 + τ / (β_k + ε)), τ = |β₀ - β₂|, ε = 1e-8, with
// the optimal weights d = (1, 6, 3) / 10 (Jiang and Shu 1996; Borges, Carmona, Costa and Don 2008).
static double weno5_face(const double* s) {
    const double a = s[0], b = s[1], c = s[2], d = s[3], e = s[4];
    double q0 = (2 * a - 7 * b + 11 * c) / 6;
    double q1 = (-b + 5 * c + 2 * d) / 6;
    double q2 = (2 * c + 5 * d - e) / 6;
    double b0 = 13.0 / 12 * (a - 2 * b + c) * (a - 2 * b + c) + 0.25 * (a - 4 * b + 3 * c) * (a - 4 * b + 3 * c);
    double b1 = 13.0 / 12 * (b - 2 * c + d) * (b - 2 * c + d) + 0.25 * (b - d) * (b - d);
    double b2 = 13.0 / 12 * (c - 2 * d + e) * (c - 2 * d + e) + 0.25 * (3 * c - 4 * d + e) * (3 * c - 4 * d + e);
    const double eps = 1e-8;
    double tau = std::fabs(b0 - b2);
    double r0 = tau / (b0 + eps), r1 = tau / (b1 + eps), r2 = tau / (b2 + eps);
    double a0 = 0.1 * (1 + r0), a1 = 0.6 * (1 + r1), a2 = 0.3 * (1 + r2);
    return (a0 * q0 + a1 * q1 + a2 * q2) / (a0 + a1 + a2);
}

// The unlimited face value of the scheme from the stencil s.
static double face_value(const nk_advection_desc& adv, const double* s) {
    if (adv.scheme == NK_ADVECTION_WENO) return weno5_face(s);
    return adv.order == 3 ? upwind3_face(s) : s[2];
}

// Stencils of the upwind cell ic of face f along x (ic = f - 1 when the flow is eastward: s(m) = H(f - 1 + m);
// ic = f when westward: s(m) = H(f - m)) and likewise along y, from the halo-filled stage thickness.
static void x_stencil(const Field& H, int f, int j, bool east, double* s) {
    for (int m = -2; m <= 2; ++m) s[m + 2] = east ? H(f - 1 + m, j) : H(f - m, j);
}
static void y_stencil(const Field& H, int i, int f, bool north, double* s) {
    for (int m = -2; m <= 2; ++m) s[m + 2] = north ? H(i, f - 1 + m) : H(i, f - m);
}

// The bounds-preserving limiter θ of cell (i, j) (Zhang and Shu 2010, applied per direction): with the cell's own
// face values W, E (x) and S, N (y), each direction's interior quadrature value p̃ = (H̄ - ω(W + E)) / (1 - 2ω),
// ω = 5/18, and M, m the largest and smallest of the six, θ = min(1, |(upper - H̄) / (M - H̄ + ε)|,
// |(lower - H̄) / (m - H̄ - ε)|), ε = 2 eps; the limited face value is H̄ + θ (face - H̄).
static double bounds_limiter(const nk_advection_desc& adv, const Field& H, int i, int j) {
    double s[5], Hc = H(i, j);
    x_stencil(H, i + 1, j, true, s);
    double E = weno5_face(s);
    x_stencil(H, i, j, false, s);
    double W = weno5_face(s);
    y_stencil(H, i, j + 1, true, s);
    double N = weno5_face(s);
    y_stencil(H, i, j, false, s);
    double S = weno5_face(s);
    const double w = 5.0 / 18, eps = 2 * std::numeric_limits<double>::epsilon();
    double px = (Hc - w * W - w * E) / (1 - 2 * w);
    double py = (Hc - w * S - w * N) / (1 - 2 * w);
    double M = std::max(std::max(std::max(px, py), std::max(W, E)), std::max(S, N));
    double m = std::min(std::min(std::min(px, py), std::min(W, E)), std::min(S, N));
    return std::min(std::min(std::fabs((adv.upper - Hc) / (M - Hc + eps)), std::fabs((adv.lower - Hc) / (m - Hc - eps))), 1.0);
}

// ------------------------------------------------------------------------------------------------
// Partial-cell front (PartialCellFront, src/Models/partial_cell_front.jl) and calving (src/Models/calving.jl).
// μ (P.mu) is the prognostic 0/1 flag of full cells, Hʳ (P.Hr) the ice thickness of a partial front cell, which covers
// the fraction H / Hʳ of its area.  Halo cells of a Bounded direction are inactive; periodic halos wrap.
// ------------------------------------------------------------------------------------------------
static inline bool full_cell(const Problem& P, int i, int j) { return P.mu(i, j) > 0; }                          // :101
static inline bool full_neighbor(const Problem& P, int i, int j) { return full_cell(P, i, j) && !P.grid.inactive_cell(i, j); }   // :102
static inline bool empty_cell(const Problem& P, const Field& H, int i, int j) {                                   // :103
    return !full_cell(P, i, j) && H(i, j) <= 0 && !P.grid.inactive_cell(i, j);
}

// initialize_front!, :80-92: every cell holding ice is full, none is partial.
static void initialize_front(Problem& P) {
    for_xy(P.grid.Nx(), P.grid.Ny(), [&](int i, int j) {
        P.mu(i, j) = P.H(i, j) > 0 ? 1.0 : 0.0;
        P.Hr(i, j) = 0.0;
    });
    fill_halo(P.mu);
    fill_halo(P.Hr);
}

// front_ice_thickness, :331: its own thickness when full or not yet given an Hʳ.
static inline double front_ice_thickness(const Problem& P, int i, int j) {
    return (full_cell(P, i, j) || P.Hr(i, j) <= 0) ? P.H(i, j) : P.Hr(i, j);
}

// remove_front_fraction!, :353-368: remove the fraction g of the cell's area; returns the part of g beyond its ice.
static double remove_front_fraction(Problem& P, int i, int j, double g) {
    double Hi = P.H(i, j), Hf = front_ice_thickness(P, i, j);
    bool calves = (g > 0) && (Hi > 0);
    double Hn = std::max(Hi - g * Hf, 0.0);
    double a = Hf > 0 ? Hi / (Hf > 0 ? Hf : 1.0) : 0.0;
    if (calves) {
        P.calved(i, j) += Hi - Hn;
        P.H(i, j) = Hn;
        P.Hr(i, j) = Hn > 0 ? Hf : 0.0;
        P.mu(i, j) = 0.0;
    }
    return calves ? std::max(g - a, 0.0) : 0.0;
}

// principal_strain_rates, calving.jl:144-152, with the velocities masked by μ (interior_u / interior_v with μ)
static void principal_strain_rates(const Problem& P, int i, int j, double& e1, double& e2) {
    const Grid& g = P.grid;
    const Field* mu = &P.mu;
    double exx = strain_rate_xx(g, i, j, P.x.u, mu), eyy = strain_rate_yy(g, i, j, P.x.v, mu);
    // ℑxyᶜᶜᵃ = ℑyᵃᶜᵃ(ℑxᶜᵃᵃ(·)) of the corner shear
    double exy = ((strain_rate_xy(g, i, j, P.x.u, P.x.v, P.ph.walls, mu) + strain_rate_xy(g, i + 1, j, P.x.u, P.x.v, P.ph.walls, mu)) / 2 +
                  (strain_rate_xy(g, i, j + 1, P.x.u, P.x.v, P.ph.walls, mu) + strain_rate_xy(g, i + 1, j + 1, P.x.u, P.x.v, P.ph.walls, mu)) / 2) / 2;
    double eb = (exx + eyy) / 2;
    double r = std::sqrt(((exx - eyy) / 2) * ((exx - eyy) / 2) + exy * exy + P.ph.eps0 * P.ph.eps0);
    e1 = eb + r;
    e2 = eb - r;
}

// front_flow_speed, calving.jl:176-181: the larger face speed along each axis.
static double front_flow_speed(const Problem& P, int i, int j) {
    const Grid& g = P.grid;
    double ut = std::max(std::fabs(interior_u(g, i, j, P.x.u, &P.mu)), std::fabs(interior_u(g, i + 1, j, P.x.u, &P.mu)));
    double vt = std::max(std::fabs(interior_v(g, i, j, P.x.v, &P.mu)), std::fabs(interior_v(g, i, j + 1, P.x.v, &P.mu)));
    double e = P.ph.eps0 * g.dx_c(i);
    return std::sqrt(ut * ut + vt * vt + e * e);
}

// calving_rate of a full cell, calving.jl:154-190
static double calving_rate(const Problem& P, int i, int j) {
    const nk_front_desc& law = P.front;
    if (law.calving == NK_CALVING_EIGEN) {
        double e1, e2;
        principal_strain_rates(P, i, j, e1, e2);
        return law.coefficient * std::max(e1, 0.0) * std::max(e2, 0.0);
    }
    if (law.calving == NK_CALVING_VON_MISES) {
        double e1, e2;
        principal_strain_rates(P, i, j, e1, e2);
        double n = P.ph.n, e0 = P.ph.eps0;
        double et2 = (std::max(e1, 0.0) * std::max(e1, 0.0) + std::max(e2, 0.0) * std::max(e2, 0.0)) / 2;
        double ee2 = effective_strain_rate2(P.grid, i, j, P.x.u, P.x.v, P.ph.walls) + e0 * e0;
        double Hi = P.H(i, j);
        double eta = P.etaH(i, j) / (Hi > 0 ? Hi : 1.0);
        double smax = P.phi(i, j) * law.stress_threshold + (1 - P.phi(i, j)) * law.floating_stress_threshold;
        double B = 2 * eta * std::pow(ee2, (n - 1) / (2 * n));
        double sig = std::sqrt(3.0) * B * et2 * std::pow(et2 + e0 * e0, (1 - 2 * n) / (2 * n));
        return front_flow_speed(P, i, j) * sig / smax;
    }
    if (law.calving == NK_CALVING_FRONT_VELOCITY) {
        double c = std::max(front_flow_speed(P, i, j) - law.front_velocity, 0.0);
        return (1 - P.phi(i, j)) * c;
    }
    return 0.0;
}

// front_calving_rate, calving.jl:197-206: a partial cell takes the mean rate of its full neighbours.
static double front_calving_rate(const Problem& P, int i, int j) {
    if (full_cell(P, i, j)) return calving_rate(P, i, j);
    double S = 0;
    int n = 0;
    const int di[4] = {-1, 1, 0, 0}, dj[4] = {0, 0, -1, 1};
    for (int k = 0; k < 4; ++k)
        if (full_neighbor(P, i + di[k], j + dj[k])) { S += calving_rate(P, i + di[k], j + dj[k]); ++n; }
    return S / std::max(n, 1);
}

// calve_front!, partial_cell_front.jl:276-296, with _compute_retreat_fraction!, _retreat_front_cells!,
// _share_residual_retreat! and _receive_residual_retreat! (:311-389) and retreat_fraction (calving.jl:212-227).
static void calve_front(Problem& P, double dt) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny();
    const int law = P.front.calving;
    fill_halo(P.bed);
    Field f(&g, CENTER, CENTER);
    // the retreat fraction of each front cell, from the state before any cell retreats
    for_xy(Nx, Ny, [&](int i, int j) {
        double dx = g.dx_c(i), dy = g.dy_c(j);
        auto ocean = [&](int a, int b, double len) { return (empty_cell(P, P.H, a, b) && P.bed(a, b) < 0) ? len : 0.0; };
        double lw = ocean(i - 1, j, dy), le = ocean(i + 1, j, dy), ls = ocean(i, j - 1, dx), ln = ocean(i, j + 1, dx);
        // front_length, :334-343
        double ub = std::fabs((interior_u(g, i, j, P.x.u, &P.mu) + interior_u(g, i + 1, j, P.x.u, &P.mu)) / 2);
        double vb = std::fabs((interior_v(g, i, j, P.x.v, &P.mu) + interior_v(g, i, j + 1, P.x.v, &P.mu)) / 2);
        double speed = std::sqrt(ub * ub + vb * vb);
        double l2 = (le - lw) * (le - lw) + (ln - ls) * (ln - ls);
        double lv = l2 > 0 ? std::sqrt(l2 > 0 ? l2 : 1.0) : lw + le + ls + ln;
        double lu = (ub * (lw + le) + vb * (ls + ln)) / (speed > 0 ? speed : 1.0);
        double l = speed > 0 ? lu : lv;
        double Hf = front_ice_thickness(P, i, j);
        bool front = P.H(i, j) > 0 && (lw + le + ls + ln > 0);
        double r = 0;
        if (front) {
            if (law == NK_CALVING_THICKNESS_THRESHOLD) r = Hf < P.front.thickness ? 1.0 : 0.0;
            else if (law == NK_CALVING_MAXIMUM_EXTENT) r = P.extent(i, j) > 0 ? 0.0 : 1.0;
            else r = std::min(1.0, front_calving_rate(P, i, j) * dt * l / g.Az_ccc(i, j));
        }
        f(i, j) = r;
    });
    // retreat (each cell changes only itself), then the area a cell could not take (rate laws only)
    const bool removal = law == NK_CALVING_THICKNESS_THRESHOLD || law == NK_CALVING_MAXIMUM_EXTENT;
    for (int j = 1; j <= Ny; ++j)
        for (int i = 1; i <= Nx; ++i) {
            double r = remove_front_fraction(P, i, j, f(i, j));
            f(i, j) = (removal ? 0.0 : r) * g.Az_ccc(i, j);
        }
    fill_halo(f);
    fill_halo(P.H);
    // _share_residual_retreat!: among the neighbours that hold ice
    Field share(&g, CENTER, CENTER);
    for_xy(Nx, Ny, [&](int i, int j) {
        auto ice = [&](int a, int b) { return (!g.inactive_cell(a, b) && P.H(a, b) > 0) ? 1 : 0; };
        int n = ice(i - 1, j) + ice(i + 1, j) + ice(i, j - 1) + ice(i, j + 1);
        share(i, j) = n > 0 ? f(i, j) / std::max(n, 1) : 0.0;
    });
    fill_halo(share);
    // _receive_residual_retreat!: what the receiving cell cannot take is not passed on
    Field A(&g, CENTER, CENTER);
    for_xy(Nx, Ny, [&](int i, int j) {
        auto area = [&](int a, int b) { return g.inactive_cell(a, b) ? 0.0 : share(a, b); };
        A(i, j) = area(i - 1, j) + area(i + 1, j) + area(i, j - 1) + area(i, j + 1);
    });
    for (int j = 1; j <= Ny; ++j)
        for (int i = 1; i <= Nx; ++i) remove_front_fraction(P, i, j, A(i, j) / g.Az_ccc(i, j));
    fill_halo(P.mu);
    fill_halo(P.Hr);
    fill_halo(P.H);
}

// advance_front!(front, model, Δt), partial_cell_front.jl:167-195.
static void advance_front(Problem& P, double dt, bool coupled) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny();
    fill_halo(P.H);
    for_xy(Nx, Ny, [&](int i, int j) { if (P.H(i, j) <= 0) P.mu(i, j) = 0.0; });          // _empty_drained_cells!, :197-200
    fill_halo(P.mu);
    fill_halo(P.x);
    // _compute_reference_thickness!, :206-230
    {
        Field Hr0 = P.Hr;
        for_xy(Nx, Ny, [&](int i, int j) {
            bool west = P.x.u(i, j) > 0, east = P.x.u(i + 1, j) < 0, south = P.x.v(i, j) > 0, north = P.x.v(i, j + 1) < 0;
            auto donor = [&](int a, int b, bool inflow) { return (inflow && full_neighbor(P, a, b)) ? P.H(a, b) : 0.0; };
            auto count = [&](int a, int b, bool inflow) { return (inflow && full_neighbor(P, a, b)) ? 1 : 0; };
            double Sin = donor(i - 1, j, west) + donor(i + 1, j, east) + donor(i, j - 1, south) + donor(i, j + 1, north);
            int nin = count(i - 1, j, west) + count(i + 1, j, east) + count(i, j - 1, south) + count(i, j + 1, north);
            double Sf = donor(i - 1, j, true) + donor(i + 1, j, true) + donor(i, j - 1, true) + donor(i, j + 1, true);
            int nf = count(i - 1, j, true) + count(i + 1, j, true) + count(i, j - 1, true) + count(i, j + 1, true);
            double Hi = P.H(i, j);
            double Hs = nf > 0 ? Sf / std::max(nf, 1) : Hi;
            double Hp = Hi > 0 ? (Hr0(i, j) > 0 ? Hr0(i, j) : Hs) : 0.0;
            double Hbar = nin > 0 ? Sin / std::max(nin, 1) : Hp;
            P.Hr(i, j) = full_cell(P, i, j) ? 0.0 : Hbar;
        });
        fill_halo(P.Hr);
    }
    // overflow passes: _fill_front_cells! then _receive_overflow!, :235-268
    for (int pass = 0; pass < P.front.passes; ++pass) {
        Field H0 = P.H, mu0 = P.mu;
        for_xy(Nx, Ny, [&](int i, int j) {
            auto empty0 = [&](int a, int b) {
                return (!(mu0(a, b) > 0) && H0(a, b) <= 0 && !g.inactive_cell(a, b)) ? 1 : 0;
            };
            int n = empty0(i - 1, j) + empty0(i + 1, j) + empty0(i, j - 1) + empty0(i, j + 1);
            double Hi = H0(i, j), Hri = P.Hr(i, j);
            bool fills = !(mu0(i, j) > 0) && (Hri > 0) && (Hi >= Hri);
            bool spills = fills && n > 0;
            P.O(i, j) = spills ? (Hi - Hri) * g.Az_ccc(i, j) / std::max(n, 1) : 0.0;
            P.H(i, j) = spills ? Hri : Hi;
            if (fills) P.mu(i, j) = 1.0;
        });
        fill_halo(P.mu);
        fill_halo(P.O);
        fill_halo(P.H);
        Field H1 = P.H;
        for_xy(Nx, Ny, [&](int i, int j) {
            bool receives = empty_cell(P, H1, i, j);
            auto vol = [&](int a, int b) { return g.inactive_cell(a, b) ? 0.0 : P.O(a, b); };
            auto donor = [&](int a, int b) { return !g.inactive_cell(a, b) && P.O(a, b) > 0; };
            double V = vol(i - 1, j) + vol(i + 1, j) + vol(i, j - 1) + vol(i, j + 1);
            double S = (donor(i - 1, j) ? H1(i - 1, j) : 0.0) + (donor(i + 1, j) ? H1(i + 1, j) : 0.0) +
                       (donor(i, j - 1) ? H1(i, j - 1) : 0.0) + (donor(i, j + 1) ? H1(i, j + 1) : 0.0);
            int n = donor(i - 1, j) + donor(i + 1, j) + donor(i, j - 1) + donor(i, j + 1);
            if (receives) P.H(i, j) = V / g.Az_ccc(i, j);
            if (receives && n > 0) P.Hr(i, j) = S / std::max(n, 1);
        });
        fill_halo(P.H);
        fill_halo(P.Hr);
    }
    if (P.front.calving != NK_CALVING_NONE) calve_front(P, dt);
    // _force_front_cells!, :271-286
    for_xy(Nx, Ny, [&](int i, int j) {
        double Hi = P.H(i, j), Hri = P.Hr(i, j);
        double m = P.grounding ? (1 - P.phi(i, j)) * P.melt(i, j) : P.melt(i, j);
        double S = P.smb(i, j) - m - (coupled ? P.gmelt(i, j) : 0.0);
        bool full = full_cell(P, i, j);
        bool forced = (Hi > 0) && (Hri > 0);
        double Hf = full ? Hi : Hri;
        bool melted = forced && (Hf + S * dt <= 0);
        double Hn = full ? Hi + S * dt : Hi / (Hri > 0 ? Hri : 1.0) * (Hri + S * dt);
        if (melted) P.clipped(i, j) += -Hn;
        P.H(i, j) = melted ? 0.0 : (forced ? Hn : Hi);
        P.Hr(i, j) = (melted || full) ? 0.0 : (forced ? Hri + S * dt : Hri);
        if (melted) P.mu(i, j) = 0.0;
    });
    fill_halo(P.mu);
    fill_halo(P.Hr);
    fill_halo(P.H);
}

// ------------------------------------------------------------------------------------------------
// One ice time step of the thickness, time_stepping.jl:15-72: three split Runge-Kutta stages
// H = max(0, H⁻ + Δτ G(H)) from the thickness H⁻ at the start of the step, with Δτ = Δt/3, Δt/2, Δt (Oceananigans
// 0.117's SplitRungeKutta3, the Wicker-Skamarock scheme), the thickness added by the clip in the last stage
// accumulated in `clipped`, and the geometry updated after every stage (update_state!).
// G = a - (1 - φ) m - mᵍ - ∇⋅(ū H), the flux through a face Δ (u H_face) with H_face the scheme's upwind-biased face
// thickness (the limited one for a bounded WENO, whose limiter is recomputed from the stage's thickness first,
// update_bounds_preserving_limiter!, :35-42, also in the first halo layer); Bounded walls pass nothing.  The
// velocities are held (no velocity solve).
// ------------------------------------------------------------------------------------------------
static void compute_geometry(Problem& P);

// The tendency and the substep of stage st (0, 1, 2) of one thickness step (rk_substep! before the front's advance);
// stage 0 records the step's starting thickness, which every stage starts from.
static void thickness_substep(Problem& P, double dt, int st, bool coupled) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny();
    const nk_advection_desc adv = P.advection;
    const bool bounded = adv.scheme == NK_ADVECTION_WENO && adv.bounded;
    fill_halo(P.x);
    for (Field* f : {&P.smb, &P.melt, &P.gmelt, &P.clipped}) fill_halo(*f);
    if (st == 0) P.H_step0 = P.H;
    Field& H0 = P.H_step0;
    Field Gt(&g, CENTER, CENTER);
    if (bounded && !P.theta.g) P.theta.init(&g, CENTER, CENTER);
    const double stages[3] = {1.0 / 3, 1.0 / 2, 1.0};
    {
        fill_halo(P.H);
        if (bounded) {
#pragma omp parallel for schedule(static)
            for (int j = 0; j <= Ny + 1; ++j)
                for (int i = 0; i <= Nx + 1; ++i) P.theta(i, j) = bounds_limiter(adv, P.H, i, j);
        }
        auto limited = [&](double v, int ic, int jc) { return bounded ? P.H(ic, jc) + P.theta(ic, jc) * (v - P.H(ic, jc)) : v; };
        // with a PartialCellFront (front_flux_x / front_flux_y, partial_cell_front.jl:114-132): the scheme's flux
        // between full cells, the upwind flux out of a full cell into a front cell, nothing out of a front cell
        const bool front = P.front.enabled != 0;
        auto xflux = [&](int i, int j) {
            if (g.peripheral_fc(i, j)) return 0.0;
            double u = P.x.u(i, j), s[5];
            bool west = !front || full_cell(P, i - 1, j), eastc = !front || full_cell(P, i, j);
            if (!(west && eastc))
                return (west || eastc) ? g.dy_c(j) * (west ? std::max(u, 0.0) * P.H(i - 1, j) : std::min(u, 0.0) * P.H(i, j)) : 0.0;
            bool east = u > 0;
            x_stencil(P.H, i, j, east, s);
            double h = limited(face_value(adv, s), east ? i - 1 : i, j);
            return g.dy_c(j) * (u * h);
        };
        auto yflux = [&](int i, int j) {
            if (g.peripheral_cf(i, j)) return 0.0;
            double v = P.x.v(i, j), s[5];
            bool south = !front || full_cell(P, i, j - 1), northc = !front || full_cell(P, i, j);
            if (!(south && northc))
                return (south || northc) ? g.dx_c(i) * (south ? std::max(v, 0.0) * P.H(i, j - 1) : std::min(v, 0.0) * P.H(i, j)) : 0.0;
            bool north = v > 0;
            y_stencil(P.H, i, j, north, s);
            double h = limited(face_value(adv, s), i, north ? j - 1 : j);
            return g.dx_c(i) * (v * h);
        };
        for_xy(Nx, Ny, [&](int i, int j) {   // _compute_thickness_tendency!, :59-63 (sources on full cells only)
            double m = P.grounding ? (1 - P.phi(i, j)) * P.melt(i, j) : P.melt(i, j);
            double S = P.smb(i, j) - m - (coupled ? P.gmelt(i, j) : 0.0);
            if (front && !full_cell(P, i, j)) S = 0.0;
            double div = (xflux(i + 1, j) - xflux(i, j) + yflux(i, j + 1) - yflux(i, j)) / g.Az_ccc(i, j);
            Gt(i, j) = S - div;
        });
        double dtau = stages[st] * dt;
        bool final_stage = st == 2;
        for_xy(Nx, Ny, [&](int i, int j) {   // _thickness_substep!, :65-72
            double Hs = H0(i, j) + dtau * Gt(i, j);
            P.H(i, j) = std::max(0.0, Hs);
            if (final_stage) P.clipped(i, j) += std::max(0.0, -Hs);
        });
        fill_halo(P.H);
    }
}

// Stage st (0, 1, 2) of one thickness step: rk_substep! (the substep, then the front's advance after the last stage,
// :23) and update_state! without the velocity solve (the geometry).
static void step_thickness_stage(Problem& P, double dt, int st, bool coupled) {
    thickness_substep(P, dt, st, coupled);
    const double stages[3] = {1.0 / 3, 1.0 / 2, 1.0};
    if (st == 2 && P.front.enabled) advance_front(P, stages[st] * dt, coupled);
    compute_geometry(P);
}

static void step_thickness(Problem& P, double dt, bool coupled) {
    for (int st = 0; st < 3; ++st) step_thickness_stage(P, dt, st, coupled);
}

// ------------------------------------------------------------------------------------------------
// The gradient through time steps with the velocities held (checkpointed_gradient!, ext/NunatakEnzymeExt.jl:245-263,
// for a model without a velocity solve): the oracle's own restatement, held to finite differences of its forward steps.
// Every stage is stored (no checkpoints); the reverse of a stage takes the chain through the clip, the sources, the
// divergence and the fluxes by hand, and the local derivatives of the face values, the limiter θ and the centre
// grounded fraction by forward differentiation (a value and one derivative) of the same formulas the forward step
// evaluates, input by input.
// ------------------------------------------------------------------------------------------------
struct Dn {
    double v, d;
};
static inline Dn operator+(Dn a, Dn b) { return {a.v + b.v, a.d + b.d}; }
static inline Dn operator-(Dn a, Dn b) { return {a.v - b.v, a.d - b.d}; }
static inline Dn operator*(Dn a, Dn b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
static inline Dn operator*(double s, Dn a) { return {s * a.v, s * a.d}; }
static inline Dn operator/(Dn a, Dn b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
static inline Dn operator/(Dn a, double s) { return {a.v / s, a.d / s}; }
static inline Dn dn_abs(Dn a) { return a.v >= 0 ? a : Dn{-a.v, -a.d}; }
static inline Dn dn_max(Dn a, Dn b) { return std::max(a.v, b.v) == a.v ? a : b; }
static inline Dn dn_min(Dn a, Dn b) { return std::min(a.v, b.v) == a.v ? a : b; }

// weno5_face, upwind3_face and face_value above, on values with a derivative
static Dn weno5_face_dn(const Dn* s) {
    const Dn a = s[0], b = s[1], c = s[2], d = s[3], e = s[4];
    Dn q0 = (2 * a - 7 * b + 11 * c) / 6.0;
    Dn q1 = ((-1.0) * b + 5 * c + 2 * d) / 6.0;
    Dn q2 = (2 * c + 5 * d - e) / 6.0;
    Dn t0 = a - 2 * b + c, u0 = a - 4 * b + 3 * c;
    Dn t1 = b - 2 * c + d, u1 = b - d;
    Dn t2 = c - 2 * d + e, u2 = 3 * c - 4 * d + e;
    Dn b0 = (13.0 / 12) * (t0 * t0) + 0.25 * (u0 * u0);
    Dn b1 = (13.0 / 12) * (t1 * t1) + 0.25 * (u1 * u1);
    Dn b2 = (13.0 / 12) * (t2 * t2) + 0.25 * (u2 * u2);
    const Dn eps{1e-8, 0.0};
    Dn tau = dn_abs(b0 - b2);
    Dn r0 = tau / (b0 + eps), r1 = tau / (b1 + eps), r2 = tau / (b2 + eps);
    Dn a0 = 0.1 * (Dn{1, 0} + r0), a1 = 0.6 * (Dn{1, 0} + r1), a2 = 0.3 * (Dn{1, 0} + r2);
    return (a0 * q0 + a1 * q1 + a2 * q2) / (a0 + a1 + a2);
}
static Dn face_value_dn(const nk_advection_desc& adv, const Dn* s) {
    if (adv.scheme == NK_ADVECTION_WENO) return weno5_face_dn(s);
    return adv.order == 3 ? ((-1.0) * s[1] + 5 * s[2] + 2 * s[3]) / 6.0 : s[2];
}
// bounds_limiter with the derivative along the stage thickness at halo position (si, sj)
static Dn bounds_limiter_dn(const nk_advection_desc& adv, const Field& H, int i, int j, int si, int sj) {
    auto h = [&](int a, int b) { return Dn{H(a, b), (a == si && b == sj) ? 1.0 : 0.0}; };
    Dn s[5];
    for (int m = -2; m <= 2; ++m) s[m + 2] = h(i + m, j);           // x_stencil(H, i + 1, j, east): H(i + m)
    Dn E = weno5_face_dn(s);
    for (int m = -2; m <= 2; ++m) s[m + 2] = h(i - m, j);           // x_stencil(H, i, j, west): H(i - m)
    Dn W = weno5_face_dn(s);
    for (int m = -2; m <= 2; ++m) s[m + 2] = h(i, j + m);
    Dn N = weno5_face_dn(s);
    for (int m = -2; m <= 2; ++m) s[m + 2] = h(i, j - m);
    Dn S = weno5_face_dn(s);
    Dn Hc = h(i, j);
    const double w = 5.0 / 18, eps = 2 * std::numeric_limits<double>::epsilon();
    Dn px = (Hc - w * W - w * E) / (1 - 2 * w);
    Dn py = (Hc - w * S - w * N) / (1 - 2 * w);
    Dn M = dn_max(dn_max(dn_max(px, py), dn_max(W, E)), dn_max(S, N));
    Dn m = dn_min(dn_min(dn_min(px, py), dn_min(W, E)), dn_min(S, N));
    Dn t1 = dn_abs((Dn{adv.upper, 0} - Hc) / (M - Hc + Dn{eps, 0}));
    Dn t2 = dn_abs((Dn{adv.lower, 0} - Hc) / (m - Hc - Dn{eps, 0}));
    return dn_min(dn_min(t1, t2), Dn{1.0, 0.0});
}
static Dn triangle_fraction_dn(Dn f1, Dn f2, Dn f3) {   // triangle_grounded_fraction
    Dn a = dn_min(dn_min(f1, f2), f3), c = dn_max(dn_max(f1, f2), f3);
    Dn b = f1 + f2 + f3 - a - c;
    auto nz = [](Dn x) { return x.v == 0.0 ? Dn{1.0, 0.0} : x; };
    Dn one_grounded = (c * c) / nz((c - a) * (c - b));
    Dn one_floating = Dn{1.0, 0.0} - (a * a) / nz((b - a) * (c - a));
    Dn phi = b.v > 0 ? one_floating : one_grounded;
    return a.v >= 0 ? Dn{1.0, 0.0} : (c.v <= 0 ? Dn{0.0, 0.0} : phi);
}
// the centre grounded fraction of compute_geometry at (i, j) with the derivative along H at halo position (si, sj)
static Dn centre_fraction_dn(const Problem& P, int i, int j, int si, int sj) {
    double rw_ri = P.ph.rho_w / P.ph.rho_i;
    auto f = [&](int a, int b) { return Dn{P.H(a, b) + rw_ri * P.bed(a, b), (a == si && b == sj) ? 1.0 : 0.0}; };
    Dn fc = f(i, j);
    Dn fe = (fc + f(i + 1, j)) / 2.0, fw = (fc + f(i - 1, j)) / 2.0, fn = (fc + f(i, j + 1)) / 2.0, fs = (fc + f(i, j - 1)) / 2.0;
    Dn fne = (fc + f(i + 1, j) + f(i, j + 1) + f(i + 1, j + 1)) / 4.0;
    Dn fnw = (fc + f(i - 1, j) + f(i, j + 1) + f(i - 1, j + 1)) / 4.0;
    Dn fse = (fc + f(i + 1, j) + f(i, j - 1) + f(i + 1, j - 1)) / 4.0;
    Dn fsw = (fc + f(i - 1, j) + f(i, j - 1) + f(i - 1, j - 1)) / 4.0;
    Dn phi = triangle_fraction_dn(fc, fe, fne) + triangle_fraction_dn(fc, fn, fne) + triangle_fraction_dn(fc, fn, fnw) +
             triangle_fraction_dn(fc, fw, fnw) + triangle_fraction_dn(fc, fw, fsw) + triangle_fraction_dn(fc, fs, fsw) +
             triangle_fraction_dn(fc, fs, fse) + triangle_fraction_dn(fc, fe, fse);
    return phi / 8.0;
}

// The interior cell a halo position of a Center-Center field copies (fill_halo: wrap, or the edge cell).
static void fold(const Grid& g, int& i, int& j) {
    i = g.x.periodic ? mod1(i, g.Nx()) : std::min(std::max(i, 1), g.Nx());
    j = g.y.periodic ? mod1(j, g.Ny()) : std::min(std::max(j, 1), g.Ny());
}

// The reverse of step_thickness_stage (no front) at the stored stage: P.H holds the stage thickness (halos filled) and
// P.phi its centre grounded fraction, P.melt the step's melt (w m); Hout is the stage output.  From λ
// of the output (lam_out) it adds λ of H0, u, v, a and the base melt m and writes λ of the stage thickness (lam_Hs).
static void stage_reverse(Problem& P, const Field& Hout, double dtau, double w, const Field& lam_out,
                          Field& lam_Hs, Field& lam_H0, VelocityVector& lam_x, Field& lam_smb, Field& lam_melt,
                          const Field* lam_phi_in = nullptr) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny();
    const nk_advection_desc adv = P.advection;
    const bool bounded = adv.scheme == NK_ADVECTION_WENO && adv.bounded;
    const Field& Hs = P.H;
    const bool front = P.front.enabled != 0;
    auto full = [&](int i, int j) { return !front || full_cell(P, i, j); };   // μ with its halo filled
    Field dv(&g, CENTER, CENTER), lam_phi(&g, CENTER, CENTER), lam_theta(&g, CENTER, CENTER);
    lam_Hs.zero();
    for (int j = 1; j <= Ny; ++j)
        for (int i = 1; i <= Nx; ++i) {
            double ls = Hout(i, j) > 0 ? lam_out(i, j) : 0.0;   // the clip max(0, H★)
            lam_H0(i, j) += ls;
            dv(i, j) = -dtau * ls / g.Az_ccc(i, j);
            double lS = full(i, j) ? dtau * ls : 0.0;           // sources on full cells only
            lam_smb(i, j) += lS;
            lam_melt(i, j) -= lS * (P.grounding ? 1 - P.phi(i, j) : 1.0) * w;
            lam_phi(i, j) = (P.grounding ? lS * P.melt(i, j) : 0.0) + (lam_phi_in ? (*lam_phi_in)(i, j) : 0.0);
        }
    auto theta = [&](int ic, int jc) { return bounded ? P.theta(ic, jc) : 1.0; };
    // a face's flux u Δ H_face: λ to the velocity, to the upwind cell (1 - θ), to its θ, and through the face value's
    // derivative to the five stencil cells
    auto face = [&](double lF, double u, double delta, bool pos, int ic, int jc, int f0x, int f0y, bool xdir, double& lam_u) {
        Dn s[5];
        double sv[5];
        int px[5], py[5];
        for (int m = -2; m <= 2; ++m) {
            int a = xdir ? (pos ? f0x - 1 + m : f0x - m) : f0x;
            int b = xdir ? f0y : (pos ? f0y - 1 + m : f0y - m);
            px[m + 2] = a;
            py[m + 2] = b;
            sv[m + 2] = Hs(a, b);
        }
        for (int m = 0; m < 5; ++m) s[m] = Dn{sv[m], 0.0};
        double h0 = face_value_dn(adv, s).v;
        double th = theta(ic, jc);
        double h = bounded ? Hs(ic, jc) + th * (h0 - Hs(ic, jc)) : h0;
        lam_u += delta * h * lF;
        double lh = delta * u * lF;
        if (bounded) {
            int fi = ic, fj = jc;
            fold(g, fi, fj);
            lam_Hs(fi, fj) += (1 - th) * lh;
            lam_theta(fi, fj) += (h0 - Hs(ic, jc)) * lh;
        }
        double lh0 = th * lh;
        for (int q = 0; q < 5; ++q) {
            for (int m = 0; m < 5; ++m) s[m] = Dn{sv[m], m == q ? 1.0 : 0.0};
            double d = face_value_dn(adv, s).d;
            int a = px[q], b = py[q];
            fold(g, a, b);
            lam_Hs(a, b) += d * lh0;
        }
    };
    // x faces f = 1 .. Nx + 1 (Nx on a periodic axis, whose face Nx + 1 is face 1)
    int fxmax = g.x.periodic ? Nx : Nx + 1, fymax = g.y.periodic ? Ny : Ny + 1;
    for (int j = 1; j <= Ny; ++j)
        for (int f = 1; f <= fxmax; ++f) {
            if (g.peripheral_fc(f, j)) continue;
            int wi = f - 1, wj = j, ei = f, ej = j;
            fold(g, wi, wj);
            fold(g, ei, ej);
            double lF = dv(wi, wj) - dv(ei, ej);
            double u = P.x.u(f, j);
            bool w = full(f - 1, j), e = full(f, j);
            if (!(w && e)) {   // front_flux_x: the upwind flux out of the full side, nothing between two front cells
                if (w) { lam_x.u(f, j) += g.dy_c(j) * (u > 0 ? Hs(f - 1, j) : 0.0) * lF; lam_Hs(wi, wj) += g.dy_c(j) * std::max(u, 0.0) * lF; }
                else if (e) { lam_x.u(f, j) += g.dy_c(j) * (u < 0 ? Hs(f, j) : 0.0) * lF; lam_Hs(ei, ej) += g.dy_c(j) * std::min(u, 0.0) * lF; }
                continue;
            }
            bool east = u > 0;
            face(lF, u, g.dy_c(j), east, east ? f - 1 : f, j, f, j, true, lam_x.u(f, j));
        }
    for (int f = 1; f <= fymax; ++f)
        for (int i = 1; i <= Nx; ++i) {
            if (g.peripheral_cf(i, f)) continue;
            int si = i, sj = f - 1, ni = i, nj = f;
            fold(g, si, sj);
            fold(g, ni, nj);
            double lF = dv(si, sj) - dv(ni, nj);
            double v = P.x.v(i, f);
            bool so = full(i, f - 1), no = full(i, f);
            if (!(so && no)) {
                if (so) { lam_x.v(i, f) += g.dx_c(i) * (v > 0 ? Hs(i, f - 1) : 0.0) * lF; lam_Hs(si, sj) += g.dx_c(i) * std::max(v, 0.0) * lF; }
                else if (no) { lam_x.v(i, f) += g.dx_c(i) * (v < 0 ? Hs(i, f) : 0.0) * lF; lam_Hs(ni, nj) += g.dx_c(i) * std::min(v, 0.0) * lF; }
                continue;
            }
            bool north = v > 0;
            face(lF, v, g.dx_c(i), north, i, north ? f - 1 : f, i, f, false, lam_x.v(i, f));
        }
    // θ of each cell, back to the thickness of its own stencils and itself
    if (bounded)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) {
                double lt = lam_theta(i, j);
                if (lt == 0.0) continue;
                for (int q = 0; q < 9; ++q) {
                    int si = q < 5 ? i + q - 2 : i, sj = q < 5 ? j : j + (q < 7 ? q - 7 : q - 6);
                    double d = bounds_limiter_dn(adv, Hs, i, j, si, sj).d;
                    int a = si, b = sj;
                    fold(g, a, b);
                    lam_Hs(a, b) += lt * d;
                }
            }
    // the centre grounded fraction of the floating melt, back to the nine flotations it reads
    if (P.grounding)
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) {
                double lp = lam_phi(i, j);
                if (lp == 0.0) continue;
                for (int b = -1; b <= 1; ++b)
                    for (int a = -1; a <= 1; ++a) {
                        double d = centre_fraction_dn(P, i, j, i + a, j + b).d;
                        int x = i + a, y = j + b;
                        fold(g, x, y);
                        lam_Hs(x, y) += lp * d;
                    }
            }
}

static void copy_in(Field& f, const double* src);
static void copy_out(const Field& f, double* dst);

// nk_checkpointed_gradient of the library with the velocities held and no front; every stage stored.
// The front's advance (advance_front without the grounded-melt coupling) as a function of its continuous inputs,
// with the flag μ and the calved thickness of the step's start held: its H and Hʳ.
struct FrontInputs {
    Field H, Hr, smb, melt, phi;
    VelocityVector x;
    Field etaH;                   // the viscosity the von Mises rates read (that law only)
};
static void front_outputs(Problem& P, const FrontInputs& in, const Field& mu0, double dt, Field& Hout, Field& Hrout) {
    Field clipped = P.clipped, calved = P.calved;
    P.H = in.H; P.Hr = in.Hr; P.mu = mu0; P.smb = in.smb; P.melt = in.melt; P.phi = in.phi; P.x = in.x;
    if (P.front.calving == NK_CALVING_VON_MISES) P.etaH = in.etaH;
    for (Field* f : {&P.H, &P.Hr, &P.mu, &P.smb, &P.melt, &P.phi}) fill_halo(*f);
    fill_halo(P.x);
    advance_front(P, dt, false);
    Hout = P.H;
    Hrout = P.Hr;
    P.clipped = clipped;
    P.calved = calved;
}
// Its reverse by the numerical Jacobian: every input entry moved by ±h, λ of the entry = Σ λ · (output(+) - output(-)) / 2h,
// with h sized to move the thickness by about 1e-7 of itself or 1e-6 m (the sources over the step), so that the
// differences keep their digits: 1e-7 of H and Hʳ (at least 1e-7 m), 1e-6 m / Δt of a and m, 1e-3 of φ and 1e-3 of a
// velocity (the calving rates and front lengths are smooth in it, and the inflow flags hold).  A velocity moves a strain
// rate by several times its own step, and the von Mises rate takes fractional powers of the strain rates, so the
// velocity columns take Richardson's (4 D(h/2) - D(h)) / 3 of the centred differences.
static void front_reverse_jacobian(Problem& P, const FrontInputs& in, const Field& mu0, double dt, const Field& lamH,
                                   const Field& lamHr, FrontInputs& lam) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny();
    Field Hp(&g, CENTER, CENTER), Rp(&g, CENTER, CENTER), Hm(&g, CENTER, CENTER), Rm(&g, CENTER, CENTER);
    auto entry = [&](Field FrontInputs::*field, bool velocity, bool u, int i, int j, double rel, double floor) {
        FrontInputs a = in;
        Field& f = velocity ? (u ? a.x.u : a.x.v) : a.*field;
        double v0 = f(i, j), h = std::max(rel * std::fabs(v0), floor);
        auto centred = [&](double step) {
            f(i, j) = v0 + step;
            front_outputs(P, a, mu0, dt, Hp, Rp);
            f(i, j) = v0 - step;
            front_outputs(P, a, mu0, dt, Hm, Rm);
            f(i, j) = v0;
            double acc = 0.0;
            for (int y = 1; y <= Ny; ++y)
                for (int x = 1; x <= Nx; ++x) acc += lamH(x, y) * (Hp(x, y) - Hm(x, y)) + lamHr(x, y) * (Rp(x, y) - Rm(x, y));
            return acc / (2 * step);
        };
        return velocity ? (4 * centred(h / 2) - centred(h)) / 3 : centred(h);
    };
    struct Spec { Field FrontInputs::*f; double rel, floor; };
    const Spec cells[5] = {{&FrontInputs::H, 1e-7, 1e-7}, {&FrontInputs::Hr, 1e-7, 1e-7}, {&FrontInputs::smb, 0.0, 1e-6 / dt},
                           {&FrontInputs::melt, 0.0, 1e-6 / dt}, {&FrontInputs::phi, 0.0, 1e-3}};
    for (const Spec& c : cells) {
        (lam.*(c.f)).zero();
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) (lam.*(c.f))(i, j) = entry(c.f, false, false, i, j, c.rel, c.floor);
    }
    lam.x.u.zero();
    lam.x.v.zero();
    for (int j = 1; j <= lam.x.u.ny(); ++j)
        for (int i = 1; i <= lam.x.u.nx(); ++i) lam.x.u(i, j) = entry(nullptr, true, true, i, j, 1e-3, 1e-15);
    for (int j = 1; j <= lam.x.v.ny(); ++j)
        for (int i = 1; i <= lam.x.v.nx(); ++i) lam.x.v(i, j) = entry(nullptr, true, false, i, j, 1e-3, 1e-15);
    if (P.front.calving == NK_CALVING_VON_MISES) {   // the rates are linear in η̄H: 1e-6 of it (at least 1)
        lam.etaH.init(&g, CENTER, CENTER);
        for (int j = 1; j <= Ny; ++j)
            for (int i = 1; i <= Nx; ++i) lam.etaH(i, j) = entry(&FrontInputs::etaH, false, false, i, j, 1e-6, 1.0);
    }
}

// The thickness part of the SSA Picard adjoint, ∂J/∂H = λᵀ ∂r/∂H with r(H) = τ(H) − A(c(x*, H)) x* at the converged
// x* held (the fixed point A(c(x)) x = τ moves with H as −(∂F/∂x)⁻¹ ∂F/∂H, and λ solves (∂F/∂x)ᵀ λ = x̄): per cell
// the centred difference of r with the geometry, the driving stress and the coefficients recomputed from H
// (update_state! without the solve), h = 1e-6 max(H, 1).  A numerical restatement of the library's hand-written
// chain through η̄H, the drag's grounded fractions and effective pressure, the slope and the front force.
// With eta_bar (the η̄H shadow of picard_adjoint) the shadow's own H part s̄ᵀ ∂η̄H/∂H joins it, by the same differences.
// The DIVA's fixed point is one of (x, s) with the lagged state s = (βᵇ, F₂, ησ): with sig (picard_adjoint's
// sig_final) the state's part σᵀ ∂S/∂H of the state update S(x*, s*, H) joins it, s* restored before each evaluation.
static void picard_thickness_gradient(Problem& P, const VelocityVector& lam, const VelocityVector& xs, Field& gH,
                                      const Field* eta_bar = nullptr, const DivaState* sig = nullptr) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny();
    const bool diva = P.stress_balance == NK_DIVA;
    Field H0 = P.H;
    Field s_bbu = P.bbu, s_bbv = P.bbv, s_F2 = P.F2;
    SigmaField s_eta = P.eta_s;
    auto restore_state = [&] {
        if (!diva) return;
        P.bbu = s_bbu; P.bbv = s_bbv; P.F2 = s_F2; P.eta_s = s_eta;
    };
    double sd = 0.0;   // σᵀ S of the last evaluation
    VelocityVector rp, rm;
    rp.init(&g);
    rm.init(&g);
    Field ep, em;
    auto residual = [&](VelocityVector& r, Field& e) {
        fill_halo(P.H);
        compute_geometry(P);
        P.x = xs;
        fill_halo(P.x);
        restore_state();
        update_coefficients(P);
        sd = 0.0;
        if (diva && sig) {
            for (int j = 1; j <= P.bbu.ny(); ++j) for (int i = 1; i <= P.bbu.nx(); ++i) sd += sig->bbu(i, j) * P.bbu(i, j);
            for (int j = 1; j <= P.bbv.ny(); ++j) for (int i = 1; i <= P.bbv.nx(); ++i) sd += sig->bbv(i, j) * P.bbv(i, j);
            for (int j = 1; j <= Ny; ++j)
                for (int i = 1; i <= Nx; ++i) {
                    sd += sig->F2(i, j) * P.F2(i, j);
                    for (size_t k = 0; k < P.eta_s.k.size(); ++k) sd += sig->eta.k[k](i, j) * P.eta_s.k[k](i, j);
                }
        }
        VelocityVector q;
        q.init(&g);
        ssa_operator(g, q, xs, coeffs(P), P.ph.walls);
        for (int j = 1; j <= r.u.ny(); ++j) for (int i = 1; i <= r.u.nx(); ++i) r.u(i, j) = P.tau.u(i, j) - q.u(i, j);
        for (int j = 1; j <= r.v.ny(); ++j) for (int i = 1; i <= r.v.nx(); ++i) r.v(i, j) = P.tau.v(i, j) - q.v(i, j);
        e = P.etaH;
    };
    gH.init(&g, CENTER, CENTER);
    for (int j = 1; j <= Ny; ++j)
        for (int i = 1; i <= Nx; ++i) {
            double h = 1e-6 * std::max(H0(i, j), 1.0);
            P.H = H0;
            P.H(i, j) += h;
            residual(rp, ep);
            double sdp = sd;
            P.H = H0;
            P.H(i, j) -= h;
            residual(rm, em);
            double acc = sdp - sd;
            if (eta_bar)
                for (int b = 1; b <= Ny; ++b) for (int a = 1; a <= Nx; ++a) acc += (*eta_bar)(a, b) * (ep(a, b) - em(a, b));
            for (int b = 1; b <= lam.u.ny(); ++b) for (int a = 1; a <= lam.u.nx(); ++a) acc += lam.u(a, b) * (rp.u(a, b) - rm.u(a, b));
            for (int b = 1; b <= lam.v.ny(); ++b) for (int a = 1; a <= lam.v.nx(); ++a) acc += lam.v(a, b) * (rp.v(a, b) - rm.v(a, b));
            gH(i, j) = acc / (2 * h);
        }
    P.H = H0;
    fill_halo(P.H);
    compute_geometry(P);
    P.x = xs;
    fill_halo(P.x);
    restore_state();
    update_coefficients(P);
    restore_state();
}

// nk_checkpointed_gradient of the library; every stage stored.  A partial-cell front's advance is reversed through its
// numerical Jacobian (the oracle's check of the library's hand-written reverse).  With velocity_solves (the SSA) each
// stage is followed by a Picard solve, and the reverse runs the oracle's Picard adjoint of each solve with
// picard_thickness_gradient, in the library's order: the step-end solve after the cost, then per stage (3, 2, 1) the
// stage's reverse and the adjoint of the solve that made its velocities; the first stage's velocities are the previous
// step's last solve's.  The front read the last stage's velocities and, under von Mises calving, the viscosity η̄H that
// stage's solve left: their λ join that solve's adjoint, η̄H's as the shadow of an overwritten coefficient.
static nk_status time_gradient(Problem& P, const nk_time_gradient_desc& d, nk_cost_fn cost, void* user, const nk_time_gradient* out,
                               nk_time_gradient_stats* st) {
    const Grid& g = P.grid;
    const int Nx = g.Nx(), Ny = g.Ny(), N = d.steps;
    const bool bounded = P.advection.scheme == NK_ADVECTION_WENO && P.advection.bounded;
    const bool front = P.front.enabled != 0;
    const double fractions[3] = {1.0 / 3, 1.0 / 2, 1.0};
    auto weight = [&](int n) { return d.melt_weights ? d.melt_weights[n] : 1.0; };
    Field base = P.melt;
    const bool solves = d.velocity_solves != 0;
    const nk_iteration_control ctl = d.adjoint_control ? *d.adjoint_control : P.sdesc.picard;
    std::vector<Field> tape;                         // H before each stage, then the final H
    std::vector<VelocityVector> xt;                  // with solves: the velocities before each stage, then the final ones
    struct Lagged { Field bbu, bbv, F2; SigmaField eta; };
    std::vector<Lagged> st_t;                        // and the DIVA's lagged state the solve left with them
    const bool diva = P.stress_balance == NK_DIVA;
    auto keep_state = [&] {
        if (solves) xt.push_back(P.x);
        if (solves && diva) st_t.push_back(Lagged{P.bbu, P.bbv, P.F2, P.eta_s});
    };
    std::vector<Field> mu_start, Hr_start, H3pre;   // a front: μ and Hʳ at each step's start, the last stage's output
    std::vector<Field> etaH_front;                   // and the viscosity its von Mises rates read
    fill_halo(P.H);
    compute_geometry(P);
    std::memset(st, 0, sizeof(*st));
    auto solve = [&] {
        nk_solve_stats ss{};
        picard_solve(P, &ss);
        ++st->picard_solves;
        if (ss.status > st->worst_solve_status) st->worst_solve_status = ss.status;
    };
    for (int n = 0; n < N; ++n) {
        for_xy(Nx, Ny, [&](int i, int j) { P.melt(i, j) = weight(n) * base(i, j); });
        if (front) {
            mu_start.push_back(P.mu);
            Hr_start.push_back(P.Hr);
        }
        for (int stg = 0; stg < 3; ++stg) {
            tape.push_back(P.H);
            keep_state();
            if (front && stg == 2) {
                thickness_substep(P, d.dt, stg, false);
                H3pre.push_back(P.H);
                etaH_front.push_back(P.etaH);
                advance_front(P, d.dt, false);
                compute_geometry(P);
            } else {
                step_thickness_stage(P, d.dt, stg, false);
            }
            if (solves) solve();
        }
    }
    tape.push_back(P.H);
    keep_state();
    VelocityVector x_end = P.x;
    Field Hfinal = P.H, clipped_end = P.clipped, mu_end = P.mu, Hr_end = P.Hr, calved_end = P.calved;
    Field lamH(&g, CENTER, CENTER), lamHs(&g, CENTER, CENTER), lamH0(&g, CENTER, CENTER), lamHr(&g, CENTER, CENTER);
    Field gsmb(&g, CENTER, CENTER), gmelt(&g, CENTER, CENTER);
    VelocityVector lamx;
    lamx.init(&g);
    FrontInputs lamf;
    if (front) {
        for (Field* f : {&lamf.H, &lamf.Hr, &lamf.smb, &lamf.melt, &lamf.phi}) f->init(&g, CENTER, CENTER);
        lamf.x.init(&g);
    }
    int nu = P.x.u.nx() * P.x.u.ny(), nv = P.x.v.nx() * P.x.v.ny();
    std::vector<double> hH(Nx * Ny), hu(nu), hv(nv), hm(Nx * Ny), gH(Nx * Ny), gu(nu), gv(nv);
    st->segments = 1;
    // with solves: λ of the velocities a solve made (the step end's, carried from the next step's first stage), and
    // the gradients in log C and log A that the solves' adjoints add up
    VelocityVector lamx_stage;
    lamx_stage.init(&g);
    Field glogC(&g, CENTER, CENTER);
    SigmaField glogA;
    glogA.init(&g, CENTER, CENTER, P.rate_layout == NK_RATE_FACTOR_SIGMA ? P.sigma.N : 1);
    auto solve_adjoint = [&](int t, const VelocityVector& xbar, Field& lam_to, const Field* eta_bar = nullptr) {
        P.H = tape[t];
        fill_halo(P.H);
        compute_geometry(P);
        P.x = xt[t];
        fill_halo(P.x);
        if (diva) { P.bbu = st_t[t].bbu; P.bbv = st_t[t].bbv; P.F2 = st_t[t].F2; P.eta_s = st_t[t].eta; }
        VelocityVector lam;
        Field gC;
        SigmaField gA;
        DivaState sig;
        nk_solve_stats ss{};
        picard_adjoint(P, xbar, ctl, lam, gC, gA, &ss, eta_bar, diva ? &sig : nullptr);
        ++st->picard_adjoints;
        st->adjoint_iterations += ss.picard_iterations;
        if (ss.status > st->worst_solve_status) st->worst_solve_status = ss.status;
        Field gHs;
        picard_thickness_gradient(P, lam, xt[t], gHs, eta_bar, diva ? &sig : nullptr);
        for_xy(Nx, Ny, [&](int i, int j) {
            lam_to(i, j) += gHs(i, j);
            glogC(i, j) += gC(i, j);
            for (size_t k = 0; k < glogA.k.size(); ++k) glogA.k[k](i, j) += gA.k[k](i, j);
        });
    };
    for (int n = N - 1; n >= 0; --n) {
        P.H = tape[3 * n + 3];
        if (solves) P.x = xt[3 * n + 3];
        if (front) P.mu = n + 1 < N ? mu_start[n + 1] : mu_end;
        fill_halo(P.H);
        fill_halo(P.mu);
        compute_geometry(P);
        copy_out(P.H, hH.data());
        copy_out(P.x.u, hu.data());
        copy_out(P.x.v, hv.data());
        copy_out(P.mu, hm.data());
        std::fill(gH.begin(), gH.end(), 0.0);
        std::fill(gu.begin(), gu.end(), 0.0);
        std::fill(gv.begin(), gv.end(), 0.0);
        nk_cost_state cs{n + 1, N, hH.data(), hu.data(), hv.data(), hm.data()};
        double J = 0.0;
        if (cost(user, &cs, &J, gH.data(), gu.data(), gv.data()) != 0) return NK_BAD_ARGUMENT;
        st->J += J;
        {
            Field t(&g, CENTER, CENTER);
            copy_in(t, gH.data());
            for_xy(Nx, Ny, [&](int i, int j) { lamH(i, j) += t(i, j); });
            Field tu(&g, FACE, CENTER), tv(&g, CENTER, FACE);
            copy_in(tu, gu.data());
            copy_in(tv, gv.data());
            for (int j = 1; j <= tu.ny(); ++j) for (int i = 1; i <= tu.nx(); ++i) lamx.u(i, j) += tu(i, j);
            for (int j = 1; j <= tv.ny(); ++j) for (int i = 1; i <= tv.nx(); ++i) lamx.v(i, j) += tv(i, j);
        }
        if (solves) {   // the solve that ended the step, for λ of its velocities; lamx then carries the next λ
            solve_adjoint(3 * n + 3, lamx, lamH);
            lamx.init(&g);
        }
        if (front) {   // the front's advance after the last stage: its inputs at the step's state
            P.H = tape[3 * n + 2];
            P.mu = mu_start[n];
            if (solves) P.x = xt[3 * n + 2];   // the velocities of the last stage
            fill_halo(P.H);
            fill_halo(P.mu);
            compute_geometry(P);   // φ of the last stage's input
            FrontInputs in;
            in.H = H3pre[n];
            in.Hr = Hr_start[n];
            in.smb = P.smb;
            in.melt = P.melt;
            for_xy(Nx, Ny, [&](int i, int j) { in.melt(i, j) = weight(n) * base(i, j); });
            in.phi = P.phi;
            in.x = P.x;
            if (P.front.calving == NK_CALVING_VON_MISES) in.etaH = etaH_front[n];
            Field phi2 = P.phi;
            front_reverse_jacobian(P, in, mu_start[n], d.dt, lamH, lamHr, lamf);
            lamH = lamf.H;
            lamHr = lamf.Hr;
            for_xy(Nx, Ny, [&](int i, int j) {
                gsmb(i, j) += lamf.smb(i, j);
                gmelt(i, j) += weight(n) * lamf.melt(i, j);
            });
            if (!solves) {   // with solves they join the last stage's velocity adjoint below
                for (int j = 1; j <= lamx.u.ny(); ++j) for (int i = 1; i <= lamx.u.nx(); ++i) lamx.u(i, j) += lamf.x.u(i, j);
                for (int j = 1; j <= lamx.v.ny(); ++j) for (int i = 1; i <= lamx.v.nx(); ++i) lamx.v(i, j) += lamf.x.v(i, j);
            }
            P.phi = phi2;
        }
        lamH0.zero();
        for (int stg = 2; stg >= 0; --stg) {
            int t = 3 * n + stg;
            P.H = tape[t];
            if (solves) P.x = xt[t];
            if (front) P.mu = mu_start[n];
            fill_halo(P.H);
            fill_halo(P.mu);
            compute_geometry(P);
            for_xy(Nx, Ny, [&](int i, int j) { P.melt(i, j) = weight(n) * base(i, j); });
            fill_halo(P.melt);
            fill_halo(P.x);
            if (bounded) {
                if (!P.theta.g) P.theta.init(&g, CENTER, CENTER);
                for (int j = 0; j <= Ny + 1; ++j)
                    for (int i = 0; i <= Nx + 1; ++i) P.theta(i, j) = bounds_limiter(P.advection, P.H, i, j);
            }
            bool after_front = front && stg == 2;
            if (solves) lamx_stage.init(&g);
            stage_reverse(P, after_front ? H3pre[n] : tape[t + 1], fractions[stg] * d.dt, weight(n), lamH, lamHs, lamH0,
                          solves ? lamx_stage : lamx, gsmb, gmelt, after_front ? &lamf.phi : nullptr);
            if (solves) {
                const Field* eta_bar = nullptr;
                if (after_front) {   // the front read the last stage's velocities and, under von Mises, the viscosity
                    for (int j = 1; j <= lamx_stage.u.ny(); ++j) for (int i = 1; i <= lamx_stage.u.nx(); ++i) lamx_stage.u(i, j) += lamf.x.u(i, j);
                    for (int j = 1; j <= lamx_stage.v.ny(); ++j) for (int i = 1; i <= lamx_stage.v.nx(); ++i) lamx_stage.v(i, j) += lamf.x.v(i, j);
                    if (P.front.calving == NK_CALVING_VON_MISES) eta_bar = &lamf.etaH;
                }
                if (stg > 0) {
                    solve_adjoint(t, lamx_stage, lamHs, eta_bar);   // the solve that made the stage's velocities from its H
                } else {                                   // made by the previous step's last solve (or the input)
                    for (int j = 1; j <= lamx.u.ny(); ++j) for (int i = 1; i <= lamx.u.nx(); ++i) lamx.u(i, j) += lamx_stage.u(i, j);
                    for (int j = 1; j <= lamx.v.ny(); ++j) for (int i = 1; i <= lamx.v.nx(); ++i) lamx.v(i, j) += lamx_stage.v(i, j);
                }
            }
            if (stg > 0) lamH = lamHs;
            else for_xy(Nx, Ny, [&](int i, int j) { lamH(i, j) = lamHs(i, j) + lamH0(i, j); });
        }
    }
    if (out) {
        if (out->grad_H) copy_out(lamH, out->grad_H);
        if (out->grad_u && out->grad_v) { copy_out(lamx.u, out->grad_u); copy_out(lamx.v, out->grad_v); }
        if (out->grad_smb) copy_out(gsmb, out->grad_smb);
        if (out->grad_melt) copy_out(gmelt, out->grad_melt);
        if (out->grad_log_C) copy_out(glogC, out->grad_log_C);
        if (out->grad_log_A) {
            int planes = P.rate_layout == NK_RATE_FACTOR_SIGMA ? P.sigma.N : 1;
            for (int k = 0; k < planes; ++k) copy_out(glogA.k[k], out->grad_log_A + (size_t)k * Nx * Ny);
        }
    }
    if (solves) P.x = x_end;
    if (solves && diva) { P.bbu = st_t.back().bbu; P.bbv = st_t.back().bbv; P.F2 = st_t.back().F2; P.eta_s = st_t.back().eta; }
    P.H = Hfinal;
    P.clipped = clipped_end;
    P.melt = base;
    if (front) {
        P.mu = mu_end;
        P.Hr = Hr_end;
        P.calved = calved_end;
        fill_halo(P.mu);
        fill_halo(P.Hr);
    }
    fill_halo(P.H);
    compute_geometry(P);
    return NK_OK;
}

// ---- field access in interior layout -------------------------------------------------------------
struct FieldRef { Field* f = nullptr; SigmaField* s = nullptr; };

static FieldRef field_ref(Problem& P, int id) {
    FieldRef r;
    switch (id) {
        case NK_FIELD_U: r.f = &P.x.u; break;
        case NK_FIELD_V: r.f = &P.x.v; break;
        case NK_FIELD_H: r.f = &P.H; break;
        case NK_FIELD_BED: r.f = &P.bed; break;
        case NK_FIELD_SURFACE: r.f = &P.s; break;
        case NK_FIELD_ICE_MASK: r.f = &P.mu; break;
        case NK_FIELD_PHI: r.f = &P.phi; break;
        case NK_FIELD_PHI_U: r.f = &P.phu; break;
        case NK_FIELD_PHI_V: r.f = &P.phv; break;
        case NK_FIELD_EFFECTIVE_PRESSURE: r.f = &P.N; break;
        case NK_FIELD_TAU_U: r.f = &P.tau.u; break;
        case NK_FIELD_TAU_V: r.f = &P.tau.v; break;
        case NK_FIELD_RATE_FACTOR: if (P.rate_layout == NK_RATE_FACTOR_SIGMA) r.s = &P.A3; else r.f = &P.A2; break;
        case NK_FIELD_FRICTION_COEFFICIENT: r.f = &P.C; break;
        case NK_FIELD_ETA_H: r.f = &P.etaH; break;
        case NK_FIELD_ETA_H_FF: r.f = &P.etaHff; break;
        case NK_FIELD_BETA_U: r.f = &P.bu; break;
        case NK_FIELD_BETA_V: r.f = &P.bv; break;
        case NK_FIELD_ETA_SIGMA: r.s = &P.eta_s; break;
        case NK_FIELD_F2: r.f = &P.F2; break;
        case NK_FIELD_BETA_B_U: r.f = &P.bbu; break;
        case NK_FIELD_BETA_B_V: r.f = &P.bbv; break;
        case NK_FIELD_U_B: r.f = &P.ub; break;
        case NK_FIELD_V_B: r.f = &P.vb; break;
        case NK_FIELD_U_SIGMA: r.s = &P.us; break;
        case NK_FIELD_V_SIGMA: r.s = &P.vs; break;
        case NK_FIELD_TEMPERATURE: r.s = &P.T; break;
        case NK_FIELD_U_PRESCRIBED: r.f = &P.ud.u; break;
        case NK_FIELD_V_PRESCRIBED: r.f = &P.ud.v; break;
        // held for every rate-factor layout here (the energy step needs them with a constant A as well); the
        // library holds them with the σ-grid rate factor only, the one its thermal diagnostics write
        case NK_FIELD_ENTHALPY: r.s = &P.E; break;
        case NK_FIELD_WATER_FRACTION: r.s = &P.omega; break;
        case NK_FIELD_SURFACE_MASS_BALANCE: r.f = &P.smb; break;
        case NK_FIELD_BASAL_MELT_RATE: r.f = &P.melt; break;
        case NK_FIELD_GROUNDED_MELT_RATE: r.f = &P.gmelt; break;
        case NK_FIELD_CLIPPED_THICKNESS: r.f = &P.clipped; break;
        case NK_FIELD_BASAL_WATER_THICKNESS: r.f = &P.Hw; break;
        case NK_FIELD_GEOTHERMAL_FLUX: r.f = &P.G; break;
        case NK_FIELD_SURFACE_TEMPERATURE: r.f = &P.Ts; break;
        case NK_FIELD_OCEAN_TEMPERATURE: r.f = &P.To; break;
        case NK_FIELD_THICKNESS_PREVIOUS: r.f = &P.Hn; break;
        case NK_FIELD_BASAL_TEMPERATE_FRACTION: r.f = &P.sb; break;
        case NK_FIELD_BASAL_HEAT_FLUX: r.f = &P.qg; break;
        case NK_FIELD_STRAIN_HEATING: r.s = &P.Phi; break;
        case NK_FIELD_FRONT_THICKNESS: r.f = &P.Hr; break;
        case NK_FIELD_CALVED_THICKNESS: r.f = &P.calved; break;
        case NK_FIELD_CALVING_EXTENT: r.f = &P.extent; break;
        default: break;
    }
    return r;
}

static int64_t field_size(Problem& P, int id) {
    FieldRef r = field_ref(P, id);
    if (r.f) return (int64_t)r.f->nx() * r.f->ny();
    if (r.s) return (int64_t)r.s->k[0].nx() * r.s->k[0].ny() * (int64_t)r.s->k.size();
    return 0;
}

static void copy_in(Field& f, const double* src) {
    int nx = f.nx(), ny = f.ny();
    for (int j = 1; j <= ny; ++j) for (int i = 1; i <= nx; ++i) f(i, j) = src[(size_t)(j - 1) * nx + (i - 1)];
    fill_halo(f);
}
static void copy_out(const Field& f, double* dst) {
    int nx = f.nx(), ny = f.ny();
    for (int j = 1; j <= ny; ++j) for (int i = 1; i <= nx; ++i) dst[(size_t)(j - 1) * nx + (i - 1)] = f(i, j);
}

}  // namespace oracle

using namespace oracle;

extern "C" {

typedef struct nko_problem nko_problem;

int nko_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

nk_status nko_problem_create(const nk_grid_desc* gd, const nk_physics_desc* pd, const nk_solver_desc* sd, nko_problem** out) {
    if (!gd || !pd || !sd || !out || gd->Nx < 1 || gd->Ny < 1 || gd->Nsigma < 1) return NK_BAD_ARGUMENT;
    auto P = new Problem();
    bool px = gd->topology_x == NK_PERIODIC, py = gd->topology_y == NK_PERIODIC;
    if (gd->x_faces) P->grid.x.build_faces(gd->Nx, gd->halo_x, px, gd->x_faces); else P->grid.x.build_regular(gd->Nx, gd->halo_x, px, gd->x0, gd->Lx);
    if (gd->y_faces) P->grid.y.build_faces(gd->Ny, gd->halo_y, py, gd->y_faces); else P->grid.y.build_regular(gd->Ny, gd->halo_y, py, gd->y0, gd->Ly);
    P->sigma.N = gd->Nsigma;
    P->sigma.faces.resize(gd->Nsigma + 1);
    for (int k = 0; k <= gd->Nsigma; ++k)
        P->sigma.faces[k] = gd->sigma_faces ? gd->sigma_faces[k] : std::pow((double)k / gd->Nsigma, gd->bed_refinement);
    P->pdesc = *pd; P->sdesc = *sd;
    P->stress_balance = pd->stress_balance;
    P->rate_layout = pd->rate_factor_layout;
    P->ph.walls = pd->side_walls; P->ph.n = pd->glen_exponent; P->ph.eps0 = pd->strain_rate_regularization;
    P->ph.friction = pd->friction; P->ph.m = pd->friction_exponent; P->ph.alpha2 = pd->coulomb_coefficient;
    P->ph.u0 = pd->velocity_regularization; P->ph.rho_i = pd->ice_density; P->ph.rho_w = pd->ocean_density;
    P->ph.g = pd->gravitational_acceleration;
    P->use_mask = pd->use_ice_mask != 0; P->use_N = pd->use_effective_pressure != 0;
    P->grounding = pd->grounding; P->gl_stress = pd->grounding_line_driving_stress;
    P->mask_min = pd->mask_minimum_thickness; P->mask_trans = pd->mask_transition_thickness;

    const Grid* g = &P->grid;
    P->x.init(g); P->tau.init(g);
    P->ud.init(g);
    std::fill(P->ud.u.d.begin(), P->ud.u.d.end(), std::nan(""));
    std::fill(P->ud.v.d.begin(), P->ud.v.d.end(), std::nan(""));
    for (Field* f : {&P->H, &P->bed, &P->s, &P->mu, &P->phi, &P->N, &P->C, &P->A2, &P->etaH, &P->F2}) f->init(g, CENTER, CENTER);
    for (Field* f : {&P->phu, &P->bu, &P->bbu, &P->ub}) f->init(g, FACE, CENTER);
    for (Field* f : {&P->phv, &P->bv, &P->bbv, &P->vb}) f->init(g, CENTER, FACE);
    P->etaHff.init(g, FACE, FACE);
    P->A3.init(g, CENTER, CENTER, gd->Nsigma); P->eta_s.init(g, CENTER, CENTER, gd->Nsigma); P->T.init(g, CENTER, CENTER, gd->Nsigma);
    P->E.init(g, CENTER, CENTER, gd->Nsigma); P->omega.init(g, CENTER, CENTER, gd->Nsigma);
    for (Field* f : {&P->Hw, &P->gmelt, &P->G, &P->Ts, &P->To, &P->melt, &P->Hn, &P->sb, &P->smb, &P->clipped, &P->qg}) f->init(g, CENTER, CENTER);
    for (Field* f : {&P->Hr, &P->calved, &P->extent, &P->O}) f->init(g, CENTER, CENTER);
    P->Phi.init(g, CENTER, CENTER, gd->Nsigma);
    P->us.init(g, FACE, CENTER, gd->Nsigma); P->vs.init(g, CENTER, FACE, gd->Nsigma);
    P->r.init(g); P->z.init(g); P->p.init(g); P->q.init(g); P->w.init(g); P->xprev.init(g);
    P->eta_prev.init(g, CENTER, CENTER);
    if (sd->preconditioner == NK_PRECONDITIONER_MULTIGRID) {
        coarse_levels(P->grid, sd->minimum_coarse_size, P->mg.levels);
        P->mg.residual.init(g); P->mg.scratch.init(g, CENTER, CENTER);
        P->mg.smoother = sd->smoother; P->mg.sweeps = sd->smoothing_sweeps; P->mg.coarsest = sd->coarsest_sweeps;
    }
    // Defaults of the geometry fields match a fresh model: φ = 1 where no grounding treatment is set.
    *out = reinterpret_cast<nko_problem*>(P);
    return NK_OK;
}

nk_status nko_problem_destroy(nko_problem* h) { delete reinterpret_cast<Problem*>(h); return NK_OK; }

int64_t nko_problem_field_size(nko_problem* h, int32_t id) { return field_size(*reinterpret_cast<Problem*>(h), id); }

nk_status nko_problem_set_field(nko_problem* h, int32_t id, const double* src, int64_t count) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    FieldRef r = field_ref(P, id);
    if ((!r.f && !r.s) || !src || count != field_size(P, id)) return NK_BAD_ARGUMENT;
    if (r.f) copy_in(*r.f, src);
    else {
        int64_t layer = (int64_t)r.s->k[0].nx() * r.s->k[0].ny();
        for (size_t k = 0; k < r.s->k.size(); ++k) copy_in(r.s->k[k], src + k * layer);
    }
    if (id == NK_FIELD_U_PRESCRIBED || id == NK_FIELD_V_PRESCRIBED) {   // the right-hand side and velocity take u_D
        P.grid.pu = &P.ud.u;
        P.grid.pv = &P.ud.v;
        impose_prescribed(P, P.tau, P.ud);
        impose_prescribed(P, P.x, P.ud);
    }
    return NK_OK;
}

nk_status nko_problem_get_field(nko_problem* h, int32_t id, double* dst, int64_t count) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    FieldRef r = field_ref(P, id);
    if ((!r.f && !r.s) || !dst || count != field_size(P, id)) return NK_BAD_ARGUMENT;
    if (r.f) copy_out(*r.f, dst);
    else {
        int64_t layer = (int64_t)r.s->k[0].nx() * r.s->k[0].ny();
        for (size_t k = 0; k < r.s->k.size(); ++k) copy_out(r.s->k[k], dst + k * layer);
    }
    return NK_OK;
}

nk_status nko_compute_geometry(nko_problem* h) { compute_geometry(*reinterpret_cast<Problem*>(h)); return NK_OK; }

// Rate factor from temperature, column_energy_solve.jl:104-110 with ω = 0 and arrhenius_rate_factor, arrhenius_rate_factor.jl:102-110
nk_status nko_compute_rate_factor(nko_problem* h, double Ac, double Aw, double Qc, double Qw, double Tt, double Tw, double R,
                                  double beta_cc, double Tm) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (P.rate_layout != NK_RATE_FACTOR_SIGMA) return NK_BAD_ARGUMENT;
    const Grid& g = P.grid;
    for (int k = 1; k <= P.sigma.N; ++k) {
        double zeta = P.sigma.zc(k);
        for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
            double p = P.ph.rho_i * P.ph.g * P.H(i, j) * (1 - zeta);          // layer_pressure, enthalpy_conversions.jl:61-64
            double Tp = P.T.k[k - 1](i, j) - (Tm - beta_cc * p) + Tm;         // T′ = T - Tₚₘ(p) + T₀
            double log_cold = std::log(Ac) - Qc / (R * Tp);
            double log_warm = std::log(Aw) - Qw / (R * Tp);
            double x = std::min(std::max((Tp - Tt) / Tw + 1.0 / 2, 0.0), 1.0);
            double s = x * x * (3 - 2 * x);
            double softening = 1 + 181.25 * std::min(0.0, 0.01);                // ω = 0
            P.A3.k[k - 1](i, j) = std::exp((1 - s) * log_cold + s * log_warm) * softening;
        });
        fill_halo(P.A3.k[k - 1]);
    }
    return NK_OK;
}

// update_thermal_diagnostics! with an ArrheniusRateFactor, src/Thermodynamics/column_energy_solve.jl:85-110:
// _compute_thermal_diagnostics! (:112-117) with temperature / water_fraction (enthalpy_conversions.jl:35, :42),
// then _compute_rate_factor! (:104-110) with arrhenius_rate_factor (arrhenius_rate_factor.jl:102-110).
nk_status nko_compute_thermal_diagnostics(nko_problem* h, const nk_thermal_params* q) {
    if (!h || !q) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (P.rate_layout != NK_RATE_FACTOR_SIGMA) return NK_BAD_ARGUMENT;
    if (!(q->heat_capacity > 0) || !(q->latent_heat > 0) || !(q->gas_constant > 0) || !(q->transition_width > 0)) return NK_BAD_ARGUMENT;
    const Grid& g = P.grid;
    for (int k = 1; k <= P.sigma.N; ++k) {
        double zeta = P.sigma.zc(k);
        for_xy(g.Nx(), g.Ny(), [&](int i, int j) {
            double p = P.ph.rho_i * P.ph.g * P.H(i, j) * (1 - zeta);                        // layer_pressure, :61-64
            double Tpm = q->melting_temperature - q->clausius_clapeyron * p;                // :6
            double Epm = q->heat_capacity * (Tpm - q->reference_temperature);              // :13
            double E = P.E.k[k - 1](i, j);
            double T = std::min(Tpm, q->reference_temperature + E / q->heat_capacity);     // :35
            double w = std::max(0.0, E - Epm) / q->latent_heat;                            // :42
            P.T.k[k - 1](i, j) = T;
            P.omega.k[k - 1](i, j) = w;
            double Tp = T - Tpm + q->melting_temperature;                                   // T′ = T - Tₚₘ + T₀
            double R = q->gas_constant;
            double log_cold = std::log(q->cold_prefactor) - q->cold_activation_energy / (R * Tp);
            double log_warm = std::log(q->warm_prefactor) - q->warm_activation_energy / (R * Tp);
            double x = std::min(std::max((Tp - q->transition_temperature) / q->transition_width + 1.0 / 2, 0.0), 1.0);
            double s = x * x * (3 - 2 * x);
            double softening = 1 + q->water_softening_coefficient * std::min(w, q->maximum_water_fraction);
            P.A3.k[k - 1](i, j) = std::exp((1 - s) * log_cold + s * log_warm) * softening;
        });
        fill_halo(P.T.k[k - 1]); fill_halo(P.omega.k[k - 1]); fill_halo(P.A3.k[k - 1]);
    }
    return NK_OK;
}

// The energy step's own fields (no library counterpart yet): which = 0 Hw, 1 mᵍ, 2 G, 3 Tₛ, 4 Tₒ, 5 basal melt rate,
// 6 Hⁿ (2-D), 7 Φ (σ grid), 8 sᵇ, 9 surface mass balance, 10 clipped thickness, 11 basal heat flux qᵍ (2-D);
// set = 1 copies data in, 0 out.
nk_status nko_energy_field(nko_problem* h, int32_t which, double* data, int64_t count, int32_t set) {
    if (!h || !data) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    Field* two[] = {&P.Hw, &P.gmelt, &P.G, &P.Ts, &P.To, &P.melt, &P.Hn, nullptr, &P.sb, &P.smb, &P.clipped, &P.qg};
    if (which >= 0 && which <= 11 && which != 7) {
        Field& f = *two[which];
        if (count != (int64_t)f.nx() * f.ny()) return NK_BAD_ARGUMENT;
        if (set) copy_in(f, data); else copy_out(f, data);
        return NK_OK;
    }
    if (which == 7) {
        size_t plane = (size_t)P.grid.Nx() * P.grid.Ny();
        if (count != (int64_t)(plane * P.Phi.k.size())) return NK_BAD_ARGUMENT;
        for (size_t k = 0; k < P.Phi.k.size(); ++k) {
            if (set) copy_in(P.Phi.k[k], data + k * plane); else copy_out(P.Phi.k[k], data + k * plane);
        }
        return NK_OK;
    }
    return NK_BAD_ARGUMENT;
}

// One energy step of length dt (step_thermodynamics!, src/Thermodynamics/column_energy_solve.jl:26-31).  prm: thermal
// conductivity, heat capacity, latent heat, Clausius-Clapeyron slope, melting and reference temperatures, temperate
// diffusivity ratio, enthalpy blend width, water layer blend thickness, minimum thickness, drainage water fraction,
// maximum drainage rate, grounded melt coupling (0 / 1): EnthalpyThermodynamics' keywords
// (src/Thermodynamics/enthalpy_thermodynamics.jl:92-110).
// One ice time step of the thickness of length dt (time_step! with a held velocity); coupled: the grounded melt
// mᵍ of the energy step thins the ice.
nk_status nko_step_thickness(nko_problem* h, double dt, int32_t coupled) {
    if (!h || !(dt > 0)) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    int halo = std::min(P.grid.x.H, P.grid.y.H);
    if (P.advection.scheme == NK_ADVECTION_WENO && P.advection.bounded && halo < 4)
        return NK_BAD_ARGUMENT;   // check_advection_halo, src/Models/ice_sheet_model.jl:131-135
    if ((P.advection.scheme == NK_ADVECTION_WENO || P.advection.order == 3) && halo < 3)
        return NK_BAD_ARGUMENT;   // the five-point stencils reach three cells beyond a face
    step_thickness(P, dt, coupled != 0);
    return NK_OK;
}

// One stage (1, 2, 3) of nko_step_thickness; the three in order equal it.
nk_status nko_step_thickness_stage(nko_problem* h, double dt, int32_t stage, int32_t coupled) {
    if (!h || !(dt > 0) || stage < 1 || stage > 3) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    int halo = std::min(P.grid.x.H, P.grid.y.H);
    if (P.advection.scheme == NK_ADVECTION_WENO && P.advection.bounded && halo < 4) return NK_BAD_ARGUMENT;
    if ((P.advection.scheme == NK_ADVECTION_WENO || P.advection.order == 3) && halo < 3) return NK_BAD_ARGUMENT;
    step_thickness_stage(P, dt, stage - 1, coupled != 0);
    return NK_OK;
}

// nk_checkpointed_gradient for a model whose velocities are held (no velocity solve).
nk_status nko_checkpointed_gradient(nko_problem* h, const nk_time_gradient_desc* d, nk_cost_fn cost, void* user,
                                    const nk_time_gradient* out, nk_time_gradient_stats* stats) {
    if (!h || !d || !cost || !(d->dt > 0) || d->steps < 1 || (d->velocity_solves != 0 && d->velocity_solves != 1))
        return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    // velocity solves: without prescribed faces; the DIVA without von Mises calving (its sweep takes no η̄H shadow)
    if (d->velocity_solves && (P.grid.pu || P.grid.pv)) return NK_BAD_ARGUMENT;
    if (d->velocity_solves && P.stress_balance == NK_DIVA && P.front.enabled && P.front.calving == NK_CALVING_VON_MISES)
        return NK_BAD_ARGUMENT;
    const nk_iteration_control ctl = d->adjoint_control ? *d->adjoint_control : P.sdesc.picard;
    if (d->velocity_solves && ctl.kind != NK_CONVERGENCE && ctl.kind != NK_FIXED_ITERATIONS) return NK_BAD_ARGUMENT;
    nk_time_gradient_stats local{};
    return time_gradient(P, *d, cost, user, out, stats ? stats : &local);
}

// PartialCellFront(grid; passes, calving) as the masking (partial_cell_front.jl:1-66, calving.jl); needs the ice mask.
nk_status nko_set_front(nko_problem* h, const nk_front_desc* f) {
    if (!h || !f) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (f->enabled && (!P.use_mask || f->passes < 0 || f->calving < NK_CALVING_NONE || f->calving > NK_CALVING_MAXIMUM_EXTENT))
        return NK_BAD_ARGUMENT;
    P.front = *f;
    return NK_OK;
}

// TillEffectivePressure as EnthalpyThermodynamics' effective_pressure (till_effective_pressure.jl:1-77).
nk_status nko_set_till(nko_problem* h, const nk_till_desc* t) {
    if (!h || !t || (t->enabled != 0 && t->enabled != 1)) return NK_BAD_ARGUMENT;
    if (t->enabled && !(t->reference_effective_pressure > 0 && t->overburden_fraction > 0 && t->compressibility > 0 &&
                        t->maximum_water_thickness > 0 && t->drainage_rate >= 0))
        return NK_BAD_ARGUMENT;
    reinterpret_cast<Problem*>(h)->till = *t;
    return NK_OK;
}

nk_status nko_initialize_front(nko_problem* h) {
    if (!h) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (!P.front.enabled) return NK_BAD_ARGUMENT;
    initialize_front(P);
    return NK_OK;
}

nk_status nko_advance_front(nko_problem* h, double dt) {
    if (!h || !(dt > 0)) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (!P.front.enabled) return NK_BAD_ARGUMENT;
    fill_halo(P.x);
    for (Field* f : {&P.smb, &P.melt, &P.gmelt, &P.clipped, &P.Hr, &P.extent}) fill_halo(*f);
    advance_front(P, dt, false);
    compute_geometry(P);
    return NK_OK;
}

// The thickness advection scheme (IceSheetModel's advection keyword): UpwindBiased(order = 1 or 3) or WENO(order = 5),
// bounded to [lower, upper] or not.
nk_status nko_set_thickness_advection(nko_problem* h, const nk_advection_desc* adv) {
    if (!h || !adv) return NK_BAD_ARGUMENT;
    bool ok = (adv->scheme == NK_ADVECTION_UPWIND && (adv->order == 1 || adv->order == 3) && !adv->bounded) ||
              (adv->scheme == NK_ADVECTION_WENO && adv->order == 5 && (!adv->bounded || adv->lower < adv->upper));
    if (!ok) return NK_BAD_ARGUMENT;
    reinterpret_cast<Problem*>(h)->advection = *adv;
    return NK_OK;
}

nk_status nko_step_enthalpy(nko_problem* h, const double* prm, double dt) {
    if (!h || !prm || !(dt > 0)) return NK_BAD_ARGUMENT;
    EnergyParams q{prm[0], prm[1], prm[2], prm[3], prm[4], prm[5], prm[6], prm[7], prm[8], prm[9], prm[10], prm[11], prm[12] != 0.0};
    step_enthalpy(*reinterpret_cast<Problem*>(h), q, dt);
    return NK_OK;
}

nk_status nko_update_coefficients(nko_problem* h) { update_coefficients(*reinterpret_cast<Problem*>(h)); return NK_OK; }

static void load_vector(VelocityVector& x, const double* u, const double* v) { copy_in(x.u, u); copy_in(x.v, v); }
static void store_vector(const VelocityVector& x, double* u, double* v) { copy_out(x.u, u); copy_out(x.v, v); }

nk_status nko_apply_operator(nko_problem* h, const double* pu, const double* pv, double* qu, double* qv) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    VelocityVector p, q; p.init(&P.grid); q.init(&P.grid);
    load_vector(p, pu, pv); load_vector(q, qu, qv);
    Coefficients c = coeffs(P);
    ssa_operator(P.grid, q, p, c, P.ph.walls);
    store_vector(q, qu, qv);
    return NK_OK;
}

nk_status nko_precondition(nko_problem* h, const double* ru, const double* rv, double* zu, double* zv) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    VelocityVector r, z; r.init(&P.grid); z.init(&P.grid);
    load_vector(r, ru, rv); load_vector(z, zu, zv);
    update_preconditioner(P);
    precondition(P, z, r);
    store_vector(z, zu, zv);
    return NK_OK;
}

nk_status nko_linear_solve(nko_problem* h, const double* bu, const double* bv, nk_solve_stats* st) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    VelocityVector b; b.init(&P.grid);
    load_vector(b, bu, bv);
    if (st) std::memset(st, 0, sizeof(*st));
    int status = NK_OK;
    impose_prescribed(P, P.x, b);   // an identity row's solution is its right-hand side
    conjugate_gradient(P, P.x, b, st, &status);
    fill_halo(P.x);
    if (st) st->status = status;
    return status == NK_NONFINITE ? NK_NONFINITE : NK_OK;
}

nk_status nko_picard_solve(nko_problem* h, nk_solve_stats* st) {
    nk_solve_stats local{};
    picard_solve(*reinterpret_cast<Problem*>(h), st ? st : &local);
    return (st ? st : &local)->status == NK_NONFINITE ? NK_NONFINITE : NK_OK;
}

nk_status nko_velocity_profile(nko_problem* h) { velocity_profile(*reinterpret_cast<Problem*>(h)); return NK_OK; }

// nk_picard_adjoint (SSA and DIVA).  Problems with prescribed velocities are refused with NK_BAD_ARGUMENT.
nk_status nko_picard_adjoint(nko_problem* h, const double* ubar, const double* vbar, const nk_iteration_control* control,
                             double* lu, double* lv, double* grad_log_C, double* grad_log_A, nk_solve_stats* stats) {
    if (!h || !ubar || !vbar) return NK_BAD_ARGUMENT;
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (P.grid.pu || P.grid.pv) return NK_BAD_ARGUMENT;
    nk_iteration_control ctl = control ? *control : P.sdesc.picard;
    if (ctl.kind != NK_CONVERGENCE && ctl.kind != NK_FIXED_ITERATIONS) return NK_BAD_ARGUMENT;
    VelocityVector xbar, lam;
    xbar.init(&P.grid);
    load_vector(xbar, ubar, vbar);
    Field gradC;
    SigmaField gradA;
    nk_solve_stats local{};
    nk_solve_stats* st = stats ? stats : &local;
    int status = picard_adjoint(P, xbar, ctl, lam, gradC, gradA, st);
    if (lu && lv) store_vector(lam, lu, lv);
    if (grad_log_C) copy_out(gradC, grad_log_C);
    if (grad_log_A) {
        size_t plane = (size_t)P.grid.Nx() * P.grid.Ny();
        for (size_t k = 0; k < gradA.k.size(); ++k) copy_out(gradA.k[k], grad_log_A + k * plane);
    }
    return status == NK_NONFINITE ? NK_NONFINITE : NK_OK;
}

nk_status nko_multigrid_levels(nko_problem* h, int32_t* count, int32_t* nx, int32_t* ny, int32_t cap) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    *count = (int32_t)P.mg.levels.size();
    for (int l = 0; l < *count && l < cap; ++l) { nx[l] = P.mg.levels[l]->grid->Nx(); ny[l] = P.mg.levels[l]->grid->Ny(); }
    return NK_OK;
}

// Transfers on level `level` (0 = first coarse level) with the current (coarsened) coefficients:
// coarse = R fine, or fine += P coarse.  Vectors in interior layout of the respective grids.
nk_status nko_multigrid_restrict(nko_problem* h, int32_t level, const double* fu, const double* fv, double* cu, double* cv) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (level < 0 || level >= (int)P.mg.levels.size()) return NK_BAD_ARGUMENT;
    update_preconditioner(P);
    const Grid& fg = level == 0 ? P.grid : *P.mg.levels[level - 1]->grid;
    const Field& feta = level == 0 ? P.etaH : P.mg.levels[level - 1]->etaH;
    Level& L = *P.mg.levels[level];
    VelocityVector f, c; f.init(&fg); c.init(L.grid.get());
    load_vector(f, fu, fv); load_vector(c, cu, cv);
    restrict_vector(*L.grid, fg, L, c, f, L.etaH, feta);
    store_vector(c, cu, cv);
    return NK_OK;
}

nk_status nko_multigrid_prolongate(nko_problem* h, int32_t level, const double* cu, const double* cv, double* fu, double* fv) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    if (level < 0 || level >= (int)P.mg.levels.size()) return NK_BAD_ARGUMENT;
    update_preconditioner(P);
    const Grid& fg = level == 0 ? P.grid : *P.mg.levels[level - 1]->grid;
    const Field& feta = level == 0 ? P.etaH : P.mg.levels[level - 1]->etaH;
    Level& L = *P.mg.levels[level];
    VelocityVector f, c; f.init(&fg); c.init(L.grid.get());
    load_vector(f, fu, fv); load_vector(c, cu, cv);
    prolongate_vector(fg, *L.grid, L, f, c, feta, L.etaH);
    store_vector(f, fu, fv);
    return NK_OK;
}

// Grid metrics for cross-checks: which = 0 Δxᶜ(1..Nx), 1 Δxᶠ(1..Nx+1), 2 Δyᶜ(1..Ny), 3 Δyᶠ(1..Ny+1).
nk_status nko_grid_metrics(nko_problem* h, int32_t which, double* out) {
    Problem& P = *reinterpret_cast<Problem*>(h);
    const Grid& g = P.grid;
    switch (which) {
        case 0: for (int i = 1; i <= g.Nx(); ++i) out[i - 1] = g.dx_c(i); break;
        case 1: for (int i = 1; i <= g.Nx() + 1; ++i) out[i - 1] = g.dx_f(i); break;
        case 2: for (int j = 1; j <= g.Ny(); ++j) out[j - 1] = g.dy_c(j); break;
        case 3: for (int j = 1; j <= g.Ny() + 1; ++j) out[j - 1] = g.dy_f(j); break;
        default: return NK_BAD_ARGUMENT;
    }
    return NK_OK;
}

}  // extern "C"
