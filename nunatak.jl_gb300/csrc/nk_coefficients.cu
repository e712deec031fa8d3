// nk_coefficients.cu — Picard coefficient update, geometry and driving stress (FP64).
//
// One thread per cell or face.  The viscosity kernel computes the membrane strain rate once per
// column and walks the sigma levels in registers, fusing compute_viscosity! with
// compute_column_integrals! (the reference launches them over Nx x Ny x Nsigma and Nx x Ny).
#include <cmath>

#include "nk_kernels.cuh"
#include "nk_transport.cuh"

namespace nk {

// ---- wall-masked velocities of the viscosity (interior_u / interior_v without η̄H, strain_rates.jl:5-6) ----
// A prescribed face on the boundary passes its value (the Dirichlet extension; `ud` NaN where free).
__device__ __forceinline__ double wall_u(const DevGrid<double>& g, const double2* __restrict__ x, const double2* ud, int i, int j) {
    return (g.peripheral_fc(i, j) && !prescribed_u(g, ud, i, j)) ? 0.0 : x[g.u_idx(i, j)].x;
}
__device__ __forceinline__ double wall_v(const DevGrid<double>& g, const double2* __restrict__ x, const double2* ud, int i, int j) {
    return (g.peripheral_cf(i, j) && !prescribed_v(g, ud, i, j)) ? 0.0 : x[g.v_idx(i, j)].y;
}
__device__ __forceinline__ double strain_xy(const DevGrid<double>& g, const double2* __restrict__ x, const double2* ud, int i, int j,
                                            double wf) {
    double dudy = (wall_u(g, x, ud, i, j) - wall_u(g, x, ud, i, j - 1)) * g.rdyf[j];
    double dvdx = (wall_v(g, x, ud, i, j) - wall_v(g, x, ud, i - 1, j)) * g.rdxf[i];
    double e = (dudy + dvdx) / 2;
    return g.peripheral_ff(i, j) ? wf * e : e;
}
// effective_strain_rate², strain_rates.jl:27-32
__device__ __forceinline__ double effective_strain_rate2(const DevGrid<double>& g, const double2* __restrict__ x, const double2* ud,
                                                         int i, int j, double wf) {
    double exx = (wall_u(g, x, ud, i + 1, j) - wall_u(g, x, ud, i, j)) * g.rdxc[i];
    double eyy = (wall_v(g, x, ud, i, j + 1) - wall_v(g, x, ud, i, j)) * g.rdyc[j];
    double e00 = strain_xy(g, x, ud, i, j, wf), e10 = strain_xy(g, x, ud, i + 1, j, wf);
    double e01 = strain_xy(g, x, ud, i, j + 1, wf), e11 = strain_xy(g, x, ud, i + 1, j + 1, wf);
    double exy2 = ((e00 * e00 + e10 * e10) / 2 + (e01 * e01 + e11 * e11) / 2) / 2;
    return exx * exx + eyy * eyy + exx * eyy + exy2;
}

// η = ½ A^(-1/n) ε̇ₑ²^((1-n)/2n) (glen_flow_law.jl:110).  For n = 3 both powers are reciprocal cube roots.
__device__ __forceinline__ double glen(double A, double ee, double n) {
    if (n == 3.0) return rcbrt(A) * rcbrt(ee) / 2;
    return pow(A, -1 / n) * pow(ee, (1 - n) / (2 * n)) / 2;
}

__device__ __forceinline__ double rate_factor(const PhysView& ph, int c, int k) {
    return ph.rate_sigma ? ph.A[(long long)k * ph.plane + c] : ph.A[c];
}

// compute_viscosity! (glen_flow_law.jl:97-111) fused with compute_column_integrals! (column_integrals.jl:54-72)
__global__ void k_viscosity(PhysView ph, const double2* __restrict__ x, double* eta_sigma, double4* coef, double* F2) {
    NK_BATCH_ENTER(ph.g, ph, x, eta_sigma, coef, F2)
    const DevGrid<double>& g = ph.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double ee = effective_strain_rate2(g, x, ph.ud, i, j, ph.wall_factor) + ph.eps0 * ph.eps0;
    double eta_bar = 0.0, F = 0.0;
    double eta_uniform = ph.rate_sigma ? 0.0 : glen(ph.A[c], ee, ph.n);
    for (int k = 0; k < ph.sig.N; ++k) {
        double eta = ph.rate_sigma ? glen(rate_factor(ph, c, k), ee, ph.n) : eta_uniform;
        eta_sigma[(long long)k * ph.plane + c] = eta;
        eta_bar += eta * ph.sig.dz[k];
        F += (1 / eta) * ph.sig.w2[k];
    }
    double H = ph.H[c];
    coef[c].x = ph.use_mask ? eta_bar * H * ph.mu[c] : eta_bar * H;
    F2[c] = F * H;
}
void launch_viscosity(const PhysView& ph, const double2* x, double* eta_sigma, double4* coef, double* F2, cudaStream_t s) {
    LaunchDims d = dims2d(ph.g.Nx, ph.g.Ny);
    k_viscosity<<<d.grid, d.block, 0, s>>>(ph, x, eta_sigma, coef, F2); count_launch();
}

// _compute_shear_viscosity! (glen_flow_law.jl:134-143): the basal stress βᵇ uᵇ drives a vertical shear
// ε̇xz = ℑxᶜ(βᵇᵘ uᵇ)(1 - ζ) / 2η⁻ with the previous viscosity η⁻ (left out where η⁻ is still zero)
__global__ void k_viscosity_diva(PhysView ph, const double2* __restrict__ x, const double2* __restrict__ bb,
                                 const double2* __restrict__ ub, double* eta_sigma, double4* coef, double* F2) {
    NK_BATCH_ENTER(ph.g, ph, x, bb, ub, eta_sigma, coef, F2)
    const DevGrid<double>& g = ph.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double e2 = effective_strain_rate2(g, x, ph.ud, i, j, ph.wall_factor);
    int u0 = g.u_idx(i, j), u1 = g.u_idx(i + 1, j), v0 = g.v_idx(i, j), v1 = g.v_idx(i, j + 1);
    double tx = (bb[u0].x * ub[u0].x + bb[u1].x * ub[u1].x) / 2;
    double ty = (bb[v0].y * ub[v0].y + bb[v1].y * ub[v1].y) / 2;
    double eta_bar = 0.0, F = 0.0;
    for (int k = 0; k < ph.sig.N; ++k) {
        long long o = (long long)k * ph.plane + c;
        double zeta = ph.sig.zc[k];
        double em = eta_sigma[o];
        em = (em == 0.0) ? INFINITY : em;
        double exz = tx * (1 - zeta) / (2 * em);
        double eyz = ty * (1 - zeta) / (2 * em);
        double ee = e2 + exz * exz + eyz * eyz + ph.eps0 * ph.eps0;
        double eta = glen(rate_factor(ph, c, k), ee, ph.n);
        eta_sigma[o] = eta;
        eta_bar += eta * ph.sig.dz[k];
        F += (1 / eta) * ph.sig.w2[k];
    }
    double H = ph.H[c];
    coef[c].x = ph.use_mask ? eta_bar * H * ph.mu[c] : eta_bar * H;
    F2[c] = F * H;
}
void launch_viscosity_diva(const PhysView& ph, const double2* x, const double2* bb, const double2* ub, double* eta_sigma,
                           double4* coef, double* F2, cudaStream_t s) {
    LaunchDims d = dims2d(ph.g.Nx, ph.g.Ny);
    k_viscosity_diva<<<d.grid, d.block, 0, s>>>(ph, x, bb, ub, eta_sigma, coef, F2); count_launch();
}

// _interpolate_to_corners! (stress_balance_coefficients.jl:26-29): ℑxyᶠᶠᵃ = ℑyᵃᶠᵃ(ℑxᶠᵃᵃ(η̄H))
template <typename T>
__global__ void k_corners(DevGrid<T> g, typename Vec4<T>::type* coef) {
    NK_BATCH_ENTER(g, g, coef)
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    T lo = (coef[g.c_idx(i - 1, j - 1)].x + coef[g.c_idx(i, j - 1)].x) / T(2);
    T hi = (coef[g.c_idx(i - 1, j)].x + coef[g.c_idx(i, j)].x) / T(2);
    coef[g.idx(i, j)].y = (lo + hi) / T(2);
}
template <typename T>
void launch_corners(const DevGrid<T>& g, typename Vec4<T>::type* coef, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx + 1, g.Ny + 1);
    k_corners<T><<<d.grid, d.block, 0, s>>>(g, coef); count_launch();
}
template void launch_corners<double>(const DevGrid<double>&, double4*, cudaStream_t);
template void launch_corners<float>(const DevGrid<float>&, float4*, cudaStream_t);

// basal_drag, frictions.jl:83-89
__device__ __forceinline__ double basal_drag(const PhysView& ph, double U, double C, double N) {
    double w = C * pow(U, ph.m - 1);
    if (ph.friction == NK_WEERTMAN) return w;
    double tc = ph.alpha2 * N;
    return w * tc / pow(pow(C, 1 / ph.m) * U + pow(tc, 1 / ph.m), ph.m);
}

// _compute_x_basal_drag! / _compute_y_basal_drag!, frictions.jl:142-160, over size(βᵘ), size(βᵛ)
__global__ void k_basal_drag(PhysView ph, const double2* __restrict__ x, double4* coef, double2* bb) {
    NK_BATCH_ENTER(ph.g, ph, x, coef, bb)
    const DevGrid<double>& g = ph.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    double u02 = ph.u0 * ph.u0;
    bool has_u = j < g.Ny && (i < g.Nx || !g.px);
    bool has_v = i < g.Nx && (j < g.Ny || !g.py);
    double bu = 0.0, bv = 0.0;
    if (has_u) {
        double vf = ((x[g.v_idx(i - 1, j)].y + x[g.v_idx(i, j)].y) / 2 + (x[g.v_idx(i - 1, j + 1)].y + x[g.v_idx(i, j + 1)].y) / 2) / 2;
        double u = x[k].x;
        double U = sqrt(u * u + vf * vf + u02);
        double Cf = (ph.C[g.c_idx(i - 1, j)] + ph.C[g.c_idx(i, j)]) / 2;
        double Nf = ph.use_N ? (ph.N[g.c_idx(i - 1, j)] + ph.N[g.c_idx(i, j)]) / 2 : 0.0;
        double b = ph.phi[k].x * basal_drag(ph, U, Cf, Nf);
        bu = g.peripheral_fc(i, j) ? 0.0 : b;
    }
    if (has_v) {
        double uf = ((x[g.u_idx(i, j - 1)].x + x[g.u_idx(i + 1, j - 1)].x) / 2 + (x[g.u_idx(i, j)].x + x[g.u_idx(i + 1, j)].x) / 2) / 2;
        double v = x[k].y;
        double U = sqrt(v * v + uf * uf + u02);
        double Cf = (ph.C[g.c_idx(i, j - 1)] + ph.C[g.c_idx(i, j)]) / 2;
        double Nf = ph.use_N ? (ph.N[g.c_idx(i, j - 1)] + ph.N[g.c_idx(i, j)]) / 2 : 0.0;
        double b = ph.phi[k].y * basal_drag(ph, U, Cf, Nf);
        bv = g.peripheral_cf(i, j) ? 0.0 : b;
    }
    if (coef) {
        if (has_u) coef[k].z = bu;
        if (has_v) coef[k].w = bv;
    } else {
        double2 o = bb[k];
        if (has_u) o.x = bu;
        if (has_v) o.y = bv;
        bb[k] = o;
    }
}
void launch_basal_drag(const PhysView& ph, const double2* x, double4* coef, double2* bb, cudaStream_t s) {
    if (ph.friction == NK_FRICTION_NONE) return;   // compute_basal_drag!(βᵘ, βᵛ, ::Nothing, ...) = nothing
    LaunchDims d = dims2d(ph.g.Nx + 1, ph.g.Ny + 1);
    k_basal_drag<<<d.grid, d.block, 0, s>>>(ph, x, coef, bb); count_launch();
}

// 1 + βᵇ ℑF₂ at the velocity points, diva.jl:1-3
__device__ __forceinline__ double x_shear_factor(const DevGrid<double>& g, double b, const double* F2, int i, int j) {
    return 1 + b * ((F2[g.c_idx(i - 1, j)] + F2[g.c_idx(i, j)]) / 2);
}
__device__ __forceinline__ double y_shear_factor(const DevGrid<double>& g, double b, const double* F2, int i, int j) {
    return 1 + b * ((F2[g.c_idx(i, j - 1)] + F2[g.c_idx(i, j)]) / 2);
}

__global__ void k_basal_velocity(PhysView ph, const double2* __restrict__ x, const double2* __restrict__ bb, const double* __restrict__ F2,
                                 double2* ub) {
    NK_BATCH_ENTER(ph.g, ph, x, bb, F2, ub)
    const DevGrid<double>& g = ph.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    bool has_u = j < g.Ny && (i < g.Nx || !g.px);
    bool has_v = i < g.Nx && (j < g.Ny || !g.py);
    double2 o = ub[k], xx = x[k], b = bb[k];
    if (has_u) o.x = xx.x / x_shear_factor(g, b.x, F2, i, j);
    if (has_v) o.y = xx.y / y_shear_factor(g, b.y, F2, i, j);
    ub[k] = o;
}
void launch_basal_velocity(const PhysView& ph, const double2* x, const double2* bb, const double* F2, double2* ub, cudaStream_t s) {
    LaunchDims d = dims2d(ph.g.Nx + 1, ph.g.Ny + 1);
    k_basal_velocity<<<d.grid, d.block, 0, s>>>(ph, x, bb, F2, ub); count_launch();
}

__global__ void k_effective_drag(PhysView ph, const double2* __restrict__ bb, const double* __restrict__ F2, double4* coef) {
    NK_BATCH_ENTER(ph.g, ph, bb, F2, coef)
    const DevGrid<double>& g = ph.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    bool has_u = j < g.Ny && (i < g.Nx || !g.px);
    bool has_v = i < g.Nx && (j < g.Ny || !g.py);
    double2 b = bb[k];
    if (has_u) coef[k].z = b.x / x_shear_factor(g, b.x, F2, i, j);
    if (has_v) coef[k].w = b.y / y_shear_factor(g, b.y, F2, i, j);
}
void launch_effective_drag(const PhysView& ph, const double2* bb, const double* F2, double4* coef, cudaStream_t s) {
    LaunchDims d = dims2d(ph.g.Nx + 1, ph.g.Ny + 1);
    k_effective_drag<<<d.grid, d.block, 0, s>>>(ph, bb, F2, coef); count_launch();
}

// shear_integral (column_integrals.jl:42): H ∫₀^ζₖ (1 - ζ′)/η dζ′
__device__ __forceinline__ double shear_integral(const PhysView& ph, const double* eta_sigma, int c, int k) {
    double I = 0.0;
    for (int kp = 0; kp <= k; ++kp) I += (1 / eta_sigma[(long long)kp * ph.plane + c]) * ph.sig.w1[k * ph.sig.N + kp];
    return I * ph.H[c];
}

// _compute_x/y_velocity_profile! (diva.jl:99-109) or _extend_depth_average! (SSA)
__global__ void k_velocity_profile(PhysView ph, int diva, const double2* __restrict__ x, const double2* __restrict__ bb,
                                   const double* __restrict__ eta_sigma, const double2* __restrict__ ub, double2* usig) {
    const DevGrid<double>& g = ph.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int c = g.idx(i, j);
    bool has_u = j < g.Ny && (i < g.Nx || !g.px);
    bool has_v = i < g.Nx && (j < g.Ny || !g.py);
    for (int k = 0; k < ph.sig.N; ++k) {
        long long o = (long long)k * ph.plane + c;
        double2 out = usig[o];
        if (!diva) {
            if (has_u) out.x = x[c].x;
            if (has_v) out.y = x[c].y;
        } else {
            if (has_u) {
                double F1 = (shear_integral(ph, eta_sigma, g.c_idx(i - 1, j), k) + shear_integral(ph, eta_sigma, g.c_idx(i, j), k)) / 2;
                out.x = ub[c].x * (1 + bb[c].x * F1);
            }
            if (has_v) {
                double F1 = (shear_integral(ph, eta_sigma, g.c_idx(i, j - 1), k) + shear_integral(ph, eta_sigma, g.c_idx(i, j), k)) / 2;
                out.y = ub[c].y * (1 + bb[c].y * F1);
            }
        }
        usig[o] = out;
    }
}
__global__ void k_copy_faces(DevGrid<double> g, const double2* __restrict__ x, double2* ub) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    ub[g.idx(i, j)] = x[g.idx(i, j)];
}
void launch_velocity_profile(const PhysView& ph, int diva, const double2* x, const double2* bb, const double* F2,
                             const double* eta_sigma, double2* ub, double2* usig, cudaStream_t s) {
    LaunchDims d = dims2d(ph.g.Nx + 1, ph.g.Ny + 1);
    if (diva) { k_basal_velocity<<<d.grid, d.block, 0, s>>>(ph, x, bb, F2, ub); count_launch(); }
    else { k_copy_faces<<<d.grid, d.block, 0, s>>>(ph.g, x, ub); count_launch(); }
    k_velocity_profile<<<d.grid, d.block, 0, s>>>(ph, diva, x, bb, eta_sigma, ub, usig); count_launch();
}

// ---- geometry ---------------------------------------------------------------------------------------------
__device__ __forceinline__ double nonzero(double x) { return x == 0.0 ? 1.0 : x; }
// segment_grounded_fraction, subgrid_grounded_fraction.jl:34-38
__device__ __forceinline__ double segment_fraction(double f1, double f2) {
    double fp = fmax(f1, 0.0) + fmax(f2, 0.0);
    double S = fabs(f1) + fabs(f2);
    return S == 0.0 ? 1.0 : fp / nonzero(S);
}
// triangle_grounded_fraction, subgrid_grounded_fraction.jl:41-49
__device__ __forceinline__ double triangle_fraction(double f1, double f2, double f3) {
    double a = fmin(fmin(f1, f2), f3);
    double c = fmax(fmax(f1, f2), f3);
    double b = f1 + f2 + f3 - a - c;
    double one_grounded = c * c / nonzero((c - a) * (c - b));
    double one_floating = 1.0 - a * a / nonzero((b - a) * (c - a));
    double phi = b > 0 ? one_floating : one_grounded;
    return a >= 0 ? 1.0 : (c <= 0 ? 0.0 : phi);
}

// effective_pressure of a TillEffectivePressure (till_effective_pressure.jl:63-70) at overburden P0 and basal water
// Hw: the saturation s and the till's own N (before the cap by the ocean-connected one)
__device__ __forceinline__ double till_pressure(const GeometryView& v, double P0, double Hw, double& sat) {
    sat = fmin(fmax(Hw / v.till_Wmax, 0.0), 1.0);
    double Pt = P0 > 0 ? P0 : v.till_N0 / v.till_delta;   // a positive stand-in where P0 = 0 (N is the cap's 0 there)
    return v.till_N0 * pow(v.till_delta * Pt / v.till_N0, sat) * pow(10.0, v.till_e0_Cc * (1 - sat));
}

// update_geometry! (ice_sheet_model_methods.jl:103-111): s, φ, φᵘ, φᵛ, N, μ
__global__ void k_geometry(GeometryView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    double rw_ri = v.rho_w / v.rho_i, ri_rw = v.rho_i / v.rho_w;
    auto f = [&](int a, int b) { int c = g.c_idx(a, b); return v.H[c] + rw_ri * v.bed[c]; };
    int k = g.idx(i, j);
    if (i < g.Nx && j < g.Ny) {
        double H = v.H[k], b = v.bed[k];
        v.s[k] = v.grounding ? fmax(b + H, (1 - ri_rw) * H) : b + H;
        double rig = v.rho_i * v.gacc, rwg = v.rho_w * v.gacc;
        double No = fmax(rig * H + rwg * fmin(b, 0.0), 0.0);
        double sat;
        v.N[k] = v.Hw ? fmin(till_pressure(v, rig * H, v.Hw[k], sat), No) : No;
        double t = fmin(fmax((H - v.mask_min) / v.mask_trans, 0.0), 1.0);
        if (!v.front) v.mu[k] = t * t * (3 - 2 * t);   // a partial-cell front's flag is prognostic
        if (v.grounding) {
            double fc = f(i, j);
            double fe = (fc + f(i + 1, j)) / 2, fw = (fc + f(i - 1, j)) / 2, fn = (fc + f(i, j + 1)) / 2, fs = (fc + f(i, j - 1)) / 2;
            double fne = (fc + f(i + 1, j) + f(i, j + 1) + f(i + 1, j + 1)) / 4;
            double fnw = (fc + f(i - 1, j) + f(i, j + 1) + f(i - 1, j + 1)) / 4;
            double fse = (fc + f(i + 1, j) + f(i, j - 1) + f(i + 1, j - 1)) / 4;
            double fsw = (fc + f(i - 1, j) + f(i, j - 1) + f(i - 1, j - 1)) / 4;
            double phi = triangle_fraction(fc, fe, fne) + triangle_fraction(fc, fn, fne) + triangle_fraction(fc, fn, fnw) +
                         triangle_fraction(fc, fw, fnw) + triangle_fraction(fc, fw, fsw) + triangle_fraction(fc, fs, fsw) +
                         triangle_fraction(fc, fs, fse) + triangle_fraction(fc, fe, fse);
            v.phi[k] = phi / 8;
        } else {
            v.phi[k] = 1.0;
        }
    }
    double2 ph = v.phi_uv[k];
    if (j < g.Ny && (i < g.Nx || !g.px)) ph.x = v.grounding ? segment_fraction(f(i - 1, j), f(i, j)) : 1.0;
    if (i < g.Nx && (j < g.Ny || !g.py)) ph.y = v.grounding ? segment_fraction(f(i, j - 1), f(i, j)) : 1.0;
    v.phi_uv[k] = ph;
}

// compute_driving_stress!, driving_stress.jl:43-125
struct DrivingStressArgs { GeometryView v; };

__device__ __forceinline__ double front_force(const GeometryView& v, int c) {   // :56-60
    double Hi = v.H[c];
    double D = fmin(fmax(Hi - v.s[c], 0.0), Hi);
    return v.gacc * (v.rho_i * Hi * Hi - v.rho_w * D * D) / 2;
}
__device__ __forceinline__ double gl_stress(const GeometryView& v, int c1, int c2, bool& straddles) {   // :84-92
    double ri = v.rho_i, rw = v.rho_w;
    double H1 = v.H[c1], H2 = v.H[c2], s1 = v.s[c1], s2 = v.s[c2], b1 = v.bed[c1], b2 = v.bed[c2];
    double f1 = H1 + rw / ri * b1, f2 = H2 + rw / ri * b2;
    straddles = ((f1 > 0) != (f2 > 0)) && (H1 > 0) && (H2 > 0);
    double theta = f1 / (straddles ? f1 - f2 : 1.0);
    double Hg = H1 + theta * (H2 - H1);
    double sg = (1 - ri / rw) * Hg;
    return -ri * v.gacc * ((H1 + Hg) * (sg - s1) + (Hg + H2) * (s2 - sg)) / 2;
}

__global__ void k_driving_stress(GeometryView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    double2 tau = v.tau[k];
    if (j < g.Ny && (i < g.Nx || !g.px)) {   // _compute_x_driving_stress!, :109-116
        int cw = g.c_idx(i - 1, j), ce = g.c_idx(i, j);
        bool wall = g.peripheral_fc(i, j) || (v.use_mask && (v.mu[cw] + v.mu[ce]) == 0.0);
        bool front = false, straddles = false;
        double tf = 0.0, tg = 0.0;
        if (v.use_mask) {
            bool w = v.mu[cw] > 0 && !(v.mu[ce] > 0), e = !(v.mu[cw] > 0) && v.mu[ce] > 0;
            double F = (w ? front_force(v, cw) : 0.0) - (e ? front_force(v, ce) : 0.0);
            front = w || e;
            tf = g.dyc[j] * F;
        }
        if (v.gl_stress) tg = g.dyc[j] * gl_stress(v, cw, ce, straddles);
        double t = -g.Az_fc(i, j) * v.rho_i * v.gacc * ((v.H[cw] + v.H[ce]) / 2) * ((v.s[ce] - v.s[cw]) * g.rdxf[i]);
        tau.x = wall ? 0.0 : (front ? tf : (straddles ? tg : t));
        if (prescribed_u(g, v.ud, i, j)) tau.x = v.ud[k].x;   // the identity row's right-hand side
    }
    if (i < g.Nx && (j < g.Ny || !g.py)) {   // _compute_y_driving_stress!, :118-125
        int cs = g.c_idx(i, j - 1), cn = g.c_idx(i, j);
        bool wall = g.peripheral_cf(i, j) || (v.use_mask && (v.mu[cs] + v.mu[cn]) == 0.0);
        bool front = false, straddles = false;
        double tf = 0.0, tg = 0.0;
        if (v.use_mask) {
            bool so = v.mu[cs] > 0 && !(v.mu[cn] > 0), no = !(v.mu[cs] > 0) && v.mu[cn] > 0;
            double F = (so ? front_force(v, cs) : 0.0) - (no ? front_force(v, cn) : 0.0);
            front = so || no;
            tf = g.dxc[i] * F;
        }
        if (v.gl_stress) tg = g.dxc[i] * gl_stress(v, cs, cn, straddles);
        double t = -g.Az_cf(i, j) * v.rho_i * v.gacc * ((v.H[cs] + v.H[cn]) / 2) * ((v.s[cn] - v.s[cs]) * g.rdyf[j]);
        tau.y = wall ? 0.0 : (front ? tf : (straddles ? tg : t));
        if (prescribed_v(g, v.ud, i, j)) tau.y = v.ud[k].y;
    }
    v.tau[k] = tau;
}

void launch_geometry(const GeometryView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx + 1, v.g.Ny + 1);
    k_geometry<<<d.grid, d.block, 0, s>>>(v); count_launch();
    k_driving_stress<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// _compute_rate_factor! with ω = 0 (column_energy_solve.jl:104-110) and arrhenius_rate_factor (arrhenius_rate_factor.jl:102-110)
__global__ void k_rate_factor(DevGrid<double> g, SigmaTable sig, int plane, const double* __restrict__ H, const double* __restrict__ T,
                              double* A, double rho_i, double gacc, const double* __restrict__ prm) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double Ac = prm[0], Aw = prm[1], Qc = prm[2], Qw = prm[3], Tt = prm[4], Tw = prm[5], R = prm[6], bcc = prm[7], Tm = prm[8];
    for (int k = 0; k < sig.N; ++k) {
        long long o = (long long)k * plane + c;
        double p = rho_i * gacc * H[c] * (1 - sig.zc[k]);
        double Tp = T[o] - (Tm - bcc * p) + Tm;
        double log_cold = log(Ac) - Qc / (R * Tp);
        double log_warm = log(Aw) - Qw / (R * Tp);
        double x = fmin(fmax((Tp - Tt) / Tw + 1.0 / 2, 0.0), 1.0);
        double s = x * x * (3 - 2 * x);
        A[o] = exp((1 - s) * log_cold + s * log_warm) * 1.0;   // water softening 1 + c min(ω, ω_max) = 1 at ω = 0
    }
}
void launch_rate_factor(const DevGrid<double>& g, const SigmaTable& sig, int plane, const double* H, const double* T, double* A,
                        double rho_i, double gacc, const double* params, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_rate_factor<<<d.grid, d.block, 0, s>>>(g, sig, plane, H, T, A, rho_i, gacc, params); count_launch();
}

// update_thermal_diagnostics! with an ArrheniusRateFactor (column_energy_solve.jl:85-110): per layer, from the
// enthalpy, the temperature and water fraction (temperature / water_fraction, enthalpy_conversions.jl:35, :42) and
// the rate factor of the pressure-adjusted temperature with the water softening (arrhenius_rate_factor.jl:102-110).
// prm: the 14 doubles of nk_thermal_params in order.
__global__ void k_thermal_diagnostics(DevGrid<double> g, SigmaTable sig, int plane, const double* __restrict__ H,
                                      const double* __restrict__ E, double* T, double* omega, double* A, double rho_i, double gacc,
                                      const double* __restrict__ prm) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double Ac = prm[0], Aw = prm[1], Qc = prm[2], Qw = prm[3], Tt = prm[4], Tw = prm[5], R = prm[6], cw = prm[7], wmax = prm[8];
    double ci = prm[9], L = prm[10], bcc = prm[11], T0 = prm[12], Tr = prm[13];
    for (int k = 0; k < sig.N; ++k) {
        long long o = (long long)k * plane + c;
        double p = rho_i * gacc * H[c] * (1 - sig.zc[k]);      // layer_pressure
        double Tpm = T0 - bcc * p;                             // pressure_melting_temperature
        double Epm = ci * (Tpm - Tr);                          // pressure_melting_enthalpy
        double e = E[o];
        double t = fmin(Tpm, Tr + e / ci);
        double w = fmax(0.0, e - Epm) / L;
        double Tp = t - Tpm + T0;
        double log_cold = log(Ac) - Qc / (R * Tp);
        double log_warm = log(Aw) - Qw / (R * Tp);
        double x = fmin(fmax((Tp - Tt) / Tw + 1.0 / 2, 0.0), 1.0);
        double s = x * x * (3 - 2 * x);
        T[o] = t;
        omega[o] = w;
        A[o] = exp((1 - s) * log_cold + s * log_warm) * (1 + cw * fmin(w, wmax));
    }
}
void launch_thermal_diagnostics(const DevGrid<double>& g, const SigmaTable& sig, int plane, const double* H, const double* E, double* T,
                                double* omega, double* A, double rho_i, double gacc, const double* params, cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx, g.Ny);
    k_thermal_diagnostics<<<d.grid, d.block, 0, s>>>(g, sig, plane, H, E, T, omega, A, rho_i, gacc, params); count_launch();
}

// ---- thickness transport -----------------------------------------------------------------------------------
// update_bounds_preserving_limiter! (src/Models/time_stepping.jl:35-42) restated as the Zhang-Shu (2010) limiter per
// direction: from cell (i, j)'s own WENO face values W, E, S, N and the interior quadrature values
// p̃ = (H̄ - ω (W + E)) / (1 - 2ω), ω = 5/18 (likewise in y), θ = min(1, |(upper - H̄) / (M - H̄ + ε)|,
// |(lower - H̄) / (m - H̄ - ε)|) with M, m the largest and smallest of the six and ε = 2 eps.
// The two WENO reconstructions of every face, once: x faces (i, j) for i in 0..Nx, j < Ny and y faces for i < Nx,
// j in 0..Ny (on a periodic axis the last face repeats the first, from the same wrapped stencils).
__global__ void k_thickness_faces(ThicknessView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    const double* __restrict__ Hs = v.Hs;
    double s[5];
    int k = g.idx(i, j);
    if (j < g.Ny) {
        double2 r;
        stencil_x(g, Hs, i, j, true, s);
        r.x = weno5_face(s);
        stencil_x(g, Hs, i, j, false, s);
        r.y = weno5_face(s);
        v.fx[k] = r;
    }
    if (i < g.Nx) {
        double2 r;
        stencil_y(g, Hs, i, j, true, s);
        r.x = weno5_face(s);
        stencil_y(g, Hs, i, j, false, s);
        r.y = weno5_face(s);
        v.fy[k] = r;
    }
}
void launch_thickness_faces(const ThicknessView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx + 1, v.g.Ny + 1);
    k_thickness_faces<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

__global__ void k_thickness_limiter(ThicknessView v) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const double* __restrict__ Hs = v.Hs;
    double Hc = Hs[g.idx(i, j)];
    // the cell's own reconstructions at its four faces (k_thickness_faces)
    double E = v.fx[g.idx(i + 1, j)].x, W = v.fx[g.idx(i, j)].y;
    double N = v.fy[g.idx(i, j + 1)].x, S = v.fy[g.idx(i, j)].y;
    const double w = 5.0 / 18, eps = 2 * 2.220446049250313e-16;
    double px = (Hc - w * W - w * E) / (1 - 2 * w);
    double py = (Hc - w * S - w * N) / (1 - 2 * w);
    double M = fmax(fmax(fmax(px, py), fmax(W, E)), fmax(S, N));
    double m = fmin(fmin(fmin(px, py), fmin(W, E)), fmin(S, N));
    v.theta[g.idx(i, j)] = fmin(fmin(fabs((v.upper - Hc) / (M - Hc + eps)), fabs((v.lower - Hc) / (m - Hc - eps))), 1.0);
}
void launch_thickness_limiter(const ThicknessView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx, v.g.Ny);
    k_thickness_limiter<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// One split Runge-Kutta stage of the mass balance, the tendency and the substep fused (_compute_thickness_tendency!
// and _thickness_substep!, src/Models/time_stepping.jl:59-72): G = a - (1 - φ) m - mᵍ - ∇⋅(ū H) at cell (i, j) from
// the stage-start thickness Hs, the flux through each face Δ (u H_face) with the scheme's upwind-biased face thickness
// (limited by the upwind cell's θ for a bounded WENO: H̄ + θ (H_face - H̄)); nothing through a Bounded wall; then
// H = max(0, H⁻ + Δτ G) from the step-start thickness H⁻, and in the last stage the clip max(0, -H★) added to Hc.
// Hs and H are distinct arrays: every cell reads its neighbours' stage-start thickness.
__global__ void k_thickness_stage(ThicknessView v, double dtau, int final_stage) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const double* __restrict__ Hs = v.Hs;
    const bool bounded = v.scheme == NK_ADVECTION_WENO && v.bounded;
    auto limited = [&](double h, int k) { return bounded ? Hs[k] + v.theta[k] * (h - Hs[k]) : h; };
    // with a partial-cell front (front_flux_x / front_flux_y, partial_cell_front.jl:114-132): the scheme's flux between
    // full cells, the upwind flux out of a full cell into a front cell, nothing out of a front cell
    auto full = [&](int k) { return !v.mu || v.mu[k] > 0; };
    auto xflux = [&](int f) {
        if (g.peripheral_fc(f, j)) return 0.0;
        double u = v.x[g.u_idx(f, j)].x, s[5];
        int kw = g.c_idx(f - 1, j), ke = g.c_idx(f, j);
        bool west = full(kw), eastc = full(ke);
        if (!(west && eastc)) return (west || eastc) ? g.dyc[j] * (west ? fmax(u, 0.0) * Hs[kw] : fmin(u, 0.0) * Hs[ke]) : 0.0;
        bool east = u > 0;
        double h0;
        if (v.fx) {
            double2 r = v.fx[g.idx(f, j)];
            h0 = east ? r.x : r.y;
        } else {
            stencil_x(g, Hs, f, j, east, s);
            h0 = face_value(v, s);
        }
        double h = limited(h0, east ? kw : ke);
        return g.dyc[j] * (u * h);
    };
    auto yflux = [&](int f) {
        if (g.peripheral_cf(i, f)) return 0.0;
        double w = v.x[g.v_idx(i, f)].y, s[5];
        int ks = g.c_idx(i, f - 1), kn = g.c_idx(i, f);
        bool south = full(ks), northc = full(kn);
        if (!(south && northc)) return (south || northc) ? g.dxc[i] * (south ? fmax(w, 0.0) * Hs[ks] : fmin(w, 0.0) * Hs[kn]) : 0.0;
        bool north = w > 0;
        double h0;
        if (v.fy) {
            double2 r = v.fy[g.idx(i, f)];
            h0 = north ? r.x : r.y;
        } else {
            stencil_y(g, Hs, i, f, north, s);
            h0 = face_value(v, s);
        }
        double h = limited(h0, north ? ks : kn);
        return g.dxc[i] * (w * h);
    };
    int c = g.idx(i, j);
    double m = v.grounding ? (1 - v.phi[c]) * v.melt[c] : v.melt[c];
    double S = v.smb[c] - m - (v.coupled ? v.gmelt[c] : 0.0);
    if (!full(c)) S = 0.0;   // sources on full cells only (ice_source_mask)
    double div = (xflux(i + 1) - xflux(i) + yflux(j + 1) - yflux(j)) / g.Az_cc(i, j);
    double Hstar = v.H0[c] + dtau * (S - div);
    v.H[c] = 0.0 < Hstar ? Hstar : 0.0;
    if (final_stage) v.clipped[c] += 0.0 < -Hstar ? -Hstar : 0.0;
}
void launch_thickness_stage(const ThicknessView& v, double dtau, int final_stage, cudaStream_t s) {
    LaunchDims d = dims2d(v.g.Nx, v.g.Ny);
    k_thickness_stage<<<d.grid, d.block, 0, s>>>(v, dtau, final_stage); count_launch();
}

// ---- the energy step ----------------------------------------------------------------------------------------
__device__ __forceinline__ double dmin(double a, double b) { return b < a ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return a < b ? b : a; }
// unit_ramp(x, w) = clamp(x / w, 0, 1), src/Thermodynamics/enthalpy_conversions.jl:69
__device__ __forceinline__ double unit_ramp(double x, double w) { return dmin(dmax(x / w, 0.0), 1.0); }

// step_thermodynamics! (src/Thermodynamics/column_energy_solve.jl:26-78) for one column (i, j), one thread:
// 1. the strain heating Φₖ = 4 ηₖ ε̇ₑ² (+ τᵇ² w₂ₖ / Δζₖ / ηₖ for the DIVA), strain_heating.jl:43-56;
// 2. the layer volume fluxes Wₖ from the basal melt up, layer_transport.jl:34-44 (upwind Hⁿ through each face);
// 3. the basal state: conductance D, friction heat F, the ramps r (warm or wet base) and s_b (temperate basal
//    layer), qᵍ = φ G + F, :127-146;
// 4. the implicit system of the Nσ layers (:148-221: storage, the upwind-or-diffusive face couplings, the basal
//    and surface boundary rows, the horizontal upwind enthalpy transport of the old E), built row by row inside the
//    forward sweep of the Thomas algorithm (row k: a[k-1] E[k-1] + b[k] E[k] + c[k] E[k+1] = f[k]), then the
//    backward sweep;
// 5. the basal water balance and the drainage of temperate ice, :223-259;
// 6. T = min(T_pm, T_r + E / c) and ω = max(0, E - E_pm) / L on every layer.
// Columns thinner than the minimum thickness hold the surface enthalpy.  E_old is a copy of E: the neighbours'
// old enthalpy is read while this column writes its new one.
__global__ void __launch_bounds__(128) k_step_enthalpy(EnergyView v, double dt) {
    const DevGrid<double>& g = v.g;
    int i = blockIdx.x * 32 + threadIdx.x, j = blockIdx.y * 4 + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    const EnergyConstants& q = v.q;
    const SigmaTable& sg = v.sig;
    const int Ns = sg.N;
    const long long P = v.plane;
    const int c = g.idx(i, j);
    const double rho = v.rho_i, ga = v.gacc, H = v.H[c], Hn = v.Hn[c];
    // The kernel is bound by the FP64 pipe, where a division costs about ten multiply-adds: divisors that stay fixed
    // through the column are inverted once and each layer's diffusivity is evaluated once (the results differ from
    // the quotients of the formulas in the last bits only).
    const double r_L = 1 / q.L, r_c = 1 / q.c, r_blend = 1 / q.blend, r_dt = 1 / dt, k_c = q.k / q.c;
    auto ramp = [](double x, double rw) { return dmin(dmax(x * rw, 0.0), 1.0); };   // unit_ramp with 1/w
    auto Tpm = [&](double p) { return q.T0 - q.beta * p; };
    auto Epm = [&](double p) { return q.c * (Tpm(p) - q.Tr); };
    auto enthalpy = [&](double T, double p) { return q.c * (dmin(T, Tpm(p)) - q.Tr) + 0.0 * q.L; };
    auto water_fraction = [&](double E, double p) { return dmax(0.0, E - Epm(p)) * r_L; };
    auto thickness = [&](double h) { return dmax(h, q.min_thickness); };
    auto layer_pressure = [&](int k) { return rho * ga * H * (1 - sg.zc[k - 1]); };
    auto Eold = [&](int k, int ii, int jj) { return v.E_old[(k - 1) * P + g.c_idx(ii, jj)]; };
    auto diffusivity = [&](int k) {
        double w = ramp(Eold(k, i, j) - Epm(layer_pressure(k)) + q.blend, r_blend);
        return k_c * (1 - w + w * q.temperate_ratio);
    };
    const double phi_g = v.grounding ? v.phi[c] : 1.0;

    // 1. strain heating
    double e2 = effective_strain_rate2(g, v.x, v.ud, i, j, v.wall_factor);
    double tb2 = 0.0;
    if (v.diva) {
        int u0 = g.u_idx(i, j), u1 = g.u_idx(i + 1, j), v0 = g.v_idx(i, j), v1 = g.v_idx(i, j + 1);
        double a0 = v.bb[u0].x * v.ub[u0].x, a1 = v.bb[u1].x * v.ub[u1].x;
        double b0 = v.bb[v0].y * v.ub[v0].y, b1 = v.bb[v1].y * v.ub[v1].y;
        tb2 = (a0 * a0 + a1 * a1) / 2 + (b0 * b0 + b1 * b1) / 2;
    }
    for (int k = 1; k <= Ns; ++k) {
        double eta = v.eta_sigma[(k - 1) * P + c];
        double ph = 4 * eta * e2;
        if (v.diva) ph += tb2 * sg.w2[k - 1] / (sg.dz[k - 1] * (eta == 0.0 ? INFINITY : eta));
        v.Phi[(k - 1) * P + c] = ph;
    }

    // 2. layer volume fluxes
    auto layer_u = [&](int f, int k) { return g.peripheral_fc(f, j) ? 0.0 : v.usig[(k - 1) * P + g.u_idx(f, j)].x; };
    auto layer_v = [&](int f, int k) { return g.peripheral_cf(i, f) ? 0.0 : v.usig[(k - 1) * P + g.v_idx(i, f)].y; };
    auto xvol = [&](int f, int k) {
        double u = layer_u(f, k);
        return g.dyc[j] * u * (u > 0 ? v.Hn[g.c_idx(f - 1, j)] : v.Hn[g.c_idx(f, j)]);
    };
    auto yvol = [&](int f, int k) {
        double w = layer_v(f, k);
        return g.dxc[i] * w * (w > 0 ? v.Hn[g.c_idx(i, f - 1)] : v.Hn[g.c_idx(i, f)]);
    };
    auto xenth = [&](int f, int k) {
        double u = v.usig[(k - 1) * P + g.u_idx(f, j)].x;
        return xvol(f, k) * (u > 0 ? Eold(k, f - 1, j) : Eold(k, f, j));
    };
    auto yenth = [&](int f, int k) {
        double w = v.usig[(k - 1) * P + g.v_idx(i, f)].y;
        return yvol(f, k) * (w > 0 ? Eold(k, i, f - 1) : Eold(k, i, f));
    };
    const double Az = g.Az_cc(i, j), r_Az = 1 / Az;
    double W[ENERGY_MAX_LAYERS + 1];
    {
        double dHdt = (thickness(H) - thickness(Hn)) * r_dt;
        double m = v.grounding ? (1 - v.phi[c]) * v.melt[c] : v.melt[c];
        W[0] = -m - (q.coupled ? v.gmelt[c] : 0.0);
        for (int k = 1; k <= Ns; ++k) {
            double div = (xvol(i + 1, k) - xvol(i, k) + yvol(j + 1, k) - yvol(j, k)) * r_Az;
            W[k] = W[k - 1] - sg.dz[k - 1] * (dHdt + div);
        }
    }

    // 3. basal state
    const double Ht = thickness(H), Hnt = thickness(Hn);
    const double kap1 = diffusivity(1);
    const double D = kap1 / (Ht * sg.zc[0]);
    double F;
    {
        int u0 = g.u_idx(i, j), u1 = g.u_idx(i + 1, j), v0 = g.v_idx(i, j), v1 = g.v_idx(i, j + 1);
        double bu0 = v.diva ? v.bb[u0].x : v.coef[u0].z, bu1 = v.diva ? v.bb[u1].x : v.coef[u1].z;
        double bv0 = v.diva ? v.bb[v0].y : v.coef[v0].w, bv1 = v.diva ? v.bb[v1].y : v.coef[v1].w;
        double ub0 = v.ub[u0].x, ub1 = v.ub[u1].x, vb0 = v.ub[v0].y, vb1 = v.ub[v1].y;
        F = (bu0 * ub0 * ub0 + bu1 * ub1 * ub1 + bv0 * vb0 * vb0 + bv1 * vb1 * vb1) / 2;
    }
    const double pb = rho * ga * H;
    const double Epm_b = Epm(pb);
    const double Hw0 = v.Hw[c], G = v.G[c];
    const double r = dmax(ramp(Eold(1, i, j) + (G + F) / D - Epm_b, r_blend), unit_ramp(Hw0, q.water_blend));
    const double sb = ramp(Eold(1, i, j) - Epm(layer_pressure(1)) + q.blend, r_blend);
    const double qg = phi_g * G + F;
    v.sb[c] = sb;
    v.qg[c] = qg;

    // 4. the column system and the Thomas algorithm
    const bool mu = H > q.min_thickness;
    const double Es = enthalpy(v.Ts[c], 0.0);
    const double chi = phi_g * r * (1 - sb);
    const double Eo = enthalpy(v.To[c], pb);
    const double Fb = rho * W[0];
    const double Lam = D * (chi + 1 - phi_g) + dmax(-Fb, 0.0);
    const double S = (1 - r) * qg + D * (chi * Epm_b + (1 - phi_g) * Eo) + dmax(Fb, 0.0) * Epm_b;
    const double Fs = rho * W[Ns];
    const double kapN = Ns == 1 ? kap1 : diffusivity(Ns);
    const double Ks = kapN / (Ht * (1 - sg.zc[Ns - 1]));
    const double Ds = Ks + dmax(Fs, 0.0), Ss = (Ks + dmax(-Fs, 0.0)) * Es;
    // interior face kf = 2..Nσ between layers of diffusivities km (below) and kp (above)
    auto couplings = [&](int kf, double km, double kp, double& lower, double& upper) {
        double zf = sg.zf[kf - 1], zm = sg.zc[kf - 2], zp = sg.zc[kf - 1];
        double theta = (zf - zm) / (zp - zm);
        double Fk = rho * W[kf - 1];
        double cond = km * kp / (Ht * ((zf - zm) * kp + (zp - zf) * km));   // 1 / (Ht ((zf - zm) / km + (zp - zf) / kp))
        double Dk = dmax(cond, dmax(dmax(Fk, 0.0) * theta, dmax(-Fk, 0.0) * (1 - theta)));
        lower = -Fk * (1 - theta) - Dk;
        upper = Fk * theta - Dk;
    };
    double t[ENERGY_MAX_LAYERS + 1], e[ENERGY_MAX_LAYERS + 1];
    double lower_m = 0, upper_m = 0, prev_a = 0, prev_c = 0, rpiv = 1;
    double kap_k = kap1;
    for (int k = 1; k <= Ns; ++k) {
        double dz = sg.dz[k - 1];
        double lower_p = 0, upper_p = 0;
        if (k < Ns) {
            double kap_n = k + 1 == Ns ? kapN : diffusivity(k + 1);
            couplings(k + 1, kap_k, kap_n, lower_p, upper_p);
            kap_k = kap_n;
        }
        double diag_m = k == 1 ? Lam : -upper_m;
        double diag_p = k == Ns ? Ds : -lower_p;
        double forcing = (k == 1 ? S : 0.0) + (k == Ns ? Ss : 0.0);
        double transport = rho * dz * ((xenth(i + 1, k) - xenth(i, k) + yenth(j + 1, k) - yenth(j, k)) * r_Az);
        double ak = mu ? lower_p : 0.0;
        double ck = mu ? upper_p : 0.0;
        double bk = mu ? rho * Ht * dz * r_dt + diag_m + diag_p : 1.0;
        double fk = mu ? rho * Hnt * dz * Eold(k, i, j) * r_dt - transport + Ht * dz * v.Phi[(k - 1) * P + c] + forcing : Es;
        if (k == 1) {
            rpiv = 1 / bk;
            e[1] = fk * rpiv;
        } else {
            t[k] = prev_c * rpiv;
            rpiv = 1 / (bk - prev_a * t[k]);
            e[k] = (fk - prev_a * e[k - 1]) * rpiv;
        }
        prev_a = ak; prev_c = ck;
        lower_m = lower_p; upper_m = upper_p;
    }
    for (int k = Ns - 1; k >= 1; --k) e[k] -= t[k + 1] * e[k + 1];

    // 5. basal water and drainage
    {
        double qb = D * (Epm_b - e[1]);
        double m = r * (qg - phi_g * (1 - sb) * qb) / (rho * q.L);
        double drained = 0;
        const double r_drain = 1 / q.drainage_fraction;
        for (int k = 1; k <= Ns; ++k) {
            double w = water_fraction(e[k], layer_pressure(k));
            double x = w * r_drain;
            double rate = q.max_drainage_rate * (dmin(dmax(x - 1, 0.0), 1.0) + 9 * dmin(dmax(x - 2, 0.0), 1.0)) * 0.1;
            double dw = dmin(dt * rate, dmax(w - q.drainage_fraction, 0.0));
            dw = mu ? dw : 0.0;
            e[k] -= q.L * dw;
            drained += Ht * sg.dz[k - 1] * dw;
        }
        double Hstar = Hw0 + dt * (mu ? m : 0.0) + drained;
        double Hplus = dmax(0.0, Hstar);
        double missing = Hplus - Hstar;
        v.gmelt[c] = (Hplus - Hw0) * r_dt;
        v.Hw[c] = v.till ? dmin(dmax(Hplus - dt * v.till_drain, 0.0), v.till_Wmax) : Hplus;   // drain_till
        e[1] -= q.L * missing / (Ht * sg.dz[0]);
    }

    // 6. the new enthalpy and its diagnostics
    for (int k = 1; k <= Ns; ++k) {
        double p = layer_pressure(k), E = e[k];
        v.E[(k - 1) * P + c] = E;
        v.T[(k - 1) * P + c] = dmin(Tpm(p), q.Tr + E * r_c);
        v.omega[(k - 1) * P + c] = water_fraction(E, p);
    }
}
void launch_step_enthalpy(const EnergyView& v, double dt, cudaStream_t s) {
    dim3 block(32, 4), grid((v.g.Nx + 31) / 32, (v.g.Ny + 3) / 4);
    k_step_enthalpy<<<grid, block, 0, s>>>(v, dt); count_launch();
}

// ---- fixed-point adjoint of the SSA Picard step -------------------------------------------------------------
// The reverse of picard_coefficient_step! (ext/NunatakEnzymeExt.jl:142-157): with q = A(c(x)) x*, the seed
// q̄ = -λ, and x* the converged velocity, it returns ȳ = -(∂q/∂x)ᵀ λ.  Only active operator rows depend on
// the coefficients (inactive rows are identities), so λ enters as λ̃ = λ masked like the operator's
// interior_u / interior_v.  The chain runs back through _compute_basal_drag!, _interpolate_to_corners! and
// compute_viscosity! exactly as they are evaluated in the forward kernels above.

// basal_drag and its derivatives with respect to the speed U and the face coefficient C (frictions.jl:83-89)
__device__ __forceinline__ void basal_drag_derivatives(const PhysView& ph, double U, double C, double N, double& b, double& dbdU,
                                                       double& dbdC) {
    double pw = pow(U, ph.m - 1);
    double w = C * pw;
    if (ph.friction == NK_WEERTMAN) {
        b = w;
        dbdU = (ph.m - 1) * w / U;
        dbdC = pw;
        return;
    }
    double tc = ph.alpha2 * N;
    double cm = pow(C, 1 / ph.m), den = cm * U + pow(tc, 1 / ph.m);
    b = w * tc / pow(den, ph.m);
    if (b == 0.0) {
        dbdU = 0.0;
        dbdC = 0.0;
        return;
    }
    dbdU = b * ((ph.m - 1) / U - ph.m * cm / den);
    dbdC = b * (1 / C - cm * U / (C * den));
}

// Speed and drag of the u face (i, j) as k_basal_drag evaluates them; returns false where βᵘ is zero or absent.
__device__ __forceinline__ bool u_drag(const PhysView& ph, const double2* __restrict__ x, int i, int j, double& u, double& vf,
                                       double& U, double& phi, double& b, double& dbdU, double& dbdC) {
    const DevGrid<double>& g = ph.g;
    if (ph.friction == NK_FRICTION_NONE || j >= g.Ny || (i >= g.Nx && g.px) || g.peripheral_fc(i, j)) return false;
    int k = g.idx(i, j);
    vf = ((x[g.v_idx(i - 1, j)].y + x[g.v_idx(i, j)].y) / 2 + (x[g.v_idx(i - 1, j + 1)].y + x[g.v_idx(i, j + 1)].y) / 2) / 2;
    u = x[k].x;
    U = sqrt(u * u + vf * vf + ph.u0 * ph.u0);
    double Cf = (ph.C[g.c_idx(i - 1, j)] + ph.C[g.c_idx(i, j)]) / 2;
    double Nf = ph.use_N ? (ph.N[g.c_idx(i - 1, j)] + ph.N[g.c_idx(i, j)]) / 2 : 0.0;
    phi = ph.phi[k].x;
    basal_drag_derivatives(ph, U, Cf, Nf, b, dbdU, dbdC);
    return true;
}
__device__ __forceinline__ bool v_drag(const PhysView& ph, const double2* __restrict__ x, int i, int j, double& v, double& uf,
                                       double& U, double& phi, double& b, double& dbdU, double& dbdC) {
    const DevGrid<double>& g = ph.g;
    if (ph.friction == NK_FRICTION_NONE || i >= g.Nx || (j >= g.Ny && g.py) || g.peripheral_cf(i, j)) return false;
    int k = g.idx(i, j);
    uf = ((x[g.u_idx(i, j - 1)].x + x[g.u_idx(i + 1, j - 1)].x) / 2 + (x[g.u_idx(i, j)].x + x[g.u_idx(i + 1, j)].x) / 2) / 2;
    v = x[k].y;
    U = sqrt(v * v + uf * uf + ph.u0 * ph.u0);
    double Cf = (ph.C[g.c_idx(i, j - 1)] + ph.C[g.c_idx(i, j)]) / 2;
    double Nf = ph.use_N ? (ph.N[g.c_idx(i, j - 1)] + ph.N[g.c_idx(i, j)]) / 2 : 0.0;
    phi = ph.phi[k].y;
    basal_drag_derivatives(ph, U, Cf, Nf, b, dbdU, dbdC);
    return true;
}

// Coefficient adjoints from λ̃ and x*: at centre (i, j) ∂(λ̃ᵀq)/∂η̄H through Δy Txx and Δx Tyy; at corner (i, j)
// ∂(λ̃ᵀq)/∂η̄Hᶠᶠ through the shear stress; at faces ∂(λ̃ᵀq)/∂β = λ̃ Az x* (ssa_operator.jl:60-89).
__global__ void k_adjoint_coefficients(AdjointView v) {
    const OpView<double>& o = v.o;
    const DevGrid<double>& g = o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    double2 cb = make_double2(0.0, 0.0), bb = make_double2(0.0, 0.0);
    if (i < g.Nx && j < g.Ny) {
        double exx = (masked_u(o, v.xs, i + 1, j) - masked_u(o, v.xs, i, j)) * g.rdxc[i];
        double eyy = (masked_v(o, v.xs, i, j + 1) - masked_v(o, v.xs, i, j)) * g.rdyc[j];
        double dlu = masked_u(o, v.lam, i + 1, j) - masked_u(o, v.lam, i, j);
        double dlv = masked_v(o, v.lam, i, j + 1) - masked_v(o, v.lam, i, j);
        cb.x = g.dyc[j] * (2.0 * (2.0 * exx + eyy)) * dlu + g.dxc[i] * (2.0 * (2.0 * eyy + exx)) * dlv;
    }
    {
        double dudy = (masked_u(o, v.xs, i, j) - masked_u(o, v.xs, i, j - 1)) * g.rdyf[j];
        double dvdx = (masked_v(o, v.xs, i, j) - masked_v(o, v.xs, i - 1, j)) * g.rdxf[i];
        double e = (dudy + dvdx) / 2;
        if (g.peripheral_ff(i, j)) e = o.wall_factor * e;
        double lu = masked_u(o, v.lam, i, j) - masked_u(o, v.lam, i, j - 1);
        double lv = masked_v(o, v.lam, i, j) - masked_v(o, v.lam, i - 1, j);
        cb.y = 2.0 * e * (g.dxf[i] * lu + g.dyf[j] * lv);
    }
    bool has_u = j < g.Ny && (i < g.Nx || !g.px), has_v = i < g.Nx && (j < g.Ny || !g.py);
    uint8_t m = o.mask[k];
    if (has_u && !(m & U_IDENTITY)) bb.x = v.lam[k].x * g.Az_fc(i, j) * v.xs[k].x;
    if (has_v && !(m & V_IDENTITY)) bb.y = v.lam[k].y * g.Az_cf(i, j) * v.xs[k].y;
    v.cbar[k] = cb;
    v.bbar[k] = bb;
}
void launch_adjoint_coefficients(const AdjointView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx + 1, v.o.g.Ny + 1);
    k_adjoint_coefficients<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// The distinct corner indices around centre index c along one axis, with the number of times _interpolate_to_corners!
// reads centre c for each (its clamped / wrapped index map can hit c twice).
__device__ __forceinline__ int corners_of_centre(int c, int n, bool periodic, int* f, int* w) {
    int a = c, b = periodic ? DevGrid<double>::wrap(c + 1, n) : c + 1;
    auto cmap = [&](int i) { return periodic ? DevGrid<double>::wrap(i, n) : DevGrid<double>::clampi(i, 0, n - 1); };
    f[0] = a;
    w[0] = (cmap(a - 1) == c) + (cmap(a) == c);
    if (b == a) return 1;
    f[1] = b;
    w[1] = (cmap(b - 1) == c) + (cmap(b) == c);
    return 2;
}

// Per centre: η̄H̄ = the centre-stress part + ¼ of the corner adjoints that _interpolate_to_corners! spreads from
// it; then back through η̄H = μ H Σₖ Δζₖ ½ Aₖ^(-1/n) S^((1-n)/2n), S = ε̇ₑ² + ε̇₀²: ḡ = η̄H̄ η̄H (1-n)/(2n) / S.
__global__ void k_adjoint_viscosity(AdjointView v) {
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    int fx[2], wx[2], fy[2], wy[2];
    int nx = corners_of_centre(i, g.Nx, g.px, fx, wx), ny = corners_of_centre(j, g.Ny, g.py, fy, wy);
    double eb = v.cbar[k].x;
    for (int a = 0; a < nx; ++a)
        for (int b = 0; b < ny; ++b) eb += (wx[a] * wy[b]) * v.cbar[g.idx(fx[a], fy[b])].y / 4;
    if (v.eta_bar_in) eb -= v.eta_bar_in[k];   // eb is λ-signed: minus the true adjoint
    const PhysView& ph = v.ph;
    double S = effective_strain_rate2(g, v.xs, ph.ud, i, j, ph.wall_factor) + ph.eps0 * ph.eps0;
    v.gbar[k] = eb * v.o.coef[k].x * ((1 - ph.n) / (2 * ph.n)) / S;
    if (v.grad_log_A) {
        // η = ½ A^(-1/n) S^((1-n)/2n): ∂η/∂log A = -η / n.  The adjoint of η̄H is -eb (eb is λ-signed and
        // p̄ = -(∂c/∂p)ᵀ eb), so with a 2-D A, which every layer shares, the cell's gradient is eb η̄H / n, and with
        // a σ-grid A layer k carries eb μ H Δζₖ ηₖ / n
        if (ph.rate_sigma) {
            double muH = (ph.use_mask ? ph.mu[k] : 1.0) * ph.H[k];
            for (int l = 0; l < ph.sig.N; ++l) {
                long long o = (long long)l * ph.plane + k;
                v.grad_log_A[o] = eb * (muH * ph.sig.dz[l] * v.eta_sigma[o]) / ph.n;
            }
        } else {
            v.grad_log_A[k] = eb * v.o.coef[k].x / ph.n;
        }
    }
}
void launch_adjoint_viscosity(const AdjointView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx, v.o.g.Ny);
    k_adjoint_viscosity<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// Map a candidate index to a stored one (wrap when periodic); false when it is outside a Bounded range [0, hi).
__device__ __forceinline__ bool map_index(int i, int n, bool periodic, int hi, int& out) {
    if (periodic) {
        out = DevGrid<double>::wrap(i, n);
        return true;
    }
    out = i;
    return i >= 0 && i < hi;
}
// Append `k` to a short list unless already there (tiny periodic grids map two candidates to one point).
__device__ __forceinline__ bool first_time(int* seen, int& n, int k) {
    for (int a = 0; a < n; ++a)
        if (seen[a] == k) return false;
    seen[n++] = k;
    return true;
}

// ∂S/∂(u or v at stored index k) for the centre (ci, cj): S = ε̇xx² + ε̇yy² + ε̇xx ε̇yy + ℑxyᶜᶜ(ε̇xy²) with the
// wall-masked velocities of effective_strain_rate2; `comp` 0 = u, 1 = v.  Every reference to the velocity is
// matched through the same index maps and masks as the forward evaluation.
__device__ double strain_sensitivity(const DevGrid<double>& g, const double2* __restrict__ x, double wf, int ci, int cj, int k, int comp) {
    auto uref = [&](int a, int b) { return !g.peripheral_fc(a, b) && g.u_idx(a, b) == k; };
    auto vref = [&](int a, int b) { return !g.peripheral_cf(a, b) && g.v_idx(a, b) == k; };
    // no prescribed faces here: the adjoint is refused for problems that have them
    double exx = (wall_u(g, x, nullptr, ci + 1, cj) - wall_u(g, x, nullptr, ci, cj)) * g.rdxc[ci];
    double eyy = (wall_v(g, x, nullptr, ci, cj + 1) - wall_v(g, x, nullptr, ci, cj)) * g.rdyc[cj];
    double d = 0.0;
    if (comp == 0) d += (2 * exx + eyy) * g.rdxc[ci] * ((double)uref(ci + 1, cj) - (double)uref(ci, cj));
    else d += (2 * eyy + exx) * g.rdyc[cj] * ((double)vref(ci, cj + 1) - (double)vref(ci, cj));
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b) {
            int fi = ci + a, fj = cj + b;
            double e = strain_xy(g, x, nullptr, fi, fj, wf);
            double sf = g.peripheral_ff(fi, fj) ? wf : 1.0;
            double de = comp == 0 ? sf / 2 * g.rdyf[fj] * ((double)uref(fi, fj) - (double)uref(fi, fj - 1))
                                  : sf / 2 * g.rdxf[fi] * ((double)vref(fi, fj) - (double)vref(fi - 1, fj));
            d += e / 2 * de;   // ∂(¼ Σ e²)/∂e = e / 2
        }
    return d;
}

// Σ over the centres whose effective strain rate reads velocity point k (u face (i, j) for comp 0, v face for
// comp 1) of gbar(centre) ∂S/∂x_k: centres ci in i-1..i (u) or i-1..i+1 (v), cj in j-1..j+1 (u) or j-1..j (v).
__device__ double viscosity_gather(const AdjointView& v, int i, int j, int k, int comp) {
    const DevGrid<double>& g = v.o.g;
    double acc = 0.0;
    int seen[6], ns = 0;
    int ilo = i - 1, ihi = comp == 0 ? i : i + 1, jlo = j - 1, jhi = comp == 0 ? j + 1 : j;
    for (int a = ilo; a <= ihi; ++a)
        for (int b2 = jlo; b2 <= jhi; ++b2) {
            int ci, cj;
            if (!map_index(a, g.Nx, g.px, g.Nx, ci) || !map_index(b2, g.Ny, g.py, g.Ny, cj)) continue;
            int c = g.idx(ci, cj);
            if (!first_time(seen, ns, c)) continue;
            double gb = v.gbar[c];
            if (gb != 0.0) acc += gb * strain_sensitivity(g, v.xs, v.ph.wall_factor, ci, cj, k, comp);
        }
    return acc;
}

// r = x̄ + ȳ with ȳ = -(∂[A(c(x)) x*]/∂x)ᵀ λ, gathered per velocity point from the centres whose strain rates
// read it (viscosity) and the faces whose speed reads it (drag).
__global__ void k_adjoint_velocity(AdjointView v) {
    const PhysView& ph = v.ph;
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    bool has_u = j < g.Ny && (i < g.Nx || !g.px), has_v = i < g.Nx && (j < g.Ny || !g.py);
    double ub = 0.0, vb = 0.0;
    double u, vf, U, phi, b, dbdU, dbdC;
    for (int comp = 0; comp < 2; ++comp) {
        if (comp == 0 ? !has_u : !has_v) continue;
        double acc = viscosity_gather(v, i, j, k, comp);
        // drag of the point itself
        if (comp == 0 && u_drag(ph, v.xs, i, j, u, vf, U, phi, b, dbdU, dbdC)) acc += v.bbar[k].x * phi * dbdU * u / U;
        if (comp == 1 && v_drag(ph, v.xs, i, j, u, vf, U, phi, b, dbdU, dbdC)) acc += v.bbar[k].y * phi * dbdU * u / U;
        // drag of the faces of the other component whose ℑxy average reads this point
        int fseen[4], nf = 0;
        for (int a = (comp == 0 ? i - 1 : i); a <= (comp == 0 ? i : i + 1); ++a)
            for (int b2 = (comp == 0 ? j : j - 1); b2 <= (comp == 0 ? j + 1 : j); ++b2) {
                int fi, fj;
                if (comp == 0) {
                    if (!map_index(a, g.Nx, g.px, g.Nx, fi) || !map_index(b2, g.Ny, g.py, g.Ny + 1, fj)) continue;
                } else {
                    if (!map_index(a, g.Nx, g.px, g.Nx + 1, fi) || !map_index(b2, g.Ny, g.py, g.Ny, fj)) continue;
                }
                int kf = g.idx(fi, fj);
                if (!first_time(fseen, nf, kf)) continue;
                double w, avg, Uf, phif, bf, dUf, dCf;
                int m;
                if (comp == 0) {
                    if (!v_drag(ph, v.xs, fi, fj, w, avg, Uf, phif, bf, dUf, dCf)) continue;
                    m = (g.u_idx(fi, fj - 1) == k) + (g.u_idx(fi + 1, fj - 1) == k) + (g.u_idx(fi, fj) == k) + (g.u_idx(fi + 1, fj) == k);
                    acc += v.bbar[kf].y * phif * dUf * avg / Uf * (m / 4.0);
                } else {
                    if (!u_drag(ph, v.xs, fi, fj, w, avg, Uf, phif, bf, dUf, dCf)) continue;
                    m = (g.v_idx(fi - 1, fj) == k) + (g.v_idx(fi, fj) == k) + (g.v_idx(fi - 1, fj + 1) == k) + (g.v_idx(fi, fj + 1) == k);
                    acc += v.bbar[kf].x * phif * dUf * avg / Uf * (m / 4.0);
                }
            }
        if (comp == 0) ub = acc; else vb = acc;
    }
    double2 xb = v.xbar[k];
    v.r[k] = make_double2(xb.x - ub, xb.y - vb);
}
void launch_adjoint_velocity(const AdjointView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx + 1, v.o.g.Ny + 1);
    k_adjoint_velocity<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// ∂J/∂log C = -C λ̃ᵀ ∂[A(c) x*]/∂C: each face coefficient is the mean of the two cells beside it (frictions.jl:142-160).
__global__ void k_adjoint_gradient(AdjointView v) {
    const PhysView& ph = v.ph;
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    double acc = 0.0, w, avg, U, phi, b, dbdU, dbdC;
    int seen[2], n = 0;
    for (int a = i; a <= i + 1; ++a) {
        int fi;
        if (!map_index(a, g.Nx, g.px, g.Nx + 1, fi)) continue;
        int kf = g.idx(fi, j);
        if (!first_time(seen, n, kf) || !u_drag(ph, v.xs, fi, j, w, avg, U, phi, b, dbdU, dbdC)) continue;
        int m = (g.c_idx(fi - 1, j) == k) + (g.c_idx(fi, j) == k);
        acc += v.bbar[kf].x * phi * dbdC * (m / 2.0);
    }
    n = 0;
    for (int b2 = j; b2 <= j + 1; ++b2) {
        int fj;
        if (!map_index(b2, g.Ny, g.py, g.Ny + 1, fj)) continue;
        int kf = g.idx(i, fj);
        if (!first_time(seen, n, kf) || !v_drag(ph, v.xs, i, fj, w, avg, U, phi, b, dbdU, dbdC)) continue;
        int m = (g.c_idx(i, fj - 1) == k) + (g.c_idx(i, fj) == k);
        acc += v.bbar[kf].y * phi * dbdC * (m / 2.0);
    }
    v.grad_log_C[k] = -ph.C[k] * acc;
}
void launch_adjoint_gradient(const AdjointView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx, v.o.g.Ny);
    k_adjoint_gradient<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// ---- ∂J/∂H of the SSA fixed point with the geometry and the driving stress recomputed from H ----------------
// J(x*(H)) where update_geometry! (ice_sheet_model_methods.jl:103-111: s, φᵘ, φᵛ, N, μ) and compute_driving_stress!
// (driving_stress.jl:43-125) take H before the Picard solve, and update_stress_balance_coefficients! reads H in
// η̄H = μ H Σ ησ Δζ (column_integrals.jl:61-71) and φᵘ, φᵛ, N in the drag (frictions.jl:142-160).  With the adjoint
// state of the fixed point (λ = ∂J/∂τ, and the λ-signed sensitivities eb of η̄H and bb of β whose true adjoints are
// -eb and -bb) each cell gathers, from its centre and its four faces:
//   ∂J/∂H = -eb η̄ μ + Σ_faces λ ∂τ/∂H + (∂J/∂s) ds/dH + (∂J/∂μ) dμ/dH + Σ_faces (-bb) β̂ ∂φ/∂f + (∂J/∂N) dN/dH
// with β = φ β̂, f = H + ρw b / ρᵢ.  The discrete switches (walls, fronts and ice-free faces from μ > 0, the branch of
// s, the clamp of D) are held where they are.

// ∂ front_force / ∂H and ∂s of the front cell c (driving_stress.jl:56-60)
__device__ __forceinline__ void front_force_partials(const GeometryView& v, int c, double& dH, double& ds) {
    double Hi = v.H[c], y = Hi - v.s[c];
    double D, dDdH, dDds;
    if (y <= 0.0) { D = 0.0; dDdH = 0.0; dDds = 0.0; }
    else if (y >= Hi) { D = Hi; dDdH = 1.0; dDds = 0.0; }
    else { D = y; dDdH = 1.0; dDds = -1.0; }
    dH = v.gacc * (v.rho_i * Hi - v.rho_w * D * dDdH);
    ds = -v.gacc * v.rho_w * D * dDds;
}

// Partials of one face's driving stress (u face: c1 west, c2 east, `w` = Δy at the face, `a` = Az ρᵢ g rdxf; v face
// likewise in y) with respect to H and s of its two centres; false when the face carries no dependence on them.
__device__ __forceinline__ bool tau_partials(const GeometryView& v, bool wall, int c1, int c2, double w, double a, double* dH, double* ds) {
    dH[0] = dH[1] = ds[0] = ds[1] = 0.0;
    if (wall) return false;
    if (v.use_mask) {
        bool m1 = v.mu[c1] > 0, m2 = v.mu[c2] > 0;
        bool ice1 = m1 && !m2, ice2 = !m1 && m2;
        if (ice1 || ice2) {   // the front: τ = Δ (ff(c1) if ice1) - Δ (ff(c2) if ice2)
            double fh, fs;
            if (ice1) { front_force_partials(v, c1, fh, fs); dH[0] = w * fh; ds[0] = w * fs; }
            else { front_force_partials(v, c2, fh, fs); dH[1] = -w * fh; ds[1] = -w * fs; }
            return true;
        }
    }
    double H1 = v.H[c1], H2 = v.H[c2], s1 = v.s[c1], s2 = v.s[c2];
    if (v.gl_stress) {   // grounding_line_stress, driving_stress.jl:84-92
        double ri = v.rho_i, rw = v.rho_w;
        double f1 = H1 + rw / ri * v.bed[c1], f2 = H2 + rw / ri * v.bed[c2];
        bool straddles = ((f1 > 0) != (f2 > 0)) && (H1 > 0) && (H2 > 0);
        if (straddles) {
            double df = f1 - f2;
            double theta = f1 / df;
            double Hg = H1 + theta * (H2 - H1);
            double cg = 1 - ri / rw;
            double sg = cg * Hg;
            double K = -ri * v.gacc / 2 * w;
            double dHg = K * ((s2 - s1) + cg * (H1 - H2));   // ∂τ/∂Hg
            double dth1 = -f2 / (df * df), dth2 = f1 / (df * df);
            double dHg1 = 1 - theta + (H2 - H1) * dth1, dHg2 = theta + (H2 - H1) * dth2;
            dH[0] = K * (sg - s1) + dHg * dHg1;
            dH[1] = K * (s2 - sg) + dHg * dHg2;
            ds[0] = -K * (H1 + Hg);
            ds[1] = K * (Hg + H2);
            return true;
        }
    }
    // τ = -Az ρᵢ g ½ (H1 + H2) (s2 - s1) / Δ
    dH[0] = dH[1] = -a * 0.5 * (s2 - s1);
    ds[1] = -a * 0.5 * (H1 + H2);
    ds[0] = -ds[1];
    return true;
}

// ∂φ/∂f₁, ∂φ/∂f₂ of segment_fraction (subgrid_grounded_fraction.jl:34-38)
__device__ __forceinline__ void segment_fraction_partials(double f1, double f2, double& d1, double& d2) {
    double S = fabs(f1) + fabs(f2);
    d1 = d2 = 0.0;
    if (S == 0.0) return;
    double fp = fmax(f1, 0.0) + fmax(f2, 0.0);
    auto sg = [](double f) { return f > 0 ? 1.0 : (f < 0 ? -1.0 : 0.0); };
    d1 = ((f1 > 0 ? 1.0 : 0.0) * S - fp * sg(f1)) / (S * S);
    d2 = ((f2 > 0 ? 1.0 : 0.0) * S - fp * sg(f2)) / (S * S);
}

// β̂ = basal_drag(U, C, N) and ∂β̂/∂N (regularised Coulomb; zero for Weertman)
__device__ __forceinline__ double basal_drag_dN(const PhysView& ph, double U, double C, double N, double& dN) {
    double w = C * pow(U, ph.m - 1);
    dN = 0.0;
    if (ph.friction == NK_WEERTMAN) return w;
    double tc = ph.alpha2 * N;
    double Q = pow(C, 1 / ph.m) * U + pow(tc, 1 / ph.m);
    double Qm = pow(Q, ph.m);
    if (tc > 0) dN = ph.alpha2 * (w / Qm) * (1 - pow(tc, 1 / ph.m) / Q);
    return w * tc / Qm;
}

// One face's drag partials for its two centres: tb β̂ ∂φ/∂f into gf, tb φ ∂β̂/∂N ½ into gN, with tb the true adjoint of
// the face's drag (β = φ β̂; the DIVA's βᵇ).
__device__ __forceinline__ void drag_partials(const AdjointView& v, const GeometryView& gv, bool has, bool wall, int k, double U,
                                              int c1, int c2, double phi, double tb, double* gf, double* gN) {
    gf[0] = gf[1] = gN[0] = gN[1] = 0.0;
    if (!has || wall || v.ph.friction == NK_FRICTION_NONE) return;
    const PhysView& ph = v.ph;
    double Cf = (ph.C[c1] + ph.C[c2]) / 2;
    double Nf = ph.use_N ? (ph.N[c1] + ph.N[c2]) / 2 : 0.0;
    double dbN;
    double bh = basal_drag_dN(ph, U, Cf, Nf, dbN);
    if (gv.grounding) {
        double rw_ri = gv.rho_w / gv.rho_i;
        double d1, d2;
        segment_fraction_partials(gv.H[c1] + rw_ri * gv.bed[c1], gv.H[c2] + rw_ri * gv.bed[c2], d1, d2);
        gf[0] = tb * bh * d1;
        gf[1] = tb * bh * d2;
    }
    if (ph.use_N) gN[0] = gN[1] = tb * phi * dbN * 0.5;
}

__global__ void k_adjoint_thickness(AdjointView v, GeometryView gv, int diva, double* grad_H) {
    const DevGrid<double>& g = v.o.g;
    const PhysView& ph = v.ph;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int c = g.idx(i, j);
    double H = gv.H[c];
    double gH, gmu, gs = 0.0, gf = 0.0, gN = 0.0;
    if (diva) {   // the centre pass of the DIVA sweep left (∂J/∂H through η̄H and F₂, ∂J/∂μ)
        gH = v.hmu[c].x;
        gmu = v.hmu[c].y;
    } else {      // η̄H = μ H η̄ with eb gathered as in k_adjoint_viscosity
        int fx[2], wx[2], fy[2], wy[2];
        int nx = corners_of_centre(i, g.Nx, g.px, fx, wx), ny = corners_of_centre(j, g.Ny, g.py, fy, wy);
        double eb = v.cbar[c].x;
        for (int a = 0; a < nx; ++a)
            for (int b = 0; b < ny; ++b) eb += (wx[a] * wy[b]) * v.cbar[g.idx(fx[a], fy[b])].y / 4;
        if (v.eta_bar_in) eb -= v.eta_bar_in[c];
        double etab = 0.0;
        for (int l = 0; l < ph.sig.N; ++l) etab += v.eta_sigma[(long long)l * ph.plane + c] * ph.sig.dz[l];
        double mu = ph.use_mask ? ph.mu[c] : 1.0;
        gH = -eb * etab * mu;
        gmu = ph.use_mask ? -eb * etab * H : 0.0;
    }
    double u02 = ph.u0 * ph.u0;
    // the four faces; `side` is this centre's place in the face's pair
    for (int f = 0; f < 4; ++f) {
        bool xf = f < 2;
        int fi = xf ? i + (f == 1) : i, fj = xf ? j : j + (f == 3);
        int side = (f == 1 || f == 3) ? 0 : 1;
        // every centre has its four faces: on a Periodic axis the east (north) face of the last column (row) is the
        // first face, reached through the wrapped index; on a Bounded one the outer faces are walls
        int k = xf ? g.u_idx(fi, fj) : g.v_idx(fi, fj);
        int c1 = xf ? g.c_idx(fi - 1, fj) : g.c_idx(fi, fj - 1), c2 = g.c_idx(fi, fj);
        bool peri = xf ? g.peripheral_fc(fi, fj) : g.peripheral_cf(fi, fj);
        // driving stress
        bool wall = peri || (gv.use_mask && (gv.mu[c1] + gv.mu[c2]) == 0.0);
        double w = xf ? g.dyc[fj] : g.dxc[fi];
        double a = xf ? g.Az_fc(fi, fj) * gv.rho_i * gv.gacc * g.rdxf[fi] : g.Az_cf(fi, fj) * gv.rho_i * gv.gacc * g.rdyf[fj];
        double dH[2], ds[2];
        if (tau_partials(gv, wall, c1, c2, w, a, dH, ds)) {
            double lam = xf ? v.lam[k].x : v.lam[k].y;
            gH += lam * dH[side];
            gs += lam * ds[side];
        }
        // drag: β = φ β̂(|x|) for the SSA, βᵇ = φ β̂(|uᵇ|) for the DIVA
        double U;
        const double2* x = diva ? v.ubs : v.xs;
        if (xf) {
            double vf = ((x[g.v_idx(fi - 1, fj)].y + x[g.v_idx(fi, fj)].y) / 2 + (x[g.v_idx(fi - 1, fj + 1)].y + x[g.v_idx(fi, fj + 1)].y) / 2) / 2;
            double u = x[k].x;
            U = sqrt(u * u + vf * vf + u02);
        } else {
            double uf = ((x[g.u_idx(fi, fj - 1)].x + x[g.u_idx(fi + 1, fj - 1)].x) / 2 + (x[g.u_idx(fi, fj)].x + x[g.u_idx(fi + 1, fj)].x) / 2) / 2;
            double vv = x[k].y;
            U = sqrt(vv * vv + uf * uf + u02);
        }
        double gfp[2], gNp[2];
        double phi = xf ? ph.phi[k].x : ph.phi[k].y;
        double tb = diva ? (xf ? v.bbt[k].x : v.bbt[k].y) : -(xf ? v.bbar[k].x : v.bbar[k].y);   // true adjoints
        drag_partials(v, gv, true, peri, k, U, c1, c2, phi, tb, gfp, gNp);
        gf += gfp[side];
        gN += gNp[side];
    }
    // chain through s, μ, f and N of this centre (update_geometry!)
    double b = gv.bed[c];
    double dsdH = gv.grounding ? ((b + H >= (1 - gv.rho_i / gv.rho_w) * H) ? 1.0 : 1 - gv.rho_i / gv.rho_w) : 1.0;
    double t = (H - gv.mask_min) / gv.mask_trans;
    double dmudH = (!gv.front && t > 0 && t < 1) ? 6 * t * (1 - t) / gv.mask_trans : 0.0;
    double rig = gv.rho_i * gv.gacc;
    double dNdH = (rig * H + gv.rho_w * gv.gacc * fmin(b, 0.0) > 0) ? rig : 0.0;
    if (gv.Hw) {   // the till's N = N0 (δ P0 / N0)^s 10^(...) where it is below the ocean-connected cap: ∂N/∂H = N s / H
        double sat, No = fmax(rig * H + gv.rho_w * gv.gacc * fmin(b, 0.0), 0.0);
        double Nt = till_pressure(gv, rig * H, gv.Hw[c], sat);
        if (Nt < No) dNdH = H > 0 ? Nt * sat / H : 0.0;
    }
    grad_H[c] = gH + gs * dsdH + gmu * dmudH + gf + gN * dNdH;
}
void launch_adjoint_thickness(const AdjointView& v, const GeometryView& gv, int diva, double* grad_H, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx, v.o.g.Ny);
    k_adjoint_thickness<<<d.grid, d.block, 0, s>>>(v, gv, diva, grad_H); count_launch();
}

// ---- DIVA: the reverse of one update_diva_coefficients! step at the fixed point ---------------------------------
// The forward step (diva.jl:61-75) reads x, the lagged βᵇ⁻, F₂⁻ and ησ⁻ and writes:
//   uᵇ = x / (1 + βᵇ⁻ ℑF₂⁻)                               (compute_basal_velocities!)
//   βᵇ = φ drag(|uᵇ|, C, N)                                (compute_basal_drag! on uᵇ)
//   ησₖ = glen(Aₖ, ε̇ₑ²(x) + (τxᵇ² + τyᵇ²) aₖ² + ε̇₀²),      τxᵇ = ℑxᶜ(βᵇᵘ uᵇ), aₖ = (1 - ζₖ) / 2ησ⁻ₖ
//   η̄H = μ H Σ ησₖ Δζₖ,  F₂ = H Σ w₂ₖ / ησₖ,  β = βᵇ / (1 + βᵇ ℑF₂)
// At the fixed point the lagged state equals the new one, so one set of arrays serves both.  True adjoints
// throughout: the operator's coefficient adjoints are minus the λ-signed cbar / bbar.

// u-face mean of F₂ (x_shear_factor) and v-face mean (y_shear_factor)
__device__ __forceinline__ double u_face_F2(const DevGrid<double>& g, const double* F2, int i, int j) {
    return (F2[g.c_idx(i - 1, j)] + F2[g.c_idx(i, j)]) / 2;
}
__device__ __forceinline__ double v_face_F2(const DevGrid<double>& g, const double* F2, int i, int j) {
    return (F2[g.c_idx(i, j - 1)] + F2[g.c_idx(i, j)]) / 2;
}

// Σ over the faces whose ℑF₂ reads centre (i, j) = k of val(face index, component) × (times read) / 2
template <typename F>
__device__ __forceinline__ double face_mean_gather(const DevGrid<double>& g, int i, int j, int k, F&& val) {
    double acc = 0.0;
    int seen[2], n = 0;
    for (int a = i; a <= i + 1; ++a) {
        int fi;
        if (!map_index(a, g.Nx, g.px, g.Nx + 1, fi)) continue;
        int kf = g.idx(fi, j);
        if (!first_time(seen, n, kf)) continue;
        int m = (g.c_idx(fi - 1, j) == k) + (g.c_idx(fi, j) == k);
        if (m) acc += val(fi, j, kf, 0) * (m / 2.0);
    }
    n = 0;
    for (int b = j; b <= j + 1; ++b) {
        int fj;
        if (!map_index(b, g.Ny, g.py, g.Ny + 1, fj)) continue;
        int kf = g.idx(i, fj);
        if (!first_time(seen, n, kf)) continue;
        int m = (g.c_idx(i, fj - 1) == k) + (g.c_idx(i, fj) == k);
        if (m) acc += val(i, fj, kf, 1) * (m / 2.0);
    }
    return acc;
}

// Centre pass: F̄₂ = σ(F₂) + the effective drags' ℑF₂; ησ̄ₖ = σ(ησₖ) + η̄̄ Δζₖ - F̄ w₂ₖ / ησₖ², through glen to
// ε̇̄ₑₖ; writes gbar = Σₖ ε̇̄ₑₖ (the membrane strain rate), txbar (the basal shear stresses), σ(ησ⁻) in place and,
// when set, ∂J/∂log A.
__global__ void k_adjoint_diva_centre(AdjointView v) {
    const PhysView& ph = v.ph;
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    int fx[2], wx[2], fy[2], wy[2];
    int nx = corners_of_centre(i, g.Nx, g.px, fx, wx), ny = corners_of_centre(j, g.Ny, g.py, fy, wy);
    double eb = v.cbar[k].x;
    for (int a = 0; a < nx; ++a)
        for (int b = 0; b < ny; ++b) eb += (wx[a] * wy[b]) * v.cbar[g.idx(fx[a], fy[b])].y / 4;
    if (v.eta_bar_in) eb -= v.eta_bar_in[k];   // λ-signed like cbar
    double H = ph.H[k];
    double etabar_b = -eb * (ph.use_mask ? ph.mu[k] : 1.0) * H;     // ∂J/∂η̄
    double F2b = v.sig_F2[k] + face_mean_gather(g, i, j, k, [&](int fi, int fj, int kf, int comp) {
        double b = comp == 0 ? v.bbs[kf].x : v.bbs[kf].y;
        double mf = comp == 0 ? u_face_F2(g, v.F2s, fi, fj) : v_face_F2(g, v.F2s, fi, fj);
        double den = 1 + b * mf;
        return (comp == 0 ? v.bbar[kf].x : v.bbar[kf].y) * b * b / (den * den);   // -β̄ ∂β/∂ℑF₂ with β̄ = -bbar
    });
    double Fb = F2b * H;
    int u0 = g.u_idx(i, j), u1 = g.u_idx(i + 1, j), v0 = g.v_idx(i, j), v1 = g.v_idx(i, j + 1);
    double tx = (v.bbs[u0].x * v.ubs[u0].x + v.bbs[u1].x * v.ubs[u1].x) / 2;
    double ty = (v.bbs[v0].y * v.ubs[v0].y + v.bbs[v1].y * v.ubs[v1].y) / 2;
    double t2 = tx * tx + ty * ty;
    double e2 = effective_strain_rate2(g, v.xs, nullptr, i, j, ph.wall_factor);
    double e2b = 0.0, txb = 0.0, tyb = 0.0, gA = 0.0, etab_sum = 0.0, F_sum = 0.0;
    for (int l = 0; l < ph.sig.N; ++l) {
        long long o = (long long)l * ph.plane + k;
        double eta = v.eta_sigma[o];
        etab_sum += eta * ph.sig.dz[l];
        F_sum += (1 / eta) * ph.sig.w2[l];
        double em = eta == 0.0 ? INFINITY : eta;
        double a = (1 - ph.sig.zc[l]) / (2 * em), a2 = a * a;
        double ee = e2 + t2 * a2 + ph.eps0 * ph.eps0;
        double etab = v.sig_eta[o] + etabar_b * ph.sig.dz[l] - Fb * ph.sig.w2[l] / (eta * eta);
        double eeb = etab * eta * ((1 - ph.n) / (2 * ph.n)) / ee;
        e2b += eeb;
        txb += eeb * 2 * tx * a2;
        tyb += eeb * 2 * ty * a2;
        v.sig_eta[o] = eta == 0.0 ? 0.0 : eeb * (-2 * t2 * a2 / em);
        if (v.grad_log_A) {
            double d = etab * (-eta / ph.n);
            if (ph.rate_sigma) v.grad_log_A[o] = d; else gA += d;
        }
    }
    if (v.grad_log_A && !ph.rate_sigma) v.grad_log_A[k] = gA;
    if (v.hmu) {   // η̄H = μ H η̄ and F₂ = H F
        double mu = ph.use_mask ? ph.mu[k] : 1.0;
        v.hmu[k] = make_double2(-eb * mu * etab_sum + F2b * F_sum, ph.use_mask ? -eb * H * etab_sum : 0.0);
    }
    v.gbar[k] = e2b;
    v.txbar[k] = make_double2(txb, tyb);
}

// Face pass: β̄ᵇ = σ(βᵇ) + β̄ / (1 + βᵇ ℑF₂)² + the basal shear stresses that read βᵇ uᵇ here; Ū = β̄ᵇ φ ∂drag/∂U.
__global__ void k_adjoint_diva_face(AdjointView v) {
    const PhysView& ph = v.ph;
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    bool has_u = j < g.Ny && (i < g.Nx || !g.px), has_v = i < g.Nx && (j < g.Ny || !g.py);
    double2 Ub = make_double2(0.0, 0.0), up = make_double2(0.0, 0.0), bt = make_double2(0.0, 0.0);
    double w, avg, U, phi, bd, dbdU, dbdC;
    if (has_u) {
        double b = v.bbs[k].x, den = 1 + b * u_face_F2(g, v.F2s, i, j);
        double bbar = v.sig_bb[k].x - v.bbar[k].x / (den * den), upf = 0.0;
        int seen[2], n = 0;
        for (int a = i - 1; a <= i; ++a) {   // τxᵇ of centre (ci, j) reads u_idx(ci, j) and u_idx(ci + 1, j)
            int ci;
            if (!map_index(a, g.Nx, g.px, g.Nx, ci)) continue;
            int kc = g.idx(ci, j);
            if (!first_time(seen, n, kc)) continue;
            int m = (g.u_idx(ci, j) == k) + (g.u_idx(ci + 1, j) == k);
            double tb = v.txbar[kc].x * (m / 2.0);
            bbar += tb * v.ubs[k].x;
            upf += tb * b;
        }
        bt.x = bbar;
        up.x = upf;
        if (u_drag(ph, v.ubs, i, j, w, avg, U, phi, bd, dbdU, dbdC)) Ub.x = bbar * phi * dbdU;
    }
    if (has_v) {
        double b = v.bbs[k].y, den = 1 + b * v_face_F2(g, v.F2s, i, j);
        double bbar = v.sig_bb[k].y - v.bbar[k].y / (den * den), upf = 0.0;
        int seen[2], n = 0;
        for (int c = j - 1; c <= j; ++c) {   // τyᵇ of centre (i, cj) reads v_idx(i, cj) and v_idx(i, cj + 1)
            int cj;
            if (!map_index(c, g.Ny, g.py, g.Ny, cj)) continue;
            int kc = g.idx(i, cj);
            if (!first_time(seen, n, kc)) continue;
            int m = (g.v_idx(i, cj) == k) + (g.v_idx(i, cj + 1) == k);
            double tb = v.txbar[kc].y * (m / 2.0);
            bbar += tb * v.ubs[k].y;
            upf += tb * b;
        }
        bt.y = bbar;
        up.y = upf;
        if (v_drag(ph, v.ubs, i, j, w, avg, U, phi, bd, dbdU, dbdC)) Ub.y = bbar * phi * dbdU;
    }
    v.Ubar[k] = Ub;
    v.ubp[k] = up;
    v.bbt[k] = bt;
}

// Velocity pass: ūᵇ = ubp + the drag speeds that read uᵇ here; then uᵇ = x / S⁻ with S⁻ = 1 + βᵇ⁻ ℑF₂⁻ gives
// x̄ += ūᵇ / S⁻, σ(βᵇ⁻) = S̄⁻ ℑF₂⁻ and the ℑF₂⁻ adjoint S̄⁻ βᵇ⁻ (mbar); r = x̄ + the membrane strain rates + ūᵇ / S⁻.
__global__ void k_adjoint_diva_velocity(AdjointView v) {
    const PhysView& ph = v.ph;
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i > g.Nx || j > g.Ny) return;
    int k = g.idx(i, j);
    bool has_u = j < g.Ny && (i < g.Nx || !g.px), has_v = i < g.Nx && (j < g.Ny || !g.py);
    double2 xb = v.xbar[k], r = xb, sb = make_double2(0.0, 0.0), mb = make_double2(0.0, 0.0);
    double u, vf, U, phi, b, dbdU, dbdC;
    for (int comp = 0; comp < 2; ++comp) {
        if (comp == 0 ? !has_u : !has_v) continue;
        double ubb = comp == 0 ? v.ubp[k].x : v.ubp[k].y;
        if (comp == 0 && u_drag(ph, v.ubs, i, j, u, vf, U, phi, b, dbdU, dbdC)) ubb += v.Ubar[k].x * u / U;
        if (comp == 1 && v_drag(ph, v.ubs, i, j, u, vf, U, phi, b, dbdU, dbdC)) ubb += v.Ubar[k].y * u / U;
        int fseen[4], nf = 0;   // the other component's drag speeds whose ℑxy average reads uᵇ here
        for (int a = (comp == 0 ? i - 1 : i); a <= (comp == 0 ? i : i + 1); ++a)
            for (int b2 = (comp == 0 ? j : j - 1); b2 <= (comp == 0 ? j + 1 : j); ++b2) {
                int fi, fj;
                if (comp == 0) {
                    if (!map_index(a, g.Nx, g.px, g.Nx, fi) || !map_index(b2, g.Ny, g.py, g.Ny + 1, fj)) continue;
                } else {
                    if (!map_index(a, g.Nx, g.px, g.Nx + 1, fi) || !map_index(b2, g.Ny, g.py, g.Ny, fj)) continue;
                }
                int kf = g.idx(fi, fj);
                if (!first_time(fseen, nf, kf)) continue;
                double w, avg, Uf, phif, bf, dUf, dCf;
                int m;
                if (comp == 0) {
                    if (!v_drag(ph, v.ubs, fi, fj, w, avg, Uf, phif, bf, dUf, dCf)) continue;
                    m = (g.u_idx(fi, fj - 1) == k) + (g.u_idx(fi + 1, fj - 1) == k) + (g.u_idx(fi, fj) == k) + (g.u_idx(fi + 1, fj) == k);
                    ubb += v.Ubar[kf].y * avg / Uf * (m / 4.0);
                } else {
                    if (!u_drag(ph, v.ubs, fi, fj, w, avg, Uf, phif, bf, dUf, dCf)) continue;
                    m = (g.v_idx(fi - 1, fj) == k) + (g.v_idx(fi, fj) == k) + (g.v_idx(fi - 1, fj + 1) == k) + (g.v_idx(fi, fj + 1) == k);
                    ubb += v.Ubar[kf].x * avg / Uf * (m / 4.0);
                }
            }
        double bl = comp == 0 ? v.bbs[k].x : v.bbs[k].y;
        double mf = comp == 0 ? u_face_F2(g, v.F2s, i, j) : v_face_F2(g, v.F2s, i, j);
        double S = 1 + bl * mf;
        double xv = comp == 0 ? v.xs[k].x : v.xs[k].y;
        double Sb = -ubb * xv / (S * S);
        double acc = (comp == 0 ? xb.x : xb.y) + viscosity_gather(v, i, j, k, comp) + ubb / S;
        if (comp == 0) { r.x = acc; sb.x = Sb * mf; mb.x = Sb * bl; }
        else { r.y = acc; sb.y = Sb * mf; mb.y = Sb * bl; }
    }
    v.r[k] = r;
    v.sig_bb[k] = sb;
    v.mbar[k] = mb;
}

// F₂⁻ pass: σ(F₂⁻) at each centre from the lagged shear factors of the faces beside it.
__global__ void k_adjoint_diva_F2(AdjointView v) {
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    v.sig_F2[k] = face_mean_gather(g, i, j, k, [&](int, int, int kf, int comp) { return comp == 0 ? v.mbar[kf].x : v.mbar[kf].y; });
}

void launch_adjoint_diva(const AdjointView& v, cudaStream_t s) {
    LaunchDims c = dims2d(v.o.g.Nx, v.o.g.Ny), f = dims2d(v.o.g.Nx + 1, v.o.g.Ny + 1);
    k_adjoint_diva_centre<<<c.grid, c.block, 0, s>>>(v); count_launch();
    k_adjoint_diva_face<<<f.grid, f.block, 0, s>>>(v); count_launch();
    k_adjoint_diva_velocity<<<f.grid, f.block, 0, s>>>(v); count_launch();
    k_adjoint_diva_F2<<<c.grid, c.block, 0, s>>>(v); count_launch();
}

// ∂J/∂log C = C Σ β̄ᵇ φ ∂drag/∂C̄ / 2 over the faces whose C̄ averages this cell (true adjoints).
__global__ void k_adjoint_diva_gradient(AdjointView v) {
    const PhysView& ph = v.ph;
    const DevGrid<double>& g = v.o.g;
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    if (i >= g.Nx || j >= g.Ny) return;
    int k = g.idx(i, j);
    double acc = face_mean_gather(g, i, j, k, [&](int fi, int fj, int kf, int comp) {
        double w, avg, U, phi, b, dbdU, dbdC;
        bool on = comp == 0 ? u_drag(ph, v.ubs, fi, fj, w, avg, U, phi, b, dbdU, dbdC) : v_drag(ph, v.ubs, fi, fj, w, avg, U, phi, b, dbdU, dbdC);
        return on ? (comp == 0 ? v.bbt[kf].x : v.bbt[kf].y) * phi * dbdC : 0.0;
    });
    v.grad_log_C[k] = ph.C[k] * acc;
}
void launch_adjoint_diva_gradient(const AdjointView& v, cudaStream_t s) {
    LaunchDims d = dims2d(v.o.g.Nx, v.o.g.Ny);
    k_adjoint_diva_gradient<<<d.grid, d.block, 0, s>>>(v); count_launch();
}

// Picard-adjoint progress (ext/NunatakEnzymeExt.jl:216-220): Δ = ‖λ⁺ - λ‖, M = ‖λ⁺‖ over the solved cells, then
// λ = λ⁺ over every stored point.
__global__ void k_adjoint_change(DevGrid<double> g, const double2* __restrict__ lam_new, double2* lam, SolverScalars* sc,
                                 double2* partials) {
    int i = blockIdx.x * BX + threadIdx.x, j = blockIdx.y * BY + threadIdx.y;
    double dd = 0.0, ll = 0.0;
    if (i <= g.Nx && j <= g.Ny) {
        int k = g.idx(i, j);
        double2 a = lam_new[k], b = lam[k];
        if (i < g.Nx && j < g.Ny) {
            double dx = a.x - b.x, dy = a.y - b.y;
            dd = dx * dx + dy * dy;
            ll = a.x * a.x + a.y * a.y;
        }
        lam[k] = a;
    }
    double tdd, tll;
    if (grid_sum2(dd, ll, partials, &sc->ticket, tdd, tll) && threadIdx.x == 0 && threadIdx.y == 0) {
        sc->p_D = sqrt(tdd);
        sc->p_X = sqrt(tll);
    }
}
void launch_adjoint_change(const DevGrid<double>& g, const double2* lam_new, double2* lam, SolverScalars* sc, double2* partials,
                           cudaStream_t s) {
    LaunchDims d = dims2d(g.Nx + 1, g.Ny + 1);
    k_adjoint_change<<<d.grid, d.block, 0, s>>>(g, lam_new, lam, sc, partials); count_launch();
}

}  // namespace nk
