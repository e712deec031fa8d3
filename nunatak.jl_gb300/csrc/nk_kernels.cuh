// nk_kernels.cuh — host-callable launchers of the kernels, shared between the translation units.
#pragma once

#include "nk_strip.cuh"

namespace nk {

// Sigma column constants (src/StressBalances/column_integrals.jl:1-45, src/Grids/sigma_grid.jl:20-22).
constexpr int MAX_SIGMA = 64;
struct SigmaTable {
    int N;
    const double* dz;     // layer_thickness(k)
    const double* w2;     // layer_weight(k, 2)
    const double* zc;     // znode(k, Center)
    const double* w1;     // profile_weight(k', k, 1) at [k * N + k'] for k' <= k
    const double* zf;     // znode(k, Face), the N + 1 faces
};
__device__ __forceinline__ void rebase(SigmaTable& t, long long d) {
    shift_ptr(t.dz, d); shift_ptr(t.w2, d); shift_ptr(t.zc, d); shift_ptr(t.w1, d); shift_ptr(t.zf, d);
}

// Fine-grid inputs of the coefficient update (all FP64, pitched; pairs interleave the u and v faces).
struct PhysView {
    DevGrid<double> g;
    SigmaTable sig;
    double n, eps0, wall_factor;
    int friction;                 // NK_FRICTION_*
    double m, alpha2, u0;
    int rate_sigma;               // A on the sigma grid
    int plane;                    // elements of one pitched plane: (Ny + 1) * pitch
    const double* A;
    const double* H;
    const double* C;
    const double* N;
    const double* mu;
    const double2* phi;           // (phi_u, phi_v)
    int use_mask, use_N;
    const double2* ud = nullptr;      // prescribed (u, v) per face, NaN where free
};
__device__ __forceinline__ void rebase(PhysView& v, long long d) {
    rebase(v.g, d);
    rebase(v.sig, d);
    shift_ptr(v.A, d); shift_ptr(v.H, d); shift_ptr(v.C, d); shift_ptr(v.N, d); shift_ptr(v.mu, d); shift_ptr(v.phi, d);
    shift_ptr(v.ud, d);
}

// ---- layout conversion ---------------------------------------------------------------------------------
// dst[(j * pitch + i) * stride + offset] = src[j * nx + i] for i < nx, j < ny, `planes` planes.
void launch_pack(double* dst, int pitch, int plane, int stride, int offset, const double* src, int nx, int ny, int planes,
                 cudaStream_t s);
void launch_unpack(double* dst, const double* src, int pitch, int plane, int stride, int offset, int nx, int ny, int planes,
                   cudaStream_t s);
void launch_fill(double* dst, int count, double value, cudaStream_t s);

// ---- operator and conjugate gradients (FP64 fine grid) --------------------------------------------------
void launch_apply(const OpView<double>& o, const double2* p, double2* q, cudaStream_t s);
// mask bits from eta_H and the topology, over 0..Nx x 0..Ny
template <typename T>
void launch_mask(const OpView<T>& o, uint8_t* mask, cudaStream_t s, const double2* ud = nullptr);
// x = val on the prescribed faces (ud finite)
void launch_impose_prescribed(const DevGrid<double>& g, double2* x, const double2* ud, const double2* val, cudaStream_t s);
// inverse diagonal (Jacobi) of the fine grid
void launch_inverse_diagonal(const OpView<double>& o, double2* invd, cudaStream_t s);
template <typename T>
void launch_inverse_row_sum(const OpView<T>& o, typename Vec2<T>::type* irs, cudaStream_t s);

struct CGView {
    OpView<double> o;
    double2* x; const double2* b; double2* r; double2* z; double2* p; double2* q; double2* zold;
    const double2* invd;          // Jacobi inverse diagonal or nullptr
    int precond;                  // NK_PRECONDITIONER_*
    SolverScalars* sc;
    double2* partials;
    unsigned long long cond;      // conditional-node handle of the conjugate-gradient while loop (0: none)
    float2* r32;                  // mixed precision: FP32 copy of r written for the V-cycle (or nullptr)
    const float2* z32;            // mixed precision: FP32 V-cycle result read back as z (or nullptr)
    float2* zold32;               // mixed precision: z_old kept as the FP32 z32 it equals exactly (or nullptr);
                                  // z itself is then never stored: each kernel that needs it rescales z32
};
__device__ __forceinline__ void rebase(CGView& v, long long d) {
    rebase(v.o, d);
    shift_ptr(v.x, d); shift_ptr(v.b, d); shift_ptr(v.r, d); shift_ptr(v.z, d); shift_ptr(v.p, d); shift_ptr(v.q, d);
    shift_ptr(v.zold, d); shift_ptr(v.invd, d); shift_ptr(v.sc, d); shift_ptr(v.partials, d);
    shift_ptr(v.r32, d); shift_ptr(v.z32, d); shift_ptr(v.zold32, d);
}
// r = b - A x; if the preconditioner is not multigrid also z = M r, p = z, rho = r.z; r0, tol, done
void launch_cg_init(const CGView& v, cudaStream_t s);
// multigrid: after z = V(r): p = z, rho = r.z, done
void launch_cg_init_finish(const CGView& v, cudaStream_t s);
void launch_cg_scale_r32(const CGView& v, cudaStream_t s);
// q = A p, alpha = rho / p.q
void launch_cg_apply(const CGView& v, cudaStream_t s);
// x += alpha p, r -= alpha q (and z = M r for Jacobi / none); dots for beta and the stopping test
void launch_cg_update(const CGView& v, cudaStream_t s);
// multigrid: z = V(r) done; dots r.z (and r.z_old when flexible), beta
void launch_cg_dots_after_precondition(const CGView& v, cudaStream_t s);
// p = z + beta p, then commit the stopping decision of this step
void launch_cg_xpby(const CGView& v, cudaStream_t s);
// z = r * invd on the Nx x Ny range, z = r on the wall faces (unit diagonal)
void launch_precondition_diagonal(const DevGrid<double>& g, double2* z, const double2* r, const double2* invd, cudaStream_t s);
// Picard: xprev = x (over the Nx x Ny range)
void launch_copy_range(const DevGrid<double>& g, double2* dst, const double2* src, cudaStream_t s);
// Picard loop control on the device: begin (iteration 0) and end of one iteration (Δ, X, stopping test),
// each setting the conditional-node handle `cond` of the Picard while loop
void launch_picard_begin(SolverScalars* sc, unsigned long long cond, long long stride, cudaStream_t s);
// sets `cond` to whether any of `slots` slots (scalars `stride` bytes apart) goes on: Picard (cg = 0) or CG (cg = 1);
// adds one to *counter (if given) when it does
void launch_batch_condition(const SolverScalars* sc, long long stride, int slots, int cg, unsigned long long cond, int* counter,
                            cudaStream_t s);
void launch_picard_end(const DevGrid<double>& g, double2* xprev, const double2* x, SolverScalars* sc, double2* partials,
                       unsigned long long cond, cudaStream_t s);
// the same under the viscosity-change rule (NK_VISCOSITY_CONVERGENCE): Δ = ‖η̄H - η̄H⁻‖, X = ‖η̄H‖, η̄H⁻ = η̄H
void launch_picard_end_viscosity(const DevGrid<double>& g, const double4* coef, double* eta_prev, SolverScalars* sc, double2* partials,
                                 unsigned long long cond, cudaStream_t s);

// ---- coefficients ---------------------------------------------------------------------------------------
// SSA membrane viscosity (glen_flow_law.jl:107-111) and column integrals (column_integrals.jl:61-72)
void launch_viscosity(const PhysView& ph, const double2* x, double* eta_sigma, double4* coef, double* F2, cudaStream_t s);
// DIVA viscosity with lagged vertical shear (glen_flow_law.jl:134-143) and column integrals
void launch_viscosity_diva(const PhysView& ph, const double2* x, const double2* bb, const double2* ub, double* eta_sigma,
                           double4* coef, double* F2, cudaStream_t s);
// eta_H_ff = ℑxyᶠᶠ(eta_H) over 0..Nx x 0..Ny (stress_balance_coefficients.jl:26-29)
template <typename T>
void launch_corners(const DevGrid<T>& g, typename Vec4<T>::type* coef, cudaStream_t s);
// basal drag at the faces from the velocity `x` (frictions.jl:142-160): writes beta into (coef.z, coef.w)
// when `coef` is given, else into the pair array `bb` (DIVA friction-law drag)
void launch_basal_drag(const PhysView& ph, const double2* x, double4* coef, double2* bb, cudaStream_t s);
// DIVA basal velocity u_b = u / (1 + beta_b ℑF2) (diva.jl:19-27)
void launch_basal_velocity(const PhysView& ph, const double2* x, const double2* bb, const double* F2, double2* ub, cudaStream_t s);
// DIVA effective drag beta = beta_b / (1 + beta_b ℑF2) (diva.jl:43-51)
void launch_effective_drag(const PhysView& ph, const double2* bb, const double* F2, double4* coef, cudaStream_t s);

// ---- fixed-point adjoint of the SSA Picard step (nk_coefficients.cu) ------------------------------------------
// One Picard step maps x to A(c(x))⁻¹ b with c = (η̄H, η̄Hᶠᶠ, βᵘ, βᵛ) from the viscosity, corner and drag
// updates.  These kernels apply the transpose of ∂[A(c(x)) x*]/∂x at the fixed point x* to an adjoint state λ.
struct AdjointView {
    PhysView ph;                  // grid, rheology and friction parameters and inputs
    OpView<double> o;             // coefficients c(x*) and the operator mask
    const double2* xs;            // converged velocity x*
    const double2* lam;           // adjoint state λ
    const double2* xbar;          // ∂J/∂x
    double2* cbar;                // (∂/∂η̄H at centre (i, j) through the centre stresses, ∂/∂η̄Hᶠᶠ at corner (i, j))
    double2* bbar;                // (∂/∂βᵘ, ∂/∂βᵛ) at faces (i, j)
    double* gbar;                 // ∂/∂(ε̇ₑ² + ε̇₀²) at centre (i, j)
    double2* r;                   // x̄ − (∂[A(c(x)) x*]/∂x)ᵀ λ
    double* grad_log_C;           // −λᵀ ∂[A(c) x*]/∂ log C per cell
    const double* eta_sigma;      // ησ of c(x*) (Nσ planes)
    double* grad_log_A;           // −λᵀ ∂[A(c) x*]/∂ log A per cell (2-D rate factor) or per cell and layer (σ);
                                  // written by k_adjoint_viscosity when not null
    // DIVA: the step also reads its own previous βᵇ, F₂ and ησ (the lagged state s), so the fixed point is one of
    // (x, s) and the adjoint carries σ = the adjoint of s next to λ.  These kernels work in true adjoints
    // (q̄ = −λ), where the SSA kernels above use λ-signed sensitivities.
    const double2* ubs = nullptr;     // basal velocities uᵇ of the step at x*
    const double2* bbs = nullptr;     // basal drag βᵇ at x* (also the lagged βᵇ of the fixed point)
    const double* F2s = nullptr;      // F₂ at x* (also the lagged F₂)
    double2* txbar = nullptr;         // per centre: ∂J/∂(ℑxᶜ βᵇᵘuᵇ), ∂J/∂(ℑyᶜ βᵇᵛvᵇ)
    double2* sig_bb = nullptr;        // σ of βᵇ per face
    double* sig_F2 = nullptr;         // σ of F₂ per centre
    double* sig_eta = nullptr;        // σ of ησ (Nσ planes)
    double2* Ubar = nullptr;          // per face: ∂J/∂U of the basal speed
    double2* ubp = nullptr;           // per face: ∂J/∂uᵇ through the basal shear stress of the centres
    double2* mbar = nullptr;          // per face: ∂J/∂(ℑF₂⁻) of the lagged shear factor
    double2* bbt = nullptr;           // per face: ∂J/∂βᵇ (all paths)
    double2* hmu = nullptr;           // when set, the centre pass writes per centre (∂J/∂H through η̄H and F₂ at
                                      // fixed μ, ∂J/∂μ through η̄H): the thickness gradient's coefficient part
    // when set, ∂J/∂η̄H per centre from outside the solve (a true adjoint): the shadow of the overwritten coefficient
    // η̄H, which the fixed point's reverse carries with the operator's own η̄H adjoint in every pass
    const double* eta_bar_in = nullptr;
};
void launch_adjoint_coefficients(const AdjointView& v, cudaStream_t s);
void launch_adjoint_viscosity(const AdjointView& v, cudaStream_t s);
void launch_adjoint_velocity(const AdjointView& v, cudaStream_t s);
void launch_adjoint_gradient(const AdjointView& v, cudaStream_t s);
struct GeometryView;
// ∂J/∂H per centre with update_geometry! and compute_driving_stress! recomputed from H, after the final pass of the
// adjoint (SSA: launch_adjoint_coefficients, eta_sigma of c(x*), λ and the drag sensitivities; DIVA: the sweep with
// v.hmu set, and bbt)
void launch_adjoint_thickness(const AdjointView& v, const GeometryView& gv, int diva, double* grad_H, cudaStream_t s);
// DIVA reverse sweep of one Picard step at the fixed point (after launch_adjoint_coefficients): the centre pass
// (viscosity, F₂, ησ; grad_log_A when set), the face pass (effective drag, basal shear stress, drag speed), the
// velocity pass (uᵇ = x / (1 + βᵇ⁻ ℑF₂⁻), strain rates; writes r and σ of βᵇ) and the F₂⁻ pass (σ of F₂)
void launch_adjoint_diva(const AdjointView& v, cudaStream_t s);
// DIVA: ∂J/∂log C from bbt
void launch_adjoint_diva_gradient(const AdjointView& v, cudaStream_t s);
// Δ = ‖λ⁺ − λ‖, M = ‖λ⁺‖ over the solved cells into sc->p_D / sc->p_X, then λ = λ⁺
void launch_adjoint_change(const DevGrid<double>& g, const double2* lam_new, double2* lam, SolverScalars* sc, double2* partials,
                           cudaStream_t s);
// DIVA velocity profile (diva.jl:99-109) / SSA depth extension (ice_sheet_model_methods.jl:167-180)
void launch_velocity_profile(const PhysView& ph, int diva, const double2* x, const double2* bb, const double* F2,
                             const double* eta_sigma, double2* ub, double2* usig, cudaStream_t s);

// ---- geometry -------------------------------------------------------------------------------------------
struct GeometryView {
    DevGrid<double> g;
    const double* H; const double* bed;
    double* s; double* N; double* mu; double* phi; double2* phi_uv; double2* tau;
    double rho_i, rho_w, gacc;
    int grounding, gl_stress, use_mask;
    double mask_min, mask_trans;
    const double2* ud = nullptr;      // prescribed (u, v) per face, NaN where free: the right-hand side there
    int front = 0;                    // a partial-cell front: the ice mask is its prognostic flag, not recomputed
    // TillEffectivePressure: when Hw is set, N follows the basal water through the till (N0, δ, e0 / Cc, W_max)
    const double* Hw = nullptr;
    double till_N0 = 0, till_delta = 0, till_e0_Cc = 0, till_Wmax = 1;
};
void launch_geometry(const GeometryView& v, cudaStream_t s);
void launch_rate_factor(const DevGrid<double>& g, const SigmaTable& sig, int plane, const double* H, const double* T, double* A,
                        double rho_i, double gacc, const double* params, cudaStream_t s);
void launch_thermal_diagnostics(const DevGrid<double>& g, const SigmaTable& sig, int plane, const double* H, const double* E, double* T,
                                double* omega, double* A, double rho_i, double gacc, const double* params, cudaStream_t s);

// ---- thickness transport --------------------------------------------------------------------------------
struct ThicknessView {
    DevGrid<double> g;
    const double2* x;                 // depth-averaged (u, v) per face, held through the step
    const double* Hs;                 // thickness at the start of the stage (read with its neighbours)
    const double* H0;                 // thickness at the start of the step (H⁻)
    const double* smb; const double* melt; const double* gmelt; const double* phi;
    double* H; double* clipped;
    int grounding, coupled;
    int scheme, order, bounded;       // nk_advection_desc
    double lower, upper;
    double* theta;                    // the bounds-preserving limiter per cell (bounded WENO only)
    const double* mu = nullptr;       // a partial-cell front's flag of full cells (null without a front)
    // WENO: each face's two reconstructions of the stage thickness, computed once by k_thickness_faces for the
    // limiter and the stage (x face (i, j): from cell i-1 (flow east), from cell i (flow west); y face likewise
    // from the south and from the north cell); null for the upwind schemes, which read the stencil directly
    double2* fx = nullptr;
    double2* fy = nullptr;
};

// ---- the partial-cell front and calving (nk_front.cu) ------------------------------------------------------------
struct FrontView {
    DevGrid<double> g;
    double* H; double* mu; double* Hr; double* O; double* calved; double* clipped;
    double* H_in; double* mu_in;      // snapshots read by the overflow passes
    double* f; double* share;         // calving: retreat fraction, then the residual area shared among neighbours
    const double2* x; const double* bed; const double* phi; const double4* coef; const double* extent;
    const double* smb; const double* melt; const double* gmelt;
    int grounding, coupled, law;
    double thickness, coefficient, stress_threshold, floating_stress_threshold, front_velocity;
    double n, eps0, wall_factor;
};
void launch_initialize_front(const FrontView& v, cudaStream_t s);
// advance_front!: the whole sequence of its kernels (with the snapshot copies of the passes) on stream s
void launch_advance_front(const FrontView& v, int passes, double dt, size_t plane, cudaStream_t s);
void launch_thickness_faces(const ThicknessView& v, cudaStream_t s);
void launch_thickness_limiter(const ThicknessView& v, cudaStream_t s);
void launch_thickness_stage(const ThicknessView& v, double dtau, int final_stage, cudaStream_t s);

// ---- the reverse of a thickness stage (nk_time_adjoint.cu) ------------------------------------------------------
// The forward view t at the stage (Hs, H0, the velocities, the effective melt, φ of Hs, and the faces and θ
// recomputed from Hs), the stage's output thickness and its adjoint λ: adds the adjoints of H0, the velocities, the
// surface mass balance and the base melt rate, and writes the adjoint of Hs (through the fluxes, the limiter, the
// reconstructions and the centre grounded fraction of the melt).
struct StageAdjointView {
    ThicknessView t;
    const double* Hout;               // the stage's output thickness (its clip: H★ > 0 where Hout > 0)
    const double* bed;                // the flotation of φ: f = H + (ρw / ρi) b
    double rw_ri;
    double dtau, melt_weight;         // Δτ of the stage; the factor of the base melt rate in the step
    const double* lam_out;            // λ of the output thickness
    double* lam_H0;                   // += λ of the step-start thickness
    double* lam_Hs;                   // = λ of the stage-start thickness
    double2* lam_x;                   // += λ of (u, v) per face
    double* lam_smb; double* lam_melt;   // += λ of the surface mass balance and of the base melt rate
    // scratch planes
    double* dv;                       // -Δτ λ★ / Az per cell (λ★ the adjoint of H★)
    double* lam_phi;                  // λ of the centre grounded fraction per cell
    double2* lamF;                    // λ of the flux through x face (i, j) (.x) and y face (i, j) (.y)
    double2* lw_x; double2* lw_y;     // λ of a cell's own reconstructions (W, E) and (S, N) through its limiter θ
    const double* lam_phi_in = nullptr;   // λ of φ from elsewhere (the front's forced melt), added before the gather
};
void launch_stage_adjoint(const StageAdjointView& a, cudaStream_t s);
// The reverse of advance_front! without calving (nk_front.cu).  f is the front's view at the end of the final stage
// with f.H the stage's output before the front, f.mu and f.Hr the flag and Hʳ before it, the stage's velocities,
// the effective melt and φ of the stage's input; snaps the advance as launch_front_record recorded it.
struct FrontAdjointView {
    FrontView f;
    int passes;
    const double* snaps;
    size_t plane;
    double dt, melt_weight;
    const double* lam_H;              // λ of H after the front
    double* lam_Hr;                   // in: λ of Hʳ after the front; out: λ of Hʳ before it
    double* lam_H3;                   // = λ of the stage output before the front
    double* lam_smb; double* lam_melt;   // +=
    double* lam_phi;                  // = λ of φ of the forced cells' melt
    double* lam_a; double* lam_b; double* lam_c; double* lam_d;   // scratch planes
    // calving (f.law a rate law or a removal law): λ of the retreat fraction, of each cell's calving rate as used and
    // as computed, of its ocean-facing length, and the λ of the velocities it adds
    double* lam_e; double* lam_f; double* lam_g; double* lam_h;
    double2* lam_x;
    // von Mises: when set, = λ of the depth-averaged viscosity η̄H (f.coef[].x) per cell that the rates read (η = η̄H / H)
    double* lam_eta = nullptr;
};
// The drain, the reference pass, the overflow passes and the calving of advance_front! on v's planes (v.H, v.mu, v.Hr
// set by the caller to the state before it), recording into snaps (front_record_planes of them): per level
// p = 0..passes the thickness, flag and Hʳ before fill p, then per pass the thickness after its fill and its overflow
// volumes, then with a calving law the retreat fraction, the thickness, flag and Hʳ after the retreat, its residual,
// the shares, and the thickness, flag and Hʳ after the receive (before the forced sources).
int front_record_planes(int passes, int law);
void launch_front_record(const FrontView& v, int passes, size_t plane, double* snaps, double dt, cudaStream_t s);
void launch_front_adjoint(const FrontAdjointView& a, cudaStream_t s);
// y += x over the interior cells of `planes` planes (each `plane` doubles apart)
void launch_add_planes(const DevGrid<double>& g, double* y, const double* x, int planes, size_t plane, cudaStream_t s);
// y += x over the pair faces 0..Nx x 0..Ny
void launch_add_pairs(const DevGrid<double>& g, double2* y, const double2* x, cudaStream_t s);
// y = a x over the interior cells
void launch_scale_plane(const DevGrid<double>& g, double* y, const double* x, double a, cudaStream_t s);

// ---- the energy step -------------------------------------------------------------------------------------
constexpr int ENERGY_MAX_LAYERS = 64;
struct EnergyConstants {
    double k, c, L, beta, T0, Tr;              // conductivity, heat capacity, latent heat, Clausius-Clapeyron, melting, reference
    double temperate_ratio, blend, water_blend, min_thickness, drainage_fraction, max_drainage_rate;
    int coupled;
};
struct EnergyView {
    DevGrid<double> g;
    SigmaTable sig;
    long long plane;
    EnergyConstants q;
    double rho_i, gacc, wall_factor;
    int diva, grounding;
    const double2* x; const double2* ud;       // depth-averaged velocities, prescribed faces (or null)
    const double2* usig;                       // layer velocities (σ planes)
    const double2* ub;                         // basal velocities
    const double4* coef;                       // SSA basal drag (βᵘ, βᵛ) in .z / .w
    const double2* bb;                         // DIVA basal drag (βᵇᵘ, βᵇᵛ)
    const double* eta_sigma;                   // layer viscosity (σ planes)
    const double* H; const double* Hn; const double* phi;
    const double* melt; const double* G; const double* Ts; const double* To;
    const double* E_old;                       // the enthalpy at the start of the step (σ planes, read with neighbours)
    double* E; double* T; double* omega;       // σ planes
    double* Hw; double* gmelt; double* sb; double* qg; double* Phi;
    int till = 0; double till_drain = 0, till_Wmax = 0;   // drain_till of TillEffectivePressure when till is set
};
void launch_step_enthalpy(const EnergyView& v, double dt, cudaStream_t s);

// ---- multigrid ------------------------------------------------------------------------------------------
template <typename T>
struct LevelView {
    OpView<T> o;
    typename Vec2<T>::type* x;
    typename Vec2<T>::type* x2;      // ping-pong partner of x for the point smoother
    typename Vec2<T>::type* b;
    typename Vec2<T>::type* q;
    T* t;                            // line-smoother scratch (one T per cell)
    const typename Vec2<T>::type* irs;  // inverse ℓ1 row sums
    int cx, cy;                      // coarsening factor from the finer level (1 or 2)
};
template <typename T>
__device__ __forceinline__ void rebase(LevelView<T>& L, long long d) {
    rebase(L.o, d);
    shift_ptr(L.x, d); shift_ptr(L.x2, d); shift_ptr(L.b, d); shift_ptr(L.q, d); shift_ptr(L.t, d); shift_ptr(L.irs, d);
}
// Mean device time in ms of `repeats` launches of one level's sweep (kind STRIP_SMOOTH, x -> x2) or residual
// (STRIP_RESIDUAL, into q) with walks of `rows` rows; negative if a CUDA call failed (the strip autotuner)
template <typename T>
float time_strip_kernel(const LevelView<T>& L, int kind, int rows, int repeats, cudaStream_t s);
// coarse coefficients from the finer level (multigrid_preconditioner.jl:331-344), then corners
template <typename T, typename TF>
void launch_coarsen(const LevelView<T>& coarse, const DevGrid<TF>& fine_g, const typename Vec4<TF>::type* fine_coef,
                    typename Vec4<T>::type* coarse_coef, cudaStream_t s);
// x_out = x_in + (b - A x_in) / rowsum (x_in = 0 when `first`: x_out = b / rowsum)
template <typename T>
void launch_smooth_point(const LevelView<T>& L, const typename Vec2<T>::type* x_in, typename Vec2<T>::type* x_out, int first,
                         const int* done, cudaStream_t s);
// the first two sweeps from a zero guess in one pass (x1 = b / rowsum formed on load)
template <typename T>
void launch_smooth_first2(const LevelView<T>& L, typename Vec2<T>::type* x_out, const int* done, cudaStream_t s);
// the coarsest level's sweeps in one thread block with the level in shared memory (x_in = nullptr: from zero;
// from_zero: the first sweep is x = b / rowsum); result in x_out
template <typename T>
bool coarsest_smem_fits(const LevelView<T>& L, int plane);
template <typename T>
void configure_coarsest_smem();
template <typename T>
void launch_coarsest_smem(const LevelView<T>& L, int plane, const typename Vec2<T>::type* x_in, int sweeps, int from_zero,
                          typename Vec2<T>::type* x_out, const int* done, cudaStream_t s);
// q = A x (line smoother first half) or q = b - A x (residual)
template <typename T>
void launch_level_apply(const LevelView<T>& L, const typename Vec2<T>::type* x, typename Vec2<T>::type* q, int residual,
                        const int* done, cudaStream_t s);
// `first`: x starts at zero (q = A x = 0 is not read, x is overwritten)
template <typename T>
void launch_line_relax(const LevelView<T>& L, typename Vec2<T>::type* x, int first, const int* done, cudaStream_t s);
// b_coarse = R r_fine; when first_out is given also first_out = b_coarse / rowsum (the coarse level's first sweep)
template <typename T>
void launch_restrict(const LevelView<T>& coarse, const LevelView<T>& fine, const typename Vec2<T>::type* r_fine,
                     typename Vec2<T>::type* b_coarse, typename Vec2<T>::type* first_out, const int* done, cudaStream_t s);
template <typename T>
void launch_prolongate(const LevelView<T>& fine, const LevelView<T>& coarse, typename Vec2<T>::type* x_fine,
                       const typename Vec2<T>::type* x_coarse, const int* done, cudaStream_t s);
template <typename T>
void launch_zero_vec(const DevGrid<T>& g, typename Vec2<T>::type* x, const int* done, cudaStream_t s);
// dst = src over the first n entries of a level's pitched plane (batch-aware device copy)
template <typename T>
void launch_copy_plane(const DevGrid<T>& g, typename Vec2<T>::type* dst, const typename Vec2<T>::type* src, int n, const int* done,
                       cudaStream_t s);
// Every level from one level down to the coarsest, handled by a single thread block.
constexpr int MAX_COARSE_LEVELS = 12;
template <typename T>
struct CoarseLevels {
    LevelView<T> lv[MAX_COARSE_LEVELS];
    int n;                  // number of levels in lv (>= 1); lv[n - 1] is the coarsest
    int sweeps, coarsest;   // smoothing_sweeps, coarsest_sweeps
    int line;               // y-line smoother
};
template <typename T>
void launch_coarse_vcycle(const CoarseLevels<T>& C, const int* done, cudaStream_t s);
// FP64 <-> FP32 conversions of vectors and of the coefficient record
void launch_to_float(const DevGrid<double>& g, const double2* src, float2* dst, const int* done, cudaStream_t s);
void launch_to_double(const DevGrid<double>& g, const float2* src, double2* dst, const int* done, cudaStream_t s);
void launch_coef_to_float(const DevGrid<double>& g, const double4* src, float4* dst, cudaStream_t s);
// FP64 vector copy on the Nx x Ny range under the done predicate
void launch_copy_vec(const DevGrid<double>& g, double2* dst, const double2* src, const int* done, cudaStream_t s);

}  // namespace nk
