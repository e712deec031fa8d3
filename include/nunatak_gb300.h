/*
 * nunatak_gb300.h — C ABI of libnunatak_gb300.so, the GB300 (sm_103a) velocity solver for
 * Nunatak.jl's depth-integrated (SSA / DIVA) stress balance.
 *
 * The entry points replace the Julia call chain of the reference at its Picard + PCG call site:
 *
 *   update_velocities!(model, ::StressBalanceSolver, ::SSA | ::DIVA)
 *       src/Models/ice_sheet_model_methods.jl:119-147
 *     -> picard_solve!(x, picard, linear_solver, update_coefficients!, b, coefficients...)
 *       src/Solvers/picard.jl:63-90
 *       -> update_stress_balance_coefficients!   src/StressBalances/stress_balance_coefficients.jl:10-20
 *          update_diva_coefficients!             src/StressBalances/diva.jl:61-75
 *       -> solve!(x, solver, b, args...)         src/Solvers/conjugate_gradient.jl:128-223
 *          -> ssa_operator!                      src/StressBalances/ssa_operator.jl:47-89
 *          -> precondition!                      src/StressBalances/diagonal_preconditioner.jl:11-54
 *                                                src/StressBalances/multigrid_preconditioner.jl:122-360
 *
 * Plain C types only: no CUDA, C++ or torch types cross this boundary.  Every function returns an
 * nk_status and never throws.  Host arrays are caller-owned; the library copies them to and from its
 * own device buffers inside the call and keeps no host pointer after the call returns.
 *
 * Array layout ("interior layout"): the memory order of Oceananigans' interior(field) — column-major,
 * x fastest, no halos.  Sizes for an Nx x Ny grid with x topology TX and y topology TY:
 *   Center-Center (H, b, s, N, mu, eta_H, F2, C, A2D) : Nx * Ny
 *   Face-Center   (u, beta_u, tau_u, phi_u, ...)      : nfx * Ny,  nfx = Nx + 1 (Bounded) or Nx (Periodic)
 *   Center-Face   (v, beta_v, tau_v, phi_v, ...)      : Nx * nfy,  nfy = Ny + 1 (Bounded) or Ny (Periodic)
 *   Face-Face     (eta_H_ff)                          : nfx * nfy
 *   sigma fields  (eta_sigma, A3D, T)                 : Nx * Ny * Nsigma  (k slowest)
 *   face sigma    (u_sigma / v_sigma)                 : nfx * Ny * Nsigma / Nx * nfy * Nsigma
 */
#ifndef NUNATAK_GB300_H
#define NUNATAK_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NK_API_VERSION 1

/* Status codes.  The reference signals these through return values, @warn and ArgumentError
 * (src/Solvers/conjugate_gradient.jl:185-200 stops silently at maxiter, src/Solvers/picard.jl:79-89 likewise,
 *  src/StressBalances/ssa_operator.jl:56 throws ArgumentError). */
typedef int32_t nk_status;
#define NK_OK               0
#define NK_NOT_CONVERGED    1   /* an iteration control with Convergence reached maxiter (result still written) */
#define NK_NONFINITE        2   /* a NaN / Inf residual or velocity */
#define NK_BREAKDOWN        3   /* p.q <= 0 in conjugate gradients (operator not SPD on the active points) */
#define NK_OOM              4   /* device allocation failed */
#define NK_BAD_ARGUMENT     5   /* invalid descriptor, field id, size or null pointer */
#define NK_TIMEOUT          6   /* a device wait ran out of its bound */
#define NK_CUDA_ERROR       7   /* any other CUDA runtime error */
#define NK_BUSY             8   /* server queue full / request not finished */

/* Topology of one horizontal direction (Oceananigans Bounded / Periodic). */
#define NK_BOUNDED   0
#define NK_PERIODIC  1

/* Tangential wall condition, src/StressBalances/depth_integrated.jl:31-45. */
#define NK_FREE_SLIP 0
#define NK_NO_SLIP   1

/* Stress balance, src/StressBalances/depth_integrated.jl:1-58 (SSA = shear nothing, DIVA = DIVAShear()). */
#define NK_SSA  0
#define NK_DIVA 1

/* Friction law, src/Frictions/frictions.jl:9-89. */
#define NK_FRICTION_NONE        0
#define NK_WEERTMAN             1
#define NK_REGULARIZED_COULOMB  2

/* Rate factor layout of GlenFlowLaw, src/Rheologies/glen_flow_law.jl:60-68. */
#define NK_RATE_FACTOR_2D     0   /* Center-Center field, uniform in depth */
#define NK_RATE_FACTOR_SIGMA  1   /* field on the sigma grid */

/* Preconditioner of the velocity conjugate-gradient solver. */
#define NK_PRECONDITIONER_NONE       0   /* precondition!(z, ::Nothing, r)          conjugate_gradient.jl:33 */
#define NK_PRECONDITIONER_DIAGONAL   1   /* StressBalanceDiagonalPreconditioner     diagonal_preconditioner.jl:9 */
#define NK_PRECONDITIONER_MULTIGRID  2   /* StressBalanceMultigridPreconditioner    multigrid_preconditioner.jl:18 */

/* Multigrid smoother, src/StressBalances/multigrid_preconditioner.jl:69-78. */
#define NK_SMOOTHER_POINT_JACOBI 0
#define NK_SMOOTHER_LINE_JACOBI  1

/* Arithmetic of the solve.  FP64 reproduces the reference; MIXED runs the multigrid preconditioner
 * (operator applies, smoother state, transfers) in FP32 under an FP64 flexible conjugate gradient whose
 * residual, dot products and Picard test stay FP64. */
#define NK_PRECISION_FP64  0
#define NK_PRECISION_MIXED 1

/* Iteration control, src/Solvers/iteration_controls.jl:1-43. */
#define NK_CONVERGENCE      0
#define NK_FIXED_ITERATIONS 1
/* An extension for the Picard control only (the reference tests the velocity change, picard.jl:79-85):
 * stop when the depth-integrated viscosity of consecutive coefficient updates changes by
 * ||etaH_k - etaH_(k-1)|| <= max(reltol ||etaH_k||, abstol) over the Nx x Ny centres, or at maxiter.  The first
 * iteration has no previous etaH (change = infinity).  picard_change / picard_norm report ||d etaH|| / ||etaH||. */
#define NK_VISCOSITY_CONVERGENCE 2

typedef struct nk_iteration_control {
    int32_t kind;        /* NK_CONVERGENCE, NK_FIXED_ITERATIONS (or NK_VISCOSITY_CONVERGENCE for Picard) */
    int32_t iterations;  /* FixedIterations(iterations) */
    int32_t maxiter;     /* Convergence: maxiter */
    int32_t reserved;
    double  reltol;      /* Convergence: reltol */
    double  abstol;      /* Convergence: abstol */
} nk_iteration_control;

/* Horizontal RectilinearGrid (Flat z) plus the sigma column of SigmaGrid, src/Grids/sigma_grid.jl:20-62. */
typedef struct nk_grid_desc {
    int32_t Nx, Ny;
    int32_t topology_x, topology_y;   /* NK_BOUNDED / NK_PERIODIC */
    int32_t halo_x, halo_y;           /* only the multigrid coarsening rule reads the halo (multigrid_preconditioner.jl:86) */
    int32_t Nsigma;                   /* number of sigma levels (>= 1) */
    int32_t reserved;
    const double* x_faces;            /* Nx+1 face coordinates, or NULL for a regular grid on [x0, x0 + Lx] */
    const double* y_faces;            /* Ny+1 face coordinates, or NULL for a regular grid on [y0, y0 + Ly] */
    double x0, Lx, y0, Ly;
    const double* sigma_faces;        /* Nsigma+1 faces zeta_0 = 0 .. zeta_Nsigma = 1, or NULL for (k/Nsigma)^bed_refinement */
    double bed_refinement;
} nk_grid_desc;

/* Physics of the solve: DepthIntegrated, GlenFlowLaw, friction law, IceSheetConstants, SmoothIceMask. */
typedef struct nk_physics_desc {
    int32_t stress_balance;           /* NK_SSA / NK_DIVA */
    int32_t side_walls;               /* NK_FREE_SLIP / NK_NO_SLIP */
    int32_t rate_factor_layout;       /* NK_RATE_FACTOR_2D / NK_RATE_FACTOR_SIGMA */
    int32_t friction;                 /* NK_FRICTION_NONE / NK_WEERTMAN / NK_REGULARIZED_COULOMB */
    double  glen_exponent;            /* n */
    double  strain_rate_regularization;   /* epsilon_0 (1/s) */
    double  friction_exponent;        /* m */
    double  coulomb_coefficient;      /* alpha^2 */
    double  velocity_regularization;  /* u_0 (m/s) */
    double  ice_density, ocean_density, gravitational_acceleration;
    int32_t use_ice_mask;             /* 1: eta_H is scaled by mu and faces with mu = 0 on both sides drop out */
    int32_t grounding;                /* 0: nothing (all grounded), 1: SubgridGroundedFraction */
    int32_t grounding_line_driving_stress;   /* SubgridGroundedFraction(driving_stress = true) */
    int32_t use_effective_pressure;   /* 1: the friction law receives N (0 passes `nothing`) */
    double  mask_minimum_thickness;   /* SmoothIceMask, src/Models/smooth_ice_mask.jl:41 */
    double  mask_transition_thickness;
} nk_physics_desc;

/* StressBalanceSolver options, src/StressBalances/stress_balance_solver.jl:43-52. */
typedef struct nk_solver_desc {
    int32_t precision;                /* NK_PRECISION_FP64 / NK_PRECISION_MIXED */
    int32_t preconditioner;           /* NK_PRECONDITIONER_* */
    int32_t smoother;                 /* NK_SMOOTHER_* */
    int32_t smoothing_sweeps;         /* default 2 */
    int32_t coarsest_sweeps;          /* default 20 */
    int32_t minimum_coarse_size;      /* default 2 */
    nk_iteration_control linear;      /* default Convergence(reltol = 1e-8, maxiter = 10_000) */
    nk_iteration_control picard;      /* default Convergence(reltol = 1e-6, maxiter = 100) */
    int32_t flags;                    /* NK_SOLVER_* bits, 0 by default */
    int32_t reserved;                 /* 0 */
} nk_solver_desc;

/* Issue the solve's kernels one by one from a host loop (conjugate-gradient steps in batches, the device stopping
 * flag read after each batch; Picard reads its decision after every iteration) instead of replaying one CUDA graph
 * with conditional WHILE nodes.  Same kernels, same arithmetic, same results; slower, and refused by
 * nk_picard_solve_async.  Kernels inside conditional graph nodes are invisible to kernel profilers; this path shows
 * every launch.  The NK_GRAPHS=0 environment variable sets it for every problem of the process. */
#define NK_SOLVER_HOST_LOOP 1

/* Field identifiers for nk_problem_set_field / nk_problem_get_field (the reference's names). */
#define NK_FIELD_U              0   /* model.velocities.u                   Face-Center */
#define NK_FIELD_V              1   /* model.velocities.v                   Center-Face */
#define NK_FIELD_H              2   /* model.geometry.H                     Center-Center */
#define NK_FIELD_BED            3   /* model.bed                            Center-Center */
#define NK_FIELD_SURFACE        4   /* model.geometry.s                     Center-Center */
#define NK_FIELD_ICE_MASK       5   /* model.geometry.ice_mask (mu)         Center-Center */
#define NK_FIELD_PHI            6   /* model.geometry.phi                   Center-Center */
#define NK_FIELD_PHI_U          7   /* model.geometry.phi_u                 Face-Center */
#define NK_FIELD_PHI_V          8   /* model.geometry.phi_v                 Center-Face */
#define NK_FIELD_EFFECTIVE_PRESSURE 9   /* model.geometry.N                 Center-Center */
#define NK_FIELD_TAU_U         10   /* model.auxiliary.tau_u (RHS)          Face-Center */
#define NK_FIELD_TAU_V         11   /* model.auxiliary.tau_v                Center-Face */
#define NK_FIELD_RATE_FACTOR   12   /* GlenFlowLaw rate factor A            Center-Center or sigma */
#define NK_FIELD_FRICTION_COEFFICIENT 13  /* friction.coefficient C         Center-Center */
#define NK_FIELD_ETA_H         14   /* model.auxiliary.eta_bar_H            Center-Center */
#define NK_FIELD_ETA_H_FF      15   /* model.auxiliary.eta_bar_H_ff         Face-Face */
#define NK_FIELD_BETA_U        16   /* model.auxiliary.beta_u               Face-Center */
#define NK_FIELD_BETA_V        17   /* model.auxiliary.beta_v               Center-Face */
#define NK_FIELD_ETA_SIGMA     18   /* model.auxiliary.eta_sigma            sigma */
#define NK_FIELD_F2            19   /* model.auxiliary.F2                   Center-Center */
#define NK_FIELD_BETA_B_U      20   /* model.auxiliary.beta_b_u (DIVA)      Face-Center */
#define NK_FIELD_BETA_B_V      21   /* model.auxiliary.beta_b_v (DIVA)      Center-Face */
#define NK_FIELD_U_B           22   /* model.velocities.u_b                 Face-Center */
#define NK_FIELD_V_B           23   /* model.velocities.v_b                 Center-Face */
#define NK_FIELD_U_SIGMA       24   /* model.velocities.u_sigma             Face-Center x sigma */
#define NK_FIELD_V_SIGMA       25   /* model.velocities.v_sigma             Center-Face x sigma */
#define NK_FIELD_TEMPERATURE   26   /* temperature on the sigma grid (input of nk_compute_rate_factor) */
/* Prescribed velocities (an extension; the reference has no velocity boundary condition): NaN = free, a finite
 * value = that face's velocity is held at it.  Such a face solves an identity row (x = u_D) and its value enters
 * the neighbouring strain rates, viscosity and stresses, also on the boundary faces that are walls otherwise
 * (an inflow at x = 0 is u_D on the faces i = 0).  Setting either field: the driving stress (the right-hand side)
 * and the velocity take u_D there, and nk_compute_geometry keeps them.  Problems with prescribed velocities
 * refuse nk_adjoint_solve and nk_picard_adjoint (the lifted operator is not symmetric) with NK_BAD_ARGUMENT. */
#define NK_FIELD_U_PRESCRIBED  27   /* u_D                                  Face-Center */
#define NK_FIELD_V_PRESCRIBED  28   /* v_D                                  Center-Face */
#define NK_FIELD_ENTHALPY      29   /* enthalpy E on the sigma grid (input of nk_compute_thermal_diagnostics) */
#define NK_FIELD_WATER_FRACTION 30  /* water fraction omega on the sigma grid (written by nk_compute_thermal_diagnostics) */
/* The thickness step's sources and its clip (nk_step_thickness), Center-Center, zero at first (allocated on first
 * use): IceSheetModel.surface_mass_balance a and basal_melt_rate m (src/Models/ice_sheet_model.jl:39-41), the
 * thermodynamics' grounded melt m^g (thermodynamics.state, read when grounded_melt_coupling is set) and
 * geometry.clipped_thickness (src/Models/time_stepping.jl:60-72), all in m s^-1 except the clip in m. */
#define NK_FIELD_SURFACE_MASS_BALANCE 31
#define NK_FIELD_BASAL_MELT_RATE      32
#define NK_FIELD_GROUNDED_MELT_RATE   33
#define NK_FIELD_CLIPPED_THICKNESS    34
/* The energy step's inputs, state and diagnostics (nk_step_enthalpy), zero at first (allocated on first use):
 * EnthalpyThermodynamics' state (src/Thermodynamics/enthalpy_thermodynamics.jl): the basal water layer H_w (m),
 * the geothermal flux G (W m^-2), the surface and ocean temperatures (K), the thickness of the last energy step
 * H^n (m; nk_step_enthalpy sets it to H), and the diagnostics of the last step: the temperate fraction of the
 * basal layer s_b, the basal heat flux q^g = phi G + friction heat (W m^-2) and the strain heating Phi on the
 * sigma grid (W m^-3).  All Center-Center; the strain heating has Nsigma planes. */
#define NK_FIELD_BASAL_WATER_THICKNESS    35
#define NK_FIELD_GEOTHERMAL_FLUX          36
#define NK_FIELD_SURFACE_TEMPERATURE      37
#define NK_FIELD_OCEAN_TEMPERATURE        38
#define NK_FIELD_THICKNESS_PREVIOUS       39
#define NK_FIELD_BASAL_TEMPERATE_FRACTION 40
#define NK_FIELD_BASAL_HEAT_FLUX          41
#define NK_FIELD_STRAIN_HEATING           42
/* The partial-cell front (nk_set_front; PartialCellFront, src/Models/partial_cell_front.jl:1-66), Center-Center, zero
 * at first: the ice thickness H^r of the partial front cells (geometry.front_thickness), the thickness removed by
 * calving (calved_thickness) and the region MaximumExtentCalving keeps ice in (extent, positive inside). */
#define NK_FIELD_FRONT_THICKNESS  43
#define NK_FIELD_CALVED_THICKNESS 44
#define NK_FIELD_CALVING_EXTENT   45
#define NK_FIELD_COUNT         46

typedef struct nk_solve_stats {
    int32_t status;                   /* nk_status of the solve */
    int32_t picard_iterations;        /* return value of picard_solve! */
    int32_t linear_iterations_last;   /* linear_solver.iteration after the last solve */
    int32_t linear_iterations_total;  /* sum over the Picard iterations */
    double  residual_norm;            /* final ||r|| of the last linear solve (unpreconditioned, FP64) */
    double  initial_residual_norm;    /* ||r0|| of the last linear solve */
    double  picard_change;            /* last ||x - x_prev|| (Convergence) */
    double  picard_norm;              /* last ||x|| (Convergence) */
    double  device_ms;                /* device time of the call, CUDA events */
    double  device_start_ms;          /* CUDA-event times of the solve's start and end, in ms after the context's */
    double  device_end_ms;            /* reference event (comparable across the problems of one context) */
} nk_solve_stats;

typedef struct nk_context nk_context;
typedef struct nk_problem nk_problem;
typedef struct nk_server  nk_server;

/* ---- context ------------------------------------------------------------------------------------ */

/* One context per device.  device = CUDA ordinal. */
nk_status   nk_context_create(int32_t device, nk_context** out);
nk_status   nk_context_destroy(nk_context* ctx);
const char* nk_last_error(const nk_context* ctx);
int32_t     nk_api_version(void);

/* ---- problem: one grid with its fields, coefficients, solver state and multigrid hierarchy ---------- */

/* IceSheetModel(grid; stress_balance, rheology, friction, grounding, masking, velocity_solver)
 * restricted to what the velocity solve reads (src/Models/ice_sheet_model.jl:79-120,
 * src/StressBalances/stress_balance_solver.jl:43-52).  Allocates every device buffer once. */
nk_status nk_problem_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics,
                            const nk_solver_desc* solver, nk_problem** out);
nk_status nk_problem_destroy(nk_problem* problem);

/* Copy an array in interior layout into a field (set!(field, array) + fill_halo_regions!).  The array may be in
 * host memory or in device memory of the problem's device (unified addressing). */
nk_status nk_problem_set_field(nk_problem* problem, int32_t field, const double* host, int64_t count);
/* Copy a field out in interior layout, to host memory or to device memory of the problem's device. */
nk_status nk_problem_get_field(const nk_problem* problem, int32_t field, double* host, int64_t count);
/* Number of values of a field in interior layout (0 for an unknown id). */
int64_t   nk_problem_field_size(const nk_problem* problem, int32_t field);
/* The same two copies with the field's Oceananigans parent array (parent(field), what set!/interior views wrap;
 * the sigma grid's z halo, src/Grids/sigma_grid.jl:57): x fastest, then y, then the level, with hx, hy halo
 * points on each side horizontally and hz levels below and above (hz = 0 for a 2-D field, whose parent has one
 * level).  The parent's x extent is the interior count plus 2 hx (Nx + 1 + 2 hx for a Face location in a Bounded
 * x), likewise in y; count is the parent's length.  set reads the interior points only; get writes them only and
 * leaves the halo values as they were.  Host or device memory, as above. */
nk_status nk_problem_set_field_parent(nk_problem* problem, int32_t field, const double* parent, int32_t hx, int32_t hy,
                                      int32_t hz, int64_t count);
nk_status nk_problem_get_field_parent(const nk_problem* problem, int32_t field, double* parent, int32_t hx, int32_t hy,
                                      int32_t hz, int64_t count);

/* update_geometry! + compute_driving_stress! (src/Models/ice_sheet_model_methods.jl:103-111, :126):
 * s, phi, phi_u, phi_v, N, mu from H and bed, then tau.  Replaces the reference's
 * compute_surface_elevation!, compute_grounded_fractions!, compute_effective_pressure!, compute_ice_mask!
 * (src/Groundings/subgrid_grounded_fraction.jl:109-232, src/Models/smooth_ice_mask.jl:60-69) and
 * compute_driving_stress! (src/StressBalances/driving_stress.jl:43-125). */
nk_status nk_compute_geometry(nk_problem* problem);

/* Rate factor on the sigma grid from the temperature field with omega = 0:
 * A = arrhenius_rate_factor(T - T_pm(p) + T_0, 0) (src/Thermodynamics/column_energy_solve.jl:104-110,
 * src/Rheologies/arrhenius_rate_factor.jl:102-110), p = rho_i g H (1 - zeta_k). */
nk_status nk_compute_rate_factor(nk_problem* problem, double cold_prefactor, double warm_prefactor,
                                 double cold_activation_energy, double warm_activation_energy,
                                 double transition_temperature, double transition_width, double gas_constant,
                                 double clausius_clapeyron, double melting_temperature);

/* Constants of the rate factor from the enthalpy: ArrheniusParameters (src/Rheologies/arrhenius_rate_factor.jl:10-29,
 * defaults :60-69: 3.61e-13, 1.73e3, 6.0e4, 13.9e4, 263.15, 1, 8.31441, 181.25, 0.01) and the EnthalpyThermodynamics
 * constants the conversions read (src/Thermodynamics/enthalpy_thermodynamics.jl:92-104: 2009, 3.34e5, 7.9e-8,
 * 273.15, 223.15). */
typedef struct nk_thermal_params {
    double cold_prefactor, warm_prefactor;                   /* Pa^-3 s^-1 */
    double cold_activation_energy, warm_activation_energy;   /* J mol^-1 */
    double transition_temperature, transition_width;         /* K */
    double gas_constant;                                     /* J mol^-1 K^-1 */
    double water_softening_coefficient;                      /* c in the softening 1 + c min(omega, omega_max) */
    double maximum_water_fraction;                           /* omega_max */
    double heat_capacity, latent_heat;                       /* c_i (J kg^-1 K^-1), L (J kg^-1) */
    double clausius_clapeyron;                               /* beta (K Pa^-1): T_pm = T_0 - beta p */
    double melting_temperature, reference_temperature;       /* T_0, T_r (K) */
} nk_thermal_params;

/* update_thermal_diagnostics! with an ArrheniusRateFactor (src/Thermodynamics/column_energy_solve.jl:85-110 and the
 * conversions of src/Thermodynamics/enthalpy_conversions.jl:1-64): on every layer k of every column, with
 * p = rho_i g H (1 - zeta_k), T_pm = T_0 - beta p and E_pm = c_i (T_pm - T_r):
 *   T = min(T_pm, T_r + E / c_i),  omega = max(0, E - E_pm) / L,  A = arrhenius_rate_factor(T - T_pm + T_0, omega).
 * Reads NK_FIELD_ENTHALPY and H; writes NK_FIELD_TEMPERATURE, NK_FIELD_WATER_FRACTION and the rate factor, which
 * must have the sigma layout.  Until an enthalpy is set the enthalpy field holds zeros. */
nk_status nk_compute_thermal_diagnostics(nk_problem* problem, const nk_thermal_params* params);

/* One ice time step of the thickness with the velocities held (replaces the three rk_substep! calls of
 * time_step!, src/Models/time_stepping.jl:15-72, with the problem's advection scheme, nk_set_thickness_advection,
 * and no PartialCellFront): Delta tau = dt/3, dt/2, dt; each stage sets H = max(0, H_start + Delta tau G(H)) with
 * G = a - (1 - phi) m - m^g - div(u H) (phi only with a grounding-line treatment, m^g only when
 * grounded_melt_coupling is non-zero), u H through each face with the scheme's upwind-biased face thickness (the
 * bounds-preserving limiter recomputed from the stage's thickness first) and nothing through a Bounded wall; the
 * last stage adds its clip max(0, -H*) to NK_FIELD_CLIPPED_THICKNESS; nk_compute_geometry runs after every
 * stage (update_state! without the velocity solve), so the surface, masks, grounded fractions, effective
 * pressure and driving stress follow the new thickness.  NK_BAD_ARGUMENT when dt is not finite and positive. */
nk_status nk_step_thickness(nk_problem* problem, double dt, int32_t grounded_melt_coupling);
/* One stage (1, 2 or 3) of nk_step_thickness: stage 1 records the step's starting thickness, which stages 2 and 3
 * start from; the three in order, with nothing between them, equal nk_step_thickness bit for bit.  The reference's
 * default velocity schedule, IterationInterval(1) (src/StressBalances/stress_balance_solver.jl:43-52), solves the
 * velocity in update_state! after every stage; a host that follows it calls stage 1, nk_picard_solve, stage 2,
 * nk_picard_solve, stage 3, nk_picard_solve, so each stage advects with the previous stage's velocities. */
nk_status nk_step_thickness_stage(nk_problem* problem, double dt, int32_t stage, int32_t grounded_melt_coupling);

/* The thickness advection scheme of nk_step_thickness, IceSheetModel's `advection` keyword
 * (src/Models/ice_sheet_model.jl:79-123):
 *   NK_ADVECTION_UPWIND, order 1 or 3   UpwindBiased(order = 1) / UpwindBiased(order = 3)
 *   NK_ADVECTION_WENO, order 5          WENO(order = 5), and with bounded = 1 WENO(order = 5, bounds = (lower, upper)),
 *                                       whose bounds-preserving limiter is recomputed before every tendency
 *                                       (update_bounds_preserving_limiter!, src/Models/time_stepping.jl:35-42).
 * A new problem starts with the reference's default for the SSA and the DIVA, WENO(order = 5, bounds = (0, 1e5))
 * (default_thickness_advection, src/Models/ice_sheet_model.jl:123).  The face value through which u H passes is the
 * upwind-biased reconstruction of H: order 1 the upwind cell; order 3 (-H₋₁ + 5 H₀ + 2 H₁) / 6; WENO-5 the
 * Jiang-Shu smoothness indicators with the WENO-Z weights (Borges et al. 2008, exponent 1, ε = 1e-8) of the three third-order
 * candidates; H₀ the upwind cell, H₋₁ the one behind it, H₁ the downwind one.  The limiter (Zhang and Shu 2010) scales
 * each cell's face values towards its mean so that they and the cell's interior quadrature value stay in
 * [lower, upper] (weights 5/18 at the faces, per direction).  NK_BAD_ARGUMENT for other schemes or orders, for
 * lower >= upper, and (at nk_step_thickness) for a bounded WENO on a grid whose smaller horizontal halo is below 4,
 * which the reference refuses (check_advection_halo, src/Models/ice_sheet_model.jl:131-135). */
#define NK_ADVECTION_UPWIND 0
#define NK_ADVECTION_WENO   1
typedef struct nk_advection_desc {
    int32_t scheme;                   /* NK_ADVECTION_UPWIND / NK_ADVECTION_WENO */
    int32_t order;                    /* 1 or 3 (upwind), 5 (WENO) */
    int32_t bounded;                  /* WENO only: 1 = bounds-preserving limiter to [lower, upper] */
    int32_t reserved;                 /* 0 */
    double lower, upper;              /* the bounds (m), lower < upper (either may be infinite) */
} nk_advection_desc;
nk_status nk_set_thickness_advection(nk_problem* problem, const nk_advection_desc* advection);

/* Calving law of a partial-cell front, src/Models/calving.jl:1-150. */
#define NK_CALVING_NONE                 0
#define NK_CALVING_THICKNESS_THRESHOLD  1   /* ThicknessThresholdCalving(thickness) */
#define NK_CALVING_EIGEN                2   /* EigenCalving(coefficient) */
#define NK_CALVING_VON_MISES            3   /* VonMisesCalving(stress_threshold, floating_stress_threshold) */
#define NK_CALVING_FRONT_VELOCITY       4   /* FrontVelocityCalving(front_velocity) */
#define NK_CALVING_MAXIMUM_EXTENT       5   /* MaximumExtentCalving(extent): NK_FIELD_CALVING_EXTENT */

/* PartialCellFront(grid; passes, calving) as the masking of a model (src/Models/partial_cell_front.jl:1-66).  With
 * `enabled`, the ice mask is the prognostic 0/1 flag of full cells: nk_compute_geometry no longer computes it from
 * H, only full cells enter the stress balance, and nk_step_thickness moves thickness only between full cells (the
 * scheme's flux), upwind from a full cell into a front cell and not out of a front cell, applies the sources to full
 * cells only, and after its last stage advances the front (advance_front!, :167-195): empties full cells that
 * drained, updates the front thickness H^r, fills front cells that reached it and spills their excess volume into
 * empty neighbours up to `passes` times, calves marine front cells under the calving law (:276-327), and applies
 * the sources of the step to the partial cells and to the cells that filled or calved.  A time-dependent front
 * velocity w(t) is set before each step with a new nk_front_desc. */
typedef struct nk_front_desc {
    int32_t enabled;                  /* 1: PartialCellFront masking; 0: the SmoothIceMask / no masking of the physics */
    int32_t passes;                   /* overflow passes per time step (the reference's default 4) */
    int32_t calving;                  /* NK_CALVING_* */
    int32_t reserved;                 /* 0 */
    double thickness;                 /* ThicknessThresholdCalving: calving below this thickness (m) */
    double coefficient;               /* EigenCalving: K (m s) */
    double stress_threshold;          /* VonMisesCalving: sigma_max of grounded ice (Pa) */
    double floating_stress_threshold; /* VonMisesCalving: sigma_max of floating ice (Pa) */
    double front_velocity;            /* FrontVelocityCalving: w (m s^-1), positive for advance */
} nk_front_desc;
nk_status nk_set_front(nk_problem* problem, const nk_front_desc* front);
/* initialize_front! (src/Models/partial_cell_front.jl:80-92), which set! calls when it sets the thickness: every cell
 * holding ice is full (mask 1, else 0) and no cell is partial (H^r = 0).  NK_BAD_ARGUMENT without a front. */
nk_status nk_initialize_front(nk_problem* problem);
/* advance_front!(front, model, dt) alone (the end of nk_step_thickness's last stage), then the geometry.
 * NK_BAD_ARGUMENT without a front or when dt is not finite and positive. */
nk_status nk_advance_front(nk_problem* problem, double dt);

/* The EnthalpyThermodynamics constants of the energy step (src/Thermodynamics/enthalpy_thermodynamics.jl:92-104,
 * defaults 2.1, 2009, 3.34e5, 7.9e-8, 273.15, 223.15, 1e-3, 1, 1e-3, 1, 0.01, 0.05 / year, coupling on). */
typedef struct nk_energy_params {
    double thermal_conductivity;          /* W m^-1 K^-1 */
    double heat_capacity, latent_heat;    /* J kg^-1 K^-1, J kg^-1 */
    double clausius_clapeyron;            /* K Pa^-1 */
    double melting_temperature, reference_temperature;   /* K */
    double temperate_diffusivity_ratio;   /* temperate / cold diffusivity */
    double enthalpy_blend_width;          /* J kg^-1 */
    double water_layer_blend_thickness;   /* m */
    double minimum_thickness;             /* m: thinner columns hold the surface enthalpy */
    double drainage_water_fraction;       /* water fraction above which temperate ice drains */
    double maximum_drainage_rate;         /* s^-1 */
    int32_t grounded_melt_coupling;       /* the thickness step reads the grounded melt (non-zero) */
    int32_t reserved;                     /* 0 */
} nk_energy_params;

#define NK_ENERGY_MAX_LAYERS 64

/* One energy step of length dt (replaces step_thermodynamics!, src/Thermodynamics/column_energy_solve.jl:26-78):
 * the strain heating of the current velocities and viscosity (strain_heating.jl:7-56), the layer volume and
 * enthalpy fluxes with first-order upwinding (layer_transport.jl:8-44), the basal state (:127-146), one implicit
 * tridiagonal system per column in the sigma direction (:148-221) solved in place, the basal water and the
 * drainage of temperate ice (:223-259), then T and omega from the new enthalpy and H^n = H.  Reads
 * NK_FIELD_ENTHALPY, H, H^n, the velocities, u_sigma / v_sigma, u_b / v_b, the basal drag and eta_sigma of the
 * last solve (nk_velocity_profile first), phi, the basal and grounded melt rates and the state fields above;
 * writes E, T, omega, H_w, the grounded melt rate, H^n and the diagnostics.  The rate factor is not updated: the
 * reference's advance_enthalpy! ends with update_thermal_diagnostics! (:85-97), so call
 * nk_compute_thermal_diagnostics after this step before the next velocity solve.  With a till (nk_set_till) the
 * basal water drains and is capped after the grounded melt rate is taken (drain_till); otherwise H_w is the water
 * balance's H+.  NK_BAD_ARGUMENT without the sigma rate-factor layout, with more than NK_ENERGY_MAX_LAYERS layers, or
 * when dt is not finite and positive. */
nk_status nk_step_enthalpy(nk_problem* problem, const nk_energy_params* params, double dt);

/* TillEffectivePressure (src/Thermodynamics/till_effective_pressure.jl), EnthalpyThermodynamics' `effective_pressure`
 * (Bueler and van Pelt 2015): with s = clamp(H_w / W_max, 0, 1) and the overburden P0 = rho_i g H,
 *   N = min(N0 (delta P0 / N0)^s 10^((e0 / Cc) (1 - s)), N_ocean),   N_ocean = max(P0 + rho_w g min(b, 0), 0),
 * with N0 / delta standing in for P0 where P0 = 0; the energy step then drains the basal water,
 * H_w = clamp(H+ - dt drainage_rate, 0, W_max).  Defaults (TillEffectivePressure(grid)): 1000 Pa, 0.02, 0.69, 0.12,
 * 2 m, 1 mm per year. */
typedef struct nk_till_desc {
    int32_t enabled;                        /* 0: the ocean-connected N and no drainage (the default) */
    int32_t reserved;                       /* 0 */
    double reference_effective_pressure;    /* N0, Pa */
    double overburden_fraction;             /* delta */
    double reference_void_ratio;            /* e0 */
    double compressibility;                 /* Cc */
    double maximum_water_thickness;         /* W_max, m */
    double drainage_rate;                   /* m s^-1 */
} nk_till_desc;
/* Set (or, enabled = 0, clear) the problem's till: nk_compute_geometry's N reads NK_FIELD_BASAL_WATER_THICKNESS
 * through it and nk_step_enthalpy drains the basal water.  NK_BAD_ARGUMENT for parameters that are not positive and
 * finite (the drainage rate may be 0). */
nk_status nk_set_till(nk_problem* problem, const nk_till_desc* till);

/* update_stress_balance_coefficients!(x, ...) (SSA) or update_diva_coefficients!(x, ...) (DIVA) at the
 * current velocity fields U, V: eta_sigma, eta_H, F2, eta_H_ff, beta (and beta_b, u_b, v_b for DIVA). */
nk_status nk_update_coefficients(nk_problem* problem);

/* ssa_operator!(q, p, eta_H, eta_H_ff, beta_u, beta_v, walls) with the problem's coefficients.
 * p and q are host arrays in interior layout (u part then v part sizes as above); q is fully written
 * on the Nx x Ny range, its other entries are left as passed. */
nk_status nk_apply_operator(nk_problem* problem, const double* pu, const double* pv, double* qu, double* qv);

/* precondition!(z, P, r, coefficients...) with the configured preconditioner (multigrid coarse
 * coefficients are rebuilt from the current coefficients first, as update_preconditioner! does). */
nk_status nk_precondition(nk_problem* problem, const double* ru, const double* rv, double* zu, double* zv);

/* solve!(x, linear_solver, b, coefficients...) from the warm start in the U, V fields; b host arrays. */
nk_status nk_linear_solve(nk_problem* problem, const double* bu, const double* bv, nk_solve_stats* stats);
/* adjoint_solve!(lambda, solver, b, ...): the operator is self-adjoint, so the same solve. */
nk_status nk_adjoint_solve(nk_problem* problem, const double* bu, const double* bv, nk_solve_stats* stats);

/* picard_solve!(x, picard, linear_solver, update_coefficients!, tau, coefficients...) on device-resident
 * fields: x = (U, V) warm start, b = (TAU_U, TAU_V).  Updates U, V and every coefficient field. */
nk_status nk_picard_solve(nk_problem* problem, nk_solve_stats* stats);

/* Fixed-point adjoint of a converged picard_solve! (the Enzyme reverse rule of ext/NunatakEnzymeExt.jl:167-240,
 * Christianson 1994) for the SSA and DIVA with Weertman or regularised-Coulomb friction.  x* = (U, V) is the problem's
 * converged velocity and x̄ = (ubar, vbar) = ∂J/∂x* in the interior layout of U, V.  The coefficients are
 * refreshed to c(x*), then λ ← A⁻¹ (x̄ - (∂[A(c(x)) x*]/∂x)ᵀ λ) is iterated from λ = 0, each step one
 * preconditioned CG solve of the problem's linear control warm-started from λ, until
 * ‖λ⁺ - λ‖ ≤ max(reltol ‖λ⁺‖, abstol) (control; NULL = the problem's Picard control).  Returns λ = ∂J/∂τ
 * (lambda_u, lambda_v, same layout as U, V), ∂J/∂log C per cell (grad_log_C, Nx x Ny) and ∂J/∂log A in the
 * layout of RATE_FACTOR (grad_log_A: Nx x Ny, or Nσ planes of them for a σ-grid rate factor); any output may be
 * NULL.  stats: picard_iterations = adjoint iterations, picard_change = ‖λ⁺ - λ‖, picard_norm = ‖λ‖,
 * status NK_NOT_CONVERGED when maxiter ended it.  U, V are left at x*.  DIVA: the step also reads its own
 * previous beta_b, F2 and eta_sigma (diva.jl:77-80), whose adjoint is swept along with lambda; the stopping test
 * watches lambda only, as the reference's does, and the lagged-state adjoint settles more slowly, so ask for a
 * tighter reltol than for the SSA.  Problems with prescribed velocities are refused (NK_BAD_ARGUMENT).  The adjoint is
 * that of the fixed point whatever stopped the forward solve: a solve that FixedIterations stopped before converging
 * is differentiated as if converged, where the reference's Enzyme, whose rule covers Convergence alone
 * (ext/NunatakEnzymeExt.jl:121), unrolls its iterations. */
nk_status nk_picard_adjoint(nk_problem* problem, const double* ubar, const double* vbar, const nk_iteration_control* control,
                            double* lambda_u, double* lambda_v, double* grad_log_C, double* grad_log_A, nk_solve_stats* stats);
/* nk_picard_adjoint plus, in grad_H (Nx x Ny, or NULL), the thickness gradient ∂J/∂H: the total derivative
 * of J(x*(H)) when H enters the way update_velocities! uses it (src/Models/ice_sheet_model_methods.jl:103-131):
 * through the geometry of update_geometry! (s, the face grounded fractions, N and the ice mask of nk_compute_geometry),
 * the driving stress of compute_driving_stress! (interior slope, calving-front force, grounding-line split), and
 * η̄H = μ H ∫η dζ and the grounded-fraction and effective-pressure factors of the drag in the coefficient update.
 * The reverse rule of picard_solve! returns the coefficient part of this as the shadow of its H argument
 * (ext/NunatakEnzymeExt.jl:226-231) and Enzyme adds the geometry and driving-stress parts through update_state!;
 * here they come in one gradient.  The discrete switches (walls, fronts and ice-free faces, the grounded or floating
 * branch of s, the clamps of the mask and of N) are held where they are: the gradient is that of the smooth piece
 * containing H.  A partial-cell front's mask is its prognostic flag and carries no H derivative.  For the DIVA H
 * also enters F2 = H ∫(1-ζ)²/η dζ, whose adjoint the DIVA sweep carries, and the drag is the basal βᵇ on |uᵇ|. */
nk_status nk_picard_adjoint_gradients(nk_problem* problem, const double* ubar, const double* vbar, const nk_iteration_control* control,
                                      double* lambda_u, double* lambda_v, double* grad_log_C, double* grad_log_A, double* grad_H,
                                      nk_solve_stats* stats);

/* ---- the gradient through time steps (checkpointed_gradient!, ext/NunatakEnzymeExt.jl:245-263) ------------------
 * The cost J = Σₙ Jₙ of the states after steps n = 1..steps of time_step!: each step the three split Runge-Kutta
 * stages of nk_step_thickness_stage with the problem's advection, each followed, with velocity_solves, by a Picard
 * solve (the reference's IterationInterval(1) velocity schedule), else with the velocities held.  The host gives Jₙ
 * and its gradient in a callback; the library returns J and its gradient with respect to the thickness and the
 * velocities at the start, the surface mass balance, the basal melt rate, and, with velocity solves, log C and log A.
 *
 * The forward run stores the state (H, U, V, a front's flag and H_r, and for the DIVA its lagged beta_b, F2 and
 * eta_sigma) every checkpoint_interval steps; the reverse pass restores each checkpoint, re-runs its segment storing
 * every stage's state, and runs the segment backwards: the cost's gradient at each step end, the fixed-point Picard adjoint of each velocity solve
 * (nk_picard_adjoint_gradients: λ of the velocities to ∂J/∂H, log C, log A) and the reverse of each stage (the clip,
 * the sources, the fluxes, the bounds-preserving limiter, the WENO or upwind reconstructions and the centre grounded
 * fraction of the floating melt; nk_time_adjoint.cu).  Only one segment's stages are held at a time.  The problem is
 * left at the final state, as checkpointed_gradient! leaves the model.
 *
 * The initial velocities are an input, as the model's stored velocities are for the reference (their gradient is
 * the shadow of the velocity fields); the geometry is recomputed from the initial H.  Discrete switches (the clip, the
 * upwind direction, the limiter's branch, walls, masks and the front's flags) are held where the forward run put them;
 * a partial-cell front's advance (its overflow passes and its calving included) is reversed with the stages.  Von Mises
 * rates read the viscosity η̄H of the solve before the front: its adjoint joins that solve's Picard adjoint, as the
 * shadow of an overwritten coefficient; with the velocities held η̄H is held too.  Not covered: the energy step and
 * its grounded-melt coupling (the stages run uncoupled), and prescribed velocities with velocity solves (refused, as
 * for nk_picard_adjoint). */
typedef struct nk_cost_state {
    int32_t step;              /* the state after this many steps, 1..steps */
    int32_t steps;
    const double* H;           /* Nx x Ny, interior layout (host) */
    const double* u;           /* the interior layouts of U, V (host) */
    const double* v;
    const double* ice_mask;    /* Nx x Ny */
} nk_cost_state;
/* Jₙ into *J and ∂Jₙ/∂(H, U, V) into the arrays (zeroed before the call; the layouts of the state's arrays).
 * Return 0; anything else stops the gradient with NK_BAD_ARGUMENT.  The library calls it once per step during the
 * reverse pass, the last step first, from the calling thread. */
typedef int32_t (*nk_cost_fn)(void* user, const nk_cost_state* state, double* J, double* dJ_dH, double* dJ_du, double* dJ_dv);

typedef struct nk_time_gradient_desc {
    double dt;
    int32_t steps;
    int32_t checkpoint_interval;            /* steps per segment; 0: ceil(sqrt(steps)) */
    int32_t velocity_solves;                /* 1: a Picard solve after every stage; 0: the velocities held */
    int32_t reserved;
    const double* melt_weights;             /* steps factors wₙ: step n melts wₙ m; NULL: all 1 */
    const nk_iteration_control* adjoint_control;   /* the Picard adjoints' control; NULL: the problem's Picard control */
} nk_time_gradient_desc;

/* Outputs, each Nx x Ny in interior layout unless noted; any may be NULL. */
typedef struct nk_time_gradient {
    double* grad_H;            /* ∂J/∂H at the start (the initial velocities held) */
    double* grad_u;            /* ∂J/∂(U, V) of the initial velocities (the interior layouts of U, V) */
    double* grad_v;
    double* grad_smb;          /* ∂J/∂a */
    double* grad_melt;         /* ∂J/∂m of the base melt rate the weights scale */
    double* grad_log_C;        /* ∂J/∂log C (velocity solves) */
    double* grad_log_A;        /* ∂J/∂log A in the layout of RATE_FACTOR (velocity solves) */
} nk_time_gradient;

typedef struct nk_time_gradient_stats {
    double J;                  /* Σₙ Jₙ */
    int32_t segments;          /* checkpoints stored */
    int32_t picard_solves;     /* forward and re-run */
    int32_t picard_adjoints;
    int32_t adjoint_iterations;     /* Picard adjoint iterations, all solves */
    int32_t worst_solve_status;     /* the worst nk_status of the Picard solves and adjoints (NK_NOT_CONVERGED kept) */
    int32_t reserved;
    double elapsed_ms;         /* wall time of the call */
} nk_time_gradient_stats;

/* Device memory: the checkpoints and one segment's stage states, (⌈steps / K⌉ + 3K + 2) states of 3 planes (DIVA:
 * 6 + Nσ; a front: 2 more, 3 with von Mises calving) plus about 25 planes of adjoints, allocated for the call and freed
 * before it returns.
 * After an error the problem's fields are those of whichever step the sweep had reached. */
nk_status nk_checkpointed_gradient(nk_problem* problem, const nk_time_gradient_desc* desc, nk_cost_fn cost, void* user,
                                   const nk_time_gradient* out, nk_time_gradient_stats* stats);

/* picard_solve! enqueued on the problem's stream without waiting (one CUDA-graph launch); independent problems
 * solved this way run concurrently on the device.  nk_problem_wait blocks until it has finished and returns its
 * statistics (the status of the solve is the return value, as for nk_picard_solve). */
nk_status nk_picard_solve_async(nk_problem* problem);
nk_status nk_problem_wait(nk_problem* problem, nk_solve_stats* stats);
/* Without blocking: *done = 1 when the pending asynchronous solve has finished (nk_problem_wait then returns at
 * once), 0 while it runs. */
nk_status nk_problem_query(nk_problem* problem, int32_t* done);

/* ---- batched solves --------------------------------------------------------------------------------------
 *
 * No counterpart in the reference, which solves one grid per picard_solve!.  A batch holds `slots` problems of one
 * configuration (the same grid, physics and solver descriptors), their device state in one allocation at a fixed
 * stride, and solves the slots chosen per call with one CUDA graph: every kernel launch of that graph covers all
 * slots (one z block row per slot), and the Picard and conjugate-gradient loops run until the last chosen slot
 * has stopped, a slot that has stopped leaving every later launch at once.  Each slot's arithmetic, and so its
 * result, is that of the same problem solved alone by nk_picard_solve.  For many small solves the GPU is limited
 * by how fast the host and the graph engine can issue launches, not by the work in them; a batch of S slots
 * issues the launches of its slowest slot once instead of S times.
 *
 * nk_batch_problem gives slot k's problem: set its fields, compute its geometry and read its results with the
 * nk_problem calls, as for any problem.  All slots share the batch's stream, so those calls and the batched
 * solve are ordered.  The slots' problems are owned by the batch (do not destroy them) and also solve alone.
 * Refused (NK_BAD_ARGUMENT): NK_SOLVER_HOST_LOOP, process-wide NK_GRAPHS=0, fused coarse multigrid levels
 * (NK_COARSE_CELLS > 0 with the mixed solver), and a batched solve of a slot with prescribed velocities. */
typedef struct nk_batch nk_batch;
#define NK_MAX_BATCH_SLOTS 1024
nk_status   nk_batch_create(nk_context* ctx, const nk_grid_desc* grid, const nk_physics_desc* physics,
                            const nk_solver_desc* solver, int32_t slots, nk_batch** out);
nk_status   nk_batch_destroy(nk_batch* batch);
int32_t     nk_batch_slots(const nk_batch* batch);
nk_problem* nk_batch_problem(nk_batch* batch, int32_t slot);   /* NULL when slot is out of range */
/* picard_solve! of the slots whose active[k] != 0 (every slot when active is NULL), enqueued on the batch's
 * stream without waiting.  nk_batch_wait blocks until it has finished and writes `slots` statistics (zeros for the
 * slots not solved); it returns NK_NONFINITE when a solved slot has, and NK_OK otherwise (read each slot's
 * status).  nk_batch_query: *done = 1 once finished, without blocking. */
nk_status   nk_batch_picard_solve_async(nk_batch* batch, const uint8_t* active);
nk_status   nk_batch_query(nk_batch* batch, int32_t* done);
nk_status   nk_batch_wait(nk_batch* batch, nk_solve_stats* stats);

/* The whole update_velocities! body for host callers: copies u, v (warm start) in, runs
 * nk_picard_solve and copies u, v out.  u, v in interior layout. */
nk_status nk_solve_velocities(nk_problem* problem, double* u, double* v, nk_solve_stats* stats);

/* DIVA: compute_velocity_profile! (src/StressBalances/diva.jl:89-109); SSA: extend_depth_average!
 * (src/Models/ice_sheet_model_methods.jl:167-180).  Fills U_B, V_B, U_SIGMA, V_SIGMA. */
nk_status nk_velocity_profile(nk_problem* problem);

/* Number of multigrid levels below the finest and the size of each (multigrid_preconditioner.jl:86-120). */
nk_status nk_multigrid_levels(const nk_problem* problem, int32_t* count, int32_t* nx, int32_t* ny, int32_t capacity);

/* Multigrid transfers between level `level` - 1 (the finest grid for level 0) and coarse level `level`,
 * with masks from the coarse coefficients rebuilt from the current ones (coarsen_coefficients!):
 *   restrict!(coarse, fine, ...)      coarse = R fine    multigrid_preconditioner.jl:182-186, :346-352
 *   prolongate!(fine, coarse, ...)    fine  += P coarse  multigrid_preconditioner.jl:188-192, :354-360
 * Vectors in interior layout of their grids (u part, v part). */
nk_status nk_multigrid_restrict(nk_problem* problem, int32_t level, const double* fine_u, const double* fine_v,
                                double* coarse_u, double* coarse_v);
nk_status nk_multigrid_prolongate(nk_problem* problem, int32_t level, const double* coarse_u, const double* coarse_v,
                                  double* fine_u, double* fine_v);

/* ---- velocity change without device allocation ---------------------------------------------------------
 *
 * No counterpart in the reference.  For callers that cannot let the library allocate device memory while
 * they run: a model whose host framework pools the whole device (a CUDA.jl or PyTorch caching allocator),
 * where an extra cudaMalloc fails and a cudaFree stalls the device, or a coupled time loop that must not
 * synchronise.  Computes the two Euclidean norms that a velocity-change stopping test compares,
 *   change_and_norm[0] = ||(u, v) - (u_prev, v_prev)||,   change_and_norm[1] = ||(u, v)||
 * over the cells of the grid (u at the west and v at the south face of each cell), with the same reduction
 * and summation order as the picard_change and picard_norm of nk_picard_solve.  u, v, u_prev, v_prev and
 * change_and_norm are DEVICE pointers: u, v in the interior layout of nk_problem_get_field (u rows of Nx + 1
 * faces when x is Bounded, Nx when Periodic; v rows of Nx), change_and_norm two doubles.  Enqueued on
 * `stream` (a cudaStream_t; NULL = the legacy default stream) without waiting; the result is there when the
 * stream reaches it.
 *
 * Scratch lives in a fixed __device__ array of 262,400 bytes that every GPU loading the library holds until
 * exit: one partial per 32 x 8 block of cells, at most NK_NOALLOC_MAX_BLOCKS, so ceil(Nx / 32) * ceil(Ny / 8)
 * must not exceed it (2048 x 2048 cells fit); larger grids return NK_BAD_ARGUMENT with the sizes in
 * nk_last_error.  The first call on a device looks the array's address up (cudaGetSymbolAddress): make that
 * first call before any stream capture.  Every call on a device shares the one array, and each clears the
 * block counter on its stream before its kernel: calls whose work overlaps on the GPU (other streams or
 * threads without ordering between them) race and give wrong results.  Nothing is allocated or freed. */
#define NK_NOALLOC_MAX_BLOCKS 16384
nk_status nk_picard_change_noalloc(nk_context* ctx, const nk_grid_desc* grid, const double* u, const double* v,
                                   const double* u_prev, const double* v_prev, double* change_and_norm,
                                   void* stream);

/* ---- serving -------------------------------------------------------------------------------------------
 *
 * A request loop for many independent velocity solves (ensemble members, inversion line-search trials,
 * requests of different grid sizes).  It has no counterpart in the reference, whose model solves one grid
 * per update_state! (src/Models/ice_sheet_model_methods.jl:80-101); each request is the reference's
 * set!(model; H) velocity solve (geometry, driving stress, picard_solve!) on its own inputs.
 *
 * The server keeps solved problems resident in HBM and reuses a resident problem for a later request with
 * the same grid, physics and solver (only the input fields change), so each problem's device buffers,
 * multigrid hierarchy and captured CUDA graph are built once.  Up to max_in_flight requests run at once, each
 * on its own stream, so requests that arrive while others are on the GPU are admitted as soon as a slot and
 * memory are free and their kernels overlap on the device.  The server reserves memory_cap_bytes of HBM (one
 * cudaMalloc) and a pinned host staging pool of a thirty-second of it (at least 64 MiB) when it is created, and
 * carves every resident problem out of them: admission by footprint, and no allocation call (which can wait on
 * running work) while requests are on the device.  When a new problem does not fit, idle problems of other
 * shapes are evicted, least recently used first.  Results do not depend on the mix: every request's arithmetic
 * is that of a solve alone. */
typedef struct nk_server_desc {
    int32_t max_in_flight;          /* requests on the device at once (>= 1) */
    int32_t flags;                  /* NK_SERVER_ADMISSION_THREAD or 0 */
    int64_t memory_cap_bytes;       /* device memory reserved for the resident problems */
    int32_t batch_slots;            /* > 1: requests of one shape are solved together, up to batch_slots per solve, by a
                                     * resident nk_batch (one launch per kernel for all of them); 0 or 1: one request per
                                     * solve.  max_in_flight still counts requests. */
    int32_t reserved;               /* 0 */
} nk_server_desc;
/* The server runs its own host thread that retires finished requests and admits queued ones as soon as a slot
 * frees, without the caller driving nk_server_progress / nk_server_wait; the calls below are then thread-safe
 * and wait on it.  Without the flag the caller's calls drive the loop (one host thread). */
#define NK_SERVER_ADMISSION_THREAD 1

typedef struct nk_request {
    nk_grid_desc grid;              /* face / sigma vectors, if any, are read during nk_server_submit */
    nk_physics_desc physics;
    nk_solver_desc solver;
    const double* H;                /* interior layout, Nx * Ny */
    const double* bed;              /* Nx * Ny */
    const double* friction_coefficient;   /* Nx * Ny, or NULL without friction */
    const double* rate_factor;      /* Nx * Ny (NK_RATE_FACTOR_2D) */
    const double* u_init;           /* warm start, or NULL for zero */
    const double* v_init;
    double* u_out;                  /* written when the request completes */
    double* v_out;
} nk_request;

nk_status nk_server_create(nk_context* ctx, const nk_server_desc* desc, nk_server** out);
nk_status nk_server_destroy(nk_server* server);
/* Queue a request; its inputs are copied before the call returns.  *ticket identifies it. */
nk_status nk_server_submit(nk_server* server, const nk_request* request, int64_t* ticket);
/* Retire finished requests and admit queued ones; never blocks.  *pending = requests not yet finished. */
nk_status nk_server_progress(nk_server* server, int32_t* pending);
/* Block until request `ticket` has finished (driving the loop meanwhile); its statistics and host
 * timestamps in seconds on the server's clock: submitted, admitted (launched), finished (seen complete). */
nk_status nk_server_wait(nk_server* server, int64_t ticket, nk_solve_stats* stats, double* t_submit, double* t_admit,
                         double* t_done);
/* Block until every submitted request has finished. */
nk_status nk_server_wait_all(nk_server* server);
/* Seconds on the server's clock (the clock of the timestamps above). */
double nk_server_clock(const nk_server* server);
/* Resident problems, their device bytes, and the largest number of requests that were on the device at once. */
nk_status nk_server_info(const nk_server* server, int32_t* resident, int64_t* device_bytes, int32_t* peak_in_flight);

/* ---- measurement ----------------------------------------------------------------------------------------- */

/* Kernels that nk_time_kernel can time. */
#define NK_KERNEL_OPERATOR_FP64   0   /* q = A p on the fine grid (FP64), the apply of every CG step */
#define NK_KERNEL_SMOOTHER        1   /* one fine-level ℓ1-Jacobi sweep x' = x + (b - A x) / rowsum, in the
                                         multigrid precision (FP32 when mixed, FP64 otherwise) */
#define NK_KERNEL_CG_UPDATE       2   /* x += alpha p, r -= alpha q with the fused r.r (and r.z) reductions */
#define NK_KERNEL_THICKNESS_STAGE 3   /* one Runge-Kutta stage of nk_step_thickness with the problem's advection scheme
                                         (the WENO face reconstructions and the bounded WENO's limiter launched once
                                         before the timed launches) */
#define NK_KERNEL_THICKNESS_LIMITER 4 /* the bounded WENO's limiter from the current thickness */
#define NK_KERNEL_STEP_ENTHALPY   5   /* the column energy step of nk_step_enthalpy with EnthalpyThermodynamics' defaults
                                         (needs the sigma rate-factor layout) */
#define NK_KERNEL_THICKNESS_FACES 6   /* the WENO schemes' two reconstructions of every face, once per stage */

/* Instrumentation (no counterpart in the reference, which times whole solves with @elapsed,
 * benchmarks/multigrid_scaling.jl:36-47): launches one hot kernel `repeats` times on the problem's
 * current state and stream, each launch bracketed by CUDA events; when flush_bytes > 0 a device buffer of
 * that size is overwritten before every launch so the launch starts with a cold L2.  Returns the mean
 * launch duration and the algorithmic bytes of one launch (every array it reads or writes counted once).
 * Leaves the solver state changed; call it after a solve, not inside one. */
nk_status nk_time_kernel(nk_problem* problem, int32_t kernel, int32_t repeats, int64_t flush_bytes,
                         double* mean_ms, double* bytes_per_launch);

/* Instrumentation (no counterpart in the reference): number of CUDA kernels this library has launched in
 * the process so far. */
int64_t nk_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* NUNATAK_GB300_H */
