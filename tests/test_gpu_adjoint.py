"""The fixed-point Picard adjoint (nk_picard_adjoint; the reverse rule of ext/NunatakEnzymeExt.jl:167-240) against
centred finite differences, following the checks of test/test_enzyme.jl:221-381.

J = ½ Σ (u - u_obs)² + (v - v_obs)² over the velocity points of a marine sheet, with u_obs from a solve with
another friction seed.  The gradients from the adjoint must match centred differences of converged solves
(Picard 1e-14, CG 1e-15):
- ∂J/∂log C at seeded grounded cells, (J(C e^ε) - J(C e^-ε)) / 2ε, on the GPU forward solve for three
  configurations (bounded / periodic x, free-slip / no-slip walls, Weertman / regularised Coulomb friction);
- ∂J/∂log A along seeded random directions d over the whole field, (J(A e^(εd)) - J(A e^(-εd))) / 2ε against
  ⟨∂J/∂log A, d⟩ (one cell's A moves J too little to be resolved against the solver tolerances), for the same
  three configurations and for a σ-grid rate factor;
- on the oracle's forward solve at one cell;
- for DIVA (Arrhenius σ-grid rate factor, regularised Coulomb friction), whose step also carries its lagged
  βᵇ, F₂ and ησ: log C and log A along random directions on the GPU forward map, log C on the oracle's.
Tolerance: 1e-4 relative to the cell's own gradient (per cell, at cells whose gradient is at least 1e-3 of the
largest entry) or to Σ|gᵢdᵢ| (directions).  The step ε is 1e-3 (1e-4 for log A, whose second derivative along d is
large against the misfit of these cases).  A per-cell difference is taken as ½ Σ (x₊ - x₋)(x₊ + x₋ - 2 x_obs) from
the two perturbed solves, not as the difference of two costs."""
import math

import numpy as np
import pytest

import nunatak_gb300 as nk
from nunatak_gb300 import model as M, workloads

pytestmark = pytest.mark.gpu

EPS = 1e-3
RTOL = 1e-4


def _solver():
    """Converged to Picard 1e-14 and CG 1e-15 (at most 5000 CG iterations per solve): a per-cell difference resolves
    1e-4 of a cell's gradient only when the perturbed solves leave less noise than that."""
    return M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-15, maxiter=5000),
                                 picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=2000),
                                 preconditioner=M.StressBalanceDiagonalPreconditioner())


def _case(kind, seed_friction, nx=40, ny=20):
    base = workloads.marine_sheet(nx, ny, seed=2, seed_friction=seed_friction, velocity_solver=_solver())
    cfg = dict(base.config)
    grid = base.grid
    if kind == "periodic_x":
        grid = M.RectilinearGrid(size=(nx, ny), x=(0.0, 512e3), y=(0.0, 256e3), halo=(4, 4), topology=("Periodic", "Bounded"))
    if kind in ("no_slip_coulomb", "till_coulomb"):
        if kind == "no_slip_coulomb":
            cfg["stress_balance"] = M.DepthIntegrated(side_walls=M.NoSlipWalls())
        cfg["friction"] = M.RegularizedCoulombFriction(coefficient=None, coulomb_coefficient=0.5, exponent=1.0 / 3.0)
    return workloads.Case(f"marine_sheet_{kind}", grid, cfg, base.fields)


def _cost(P, uo, vo):
    u, v = P.get("u"), P.get("v")
    return 0.5 * (np.sum((u - uo) ** 2) + np.sum((v - vo) ** 2)), u - uo, v - vo


def _cost_difference(plus, minus, uo, vo):
    """J(+) - J(-) as ½ Σ (x₊ - x₋)(x₊ + x₋ - 2 x_obs), without forming either cost: subtracting two rounded sums
    of the whole field would bury the small differences of weakly sensitive cells."""
    (up, vp), (um, vm) = plus, minus
    return 0.5 * (float(np.sum((up - um) * (up + um - 2 * uo))) + float(np.sum((vp - vm) * (vp + vm - 2 * vo))))


def _fd(P, case, cell, xs, uo, vo, name="C"):
    """Centred difference of J in log `name` at `cell` (an index of that field) from converged solves warm-started
    at x*."""
    vel = []
    for s in (1.0, -1.0):
        p = case.fields[name].copy()
        p[cell] *= math.exp(s * EPS)
        P.set(name, p)
        P.set("u", xs[0])
        P.set("v", xs[1])
        P.picard_solve()
        vel.append((P.get("u"), P.get("v")))
    P.set(name, case.fields[name])
    return _cost_difference(vel[0], vel[1], uo, vo) / (2 * EPS)


def _cells(grad, n, seed, floor=1e-3):
    """n seeded cells among those whose gradient is at least `floor` of the largest entry: each is checked against
    its own value, and a centred difference cannot resolve cells far below that."""
    cand = np.argwhere(np.abs(grad) >= floor * np.max(np.abs(grad)))
    rng = np.random.default_rng(seed)
    return [tuple(cand[k]) for k in rng.choice(len(cand), size=min(n, len(cand)), replace=False)]


def _with_till(P, kind):
    """till_coulomb: the effective pressure of a till holding 1.8 m of water (s = 0.9; below the ocean-connected value
    on the grounded ice, where it scales as P₀^s)."""
    if kind == "till_coulomb":
        P.set_till(M.TillEffectivePressure())
        P.energy_set("Hw", 1.8)
        P.compute_geometry()
    return P


def _adjoint(cls, kind):
    case = _case(kind, 1100)
    obs = _with_till(_case(kind, 1200).problem(cls), kind)
    obs.picard_solve()
    uo, vo = obs.get("u"), obs.get("v")
    P = _with_till(case.problem(cls), kind)
    P.picard_solve()
    J0, ub, vb = _cost(P, uo, vo)
    return case, P, uo, vo, ub, vb


@pytest.mark.parametrize("kind", ["bounded", "periodic_x", "no_slip_coulomb"])
def test_picard_adjoint_matches_finite_differences(gpu_cls, kind):
    case, P, uo, vo, ub, vb = _adjoint(gpu_cls, kind)
    xs = (P.get("u"), P.get("v"))
    lu, lv, grad, grad_a, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500))
    assert st.status == 0 and st.picard_iterations > 1
    assert np.array_equal(P.get("u"), xs[0])              # the forward state is left at x*
    scale, scale_a = np.max(np.abs(grad)), np.max(np.abs(grad_a))
    assert scale > 0 and scale_a > 0
    for cell in _cells(grad, 6, 7):
        fd = _fd(P, case, cell, xs, uo, vo)
        assert abs(fd - grad[cell]) <= RTOL * abs(grad[cell]), (kind, cell, fd, grad[cell], scale)
    A0 = P.get("A")
    d = np.random.default_rng(31).standard_normal(A0.shape)
    fd = _directional_fd(P, "A", A0, d, xs, uo, vo, eps=1e-6)
    ad = float(np.sum(grad_a * d))
    assert abs(fd - ad) <= RTOL * np.sum(np.abs(grad_a * d)), (kind, "A", fd, ad)


def test_picard_adjoint_rate_factor_on_the_sigma_grid(gpu_cls):
    """∂J/∂log A for a σ-grid rate factor: one layer of one cell against a centred difference."""
    base = _case("bounded", 1100)
    cfg = dict(base.config)
    cfg["rheology"] = M.GlenFlowLaw(rate_factor="sigma", strain_rate_regularization=1e-13)
    A2 = base.fields["A"]
    ns = cfg["Nsigma"]
    fields = dict(base.fields)
    fields["A"] = np.stack([A2 * (1.0 + 0.5 * k / ns) for k in range(ns)])
    case = workloads.Case("marine_sheet_sigma_A", base.grid, cfg, fields)
    obs = workloads.Case("obs", base.grid, cfg, dict(_case("bounded", 1200).fields, A=fields["A"])).problem(gpu_cls)
    obs.picard_solve()
    uo, vo = obs.get("u"), obs.get("v")
    P = case.problem(gpu_cls)
    P.picard_solve()
    _, ub, vb = _cost(P, uo, vo)
    xs = (P.get("u"), P.get("v"))
    _, _, _, grad_a, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500))
    assert st.status == 0 and grad_a.shape == (ns,) + A2.shape
    rng = np.random.default_rng(37)
    for layer in (None, 1, ns - 2):   # every layer at once, then single layers
        d = rng.standard_normal(grad_a.shape)
        if layer is not None:
            d[np.arange(ns) != layer] = 0.0
        fd = _directional_fd(P, "A", fields["A"], d, xs, uo, vo, eps=1e-4)
        ad = float(np.sum(grad_a * d))
        assert abs(fd - ad) <= RTOL * np.sum(np.abs(grad_a * d)), (layer, fd, ad)


def test_picard_adjoint_matches_oracle_finite_difference(gpu_cls, oracle_cls):
    """The adjoint gradient of the GPU library against a centred difference of the oracle's forward solve."""
    case, P, uo, vo, ub, vb = _adjoint(gpu_cls, "bounded")
    _, _, grad, _, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500))
    assert st.status == 0
    O = case.problem(oracle_cls)
    O.picard_solve()
    xs = (O.get("u"), O.get("v"))
    for cell in _cells(grad, 2, 11):
        fd = _fd(O, case, cell, xs, uo, vo)
        assert abs(fd - grad[cell]) <= RTOL * abs(grad[cell]), (cell, fd, grad[cell])


def _diva(friction, obs=False):
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-13, maxiter=1000),
                                   preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4))
    case = workloads.diva_sheet(48, 24, dx=32e3, velocity_solver=solver, Nsigma=6)
    cfg = dict(case.config)
    if friction == "weertman":
        cfg["friction"] = M.WeertmanFriction(coefficient=None, exponent=1.0 / 3.0)
    fields = dict(case.fields)
    if obs:   # other friction and a thinner sheet, so that the misfit dominates J's second-order terms
        fields["C"] = fields["C"] * np.exp(0.3 * np.random.default_rng(5).standard_normal(fields["C"].shape))
        fields["H"] = 0.97 * fields["H"]
    return workloads.Case(f"diva_{friction}", case.grid, cfg, fields, temperature=case.temperature)


def _directional_fd(P, name, p0, d, xs, uo, vo, eps=EPS):
    """(J(p e^(εd)) - J(p e^(-εd))) / 2ε: the derivative of J along the log-space direction d, from converged solves
    warm-started at x*."""
    J = []
    for sgn in (1.0, -1.0):
        P.set(name, p0 * np.exp(sgn * eps * d))
        P.set("u", xs[0])
        P.set("v", xs[1])
        assert P.picard_solve().status == 0
        J.append(_cost(P, uo, vo)[0])
    P.set(name, p0)
    return (J[0] - J[1]) / (2 * eps)


def _diva_setup(cls, friction):
    obs = _diva(friction, obs=True).problem(cls)
    assert obs.picard_solve().status == 0
    uo, vo = obs.get("u"), obs.get("v")
    case = _diva(friction)
    P = case.problem(cls)
    assert P.picard_solve().status == 0
    return case, P, uo, vo


# The DIVA adjoint's stopping test watches λ (as the reference's does); the lagged-state adjoint σ settles more
# slowly, so these checks iterate to 1e-14.
DIVA_ADJOINT = M.Convergence(reltol=1e-14, maxiter=3000)


@pytest.mark.parametrize("friction", ["weertman", "coulomb"])
def test_picard_adjoint_diva_matches_finite_differences(gpu_cls, friction):
    """DIVA: ⟨∂J/∂log C, d⟩ and ⟨∂J/∂log A, d⟩ against directional differences along seeded random directions.
    The Coulomb cap (τᵇ ≤ α²N) leaves J nearly insensitive to C, so there the C difference takes ε = 1e-2 and is
    resolved to 1e-3 only."""
    case, P, uo, vo = _diva_setup(gpu_cls, friction)
    _, ub, vb = _cost(P, uo, vo)
    xs = (P.get("u"), P.get("v"))
    C0, A0 = P.get("C"), P.get("A")
    lu, lv, grad, grad_a, st = P.picard_adjoint(ub, vb, DIVA_ADJOINT)
    assert st.status == 0 and st.picard_iterations > 1
    assert grad_a.shape == A0.shape
    rng = np.random.default_rng(17)
    checks = (("C", C0, grad, 1e-2 if friction == "coulomb" else EPS, 1e-3 if friction == "coulomb" else RTOL),
              ("A", A0, grad_a, 1e-4, RTOL))
    for name, p0, g, eps, tol in checks:
        d = rng.standard_normal(p0.shape)
        fd = _directional_fd(P, name, p0, d, xs, uo, vo, eps=eps)
        ad = float(np.sum(g * d))
        assert abs(fd - ad) <= tol * np.sum(np.abs(g * d)), (name, fd, ad)


def test_picard_adjoint_diva_matches_oracle_finite_difference(gpu_cls, oracle_cls):
    """The GPU DIVA adjoint against a directional difference of the oracle's forward solves (Weertman drag)."""
    case, P, uo, vo = _diva_setup(gpu_cls, "weertman")
    _, ub, vb = _cost(P, uo, vo)
    _, _, grad, _, st = P.picard_adjoint(ub, vb, DIVA_ADJOINT)
    assert st.status == 0
    O = case.problem(oracle_cls)
    assert O.picard_solve().status == 0
    xs = (O.get("u"), O.get("v"))
    d = np.random.default_rng(23).standard_normal(grad.shape)
    fd = _directional_fd(O, "C", O.get("C"), d, xs, uo, vo)
    ad = float(np.sum(grad * d))
    assert abs(fd - ad) <= RTOL * np.sum(np.abs(grad * d)), (fd, ad)


# ---- ∂J/∂H (nk_picard_adjoint_gradients) -----------------------------------------------------------------------------
def _fd_thickness(P, case, cell, xs, uo, vo, delta):
    """Centred difference of J in H at `cell`, the geometry and the driving stress recomputed from the perturbed H
    (nk_compute_geometry), from converged solves warm-started at x*."""
    vel = []
    for sgn in (1.0, -1.0):
        H = case.fields["H"].copy()
        H[cell] += sgn * delta
        P.set("H", H)
        P.compute_geometry()
        P.set("u", xs[0])
        P.set("v", xs[1])
        assert P.picard_solve().status == 0
        vel.append((P.get("u"), P.get("v")))
    P.set("H", case.fields["H"])
    P.compute_geometry()
    return _cost_difference(vel[0], vel[1], uo, vo) / (2 * delta)


def _fd_thickness_extrapolated(P, case, cell, xs, uo, vo, rel=1e-3):
    """Richardson extrapolation (16 D(δ/4) - D(δ)) / 15 of centred differences with δ = rel H: near the calving front
    the response to H curves strongly (the front force grows as H²), and the O(δ²) error of one centred difference
    there reaches 1e-2 while the two-step combination is accurate to O(δ⁴)."""
    delta = rel * max(case.fields["H"][cell], 10.0)
    d1 = _fd_thickness(P, case, cell, xs, uo, vo, delta)
    d4 = _fd_thickness(P, case, cell, xs, uo, vo, delta / 4)
    return (16 * d4 - d1) / 15


def _switch_free(case, margin):
    """Cells with ice (H > 20 m, so the ice mask is 1 on both sides of a difference) whose flotation function
    f = H + ρw b / ρᵢ and that of their four neighbours is farther than margin·H from zero (the grounded fractions, s
    and N switch branch at f = 0)."""
    H, b = case.fields["H"], case.fields["bed"]
    f = H + 1028.0 / 918.0 * b
    ny, nx = H.shape
    ok = np.zeros_like(H, dtype=bool)
    for j in range(ny):
        for i in range(nx):
            nb = [f[j, i]] + [f[jj, ii] for jj, ii in ((j, i - 1), (j, i + 1), (j - 1, i), (j + 1, i)) if 0 <= jj < ny and 0 <= ii < nx]
            ok[j, i] = H[j, i] > 20.0 and min(abs(x) for x in nb) > margin * max(H[j, i], 10.0)
    return ok


def _smooth_cells(case, grad, n, seed, delta_rel=1e-3):
    """Seeded switch-free cells (100 steps of δ = delta_rel H from the flotation switch) whose gradient is at least
    1e-3 of the largest entry."""
    ok = _switch_free(case, 100 * delta_rel)
    cand = np.argwhere(ok & (np.abs(grad) >= 1e-3 * np.max(np.abs(grad))))
    rng = np.random.default_rng(seed)
    return [tuple(cand[k]) for k in rng.choice(len(cand), size=min(n, len(cand)), replace=False)]


@pytest.mark.parametrize("kind", ["bounded", "periodic_x", "no_slip_coulomb", "till_coulomb"])
def test_thickness_gradient_matches_finite_differences(gpu_cls, kind):
    """∂J/∂H per cell against extrapolated centred differences in H with the geometry (s, φᵘ, φᵛ, N, μ) and the
    driving stress recomputed: through η̄H = μ H ∫η dζ, the drag's grounded fractions and effective pressure (the
    ocean-connected one, or a till's), the surface slope and the calving-front force of the driving stress."""
    case, P, uo, vo, ub, vb = _adjoint(gpu_cls, kind)
    xs = (P.get("u"), P.get("v"))
    ctl = M.Convergence(reltol=1e-12, maxiter=500)
    lu, lv, grad, grad_a, grad_h, st = P.picard_adjoint(ub, vb, ctl, thickness=True)
    assert st.status == 0
    # the same call computes the other gradients unchanged
    lu2, lv2, grad2, grad_a2, st2 = P.picard_adjoint(ub, vb, ctl)
    assert np.array_equal(grad, grad2) and np.array_equal(lu, lu2)
    assert np.max(np.abs(grad_h)) > 0
    cells = _smooth_cells(case, grad_h, 8, 13)
    assert len(cells) >= 4
    # under the till's small N the Coulomb drag of a grounding-line cell curves so strongly that the first derivative
    # there is small beside the higher ones: the O(δ⁴) remainder of the extrapolation at δ = 1e-3 H is 2e-3 of it
    # (the oracle's differences at δ, δ/4 and δ/16 show it), so its differences start at δ = 2.5e-4 H
    rel = 2.5e-4 if kind == "till_coulomb" else 1e-3
    for cell in cells:
        fd = _fd_thickness_extrapolated(P, case, cell, xs, uo, vo, rel)
        assert abs(fd - grad_h[cell]) <= RTOL * abs(grad_h[cell]), (kind, cell, fd, grad_h[cell])


def test_thickness_gradient_front_cells():
    """The last ice cells of the rows (the calving-front force path) against extrapolated centred differences."""
    case, P, uo, vo, ub, vb = _adjoint(nk.Problem, "bounded")
    xs = (P.get("u"), P.get("v"))
    *_, grad_h, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500), thickness=True)
    H = case.fields["H"]
    checked = 0
    for j in range(2, H.shape[0] - 2, 3):
        i = int(np.max(np.nonzero(H[j] > 0)[0]))
        cell = (j, i)
        if abs(grad_h[cell]) < 1e-3 * np.max(np.abs(grad_h)) or cell not in _smooth_cells(case, grad_h, 10**6, 0):
            continue
        checked += 1
        fd = _fd_thickness_extrapolated(P, case, cell, xs, uo, vo)
        assert abs(fd - grad_h[cell]) <= RTOL * abs(grad_h[cell]), (cell, fd, grad_h[cell])
    assert checked >= 2


@pytest.mark.parametrize("friction", ["weertman", "coulomb"])
def test_thickness_gradient_diva_matches_directional_differences(gpu_cls, friction):
    """DIVA ∂J/∂H (H also in F₂ = H ∫(1-ζ)²/η dζ and in the basal drag's grounded fractions on |uᵇ|) against
    Richardson-extrapolated directional differences along a seeded direction d H over the cells away from the
    flotation switch (one cell moves J too little against the solver tolerances); the rate factor is held."""
    case, P, uo, vo = _diva_setup(gpu_cls, friction)
    _, ub, vb = _cost(P, uo, vo)
    xs = (P.get("u"), P.get("v"))
    *_, gh, st = P.picard_adjoint(ub, vb, DIVA_ADJOINT, thickness=True)
    assert st.status == 0 and np.max(np.abs(gh)) > 0
    H0 = case.fields["H"]
    keep = _switch_free(case, 1e-2)   # the differences below move H by at most ~4e-4 H
    assert keep.sum() > 20
    d = np.random.default_rng(23).standard_normal(H0.shape) * keep * H0

    def fd(eps):
        vel = []
        for sgn in (1.0, -1.0):
            P.set("H", H0 + sgn * eps * d)
            P.compute_geometry()
            P.set("u", xs[0])
            P.set("v", xs[1])
            assert P.picard_solve().status == 0
            vel.append((P.get("u"), P.get("v")))
        P.set("H", H0)
        P.compute_geometry()
        return _cost_difference(vel[0], vel[1], uo, vo) / (2 * eps)

    eps = 1e-4
    rich = (16 * fd(eps / 4) - fd(eps)) / 15
    ad = float(np.sum(gh * d))
    assert abs(rich - ad) <= RTOL * np.sum(np.abs(gh * d)), (friction, rich, ad)


@pytest.mark.parametrize("diva", [False, True], ids=["ssa", "diva"])
def test_thickness_gradient_on_the_periodic_seam(gpu_cls, diva):
    """∂J/∂H of the cells whose north (east) face is the periodic axis's first face, read through the wrapped index:
    the top row of a ridge periodic in y and Bounded in x (test/test_enzyme.jl:79-88), against extrapolated centred
    differences of a seeded linear cost Σ w·x (Picard 1e-14), per cell to 1e-6 of the cell's own gradient, beside
    interior cells (1e-8 of the largest entry at the weakly sensitive ones)."""
    from support import ice_sheet_model
    L = 64e3
    grid = M.RectilinearGrid(size=(16, 4), x=(0.0, L), y=(0.0, 16e3), topology=("Bounded", "Periodic"), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-15, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=1000))

    def build():
        P, st = ice_sheet_model(gpu_cls, grid,
                                H=lambda x, y: 500 + 300 * math.exp(-((x - L / 2) / 12e3) ** 2) * (1 + math.sin(2 * math.pi * y / 16e3) / 5),
                                bed=0.0, rheology=M.GlenFlowLaw(rate_factor=1e-24),
                                friction=M.WeertmanFriction(coefficient=lambda x, y: 3e6 * (1 + x / L)),
                                stress_balance=M.DepthIntegrated(shear=M.DIVAShear()) if diva else None,
                                velocity_solver=solver, Nsigma=6 if diva else 4)
        return P

    P = build()
    u0, v0, H0 = P.get("u"), P.get("v"), P.get("H")
    rng = np.random.default_rng(5)
    wu, wv = rng.standard_normal(u0.shape), rng.standard_normal(v0.shape)
    *_, gh, st = P.picard_adjoint(wu, wv, M.Convergence(reltol=1e-14, maxiter=3000), thickness=True)
    assert st.status == 0

    def difference(cell, d):
        out = []
        for sgn in (1.0, -1.0):
            Q = build()
            H = H0.copy()
            H[cell] += sgn * d
            Q.set("H", H)
            Q.compute_geometry()
            Q.set("u", u0)
            Q.set("v", v0)
            Q.picard_solve()
            out.append((Q.get("u"), Q.get("v")))
        return (np.sum(wu * (out[0][0] - out[1][0])) + np.sum(wv * (out[0][1] - out[1][1]))) / (2 * d)

    for cell in ((3, 15), (3, 7), (3, 0), (1, 5), (0, 8)):
        d = 1e-3 * H0[cell]
        fd = (16 * difference(cell, d / 4) - difference(cell, d)) / 15
        assert abs(fd - gh[cell]) <= 1e-6 * abs(fd) + 1e-8 * np.max(np.abs(gh)), (cell, fd, gh[cell])


@pytest.mark.parametrize("driving_stress", [False, True], ids=["centred", "split"])
def test_thickness_gradient_across_the_grounding_line(gpu_cls, driving_stress):
    """∂J/∂H of J = Σ u² + v² across a grounding line (test/test_enzyme.jl:584-608): a 16 x 4 marine sheet on a bed
    sloping down from 200 m, H = 1000 - 0.01 x - 100 ((y - 8 km) / 8 km)² up to a front at 56 km, Weertman drag,
    the subgrid grounded fraction with and without the grounding-line split of the driving stress, at the reference's
    four cells (two with 0 < φ < 1), to 1e-4 against extrapolated centred differences.  The reference differentiates
    four fixed Picard iterations; here the solves are converged (Picard 1e-14) and the adjoint is the fixed point's."""
    from support import ice_sheet_model
    grid = M.RectilinearGrid(size=(16, 4), x=(0.0, 64e3), y=(0.0, 16e3), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-15, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=1000))

    def build():
        P, st = ice_sheet_model(gpu_cls, grid, H=lambda x, y: 1000 - 1e-2 * x - 100 * ((y - 8e3) / 8e3) ** 2 if x < 56e3 else 0.0,
                                bed=lambda x, y: -200 - 1e-2 * x, rheology=M.GlenFlowLaw(rate_factor=1e-24),
                                friction=M.WeertmanFriction(coefficient=3e6),
                                grounding=M.SubgridGroundedFraction(driving_stress=driving_stress), velocity_solver=solver)
        assert st.status == 0
        return P

    P = build()
    phi = P.get("phi")
    assert 0 < phi[1, 8] < 1 and 0 < phi[1, 9] < 1
    u0, v0, H0 = P.get("u"), P.get("v"), P.get("H")
    *_, gh, st = P.picard_adjoint(2 * u0, 2 * v0, M.Convergence(reltol=1e-14, maxiter=3000), thickness=True)
    assert st.status == 0

    def difference(cell, d):
        out = []
        for sgn in (1.0, -1.0):
            Q = build()
            H = H0.copy()
            H[cell] += sgn * d
            Q.set("H", H)
            Q.compute_geometry()
            Q.set("u", u0)
            Q.set("v", v0)
            Q.picard_solve()
            out.append((Q.get("u"), Q.get("v")))
        (up, vp), (um, vm) = out
        return (np.sum((up - um) * (up + um)) + np.sum((vp - vm) * (vp + vm))) / (2 * d)

    for cell in ((1, 7), (2, 8), (1, 9), (1, 11)):
        d = 1e-3 * H0[cell]
        fd = (16 * difference(cell, d / 4) - difference(cell, d)) / 15
        assert abs(fd - gh[cell]) <= 1e-4 * abs(fd), (driving_stress, cell, fd, gh[cell])
