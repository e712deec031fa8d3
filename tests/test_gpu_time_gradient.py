"""The gradient through time steps (nk_checkpointed_gradient; checkpointed_gradient!, ext/NunatakEnzymeExt.jl:245-263)
against centred finite differences of the forward time steps, following the checks of test/test_enzyme.jl:391-488.

Each case builds its problem afresh for every evaluation, so the finite differences and the gradient start from
the same state; the forward map is the public one a host steps with (step_thickness with the velocities held, or
step_thickness_stage followed by picard_solve for each stage), J = Σ H² after the last step unless noted.
- thickness transport through the time steps, velocities held (:447-488): 16 x 4, Bounded x Periodic, the default
  bounded WENO-5, sources a and m, eight steps of half the advective time scale; ∂J/∂a, ∂J/∂m, ∂J/∂u and ∂J/∂H₀ at
  the reference's cells to 1e-6, and segments of 3, 3 and 2 steps against one segment to 1e-12; the same for
  first-order upwinding; ∂J/∂u and ∂J/∂H₀ also against the oracle's forward steps;
- converged Picard time steps (:421-445): the reference's ridge (SSA, Weertman, a = 1e-8), six steps of 1/200 of
  the advective time scale, checkpoints every two steps; ∂J/∂H₀ at two cells, ∂J/∂C and ∂J/∂a at one each, to 1e-5;
  the same ridge under the DIVA (Nσ = 6) to 1e-4; ∂J/∂H₀ against the oracle's forward steps;
- checkpoint intervals 1, 2 and 6 give one gradient, J is the forward cost and the problem ends at the forward's
  final state;
- the floating melt across a grounding line (SubgridGroundedFraction, velocities held): ∂J/∂H₀ at cells with
  0 < φ < 1 runs through the centre grounded fraction of the melt source, and ∂J/∂m at floating cells;
- a cost at two steps with per-step melt factors (the structure of the STREAMICE halfpipe adjoint,
  benchmarks/halfpipe_streamice_adjoint.jl:50-64: velocities after step 2, thickness after step 3, melt weights
  0.5, 1, 0.5): ∂J/∂m and ∂J/∂H₀ on the ridge to 1e-5;
- a partial-cell front with its overflow passes and its calving laws (test/test_enzyme.jl:490-536), von Mises calving
  with the velocities held and, on a confined floating shelf, through Picard solves (its rates read the viscosity of
  the solve before the front);
- with the velocities held, the library's gradient equals the oracle's restatement over every cell and face.
A difference is formed as Σ (x₊ - x₋)(x₊ + x₋) / 2δ from the two perturbed runs, never as the difference of two
rounded costs."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import evaluate, ice_sheet_model, make, set_fn

pytestmark = pytest.mark.gpu


# ---- cases: a fresh problem at its initial state, the time step and the step count ---------------------------------
class Case:
    def __init__(self, build, dt, steps, solves):
        self.build, self.dt, self.steps, self.solves = build, dt, steps, solves

    def forward(self, cls, mutate=None, record=None):
        """Run the steps on a fresh problem after mutate(P); record(step, P) after each step."""
        P = self.build(cls)
        if mutate is not None:
            mutate(P)
            P.compute_geometry()
        for n in range(1, self.steps + 1):
            if self.solves:
                for stage in (1, 2, 3):
                    P.step_thickness_stage(self.dt, stage)
                    P.picard_solve()
            else:
                P.step_thickness(self.dt)
            if record is not None:
                record(n, P)
        return P


def _advective_timescale(P):
    """cell_advection_timescale: the shortest time for the depth-averaged flow to cross a cell."""
    g = P.grid
    dx, dy = (g.x[1] - g.x[0]) / g.Nx, (g.y[1] - g.y[0]) / g.Ny
    u, v = np.abs(P.get("u")), np.abs(P.get("v"))
    rate = u[:, :g.Nx] / dx + v[:g.Ny, :] / dy
    return 1.0 / float(np.max(rate))


def transport_case(advection=None):
    L = 16e3
    grid = M.RectilinearGrid(size=(16, 4), x=(0.0, L), y=(0.0, 4e3), topology=("Bounded", "Periodic"), halo=(4, 4))

    def build(cls):
        P = make(cls, grid, advection=advection, Nsigma=2)
        set_fn(P, "H", lambda x, y: 100 + 50 * math.exp(-((x - L / 4) / 2e3) ** 2))
        P.set("bed", 0.0)
        P.compute_geometry()
        set_fn(P, "u", lambda x, y: 1e-6 * math.sin(math.pi * x / L))
        P.set("v", 0.0)
        P.energy_set("surface_mass_balance", 1e-8)
        P.energy_set("basal_melt_rate", evaluate(grid, "H", lambda x, y: 1e-9 * x / L))
        P.energy_set("clipped_thickness", 0.0)
        return P

    return Case(build, 0.5 * (L / 16) / 1e-6, 8, solves=False)


def ridge_case(cls_for_dt, diva=False, steps=6, melt=0.0):
    L = 64e3
    grid = M.RectilinearGrid(size=(16, 4), x=(0.0, L), y=(0.0, 16e3), topology=("Bounded", "Periodic"), halo=(4, 4))
    # Picard to 1e-14, CG to 1e-15: a perturbed solve stops once its change falls below reltol ‖u‖, so with the
    # reference's 1e-12 a difference in one cell's H (a velocity response of ~1e-6 ‖u‖) keeps a bias of ~1e-5 of
    # its own size from the Picard iterations not run; the adjoint is the converged fixed point's
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-15, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=1000),
                                   adjoint_iteration_control=M.Convergence(reltol=1e-14, maxiter=2000))
    sb = M.DepthIntegrated(shear=M.DIVAShear()) if diva else None

    def build(cls):
        P, _ = ice_sheet_model(cls, grid,
                               H=lambda x, y: 500 + 300 * math.exp(-((x - L / 2) / 12e3) ** 2) * (1 + math.sin(2 * math.pi * y / 16e3) / 5),
                               bed=0.0, rheology=M.GlenFlowLaw(rate_factor=1e-24),
                               friction=M.WeertmanFriction(coefficient=lambda x, y: 3e6 * (1 + x / L)),
                               stress_balance=sb, velocity_solver=solver, Nsigma=6 if diva else 4)
        P.energy_set("surface_mass_balance", 1e-8)
        P.energy_set("basal_melt_rate", evaluate(grid, "H", melt) if callable(melt) else melt)
        P.energy_set("clipped_thickness", 0.0)
        return P

    dt = _advective_timescale(build(cls_for_dt)) / 200
    return Case(build, dt, steps, solves=True)


def grounding_line_case(advection):
    L = 32e3
    grid = M.RectilinearGrid(size=(16, 6), x=(0.0, L), y=(0.0, 12e3), topology=("Bounded", "Periodic"), halo=(4, 4))

    def build(cls):
        P = make(cls, grid, advection=advection, Nsigma=2, grounding=M.SubgridGroundedFraction())
        # curved along the flow: on linear data WENO-Z's τ = |β₀ - β₂| sits at its kink, where a difference and the
        # derivative of one branch part; the phase keeps rows apart (equal flotations tie in the grounded fraction's
        # sort, where the derivative is one-sided)
        set_fn(P, "H", lambda x, y: 700 - 400 * x / L + 40 * math.cos(2 * math.pi * x / L) + 30 * math.sin(2 * math.pi * y / 12e3 + 0.4))
        set_fn(P, "bed", lambda x, y: -300 - 700 * x / L)
        P.compute_geometry()
        P.set("u", 2e-6)
        set_fn(P, "v", lambda x, y: 2e-7 * math.cos(2 * math.pi * y / 12e3))
        P.energy_set("surface_mass_balance", 0.0)
        P.energy_set("basal_melt_rate", 3e-8)
        P.energy_set("clipped_thickness", 0.0)
        return P

    return Case(build, 0.1 * (L / 16) / 2e-6, 4, solves=False)


# ---- costs ----------------------------------------------------------------------------------------------------------
def thickness_cost(steps):
    def cost(step, H, u, v, mask):
        if step != steps:
            return None
        return float(np.sum(H * H)), 2 * H, None, None
    return cost


def _difference(plus, minus):
    return float(np.sum((plus - minus) * (plus + minus)))


def fd_final_thickness(case, cls, field, index, h):
    """Centred difference of Σ H² after the steps in one entry of a field (an energy-step source or a problem field)."""
    def mutate(sign):
        def m(P):
            src = field in ("surface_mass_balance", "basal_melt_rate")
            a = P.energy_get(field) if src else P.get(field)
            a[index] += sign * h
            (P.energy_set if src else P.set)(field, a)
        return m
    Hp = case.forward(cls, mutate(+1)).get("H")
    Hm = case.forward(cls, mutate(-1)).get("H")
    return _difference(Hp, Hm) / (2 * h)


def fd_extrapolated(case, cls, field, index, h):
    """Richardson's (16 D(h/4) - D(h)) / 15 of fd_final_thickness: accurate to O(h⁴) where the response curves."""
    return (16 * fd_final_thickness(case, cls, field, index, h / 4) - fd_final_thickness(case, cls, field, index, h)) / 15


def gradient(case, cls, cost=None, **kw):
    P = case.build(cls)
    return P, P.checkpointed_gradient(cost or thickness_cost(case.steps), case.dt, case.steps,
                                      velocity_solves=case.solves, **kw)


def _close(ad, fd, rtol):
    assert fd != 0.0
    assert abs(ad - fd) <= rtol * abs(fd), (ad, fd, abs(ad - fd) / abs(fd))


# ---- thickness transport, velocities held (test/test_enzyme.jl:447-488) --------------------------------------------
@pytest.mark.parametrize("advection", [None, M.UpwindBiased(order=1)], ids=["bounded_weno5", "upwind1"])
def test_transport_gradient_matches_differences(gpu_cls, advection):
    case = transport_case(advection)
    _, g = gradient(case, gpu_cls)
    a_checks = (("surface_mass_balance", "smb", (1, 4), 1e-8), ("basal_melt_rate", "melt", (2, 8), 1e-9 * 8.5 / 16))
    for field, key, idx, val in a_checks:
        _close(g[key][idx], fd_final_thickness(case, gpu_cls, field, idx, 1e-6 * val), 1e-6)
    u0 = case.build(gpu_cls).get("u")
    for idx in ((0, 5), (3, 10)):
        _close(g["u"][idx], fd_final_thickness(case, gpu_cls, "u", idx, 1e-6 * abs(u0[idx])), 1e-6)
    H0 = case.build(gpu_cls).get("H")
    for idx in ((1, 3), (2, 8)):
        _close(g["H"][idx], fd_final_thickness(case, gpu_cls, "H", idx, 1e-6 * H0[idx]), 1e-6)
    assert g["stats"]["picard_solves"] == 0 and g["stats"]["segments"] == 3


@pytest.mark.parametrize("advection", [None, M.UpwindBiased(order=1)], ids=["bounded_weno5", "upwind1"])
def test_transport_segments_reproduce_one_pass(gpu_cls, advection):
    case = transport_case(advection)
    _, whole = gradient(case, gpu_cls, checkpoint_interval=case.steps)
    _, split = gradient(case, gpu_cls, checkpoint_interval=3)
    assert whole["stats"]["segments"] == 1 and split["stats"]["segments"] == 3
    for key in ("smb", "melt", "u", "H"):
        np.testing.assert_allclose(split[key], whole[key], rtol=1e-12, atol=1e-12 * np.max(np.abs(whole[key])))
    J = float(np.sum(case.forward(gpu_cls).get("H") ** 2))
    assert abs(whole["J"] - J) <= 1e-13 * J


def test_transport_gradient_against_the_oracle_forward(gpu_cls, oracle_cls):
    case = transport_case()
    _, g = gradient(case, gpu_cls)
    u0 = case.build(oracle_cls).get("u")
    _close(g["u"][0, 5], fd_final_thickness(case, oracle_cls, "u", (0, 5), 1e-6 * abs(u0[0, 5])), 1e-6)
    H0 = case.build(oracle_cls).get("H")
    _close(g["H"][1, 3], fd_final_thickness(case, oracle_cls, "H", (1, 3), 1e-6 * H0[1, 3]), 1e-6)


# ---- converged Picard time steps (test/test_enzyme.jl:421-445) ----------------------------------------------------
@pytest.mark.parametrize("diva", [False, True], ids=["ssa", "diva"])
def test_picard_time_steps_gradient_matches_differences(gpu_cls, diva):
    case = ridge_case(gpu_cls, diva=diva)
    P, g = gradient(case, gpu_cls, checkpoint_interval=2)
    rtol = 1e-4 if diva else 1e-5
    assert g["stats"]["segments"] == 3 and g["stats"]["picard_adjoints"] == 3 * case.steps
    assert g["stats"]["worst_solve_status"] == 0
    H0 = case.build(gpu_cls).get("H")
    for idx in ((1, 5), (2, 9)):
        _close(g["H"][idx], fd_extrapolated(case, gpu_cls, "H", idx, 1e-3 * H0[idx]), rtol)
    C = case.build(gpu_cls).get("C")
    _close(g["log_C"][1, 6] / C[1, 6], fd_extrapolated(case, gpu_cls, "C", (1, 6), 1e-3 * C[1, 6]), rtol)
    _close(g["smb"][2, 8], fd_extrapolated(case, gpu_cls, "surface_mass_balance", (2, 8), 1e-2 * 1e-8), rtol)


def test_picard_time_steps_against_the_oracle_forward(gpu_cls, oracle_cls):
    case = ridge_case(gpu_cls)
    _, g = gradient(case, gpu_cls, checkpoint_interval=2)
    H0 = case.build(oracle_cls).get("H")
    _close(g["H"][1, 5], fd_final_thickness(case, oracle_cls, "H", (1, 5), 1e-4 * H0[1, 5]), 1e-5)


@pytest.mark.parametrize("diva", [False, True], ids=["ssa", "diva"])
def test_checkpoint_intervals_agree_and_the_problem_ends_at_the_final_state(gpu_cls, diva):
    case = ridge_case(gpu_cls, diva=diva)
    runs = []
    for k in (1, 2, case.steps):
        P, g = gradient(case, gpu_cls, checkpoint_interval=k)
        runs.append((P.get("H"), P.get("u"), g))
    ref = case.forward(gpu_cls)
    J = float(np.sum(ref.get("H") ** 2))
    for H, u, g in runs:
        np.testing.assert_array_equal(H, ref.get("H"))
        np.testing.assert_array_equal(u, ref.get("u"))
        assert abs(g["J"] - J) <= 1e-14 * J
        for key in ("H", "u", "v", "smb", "log_C", "log_A"):
            np.testing.assert_allclose(g[key], runs[0][2][key], rtol=1e-12, atol=1e-12 * np.max(np.abs(runs[0][2][key])))


# ---- the floating melt across a grounding line ---------------------------------------------------------------------
@pytest.mark.parametrize("advection", [None, M.UpwindBiased(order=1)], ids=["bounded_weno5", "upwind1"])
def test_floating_melt_gradient_through_the_grounded_fraction(gpu_cls, advection):
    case = grounding_line_case(advection)
    P0 = case.build(gpu_cls)
    phi, H0 = P0.get("phi"), P0.get("H")
    _, g = gradient(case, gpu_cls)
    partial = [tuple(ix) for ix in np.argwhere((phi > 0.05) & (phi < 0.95))]
    assert len(partial) >= 3
    for idx in partial[:4]:
        _close(g["H"][idx], fd_final_thickness(case, gpu_cls, "H", idx, 1e-6 * H0[idx]), 1e-5)
    floating = [tuple(ix) for ix in np.argwhere(phi == 0.0)]
    for idx in (floating[0], floating[len(floating) // 2]):
        _close(g["melt"][idx], fd_final_thickness(case, gpu_cls, "basal_melt_rate", idx, 1e-6 * 3e-8), 1e-6)
    assert np.all(g["melt"][:, :2] == 0.0)   # the grounded cells upstream melt nothing


# ---- costs at two steps, melt weights (the structure of the STREAMICE halfpipe adjoint) -----------------------------
def test_costs_at_two_steps_with_melt_weights(gpu_cls):
    L = 64e3
    case = ridge_case(gpu_cls, steps=3, melt=lambda x, y: 1e-9 * (1 + x / L))
    weights = (0.5, 1.0, 0.5)
    year = 31556926.0

    def cost(step, H, u, v, mask):
        if step == 2:
            return float(np.sum(u * u) + np.sum(v * v)) * year ** 2, None, 2 * u * year ** 2, 2 * v * year ** 2
        if step == 3:
            return float(np.sum(H * H)), 2 * H, None, None
        return None

    _, g = gradient(case, gpu_cls, cost=cost, melt_weights=weights)

    def run(mutate):
        out = {}

        def weighted(P):
            mutate(P)
            base = P.energy_get("basal_melt_rate")
            out["base"] = base

        def record(n, P):
            out[n] = (P.get("H"), P.get("u"), P.get("v"))
            if n < case.steps:
                P.energy_set("basal_melt_rate", weights[n] * out["base"])

        def first(P):
            weighted(P)
            P.energy_set("basal_melt_rate", weights[0] * out["base"])
        case.forward(gpu_cls, first, record)
        return out

    def fd(mutate_plus, mutate_minus, h):
        p, m = run(mutate_plus), run(mutate_minus)
        d = _difference(p[3][0], m[3][0]) + year ** 2 * (_difference(p[2][1], m[2][1]) + _difference(p[2][2], m[2][2]))
        return d / (2 * h)

    def melt_at(idx, h):
        def f(P):
            a = P.energy_get("basal_melt_rate")
            a[idx] += h
            P.energy_set("basal_melt_rate", a)
        return f

    for idx in ((1, 6), (3, 12)):
        h = 1e-2 * 1e-9 * (1 + (idx[1] + 0.5) / 16)
        _close(g["melt"][idx], fd(melt_at(idx, h), melt_at(idx, -h), h), 1e-5)

    H0 = case.build(gpu_cls).get("H")

    def thick_at(idx, h):
        def f(P):
            a = P.get("H")
            a[idx] += h
            P.set("H", a)
        return f
    h = 1e-4 * H0[2, 9]
    _close(g["H"][2, 9], fd(thick_at((2, 9), h), thick_at((2, 9), -h), h), 1e-5)


def test_refusals(gpu_cls):
    case = transport_case()
    P = case.build(gpu_cls)
    with pytest.raises(Exception):
        P.checkpointed_gradient(thickness_cost(2), -1.0, 2, velocity_solves=False)
    with pytest.raises(Exception):
        P.checkpointed_gradient(thickness_cost(2), case.dt, 0, velocity_solves=False)

    def broken(step, H, u, v, mask):
        raise ValueError("the host's cost failed")
    with pytest.raises(ValueError):
        P.checkpointed_gradient(broken, case.dt, 2, velocity_solves=False)


# ---- the partial-cell front (test/test_enzyme.jl:490-514) -------------------------------------------------------------
def channel_front_case(passes=4):
    dx, U, Hi = 1e3, 1.0, 100.0
    grid = M.RectilinearGrid(size=(16, 4), x=(0.0, 16 * dx), y=(0.0, 4 * dx), topology=("Bounded", "Periodic"), halo=(4, 4))

    def build(cls):
        P = make(cls, grid, advection=M.UpwindBiased(order=1), Nsigma=2, masking=M.PartialCellFront(passes=passes))
        set_fn(P, "H", lambda x, y: Hi if x < 4 * dx else 0.0)
        P.set("bed", 0.0)
        P.initialize_front()
        P.compute_geometry()
        set_fn(P, "u", lambda x, y: U if 0 < x < 16 * dx else 0.0)
        P.set("v", 0.0)
        P.energy_set("surface_mass_balance", evaluate(grid, "H", lambda x, y: U * Hi / dx if x < dx else -1e-6))
        P.energy_set("basal_melt_rate", 0.0)
        P.energy_set("clipped_thickness", 0.0)
        return P

    return Case(build, dx / U / 4, 6, solves=False)


@pytest.mark.parametrize("passes", [4, 0])
def test_surface_mass_balance_through_the_partial_cell_front(gpu_cls, passes):
    """∂J/∂a of J = Σ H² after six steps of a front advancing through partially filled cells, at a full cell and at a
    cell the front reaches (its sources forced onto the partial cell), to 1e-6 (the reference's h = 1e-9); with the
    reference's default four overflow passes (filled cells spill their excess into empty neighbours) and without."""
    case = channel_front_case(passes)
    _, g = gradient(case, gpu_cls)
    assert not np.any(np.isnan(g["smb"]))
    for idx in ((1, 2), (2, 4)):
        _close(g["smb"][idx], fd_final_thickness(case, gpu_cls, "surface_mass_balance", idx, 1e-9), 1e-6)
    H0 = case.build(gpu_cls).get("H")
    for idx in ((1, 2), (2, 3)):   # (2, 3): the last full cell, the inflowing donor of the first front cell
        _close(g["H"][idx], fd_final_thickness(case, gpu_cls, "H", idx, 1e-6 * H0[idx]), 1e-6)


# ---- calving (test/test_enzyme.jl:516-536) -----------------------------------------------------------------------------
def calving_case(law, steps=1, grounding=None):
    """The reference's eigencalving case: a 12 x 6 shelf on a bed 500 m deep, 100 m of ice west of 4 km, spreading at
    u = a x, v = b y (a = b = 1e-9 /s), the front's four overflow passes; one step of 1e7 s with the velocities held
    (the stages move ice too, where the reference's cost advances the front alone).  The front-velocity law calves
    floating ice only ((1 - φ) c), so its case takes the subgrid grounded fraction.  η̄H = 10¹⁴ H (held with the
    velocities) is read by the von Mises law alone."""
    dx, Hi, a, b = 1e3, 100.0, 1e-9, 1e-9
    grid = M.RectilinearGrid(size=(12, 6), x=(0.0, 12 * dx), y=(0.0, 6 * dx), halo=(4, 4))

    def build(cls):
        P = make(cls, grid, advection=M.UpwindBiased(order=1), Nsigma=2, masking=M.PartialCellFront(calving=law),
                 grounding=grounding)
        set_fn(P, "H", lambda x, y: Hi if x < 4 * dx else 0.0)
        P.set("bed", -500.0)
        P.initialize_front()
        P.compute_geometry()
        set_fn(P, "u", lambda x, y: a * x)
        set_fn(P, "v", lambda x, y: b * y)
        P.set("eta_H", 1e14 * np.maximum(P.get("H"), 1.0))
        P.energy_set("surface_mass_balance", 0.0)
        P.energy_set("basal_melt_rate", 0.0)
        P.energy_set("clipped_thickness", 0.0)
        return P

    return Case(build, 1e7, steps, solves=False)


VON_MISES = M.VonMisesCalving(stress_threshold=1e6, floating_stress_threshold=2e5)


@pytest.mark.parametrize("law", [M.EigenCalving(coefficient=1e13), M.FrontVelocityCalving(front_velocity=1e-6), VON_MISES],
                         ids=["eigen", "front_velocity", "von_mises"])
def test_velocity_gradient_through_calving(gpu_cls, law):
    """∂J/∂u of J = Σ H² at the faces the reference checks (its cells (4, 2) and (4, 3)), through the retreat the rate
    law sets from the strain rates or the front speed, to 1e-5 (the reference's tolerance and h = 1e-12); ∂J/∂H₀ also
    runs through η = η̄H / H of the von Mises rate."""
    grounded = isinstance(law, (M.FrontVelocityCalving, M.VonMisesCalving))
    case = calving_case(law, grounding=M.SubgridGroundedFraction() if grounded else None)
    P0 = case.build(gpu_cls)
    _, g = gradient(case, gpu_cls)
    assert not np.any(np.isnan(g["u"]))
    for idx in ((1, 3), (2, 3)):
        fd = fd_final_thickness(case, gpu_cls, "u", idx, 1e-12)
        _close(g["u"][idx], fd, 1e-5)
    P1 = case.forward(gpu_cls)
    assert np.sum(P1.get("calved_thickness")) > 0   # the law calved
    H0 = P0.get("H")
    _close(g["H"][2, 3], fd_final_thickness(case, gpu_cls, "H", (2, 3), 1e-6 * H0[2, 3]), 1e-5)


def test_thickness_gradient_through_threshold_calving(gpu_cls):
    """A removal law (thickness threshold): the calved cells hold no ice afterwards; ∂J/∂H₀ and ∂J/∂a elsewhere through
    the front's advance, two steps, to 1e-6."""
    case = calving_case(M.ThicknessThresholdCalving(thickness=150.0), steps=2)
    P0 = case.build(gpu_cls)
    _, g = gradient(case, gpu_cls)
    H0 = P0.get("H")
    for idx in ((2, 1), (3, 2)):
        _close(g["H"][idx], fd_final_thickness(case, gpu_cls, "H", idx, 1e-6 * H0[idx]), 1e-6)


def shelf_case(diva=False):
    """A floating shelf in a channel with free-slip walls (Bounded x Bounded, 16 x 4 cells of 2 km, 400 m thinning
    east and thicker mid-channel, ice west of 20 km over a bed 2 km deep), PartialCellFront under von Mises calving,
    a converged Picard solve after every stage, two steps of 2e8 s: the rates read the viscosity η̄H of the solve
    before the front."""
    L, Ly, xf = 32e3, 8e3, 20e3
    grid = M.RectilinearGrid(size=(16, 4), x=(0.0, L), y=(0.0, Ly), topology=("Bounded", "Bounded"), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-15, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=1000),
                                   adjoint_iteration_control=M.Convergence(reltol=1e-14, maxiter=2000))
    sb = M.DepthIntegrated(shear=M.DIVAShear()) if diva else None
    law = M.VonMisesCalving(stress_threshold=3e6, floating_stress_threshold=1e6)

    def build(cls):
        P = make(cls, grid, advection=M.UpwindBiased(order=1), Nsigma=6 if diva else 4, masking=M.PartialCellFront(calving=law),
                 rheology=M.GlenFlowLaw(rate_factor=1e-24), friction=M.WeertmanFriction(coefficient=1e6),
                 grounding=M.SubgridGroundedFraction(), stress_balance=sb, velocity_solver=solver)
        set_fn(P, "H", lambda x, y: 400 - 4e-3 * x + 20 * math.sin(math.pi * y / Ly) if x < xf else 0.0)
        P.set("bed", -2000.0)
        P.set("A", 1e-24)
        P.set("C", 1e6)
        P.compute_geometry()
        P.initialize_front()
        P.compute_geometry()
        set_fn(P, "u", lambda x, y: 1e-9 * x)
        P.set("v", 0.0)
        P.energy_set("surface_mass_balance", 0.0)
        P.energy_set("basal_melt_rate", 0.0)
        P.energy_set("clipped_thickness", 0.0)
        P.picard_solve()
        return P

    return Case(build, 2e7, 2, solves=True)


@pytest.mark.parametrize("diva", [False, True], ids=["ssa", "diva"])
def test_gradient_through_von_mises_calving_with_solves(gpu_cls, diva):
    """Von Mises calving with the velocities solved: ∂J/∂H₀ at a shelf cell and at the front column, and ∂J/∂log A at a
    cell near the front (A enters the velocities and the viscosity η̄H the rates read, whose adjoint joins the Picard
    adjoint of the solve before the front) against Richardson-extrapolated differences, to 1e-5 (SSA) and 1e-4 (DIVA)."""
    case = shelf_case(diva)
    P0 = case.build(gpu_cls)
    H0, A0 = P0.get("H"), P0.get("A")
    _, g = gradient(case, gpu_cls)
    P1 = case.forward(gpu_cls)
    assert np.sum(P1.get("calved_thickness")) > 0   # the law calved
    rtol = 1e-4 if diva else 1e-5
    for idx in ((1, 4), (2, 9)):
        _close(g["H"][idx], fd_extrapolated(case, gpu_cls, "H", idx, 1e-5 * H0[idx]), rtol)
    idx = (1, 8)
    _close(g["log_A"][idx], A0[idx] * fd_extrapolated(case, gpu_cls, "A", idx, 1e-4 * A0[idx]), rtol)


# ---- the library against the oracle's own restatement, every cell ------------------------------------------------------
@pytest.mark.parametrize("which", ["transport_weno5", "transport_upwind1", "grounding_line_weno5", "front_passes4", "front_passes0",
                                   "eigencalving", "front_velocity_calving", "von_mises_calving"])
def test_gradient_equals_the_oracle_restatement(gpu_cls, oracle_cls, which):
    """With the velocities held, the oracle restates the gradient through the time steps (nko_checkpointed_gradient: the
    chain by hand, the local derivatives by forward differentiation of its own forward formulas, and a partial-cell
    front's advance through its numerical Jacobian); the library's ∂J/∂H₀, ∂J/∂(u, v), ∂J/∂a and ∂J/∂m agree with it at
    every cell and face to 1e-9 of each field's largest entry, and to 1e-6 with a front (the Jacobian's differences)."""
    cases = {"transport_weno5": lambda: transport_case(None), "transport_upwind1": lambda: transport_case(M.UpwindBiased(order=1)),
             "grounding_line_weno5": lambda: grounding_line_case(None), "front_passes4": lambda: channel_front_case(4),
             "front_passes0": lambda: channel_front_case(0), "eigencalving": lambda: calving_case(M.EigenCalving(coefficient=1e13)),
             "front_velocity_calving": lambda: calving_case(M.FrontVelocityCalving(front_velocity=1e-6),
                                                            grounding=M.SubgridGroundedFraction()),
             "von_mises_calving": lambda: calving_case(VON_MISES, grounding=M.SubgridGroundedFraction())}
    case = cases[which]()
    rtol = 1e-9 if which.startswith(("transport", "grounding")) else 1e-6
    _, ga = gradient(case, gpu_cls)
    _, go = gradient(case, oracle_cls)
    assert abs(ga["J"] - go["J"]) <= 1e-12 * abs(go["J"])
    for key in ("H", "u", "v", "smb", "melt"):
        scale = max(np.max(np.abs(go[key])), 1e-300)
        assert np.max(np.abs(ga[key] - go[key])) <= rtol * scale, (which, key, np.max(np.abs(ga[key] - go[key])) / scale)


def test_gradient_through_solves_equals_the_oracle_restatement(gpu_cls, oracle_cls):
    """With a Picard solve after every stage (the reference's SSA ridge, two steps) the oracle restates the gradient
    through its own Picard adjoints, the thickness part by differences of the solve's residual τ − A(c(x*, H)) x*;
    the library's ∂J/∂H₀, ∂J/∂(u, v), ∂J/∂a, ∂J/∂m, ∂J/∂log C and ∂J/∂log A agree with it at every cell and face to
    1e-6 of each field's largest entry."""
    case = ridge_case(gpu_cls, steps=2)
    _, ga = gradient(case, gpu_cls)
    _, go = gradient(case, oracle_cls)
    assert abs(ga["J"] - go["J"]) <= 1e-10 * abs(go["J"])
    for key in ("H", "u", "v", "smb", "melt", "log_C", "log_A"):
        scale = max(np.max(np.abs(go[key])), 1e-300)
        assert np.max(np.abs(ga[key] - go[key])) <= 1e-6 * scale, (key, np.max(np.abs(ga[key] - go[key])) / scale)
