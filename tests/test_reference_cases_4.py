"""The checks of the reference's conjugate-gradient testset (test/test_conjugate_gradient.jl:7-54) and the three
doctests of src/Solvers/conjugate_gradient.jl, restated on the library's own linear operation.

The reference runs them on toy_operator! (test/toy_problems.jl:6-21: identity plus a weighted graph Laplacian on
an 8 x 8 Periodic x Periodic grid).  The library's solver has exactly one linear operation, the SSA operator, so
the same checks run on it, on the same grid, with η̄H = 1 + sin²(2πx) + cos²(2πy)/2 (toy_viscosity,
test/toy_problems.jl:29-34), the right-hand side of toy_right_hand_side (:36-41), and a drag β = 1/Az, so the
drag term is the identity as in toy_operator!:
- Convergence(reltol = 1e-12, maxiter = 500) stops within 0 < iterations < 500 with ‖A x − b‖ < 1e-10 ‖b‖;
- adjoint_solve! gives the forward solution (the operator is self-adjoint);
- dot(A x, y) ≈ dot(x, A y) (Julia's default ≈, rtol √eps);
- the Jacobi-preconditioned solve gives the plain solution (≈);
- Picard(FixedIterations(3)) around CG(FixedIterations(4)) leaves the linear iteration count at 4.
The reference's zero-allocation check (:51-53) has its counterpart in nk_picard_change_noalloc
(tests/test_zz_no_alloc.py).  Every case runs on the oracle and on the GPU library (marked gpu)."""
import inspect
import math
import re

import numpy as np
import pytest

from nunatak_gb300 import model as M
from nunatak_gb300 import workloads
from support import evaluate, isapprox, julia_value, make, reference_doctest, reference_doctests, set_fn, vector_dot

N = 8
RTOL_APPROX = math.sqrt(np.finfo(np.float64).eps)


def toy_grid():
    return M.RectilinearGrid(size=(N, N), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Periodic", "Periodic"), halo=(3, 3))


def toy_viscosity(x, y):
    return 1 + math.sin(2 * math.pi * x) ** 2 + math.cos(2 * math.pi * y) ** 2 / 2


def toy_problem(cls, preconditioner=None, control=None):
    g = toy_grid()
    solver = M.StressBalanceSolver(linear_iteration_control=control or M.Convergence(reltol=1e-12, maxiter=500),
                                   preconditioner=preconditioner)
    P = make(cls, g, stress_balance=M.DepthIntegrated(side_walls=M.FreeSlipWalls()), masking=None, velocity_solver=solver)
    set_fn(P, "eta_H", toy_viscosity)
    set_fn(P, "eta_H_ff", toy_viscosity)
    P.set("beta_u", float(N * N))   # Az β = 1: the drag term is the identity
    P.set("beta_v", float(N * N))
    return P


def toy_right_hand_side(g):
    bu = evaluate(g, "u", lambda x, y: math.sin(2 * math.pi * x) * math.cos(4 * math.pi * y))
    bv = evaluate(g, "v", lambda x, y: math.cos(2 * math.pi * x) + x * y)
    return bu, bv


def _solve(P, bu, bv, adjoint=False):
    P.set("u", 0.0)
    P.set("v", 0.0)
    st = (P.adjoint_solve if adjoint else P.linear_solve)(bu, bv)
    return P.get("u"), P.get("v"), st


def test_cg_converges_and_adjoint_equals_forward(backend):
    P = toy_problem(backend)
    g = P.grid
    bu, bv = toy_right_hand_side(g)
    xu, xv, st = _solve(P, bu, bv)
    assert st.status == 0 and 0 < st.linear_iterations_last < 500
    Au, Av = P.apply_operator(xu, xv)
    residual = math.sqrt(np.sum((Au - bu) ** 2) + np.sum((Av - bv) ** 2))
    assert residual < 1e-10 * math.sqrt(vector_dot(g, bu, bv, bu, bv))
    lu, lv, st_adj = _solve(P, bu, bv, adjoint=True)
    assert st_adj.status == 0
    assert isapprox(lu, xu, rtol=RTOL_APPROX) and isapprox(lv, xv, rtol=RTOL_APPROX)
    yu = evaluate(g, "u", lambda x, y: math.cos(6 * math.pi * y))
    yv = bv
    Ayu, Ayv = P.apply_operator(yu, yv)
    a, b = vector_dot(g, Au, Av, yu, yv), vector_dot(g, xu, xv, Ayu, Ayv)
    assert abs(a - b) <= RTOL_APPROX * max(abs(a), abs(b))


def test_jacobi_preconditioned_solve_equals_plain(backend):
    bu, bv = toy_right_hand_side(toy_grid())
    xu, xv, _ = _solve(toy_problem(backend), bu, bv)
    pu, pv, st = _solve(toy_problem(backend, preconditioner=M.StressBalanceDiagonalPreconditioner()), bu, bv)
    assert st.status == 0 and 0 < st.linear_iterations_last < 500
    assert isapprox(pu, xu, rtol=RTOL_APPROX) and isapprox(pv, xv, rtol=RTOL_APPROX)


# ---- doctests of src/Solvers/conjugate_gradient.jl on a 4 x 4 Periodic x Periodic grid --------------------
# The doctests use a stored diagonal 2 and the operator double!(q, p) = 2p.  The SSA operator reproduces both
# exactly on that grid: with η̄H = η̄Hᶠᶠ = 1/8 and Az β = 3/4 its diagonal is 3/4 + 2 (4 Δy η̄H / Δx) +
# 2 (Δx η̄Hᶠᶠ / Δy) = 2, and with Az β = 2 it maps every constant vector to twice itself (the strain rates of a
# constant field are zero), so one CG iteration from zero reaches x = b / 2 exactly.  Every number involved
# is a power of two or a small sum of them, so the answers are exact, as in the doctests.

def _doctest_problem(cls, eta, beta, preconditioner=None):
    g = M.RectilinearGrid(size=(4, 4), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Periodic", "Periodic"), halo=(3, 3))
    solver = M.StressBalanceSolver(preconditioner=preconditioner)
    P = make(cls, g, stress_balance=M.DepthIntegrated(side_walls=M.FreeSlipWalls()), masking=None, velocity_solver=solver)
    for name in ("eta_H", "eta_H_ff"):
        P.set(name, eta)
    for name in ("beta_u", "beta_v"):
        P.set(name, beta)
    return P


def test_jacobi_precondition_doctest(backend):
    """src/Solvers/conjugate_gradient.jl:18-31: z = r / diagonal with r = 3 and diagonal 2 gives 1.5."""
    P = _doctest_problem(backend, 0.125, 12.0, preconditioner=M.StressBalanceDiagonalPreconditioner())
    zu, zv = P.precondition(np.full(P.shape("u"), 3.0), np.full(P.shape("v"), 3.0))
    expected = julia_value(reference_doctest("src/Solvers/conjugate_gradient.jl", 18)[0])   # extrema (1.5, 1.5)
    assert (zu.min(), zu.max()) == expected and (zv.min(), zv.max()) == expected


def test_solve_and_adjoint_solve_doctests(backend):
    """src/Solvers/conjugate_gradient.jl:109-126 (solve!) and :136-153 (adjoint_solve!): A = 2I, b = 1 gives
    x = λ = 0.5 everywhere, starting from zero."""
    P = _doctest_problem(backend, 0.125, 32.0)
    one_u, one_v = np.ones(P.shape("u")), np.ones(P.shape("v"))
    qu, qv = P.apply_operator(one_u, one_v)
    assert np.all(qu == 2.0) and np.all(qv == 2.0)
    for adjoint, line in ((False, 109), (True, 136)):
        expected = julia_value(reference_doctest("src/Solvers/conjugate_gradient.jl", line)[0])   # (0.5, 0.5)
        xu, xv, st = _solve(P, one_u, one_v, adjoint=adjoint)
        assert st.status == 0 and st.linear_iterations_last == 1
        assert (xu.min(), xu.max()) == expected and (xv.min(), xv.max()) == expected


def test_fixed_picard_around_fixed_cg_reports_the_linear_count(backend):
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(4), picard_iteration_control=M.FixedIterations(3),
                                   preconditioner=None)
    P = workloads.channel_shelf(velocity_solver=solver).problem(backend)
    st = P.picard_solve()
    assert st.status == 0
    assert (st.picard_iterations, st.linear_iterations_last, st.linear_iterations_total) == (3, 4, 12)
    st = P.picard_solve()   # a second call with the same workspaces counts the same way
    assert (st.picard_iterations, st.linear_iterations_last, st.linear_iterations_total) == (3, 4, 12)


# ---- constructor doctests of the configuration objects (host side, no device) ---------------------------

def _numbers(text):
    """The numbers between the parentheses of a printed constructor call, e.g. Convergence{Float64}(1.0e-10, 0.0, 50)."""
    return [float(x) for x in re.findall(r"[-+]?\d+\.?\d*(?:e[-+]?\d+)?", text[text.index("("):])]


def test_configuration_doctests():
    """The reference's constructor doctests, on the host-side mirrors of its configuration objects, with the
    printed values of tests/golden/reference_doctests.json:
    Convergence(; reltol = 1e-10, maxiter = 50) (src/Solvers/iteration_controls.jl:21-26);
    PicardIteration's adjoint control defaults to its control (src/Solvers/picard.jl:27-34), here
    StressBalanceSolver's (src/StressBalances/stress_balance_solver.jl:46);
    the linear and Picard controls given (src/Solvers/conjugate_gradient.jl:80-91,
    src/StressBalances/stress_balance_solver.jl:29-41);
    DepthIntegrated(side_walls = NoSlipWalls()) (src/StressBalances/depth_integrated.jl:22-27);
    SubgridGroundedFraction(driving_stress = true) (src/Groundings/subgrid_grounded_fraction.jl:14-19);
    WeertmanFriction(grid; coefficient = 3e4).exponent (src/Frictions/frictions.jl:23-32);
    GlenFlowLaw(grid; rate_factor = 1e-24).exponent (src/Rheologies/glen_flow_law.jl:25-34);
    IceSheetConstants(grid): ρw / ρᵢ (src/Models/ice_sheet_constants.jl:22-31);
    the Arrhenius transition temperature default (src/Rheologies/arrhenius_rate_factor.jl:51-58);
    sigma_faces(4; bed_refinement = 1) (src/Grids/sigma_grid.jl:8-18)."""
    c = M.Convergence(reltol=1e-10, maxiter=50)
    assert [c.reltol, c.abstol, c.maxiter] == _numbers(reference_doctest("src/Solvers/iteration_controls.jl", 21)[0])
    a = M.StressBalanceSolver(picard_iteration_control=M.Convergence(reltol=1e-8)).adjoint_control
    assert [a.reltol, a.abstol, a.maxiter] == _numbers(reference_doctest("src/Solvers/picard.jl", 27)[0])
    fixed = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(2)).linear_iteration_control
    assert f"FixedIterations({fixed.iterations})" == reference_doctest("src/Solvers/conjugate_gradient.jl", 80)[0]
    fixed = M.StressBalanceSolver(picard_iteration_control=M.FixedIterations(5)).picard_iteration_control
    assert f"FixedIterations({fixed.iterations})" == reference_doctest("src/StressBalances/stress_balance_solver.jl", 29)[0]
    d = M.DepthIntegrated(side_walls=M.NoSlipWalls())
    assert d.shear is None and isinstance(d.side_walls, M.NoSlipWalls)
    assert reference_doctest("src/StressBalances/depth_integrated.jl", 22)[0] == \
        "DepthIntegrated{Nothing, NoSlipWalls}(nothing, NoSlipWalls())"
    assert M.SubgridGroundedFraction(driving_stress=True).driving_stress is True
    assert reference_doctest("src/Groundings/subgrid_grounded_fraction.jl", 14)[0] == "SubgridGroundedFraction{true}()"
    assert M.WeertmanFriction(coefficient=3e4).exponent == julia_value(reference_doctest("src/Frictions/frictions.jl", 23)[0])
    assert M.GlenFlowLaw(rate_factor=1e-24).exponent == julia_value(reference_doctest("src/Rheologies/glen_flow_law.jl", 25)[0])
    k = M.IceSheetConstants()
    assert k.ocean_density / k.ice_density == julia_value(reference_doctest("src/Models/ice_sheet_constants.jl", 22)[0])
    from nunatak_gb300 import Problem
    default_t = inspect.signature(Problem.compute_rate_factor).parameters["transition_temperature"].default
    assert default_t == julia_value(reference_doctest("src/Rheologies/arrhenius_rate_factor.jl", 51)[0])
    assert M.sigma_faces(4, bed_refinement=1) == julia_value(reference_doctest("src/Grids/sigma_grid.jl", 8)[0])
    desc = M.make_descriptors(toy_grid(), velocity_solver=M.StressBalanceSolver(adjoint_iteration_control=M.FixedIterations(7)))
    assert desc.adjoint_control == M.FixedIterations(7)


def test_velocity_vector_doctest(backend):
    """src/Solvers/velocity_vector.jl:22-31: on a 4 x 3 Periodic x Bounded grid u holds 4 x 3 and v 4 x 4 values."""
    g = M.RectilinearGrid(size=(4, 3), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Periodic", "Bounded"), halo=(3, 3))
    P = make(backend, g, masking=None)
    (ux, uy, _), (vx, vy, _) = julia_value(reference_doctest("src/Solvers/velocity_vector.jl", 22)[0])
    assert P.shape("u") == (uy, ux) and P.shape("v") == (vy, vx)   # numpy (y, x) order
    assert P.get("u").shape == (uy, ux) and P.get("v").shape == (vy, vx)


def test_smooth_ice_mask_doctest(backend):
    """src/Models/smooth_ice_mask.jl:23-39: minimum 1, transition 2 gives μ = 0, 0, 0.5, 1, 1 for
    H = 0.5, 1, 2, 3, 10."""
    g = M.RectilinearGrid(size=(5, 1), x=(0.0, 5.0), y=(0.0, 1.0), topology=("Bounded", "Periodic"), halo=(3, 3))
    Hs = [0.5, 1.0, 2.0, 3.0, 10.0]
    P = make(backend, g, masking=M.SmoothIceMask(minimum_thickness=1.0, transition_thickness=2.0))
    P.set("H", np.array([Hs]))
    P.set("bed", 0.0)
    P.compute_geometry()
    assert P.get("ice_mask")[0].tolist() == julia_value(reference_doctest("src/Models/smooth_ice_mask.jl", 23)[0])


def test_sigma_grid_doctest(backend):
    """src/Grids/sigma_grid.jl:32-41: SigmaGrid of a 4 x 3 grid with Nσ = 6 has size (4, 3, 6)."""
    g = M.RectilinearGrid(size=(4, 3), x=(0.0, 4e3), y=(0.0, 3e3), topology=("Periodic", "Bounded"), halo=(3, 3))
    P = make(backend, g, Nsigma=6, masking=None)
    nx, ny, ns = julia_value(reference_doctest("src/Grids/sigma_grid.jl", 32)[0])
    assert P.shape("eta_sigma") == (ns, ny, nx) and P.get("eta_sigma").shape == (ns, ny, nx)


def test_library_sigma_faces_follow_sigma_faces(backend):
    """With no face list the library places the σ faces by the rule of sigma_faces (src/Grids/sigma_grid.jl:20-22):
    a DIVA solve (Arrhenius rate factor from a temperature, so the layer pressures see the faces too) and its
    velocity profile are bit for bit those of the same solve given sigma_faces(Nσ; bed_refinement) explicitly,
    and the refinement changes them."""
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(10), picard_iteration_control=M.FixedIterations(2))
    base = workloads.diva_sheet(24, 12, dx=32e3, Nsigma=4, velocity_solver=solver)
    profiles = {}
    for r in (1.0, 1.5):
        for how in ("rule", "list"):
            extra = {"bed_refinement": r} if how == "rule" else {"sigma_faces": M.sigma_faces(4, r)}
            case = workloads.Case("diva_faces", base.grid, dict(base.config, **extra), base.fields, temperature=base.temperature)
            P = case.problem(backend)
            P.picard_solve()
            P.velocity_profile()
            profiles[r, how] = P.get("u_sigma")
        assert np.array_equal(profiles[r, "rule"], profiles[r, "list"])
    assert not np.array_equal(profiles[1.0, "rule"], profiles[1.5, "rule"])


# Every doctest of tests/golden/reference_doctests.json and the test that restates it, or why none can.
DOCTEST_RESTATEMENTS = {
    ("src/Solvers/velocity_vector.jl", 22): "test_reference_cases_4::test_velocity_vector_doctest",
    ("src/Solvers/iteration_controls.jl", 21): "test_reference_cases_4::test_configuration_doctests",
    ("src/Solvers/conjugate_gradient.jl", 18): "test_reference_cases_4::test_jacobi_precondition_doctest",
    ("src/Solvers/conjugate_gradient.jl", 80): "test_reference_cases_4::test_configuration_doctests",
    ("src/Solvers/conjugate_gradient.jl", 109): "test_reference_cases_4::test_solve_and_adjoint_solve_doctests",
    ("src/Solvers/conjugate_gradient.jl", 136): "test_reference_cases_4::test_solve_and_adjoint_solve_doctests",
    ("src/Solvers/picard.jl", 27): "test_reference_cases_4::test_configuration_doctests",
    # picard_solve! with the toy double! and a no-op coefficient update returns 3 for FixedIterations(3); the
    # library's Picard step always updates the coefficients from the physics, so the count is checked on the
    # channel shelf instead.
    ("src/Solvers/picard.jl", 46): "test_reference_cases_4::test_fixed_picard_around_fixed_cg_reports_the_linear_count",
    ("src/StressBalances/ssa_operator.jl", 20): "test_reference_cases::test_ssa_operator_doctest",
    ("src/StressBalances/depth_integrated.jl", 22): "test_reference_cases_4::test_configuration_doctests",
    ("src/StressBalances/driving_stress.jl", 13): "test_reference_cases::test_driving_stress_doctests",
    ("src/StressBalances/multigrid_preconditioner.jl", 41): "test_reference_cases::test_multigrid_levels",
    # the second output, IterationInterval(48, 0), is the velocity-solve schedule of the time loop (out of scope)
    ("src/StressBalances/stress_balance_solver.jl", 29): "test_reference_cases_4::test_configuration_doctests",
    ("src/Rheologies/glen_flow_law.jl", 25): "test_reference_cases_4::test_configuration_doctests",
    ("src/Rheologies/glen_flow_law.jl", 78): "test_reference_cases::test_viscosity_doctest",
    ("src/Rheologies/arrhenius_rate_factor.jl", 51): "test_reference_cases_4::test_configuration_doctests",
    ("src/Rheologies/arrhenius_rate_factor.jl", 89): "test_reference_cases::test_arrhenius_doctest",
    ("src/Frictions/frictions.jl", 23): "test_reference_cases_4::test_configuration_doctests",
    ("src/Frictions/frictions.jl", 102): "test_reference_cases::test_basal_drag_doctest",
    ("src/Groundings/subgrid_grounded_fraction.jl", 14): "test_reference_cases_4::test_configuration_doctests",
    ("src/Groundings/subgrid_grounded_fraction.jl", 82): "test_reference_cases::test_grounded_fraction_doctest",
    ("src/Groundings/subgrid_grounded_fraction.jl", 149): "test_reference_cases::test_effective_pressure_and_surface_doctests",
    ("src/Groundings/subgrid_grounded_fraction.jl", 192): "test_reference_cases::test_effective_pressure_and_surface_doctests",
    ("src/Models/smooth_ice_mask.jl", 23): "test_reference_cases_4::test_smooth_ice_mask_doctest",
    ("src/Models/ice_sheet_constants.jl", 22): "test_reference_cases_4::test_configuration_doctests",
    ("src/Grids/sigma_grid.jl", 8): "test_reference_cases_4::test_configuration_doctests",
    ("src/Grids/sigma_grid.jl", 32): "test_reference_cases_4::test_sigma_grid_doctest",
    ("src/Thermodynamics/enthalpy_conversions.jl", 20): "test_thermal_diagnostics::test_enthalpy_doctest",
}


def test_every_reference_doctest_is_restated():
    """The golden file holds the 28 doctests of the velocity solve's sources and of the enthalpy conversions,
    and each has its restating test."""
    import importlib
    found = {(d["file"], d["lines"][0]) for d in reference_doctests()}
    assert found == set(DOCTEST_RESTATEMENTS)
    for target in DOCTEST_RESTATEMENTS.values():
        module, name = target.split("::")
        assert callable(getattr(importlib.import_module(module), name)), target


@pytest.mark.gpu
def test_picard_adjoint_defaults_to_the_solver_adjoint_control(gpu_cls):
    """StressBalanceSolver(adjoint_iteration_control = ...) sets the control of Problem.picard_adjoint when none
    is passed (the reference's PicardIteration keeps it beside the forward control); an explicit control wins.
    The 40 x 20 marine sheet with Weertman drag of the adjoint finite-difference tests."""
    def run(adjoint_control, explicit=None):
        solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                       picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=500),
                                       preconditioner=M.StressBalanceDiagonalPreconditioner(),
                                       adjoint_iteration_control=adjoint_control)
        P = workloads.marine_sheet(40, 20, seed=2, seed_friction=1100, velocity_solver=solver).problem(gpu_cls)
        assert P.picard_solve().status == 0
        lu, _, _, _, st = P.picard_adjoint(1e-3 * P.get("u"), 1e-3 * P.get("v"), explicit)
        P.close()
        return lu, st
    _, st = run(M.FixedIterations(4))
    assert st.picard_iterations == 4
    _, st = run(M.FixedIterations(4), explicit=M.FixedIterations(2))
    assert st.picard_iterations == 2
    l_default, st_default = run(None)
    l_picard, st_picard = run(None, explicit=M.Convergence(reltol=1e-12, maxiter=500))
    assert st_default.status == 0 and st_default.picard_iterations == st_picard.picard_iterations
    assert np.array_equal(l_default, l_picard)
