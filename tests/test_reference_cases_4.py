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
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from nunatak_gb300 import workloads
from support import evaluate, isapprox, make, set_fn, vector_dot

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
    assert (zu.min(), zu.max()) == (1.5, 1.5) and (zv.min(), zv.max()) == (1.5, 1.5)


def test_solve_and_adjoint_solve_doctests(backend):
    """src/Solvers/conjugate_gradient.jl:109-126 (solve!) and :136-153 (adjoint_solve!): A = 2I, b = 1 gives
    x = λ = 0.5 everywhere, starting from zero."""
    P = _doctest_problem(backend, 0.125, 32.0)
    one_u, one_v = np.ones(P.shape("u")), np.ones(P.shape("v"))
    qu, qv = P.apply_operator(one_u, one_v)
    assert np.all(qu == 2.0) and np.all(qv == 2.0)
    for adjoint in (False, True):
        xu, xv, st = _solve(P, one_u, one_v, adjoint=adjoint)
        assert st.status == 0 and st.linear_iterations_last == 1
        assert (xu.min(), xu.max()) == (0.5, 0.5) and (xv.min(), xv.max()) == (0.5, 0.5)


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

def test_configuration_doctests():
    """The reference's constructor doctests, on the host-side mirrors of its configuration objects:
    Convergence(; reltol = 1e-10, maxiter = 50) = (1e-10, 0, 50) (src/Solvers/iteration_controls.jl:21-26);
    DepthIntegrated(side_walls = NoSlipWalls()) is SSA with no-slip walls (src/StressBalances/depth_integrated.jl:22-27);
    WeertmanFriction(grid; coefficient = 3e4).exponent = 1/3 (src/Frictions/frictions.jl:23-32);
    GlenFlowLaw(grid; rate_factor = 1e-24).exponent = 3 (src/Rheologies/glen_flow_law.jl:25-34);
    IceSheetConstants(grid) has ρw/ρᵢ = 1.1198257080610021 (src/Models/ice_sheet_constants.jl:22-31);
    the adjoint control defaults to the Picard control (src/Solvers/picard.jl:27-34,
    src/StressBalances/stress_balance_solver.jl:46); the solver's linear control is the one given
    (src/Solvers/conjugate_gradient.jl:80-91, src/StressBalances/stress_balance_solver.jl:29-41 for the Picard one)."""
    c = M.Convergence(reltol=1e-10, maxiter=50)
    assert (c.reltol, c.abstol, c.maxiter) == (1e-10, 0.0, 50)
    d = M.DepthIntegrated(side_walls=M.NoSlipWalls())
    assert d.shear is None and isinstance(d.side_walls, M.NoSlipWalls)
    assert M.WeertmanFriction(coefficient=3e4).exponent == 0.3333333333333333
    assert M.GlenFlowLaw(rate_factor=1e-24).exponent == 3.0
    k = M.IceSheetConstants()
    assert k.ocean_density / k.ice_density == 1.1198257080610021
    s = M.StressBalanceSolver(picard_iteration_control=M.Convergence(reltol=1e-8))
    assert s.adjoint_control == M.Convergence(reltol=1e-8, abstol=0.0, maxiter=1000)
    assert M.StressBalanceSolver(picard_iteration_control=M.FixedIterations(5)).picard_iteration_control == M.FixedIterations(5)
    assert M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(2)).linear_iteration_control == M.FixedIterations(2)
    desc = M.make_descriptors(toy_grid(), velocity_solver=M.StressBalanceSolver(adjoint_iteration_control=M.FixedIterations(7)))
    assert desc.adjoint_control == M.FixedIterations(7)


def test_velocity_vector_doctest(backend):
    """src/Solvers/velocity_vector.jl:22-31: on a 4 x 3 Periodic x Bounded grid u holds 4 x 3 and v 4 x 4 values."""
    g = M.RectilinearGrid(size=(4, 3), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Periodic", "Bounded"), halo=(3, 3))
    P = make(backend, g, masking=None)
    assert P.shape("u") == (3, 4) and P.shape("v") == (4, 4)   # numpy (y, x) order
    assert P.get("u").shape == (3, 4) and P.get("v").shape == (4, 4)


def test_smooth_ice_mask_doctest(backend):
    """src/Models/smooth_ice_mask.jl:23-39: minimum 1, transition 2 gives μ = 0, 0, 0.5, 1, 1 for
    H = 0.5, 1, 2, 3, 10."""
    g = M.RectilinearGrid(size=(5, 1), x=(0.0, 5.0), y=(0.0, 1.0), topology=("Bounded", "Periodic"), halo=(3, 3))
    Hs = [0.5, 1.0, 2.0, 3.0, 10.0]
    P = make(backend, g, masking=M.SmoothIceMask(minimum_thickness=1.0, transition_thickness=2.0))
    P.set("H", np.array([Hs]))
    P.set("bed", 0.0)
    P.compute_geometry()
    assert P.get("ice_mask")[0].tolist() == [0.0, 0.0, 0.5, 1.0, 1.0]


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
