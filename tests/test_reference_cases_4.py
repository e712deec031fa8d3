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
