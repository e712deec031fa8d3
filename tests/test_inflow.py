"""Prescribed velocities: an inflow boundary, an extension with no counterpart in the reference.

The reference's Bounded walls are impenetrable (u = 0 on the wall faces, which are identity rows and are
masked out of the strain rates).  NK_FIELD_U_PRESCRIBED / NK_FIELD_V_PRESCRIBED turn faces of the solved rows
into identity rows x = u_D whose value still enters the neighbouring strain rates, viscosity and stresses (the
lifting of a Dirichlet condition).  The oracle restates the same rule (prescribed_fc / prescribed_cf in
oracle/nunatak_oracle.cpp).  Workload: the 84 x 40 floating channel shelf with 100 m/yr at x = 0.

On both backends (the oracle on the CPU, the GPU library marked gpu):
- the prescribed faces hold u_D exactly after the solve, and the driving stress there is u_D;
- u_D = 0 on the west faces gives bit for bit the solution without prescribed faces (the reference's wall);
- a value on the east boundary faces (no solved row) changes nothing;
- the converged solution satisfies A x = τ (relative residual ≤ 1e-8 of ‖τ‖, exactly on the prescribed faces).
GPU against the oracle (relative L2 of the velocities, the tolerances of the other parity tests): the channel
inflow with Picard(3) x CG(40) fixed ≤ 1e-10 and converged tightly ≤ 1e-10; the marine sheet with a west
inflow on the FP64 multigrid ≤ 1e-10 (fixed) and mixed precision ≤ 1e-6 (converged); a periodic-x sheet with
prescribed u and v faces inside the domain and across the wrap ≤ 1e-10; DIVA ≤ 1e-10 (fixed).  The adjoint
entry points refuse problems with prescribed faces."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from nunatak_gb300 import workloads

YEAR = M.YEAR
TIGHT = dict(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
             picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=300))


def rel_l2(ua, va, ub, vb):
    return math.sqrt(np.sum((ua - ub) ** 2) + np.sum((va - vb) ** 2)) / math.sqrt(np.sum(ub ** 2) + np.sum(vb ** 2))


def _with(case, name, **fields):
    return workloads.Case(name, case.grid, case.config, dict(case.fields, **fields), dict(case.initial), case.temperature)


def test_inflow_faces_hold_the_prescribed_velocity(backend):
    P = workloads.channel_shelf(inflow=100.0).problem(backend)
    assert np.all(P.get("tau_u")[:, 0] == 100.0 / YEAR)
    st = P.picard_solve()
    assert st.status == 0 and st.picard_iterations > 1
    u = P.get("u")
    assert np.all(u[:, 0] == 100.0 / YEAR)
    assert np.all(np.isnan(P.get("u_prescribed")[:, 1:])) and np.all(np.isnan(P.get("v_prescribed")))
    # ice enters at the west face and is faster everywhere than behind the impenetrable wall
    P0 = workloads.channel_shelf().problem(backend)
    P0.picard_solve()
    assert np.all(u[:, 1:80] > P0.get("u")[:, 1:80])


def test_zero_inflow_is_the_reference_wall(backend):
    """u_D = 0 on the west faces: identity rows with b = 0 whose value 0 enters the strain rates, exactly what the
    masked wall gives, so the solution is bit for bit the reference's."""
    runs = []
    for inflow in (None, 0.0):
        P = workloads.channel_shelf(inflow=inflow).problem(backend)
        st = P.picard_solve()
        runs.append((P.get("u"), P.get("v"), st.picard_iterations, st.linear_iterations_total))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    assert runs[0][2:] == runs[1][2:]


def test_east_boundary_values_are_ignored(backend):
    """The east boundary faces (i = Nx) are no solved row: a value there prescribes nothing."""
    base = workloads.channel_shelf(inflow=100.0)
    ud = base.fields["u_prescribed"].copy()
    ud[:, -1] = 50.0 / YEAR
    runs = []
    for case in (base, _with(base, "east", u_prescribed=ud)):
        P = case.problem(backend)
        P.picard_solve()
        runs.append((P.get("u"), P.get("v")))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])
    assert np.all(runs[1][0][:, -1] == 0.0)


def test_converged_inflow_solves_the_lifted_system(backend):
    solver = M.StressBalanceSolver(**TIGHT)
    P = workloads.channel_shelf(inflow=100.0, velocity_solver=solver).problem(backend)
    assert P.picard_solve().status == 0
    u, v = P.get("u"), P.get("v")
    qu, qv = P.apply_operator(u, v)
    tu, tv = P.get("tau_u"), P.get("tau_v")
    assert np.all(qu[:, 0] == tu[:, 0])
    r = math.sqrt(np.sum((qu[:, :-1] - tu[:, :-1]) ** 2) + np.sum((qv[:-1, :] - tv[:-1, :]) ** 2))
    assert r <= 1e-8 * math.sqrt(np.sum(tu ** 2) + np.sum(tv ** 2))


def _solve_both(oracle_cls, gpu_cls, case):
    res = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P = case.problem(cls)
        st = P.picard_solve()
        res[key] = (P.get("u"), P.get("v"), st)
    return res


@pytest.mark.gpu
def test_channel_inflow_fixed_iterations_matches_oracle(oracle_cls, gpu_cls):
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(40), picard_iteration_control=M.FixedIterations(3))
    r = _solve_both(oracle_cls, gpu_cls, workloads.channel_shelf(inflow=100.0, velocity_solver=solver))
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10


@pytest.mark.gpu
def test_channel_inflow_converged_matches_oracle(oracle_cls, gpu_cls):
    r = _solve_both(oracle_cls, gpu_cls, workloads.channel_shelf(inflow=100.0, velocity_solver=M.StressBalanceSolver(**TIGHT)))
    assert r["g"][2].status == 0 and r["o"][2].status == 0
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10
    assert abs(r["g"][2].picard_iterations - r["o"][2].picard_iterations) <= 1


def _sheet_inflow(solver):
    base = workloads.marine_sheet(64, 32, seed=2, velocity_solver=solver)
    return _with(base, "marine_sheet_inflow", u_prescribed=workloads.west_inflow(base.grid, 50.0))


@pytest.mark.gpu
def test_sheet_inflow_multigrid_fp64_fixed_matches_oracle(oracle_cls, gpu_cls):
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(25), picard_iteration_control=M.FixedIterations(3),
                                   preconditioner=mg)
    r = _solve_both(oracle_cls, gpu_cls, _sheet_inflow(solver))
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10
    assert np.all(r["g"][0][:, 0] == 50.0 / YEAR)


@pytest.mark.gpu
def test_sheet_inflow_mixed_precision_vs_fp64_oracle(oracle_cls, gpu_cls):
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)
    tight = dict(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=2000),
                 picard_iteration_control=M.Convergence(reltol=1e-9, maxiter=300), preconditioner=mg)
    ref = _sheet_inflow(M.StressBalanceSolver(**tight)).problem(oracle_cls)
    assert ref.picard_solve().status == 0
    P = _sheet_inflow(M.StressBalanceSolver(precision="mixed", **tight)).problem(gpu_cls)
    st = P.picard_solve()
    assert st.status == 0
    assert rel_l2(P.get("u"), P.get("v"), ref.get("u"), ref.get("v")) < 1e-6
    assert np.all(P.get("u")[:, 0] == 50.0 / YEAR)


@pytest.mark.gpu
@pytest.mark.parametrize("smoother", [M.PointJacobi(), M.LineJacobi()])
def test_periodic_interior_prescribed_faces_match_oracle(oracle_cls, gpu_cls, smoother):
    """Periodic x: u prescribed on the column i = 0 (neighbour of i = Nx - 1 across the wrap) and at an interior
    column, v on part of one row."""
    nx, ny = 40, 20
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4, smoother=smoother)
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(25), picard_iteration_control=M.FixedIterations(3),
                                   preconditioner=mg)
    base = workloads.marine_sheet(nx, ny, seed=2, velocity_solver=solver)
    grid = M.RectilinearGrid(size=(nx, ny), x=(0.0, 512e3), y=(0.0, 256e3), halo=(4, 4), topology=("Periodic", "Bounded"))
    ud = np.full((ny, nx), np.nan)
    ud[:, 0] = 80.0 / YEAR
    ud[4:16, 17] = 40.0 / YEAR
    vd = np.full((ny + 1, nx), np.nan)
    vd[6, 5:15] = -20.0 / YEAR
    case = workloads.Case("periodic_prescribed", grid, base.config, dict(base.fields, u_prescribed=ud, v_prescribed=vd))
    r = _solve_both(oracle_cls, gpu_cls, case)
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10
    assert np.all(r["g"][0][:, 0] == 80.0 / YEAR) and np.all(r["g"][1][6, 5:15] == -20.0 / YEAR)


@pytest.mark.gpu
def test_diva_inflow_fixed_iterations_matches_oracle(oracle_cls, gpu_cls):
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(30), picard_iteration_control=M.FixedIterations(3),
                                   preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4))
    base = workloads.diva_sheet(64, 32, dx=32e3, velocity_solver=solver, Nsigma=6)
    case = _with(base, "diva_inflow", u_prescribed=workloads.west_inflow(base.grid, 50.0))
    res = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P = case.problem(cls)
        P.picard_solve()
        P.velocity_profile()
        res[key] = {k: P.get(k) for k in ("u", "v", "u_sigma", "u_b")}
    assert rel_l2(res["g"]["u"], res["g"]["v"], res["o"]["u"], res["o"]["v"]) < 1e-10
    for k in ("u_sigma", "u_b"):
        a, b = res["g"][k], res["o"][k]
        assert np.linalg.norm(a - b) <= 1e-10 * np.linalg.norm(b), k


@pytest.mark.gpu
def test_adjoints_refuse_prescribed_faces(gpu_cls):
    P = workloads.channel_shelf(inflow=100.0).problem(gpu_cls)
    P.picard_solve()
    u, v = P.get("u"), P.get("v")
    with pytest.raises(ValueError):
        P.picard_adjoint(u, v, M.Convergence(reltol=1e-8, maxiter=10))
    with pytest.raises(ValueError):
        P.adjoint_solve(u, v)
