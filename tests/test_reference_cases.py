"""The reference's own known answers, restated.  Each test follows a doctest or testset of Nunatak.jl
(file:line given) and runs on both backends: the FP64 CPU oracle (pins the oracle to the reference) and
the GPU library (marked gpu; checks the CUDA path against the same known answers)."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import evaluate, ice_sheet_model, isapprox, julia_value, make, reference_doctest, set_fn, vector_dot


def grid(size, x=(0.0, 1.0), y=(0.0, 1.0), topology=("Bounded", "Bounded"), halo=(3, 3)):
    return M.RectilinearGrid(size=size, x=x, y=y, topology=topology, halo=halo)


def coefficients_problem(cls, g, eta=lambda x, y: 1 + x**2 + math.sin(2 * math.pi * y)**2 / 2,
                         beta=lambda x, y: 1 + x * y, walls=None, **kw):
    """ssa_coefficients(grid; η̄H, β), test/test_ssa_operator.jl:6-18: η̄H and η̄Hᶠᶠ from the same function."""
    P = make(cls, g, stress_balance=M.DepthIntegrated(side_walls=walls or M.FreeSlipWalls()), masking=None, **kw)
    set_fn(P, "eta_H", eta)
    set_fn(P, "eta_H_ff", eta)
    set_fn(P, "beta_u", beta)
    set_fn(P, "beta_v", beta)
    return P


def apply(P, pu, pv):
    return P.apply_operator(evaluate(P.grid, "u", pu), evaluate(P.grid, "v", pv))


# ---- doctests ---------------------------------------------------------------------------------------
# The expected values are the doctests' printed outputs, read from tests/golden/reference_doctests.json.

def test_ssa_operator_doctest(backend):
    """src/StressBalances/ssa_operator.jl:20-45: rigid translation feels only the drag, 2 × 3 × (1/4)² = 0.375."""
    g = grid((4, 4), topology=("Periodic", "Periodic"))
    P = coefficients_problem(backend, g, eta=1.0, beta=2.0)
    qu, qv = apply(P, 3.0, 0.0)
    assert qu[0, 0] == julia_value(reference_doctest("src/StressBalances/ssa_operator.jl", 20)[0])   # 0.375


def test_driving_stress_doctests(backend):
    """src/StressBalances/driving_stress.jl:13-41."""
    g = grid((4, 4))
    expected = [julia_value(o) for o in reference_doctest("src/StressBalances/driving_stress.jl", 13)]
    c = M.IceSheetConstants(1.0, 1.0, 1.0)
    # s = x with H = 1 and no grounding treatment: s = b + H, so b = x - 1.
    P, _ = ice_sheet_model(backend, g, H=1.0, bed=lambda x, y: x - 1, masking=None, constants=c, solve=False)
    assert P.get("tau_u")[0, 1] == expected[0]   # -0.0625
    # Grounding line inside the face: b = -2x, H = 2 - 2x, s = max(2 - 4x, 1 - x) with ρw = 2.
    c2 = M.IceSheetConstants(1.0, 2.0, 1.0)
    P, _ = ice_sheet_model(backend, g, H=lambda x, y: 2 - 2 * x, bed=lambda x, y: -2 * x, masking=None, constants=c2,
                           grounding=M.SubgridGroundedFraction(driving_stress=True), solve=False)
    assert abs(P.get("tau_u")[0, 1] - expected[1]) < 1e-15   # 0.33463541666666663


def test_viscosity_doctest(backend):
    """src/Rheologies/glen_flow_law.jl:78-95: A = 1, n = 1 gives η = 1/2."""
    g = grid((4, 4), topology=("Periodic", "Periodic"))
    P = make(backend, g, Nsigma=3, rheology=M.GlenFlowLaw(rate_factor=1.0, exponent=1.0), masking=None)
    P.set("A", 1.0)
    P.update_coefficients()
    assert P.get("eta_sigma")[0, 0, 0] == julia_value(reference_doctest("src/Rheologies/glen_flow_law.jl", 78)[0])   # 0.5


def test_basal_drag_doctest(backend):
    """src/Frictions/frictions.jl:102-125: Weertman C = 2, u = 1, u₀ = 0 gives β = 2."""
    g = grid((4, 4), topology=("Periodic", "Periodic"))
    fr = M.WeertmanFriction(coefficient=2.0, velocity_regularization=0.0)
    P = make(backend, g, friction=fr, masking=None, use_effective_pressure=False)
    P.set("C", 2.0)
    P.set("A", 1e-24)
    P.set("phi_u", 1.0)
    P.set("phi_v", 1.0)
    P.set("u", 1.0)
    P.update_coefficients()
    assert P.get("beta_u")[0, 1] == julia_value(reference_doctest("src/Frictions/frictions.jl", 102)[0])   # 2.0


def test_grounded_fraction_doctest(backend):
    """src/Groundings/subgrid_grounded_fraction.jl:82-107: φ = [1, 0.75, 0, 0]."""
    g = grid((4, 1), x=(0.0, 4.0), topology=("Bounded", "Periodic"))
    c = M.IceSheetConstants(1.0, 1.0, 9.81)
    P, _ = ice_sheet_model(backend, g, H=100.0, bed=lambda x, y: -100 * (x - 0.75), constants=c,
                           grounding=M.SubgridGroundedFraction(), solve=False)
    np.testing.assert_array_equal(P.get("phi")[0], julia_value(reference_doctest("src/Groundings/subgrid_grounded_fraction.jl", 82)[0]))


def test_effective_pressure_and_surface_doctests(backend):
    """src/Groundings/subgrid_grounded_fraction.jl:149-166 (N = [10, 5]) and :192-209 (s = [80, 50])."""
    g = grid((2, 1), x=(0.0, 2.0), topology=("Bounded", "Periodic"))
    P, _ = ice_sheet_model(backend, g, H=10.0, bed=lambda x, y: 5.0 if x < 1 else -5.0,
                           constants=M.IceSheetConstants(1.0, 1.0, 1.0), grounding=M.SubgridGroundedFraction(), solve=False)
    np.testing.assert_array_equal(P.get("N")[0], julia_value(reference_doctest("src/Groundings/subgrid_grounded_fraction.jl", 149)[0]))
    P, _ = ice_sheet_model(backend, g, H=100.0, bed=lambda x, y: -20.0 if x < 1 else -500.0,
                           constants=M.IceSheetConstants(1.0, 2.0, 9.81), grounding=M.SubgridGroundedFraction(), solve=False)
    np.testing.assert_array_equal(P.get("s")[0], julia_value(reference_doctest("src/Groundings/subgrid_grounded_fraction.jl", 192)[0]))


def test_multigrid_levels(backend):
    """src/StressBalances/multigrid_preconditioner.jl:41-55 and test/test_multigrid_preconditioner.jl:30-37."""
    mg = M.StressBalanceSolver(preconditioner=M.StressBalanceMultigridPreconditioner())
    doc = [[(int(nx), int(ny)) for nx, ny, _ in julia_value(o)]
           for o in reference_doctest("src/StressBalances/multigrid_preconditioner.jl", 41)]
    cases = [((32, 16), ("Bounded", "Periodic"), (3, 3), doc[0]),     # (16, 8), (8, 4), (4, 4)
             ((64, 4), ("Bounded", "Bounded"), (4, 4), doc[1]),       # (32, 4), (16, 4), (8, 4), (4, 4)
             ((15, 8), ("Bounded", "Periodic"), (3, 3), [(15, 4)]),
             ((15, 5), ("Bounded", "Periodic"), (3, 3), [])]
    for size, topo, halo, levels in cases:
        P = make(backend, grid(size, topology=topo, halo=halo), velocity_solver=mg)
        assert P.multigrid_levels() == levels


def test_arrhenius_doctest(backend):
    """src/Rheologies/arrhenius_rate_factor.jl:89-100: A(253.15 K, ω = 0) ≈ 1.5e-25 (3 significant digits)."""
    g = grid((2, 2))
    P = make(backend, g, Nsigma=2, rheology=M.GlenFlowLaw(rate_factor="sigma"))
    P.set("H", 0.0)          # zero pressure, so T′ = T
    P.set("T", 253.15)
    P.compute_rate_factor()
    A = P.get("A")
    assert float(f"{A[0, 0, 0]:.2e}") == julia_value(reference_doctest("src/Rheologies/arrhenius_rate_factor.jl", 89)[0])


# ---- SSA operator (test/test_ssa_operator.jl) --------------------------------------------------------

def test_ssa_operator_symmetric_positive_and_cg_recovers(backend):
    """test/test_ssa_operator.jl:51-77 on a stretched Bounded x Periodic grid."""
    Nx, Ny = 12, 10
    xs = list(np.linspace(0, 1, Nx + 1) ** 1.3)
    g = grid((Nx, Ny), x=xs, topology=("Bounded", "Periodic"))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000), preconditioner=None)
    P = coefficients_problem(backend, g, velocity_solver=solver)
    pu = evaluate(g, "u", lambda x, y: math.sin(math.pi * x) * (math.cos(2 * math.pi * y) + 2))
    pv = evaluate(g, "v", lambda x, y: math.cos(2 * x) + math.sin(4 * math.pi * y) * x)
    yu = evaluate(g, "u", lambda x, y: x**2 - math.cos(2 * math.pi * y))
    yv = evaluate(g, "v", lambda x, y: math.exp(-x) * math.sin(2 * math.pi * y))
    Apu, Apv = P.apply_operator(pu, pv)
    Ayu, Ayv = P.apply_operator(yu, yv)
    a, b = vector_dot(g, Apu, Apv, yu, yv), vector_dot(g, pu, pv, Ayu, Ayv)
    assert abs(a - b) <= 1e-8 * max(abs(a), abs(b))
    assert vector_dot(g, Apu, Apv, pu, pv) > 0 and vector_dot(g, Ayu, Ayv, yu, yv) > 0
    P.set("u", 0.0)
    P.set("v", 0.0)
    P.linear_solve(Apu, Apv)
    xu, xv = P.get("u"), P.get("v")
    assert isapprox(xu, pu, rtol=1e-8)
    assert isapprox(xv, pv, rtol=1e-8)
    assert np.all(xu[:, [0, Nx]] == 0)


def manufactured_ssa_error(cls, N):
    """manufactured_ssa_error, test/test_ssa_operator.jl:27-49."""
    g = grid((N, N), topology=("Periodic", "Periodic"))
    eta0, beta0, a, b = 1.0, 1.0, 2 * math.pi, 4 * math.pi
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000), preconditioner=None)
    P = coefficients_problem(cls, g, eta=eta0, beta=beta0, velocity_solver=solver)
    A = 1 / N**2
    ue = lambda x, y: math.sin(a * x) * math.cos(b * y)
    ve = lambda x, y: math.cos(a * x) * math.sin(b * y)
    ru = evaluate(g, "u", lambda x, y: A * (eta0 * (4 * a**2 + b**2 + 3 * a * b) + beta0) * ue(x, y))
    rv = evaluate(g, "v", lambda x, y: A * (eta0 * (4 * b**2 + a**2 + 3 * a * b) + beta0) * ve(x, y))
    P.linear_solve(ru, rv)
    return max(np.max(np.abs(P.get("u") - evaluate(g, "u", ue))), np.max(np.abs(P.get("v") - evaluate(g, "v", ve))))


def test_manufactured_solution_second_order(backend):
    """test/test_ssa_operator.jl:79-82."""
    e = [manufactured_ssa_error(backend, N) for N in (32, 64)]
    assert e[1] < 5e-3
    assert e[0] / e[1] > 3.5


def test_free_slip_walls_rigid_translation(backend):
    """test/test_ssa_operator.jl:85-111."""
    Nx, Ny, b0, U = 6, 5, 2.0, 3.0
    for topology in (("Periodic", "Bounded"), ("Bounded", "Periodic")):
        g = grid((Nx, Ny), topology=topology)
        P = coefficients_problem(backend, g, beta=b0)
        along_x = topology[0] == "Periodic"
        qu, qv = apply(P, U if along_x else 0.0, 0.0 if along_x else U)
        q = qu if along_x else qv
        q = q[:Ny, :Nx] if along_x else q[:, :Nx]
        np.testing.assert_allclose(q, b0 * U / (Nx * Ny), rtol=1e-13)
    xs = list(np.linspace(0, 1, Nx + 1) ** 1.3)
    g = grid((Nx, Ny), x=xs)
    P = coefficients_problem(backend, g)
    pu, pv = evaluate(g, "u", lambda x, y: math.sin(math.pi * x) + y), evaluate(g, "v", lambda x, y: x * y**2)
    yu, yv = evaluate(g, "u", lambda x, y: math.cos(x) * y), evaluate(g, "v", lambda x, y: math.sin(3 * y) + x)
    Apu, Apv = P.apply_operator(pu, pv)
    Ayu, Ayv = P.apply_operator(yu, yv)
    a, b = vector_dot(g, Apu, Apv, yu, yv), vector_dot(g, pu, pv, Ayu, Ayv)
    assert abs(a - b) <= 1e-8 * abs(a)
    assert vector_dot(g, Apu, Apv, pu, pv) > 0


def channel_flow_error(cls, N, along_x=True, stretched=False):
    """channel_flow_error, test/test_ssa_operator.jl:113-139: Poiseuille flow between no-slip walls."""
    W, eta0, f = 1.0, 2.0, 3.0
    topology = ("Periodic", "Bounded") if along_x else ("Bounded", "Periodic")
    across = [W * (xi - 0.6 * math.sin(2 * math.pi * xi) / (2 * math.pi)) for xi in np.linspace(0, 1, N + 1)] if stretched else (0.0, W)
    g = grid((4, N) if along_x else (N, 4), x=(0.0, 1.0) if along_x else across, y=across if along_x else (0.0, 1.0), topology=topology)
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=10_000))
    P = coefficients_problem(cls, g, eta=eta0, beta=0.0, walls=M.NoSlipWalls(), velocity_solver=solver)
    # right-hand side f × the area of each velocity cell
    fx, fy = g.faces(0), g.faces(1)
    dxc, dyc = np.diff(fx), np.diff(fy)
    cx, cy = g.centers(0), g.centers(1)
    if along_x:
        dxf = np.diff(np.concatenate(([cx[-1] - (fx[-1] - fx[0])], cx)))   # periodic centre spacing at faces 1..N
        ru = f * np.outer(dyc, dxf)
        rv = np.zeros(P.shape("v"))
    else:
        dyf = np.diff(np.concatenate(([cy[-1] - (fy[-1] - fy[0])], cy)))
        ru = np.zeros(P.shape("u"))
        rv = f * np.outer(dyf, dxc)
    P.linear_solve(ru, rv)
    if along_x:
        U, Ue = P.get("u"), evaluate(g, "u", lambda x, y: f * y * (W - y) / (2 * eta0))
        cross = P.get("v")
    else:
        U, Ue = P.get("v"), evaluate(g, "v", lambda x, y: f * x * (W - x) / (2 * eta0))
        cross = P.get("u")
    return np.max(np.abs(U - Ue)) / np.max(np.abs(Ue)), np.max(np.abs(cross))


def test_no_slip_channel_poiseuille(backend):
    """test/test_ssa_operator.jl:141-148."""
    for along_x in (True, False):
        for stretched in (False, True):
            (e1, a1), (e2, a2) = channel_flow_error(backend, 16, along_x, stretched), channel_flow_error(backend, 32, along_x, stretched)
            assert e2 < (3e-3 if stretched else 2e-3)
            assert e1 / e2 > 3.5
            assert max(a1, a2) < 1e-12


def test_no_slip_stiffer_and_viscosity_symmetric(backend):
    """test/test_ssa_operator.jl:150-174."""
    Nx, Ny = 6, 5
    xs = list(np.linspace(0, 1, Nx + 1) ** 1.3)
    g = grid((Nx, Ny), x=xs)
    P = coefficients_problem(backend, g, walls=M.NoSlipWalls())
    Pf = coefficients_problem(backend, g, walls=M.FreeSlipWalls())
    pu, pv = evaluate(g, "u", lambda x, y: math.sin(math.pi * x) + y), evaluate(g, "v", lambda x, y: x * y**2)
    yu, yv = evaluate(g, "u", lambda x, y: math.cos(x) * y), evaluate(g, "v", lambda x, y: math.sin(3 * y) + x)
    Apu, Apv = P.apply_operator(pu, pv)
    Ayu, Ayv = P.apply_operator(yu, yv)
    a, b = vector_dot(g, Apu, Apv, yu, yv), vector_dot(g, pu, pv, Ayu, Ayv)
    assert abs(a - b) <= 1e-8 * abs(a)
    Fpu, Fpv = Pf.apply_operator(pu, pv)
    assert vector_dot(g, Apu, Apv, pu, pv) > vector_dot(g, pu, pv, Fpu, Fpv)

    channel = grid((4, 4), topology=("Periodic", "Bounded"))
    out = {}
    for walls in (M.FreeSlipWalls(), M.NoSlipWalls()):
        Q = make(backend, channel, Nsigma=2, rheology=M.GlenFlowLaw(rate_factor=1.0, exponent=3.0),
                 stress_balance=M.DepthIntegrated(side_walls=walls), masking=None)
        Q.set("A", 1.0)
        Q.set("u", 1.0)
        Q.update_coefficients()
        out[walls.code] = Q.get("eta_sigma")
    free, noslip = out[0], out[1]
    np.testing.assert_allclose(noslip[:, 0, :], noslip[:, 3, :], rtol=1e-14)
    assert np.all(noslip[:, 0, :] < free[:, 0, :])
    np.testing.assert_allclose(noslip[:, 1:3, :], free[:, 1:3, :], rtol=1e-14)


# ---- Glen viscosity and driving stress (test/test_glen_viscosity.jl) --------------------------------------

def uniform_strain_viscosity(cls, g, ue):
    P = make(cls, g, Nsigma=3, rheology=M.GlenFlowLaw(rate_factor=1.0, strain_rate_regularization=0.0), masking=None)
    P.set("A", 1.0)
    set_fn(P, "u", ue)
    P.update_coefficients()
    return P.get("eta_sigma")   # (Nσ, Ny, Nx)


def test_uniform_strain_viscosity(backend):
    """test/test_glen_viscosity.jl:48-55."""
    a = 2.0
    eta = uniform_strain_viscosity(backend, grid((8, 4), topology=("Bounded", "Periodic")), lambda x, y: a * x)
    np.testing.assert_allclose(eta[:, :, 1:7], a ** (-2 / 3) / 2, rtol=1e-12)
    eta = uniform_strain_viscosity(backend, grid((4, 8), topology=("Periodic", "Bounded")), lambda x, y: a * y)
    np.testing.assert_allclose(eta[:, 1:7, :], (a / 2) ** (-2 / 3) / 2, rtol=1e-12)


def test_driving_stress_closed_form(backend):
    """test/test_glen_viscosity.jl:57-72."""
    g = grid((6, 5), x=(0.0, 3.0))
    P, _ = ice_sheet_model(backend, g, H=lambda x, y: 1 + x, bed=lambda x, y: 2 * x + 3 * y - (1 + x), masking=None,
                           constants=M.IceSheetConstants(2.0, 2.0, 5.0), solve=False)
    Az = 0.5 * 0.2
    xf = np.arange(0.5, 2.5 + 1e-9, 0.5)
    xc = np.arange(0.25, 2.75 + 1e-9, 0.5)
    tu, tv = P.get("tau_u"), P.get("tau_v")
    np.testing.assert_allclose(tu[:, 1:6], np.tile(-Az * 10 * (1 + xf) * 2, (5, 1)), rtol=1e-12)
    np.testing.assert_allclose(tv[1:5, :], np.tile(-Az * 10 * (1 + xc) * 3, (4, 1)), rtol=1e-12)
    assert np.all(tu[:, [0, 6]] == 0) and np.all(tv[[0, 5], :] == 0)


def ice_stream_error(cls, Nx, L=100e3, H0=500.0, delta=20.0, rho=917.0, gacc=9.81, A=1e-24):
    """ice_stream_error, test/test_glen_viscosity.jl:14-45 (n = 3 analytic ice stream)."""
    g = grid((Nx, 4), x=(0.0, L), y=(0.0, L / Nx * 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-10, maxiter=300), preconditioner=None)
    s = lambda x, y: H0 + delta * math.cos(math.pi * x / L)
    P, st = ice_sheet_model(cls, g, H=H0, bed=lambda x, y: s(x, y) - H0, rheology=M.GlenFlowLaw(rate_factor=A),
                            masking=None, constants=M.IceSheetConstants(rho, rho, gacc), velocity_solver=solver, Nsigma=4)
    U = A * (rho * gacc * delta / 2) ** 3 * L / math.pi
    ue = evaluate(g, "u", lambda x, y: U * (math.sin(math.pi * x / L) - math.sin(math.pi * x / L) ** 3 / 3))
    err = np.max(np.abs(P.get("u") - ue)) / (2 * U / 3)
    return err, st.picard_iterations, np.max(np.abs(P.get("v"))) / (2 * U / 3)


def test_ice_stream_n3(backend):
    """test/test_glen_viscosity.jl:74-80."""
    r = [ice_stream_error(backend, N) for N in (32, 64)]
    assert all(it < 300 for _, it, _ in r)
    assert all(v < 1e-10 for _, _, v in r)
    assert r[1][0] < 1e-3
    assert r[0][0] / r[1][0] > 3.5


# ---- friction and diagonal preconditioner (test/test_friction.jl) ------------------------------------------

def uniform_drag(cls, friction, U, phi0=1.0, N0=None):
    g = grid((4, 4), topology=("Periodic", "Periodic"))
    P = make(cls, g, friction=friction, masking=None, use_effective_pressure=N0 is not None)
    P.set("A", 1e-24)
    P.set("C", friction.coefficient)
    P.set("phi_u", phi0)
    P.set("phi_v", phi0)
    if N0 is not None:
        P.set("N", N0)
    P.set("u", U)
    P.update_coefficients()
    return P.get("beta_u")


def test_friction_laws(backend):
    """test/test_friction.jl:59-68."""
    m, C, U = 1 / 3, 3e4, 1e-5
    w = M.WeertmanFriction(coefficient=C, exponent=m, velocity_regularization=0.0)
    np.testing.assert_allclose(uniform_drag(backend, w, U), C * U ** (m - 1), rtol=1e-12)
    np.testing.assert_allclose(uniform_drag(backend, w, U, phi0=0.5), C * U ** (m - 1) / 2, rtol=1e-12)
    a2, N0 = 0.5, 1e6
    c = M.RegularizedCoulombFriction(coefficient=C, coulomb_coefficient=a2, exponent=m, velocity_regularization=0.0)
    assert abs(uniform_drag(backend, c, 1e-12, N0=N0)[0, 0] / (C * 1e-12 ** (m - 1)) - 1) < 1e-3
    assert abs(uniform_drag(backend, c, 1e8, N0=N0)[0, 0] * 1e8 / (a2 * N0) - 1) < 1e-3


def sliding_slab_speed(cls, friction, tau0, N0):
    """sliding_slab_speed, test/test_friction.jl:18-40."""
    g = grid((4, 4), x=(0.0, 1e3), y=(0.0, 1e3), topology=("Periodic", "Periodic"))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=100),
                                   picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=300), preconditioner=None)
    P = make(cls, g, Nsigma=2, friction=friction, masking=None, velocity_solver=solver)
    P.set("H", 500.0)
    P.set("phi_u", 1.0)
    P.set("phi_v", 1.0)
    P.set("N", N0)
    P.set("A", 1e-24)
    P.set("C", friction.coefficient)
    P.set("tau_u", tau0 * 250**2)
    st = P.picard_solve()
    return P.get("u"), st.picard_iterations


def test_sliding_slab(backend):
    """test/test_friction.jl:70-81."""
    m, C, N0, tau0 = 1 / 3, 3e4, 1e6, 1e5
    u, it = sliding_slab_speed(backend, M.WeertmanFriction(coefficient=C, exponent=m, velocity_regularization=1e-12), tau0, N0)
    assert it < 300
    np.testing.assert_allclose(u, (tau0 / C) ** (1 / m), rtol=1.5e-8)
    a2 = 0.5
    u, it = sliding_slab_speed(backend, M.RegularizedCoulombFriction(coefficient=C, coulomb_coefficient=a2, exponent=m,
                                                                     velocity_regularization=1e-12), tau0, N0)
    tc = a2 * N0
    Ue = (tau0 * tc) ** (1 / m) / (C ** (1 / m) * (tc ** (1 / m) - tau0 ** (1 / m)))
    assert it < 300
    np.testing.assert_allclose(u, Ue, rtol=1.5e-8)


def test_diagonal_preconditioner_is_operator_diagonal(backend):
    """test/test_friction.jl:83-95: z = r / diag with the diagonal probed by unit vectors."""
    Nx, Ny = 7, 6
    xs = list(np.linspace(0, 1, Nx + 1) ** 1.4)
    g = grid((Nx, Ny), x=xs)
    for walls in (M.FreeSlipWalls(), M.NoSlipWalls()):
        P = coefficients_problem(backend, g, walls=walls)
        du, dv = np.zeros(P.shape("u")), np.zeros(P.shape("v"))
        for comp, d in (("u", du), ("v", dv)):
            ny, nx = d.shape
            for j in range(ny):
                for i in range(nx):
                    eu, ev = np.zeros(P.shape("u")), np.zeros(P.shape("v"))
                    (eu if comp == "u" else ev)[j, i] = 1.0
                    qu, qv = P.apply_operator(eu, ev)
                    d[j, i] = (qu if comp == "u" else qv)[j, i]
        zu, zv = P.precondition(np.ones(P.shape("u")), np.ones(P.shape("v")))
        np.testing.assert_allclose(zu[:, 1:Nx] * du[:, 1:Nx], 1.0, rtol=1e-13)
        np.testing.assert_allclose(zv[1:Ny, :] * dv[1:Ny, :], 1.0, rtol=1e-13)


def test_jacobi_beats_plain_cg(backend):
    """test/test_friction.jl:97-110."""
    g = grid((48, 32), topology=("Bounded", "Periodic"))
    control = M.Convergence(reltol=1e-10, maxiter=10_000)
    res = {}
    for name, pre in (("plain", None), ("jacobi", M.StressBalanceDiagonalPreconditioner())):
        P = coefficients_problem(backend, g, eta=lambda x, y: 1 + 1e3 * x**4, beta=lambda x, y: 1e4 * math.exp(-20 * x),
                                 velocity_solver=M.StressBalanceSolver(linear_iteration_control=control, preconditioner=pre))
        st = P.linear_solve(evaluate(g, "u", lambda x, y: math.sin(math.pi * x) * math.cos(2 * math.pi * y)),
                            evaluate(g, "v", lambda x, y: x * math.sin(2 * math.pi * y)))
        res[name] = (st.linear_iterations_last, P.get("u"))
    assert res["jacobi"][0] < res["plain"][0]
    assert isapprox(res["jacobi"][1], res["plain"][1], rtol=1e-7)
