"""More of the reference's own known answers, restated from test/test_rate_factor.jl, test/test_sigma_grid.jl and
test/test_model.jl (file:line given per test).  Each runs on both backends: the FP64 CPU oracle and the GPU library
(marked gpu)."""
import math

import numpy as np

from nunatak_gb300 import model as M
from support import make


def grid(size, x=(0.0, 1.0), y=(0.0, 1.0), topology=("Bounded", "Bounded"), halo=(4, 4)):
    return M.RectilinearGrid(size=size, x=x, y=y, topology=topology, halo=halo)


# Paterson-Budd branches of the Arrhenius law with the reference's constants (test/test_rate_factor.jl:7-8).
def cold_branch(t):
    return 3.61e-13 * math.exp(-6.0e4 / (8.31441 * t))


def warm_branch(t):
    return 1.73e3 * math.exp(-13.9e4 / (8.31441 * t))


def sigma_nodes(Nsigma, refinement=2.0):
    """Faces (k / Nσ)^refinement and the layer centres (sigma_faces, src/Grids/sigma_grid.jl:20-22)."""
    f = np.array([(k / Nsigma) ** refinement for k in range(Nsigma + 1)])
    return f, (f[1:] + f[:-1]) / 2


def rate_factor_at(cls, temperatures, H=0.0, Nsigma=1, clausius_clapeyron=0.0, ice_density=918.0):
    """A from nk_compute_rate_factor for one temperature per cell (a row of cells, Nσ layers)."""
    t = np.asarray(temperatures, dtype=np.float64)
    g = grid((t.size, 1), x=(0.0, float(t.size)))
    P = make(cls, g, Nsigma=Nsigma, rheology=M.GlenFlowLaw(rate_factor="sigma"),
             constants=M.IceSheetConstants(ice_density=ice_density))
    P.set("H", H)
    P.set("T", np.broadcast_to(t.reshape(1, 1, -1), (Nsigma, 1, t.size)))
    P.compute_rate_factor(clausius_clapeyron=clausius_clapeyron)
    return P.get("A")


def test_arrhenius_values(backend):
    """test/test_rate_factor.jl:70-79: A(T', ω = 0) equals the cold branch below 263.15 K and the warm one above,
    to 1e-13 (zero pressure, so T' = T)."""
    cold, warm = (223.15, 243.15, 262.6), (263.7, 268.15, 273.15)
    A = rate_factor_at(backend, cold + warm)[0, 0]
    for k, t in enumerate(cold):
        assert abs(A[k] - cold_branch(t)) <= 1e-13 * cold_branch(t), t
    for k, t in enumerate(warm):
        assert abs(A[3 + k] - warm_branch(t)) <= 1e-13 * warm_branch(t), t


def test_arrhenius_smooth_transition(backend):
    """test/test_rate_factor.jl:81-89: across 262-264 K A rises monotonically, log A has no kink, and at the
    transition temperature A is the geometric mean of the two branches."""
    t = np.linspace(262.0, 264.0, 2001)
    A = rate_factor_at(backend, t)[0, 0]
    assert np.all(np.diff(A) > 0)
    slope = np.diff(np.log(A)) / (t[1] - t[0])
    assert np.max(np.abs(np.diff(slope))) * 2000 / 2 < 1
    mid = rate_factor_at(backend, [263.15])[0, 0, 0]
    ref = math.sqrt(cold_branch(263.15) * warm_branch(263.15))
    assert abs(mid - ref) <= 1e-13 * ref


def test_rate_factor_with_pressure_melting(backend):
    """test/test_rate_factor.jl:166-174: with the Clausius-Clapeyron slope β, T' = T + β ρ g H (1 - ζ), and A is
    the cold branch there (ρ = 910, H = 1000 m, T = 253.15 K), to 1e-12."""
    Nsigma, beta, rho, H = 10, 7.9e-8, 910.0, 1000.0
    A = rate_factor_at(backend, [253.15] * 4, H=H, Nsigma=Nsigma, clausius_clapeyron=beta, ice_density=rho)
    _, zeta = sigma_nodes(Nsigma)
    g = M.IceSheetConstants().gravitational_acceleration
    expected = np.array([cold_branch(253.15 + beta * rho * g * H * (1 - z)) for z in zeta])
    for cell in range(4):
        np.testing.assert_allclose(A[:, 0, cell], expected, rtol=1e-12)


def _viscosity_problem(cls, Nsigma, rate_factor, diva=False):
    g = grid((8, 8), x=(0.0, 1e5), y=(0.0, 1e5), topology=("Periodic", "Periodic"))
    sb = M.DepthIntegrated(shear=M.DIVAShear()) if diva else M.DepthIntegrated()
    P = make(cls, g, Nsigma=Nsigma, stress_balance=sb, rheology=M.GlenFlowLaw(rate_factor=rate_factor),
             friction=M.WeertmanFriction(coefficient=1e10, exponent=1.0), use_effective_pressure=False, masking=None)
    x = g.faces(0)[:-1]
    y = g.faces(1)[:-1]
    P.set("u", np.broadcast_to(1e-6 * np.sin(2 * np.pi * x / 1e5), (8, 8)))
    P.set("v", np.broadcast_to((2e-6 * np.cos(2 * np.pi * y / 1e5)).reshape(-1, 1), (8, 8)))
    P.set("H", 1000.0)
    P.set("C", 1e10)
    P.set("phi_u", 1.0)
    P.set("phi_v", 1.0)
    return P


def test_uniform_sigma_rate_factor_equals_the_2d_one(backend):
    """test/test_rate_factor.jl:91-115: a σ-grid A of uniform value gives the same layer viscosities, bit for bit,
    as the 2-D A of that value, for the SSA and the DIVA viscosity."""
    Nsigma = 4
    for diva in (False, True):
        P2 = _viscosity_problem(backend, Nsigma, 1e-24, diva)
        P3 = _viscosity_problem(backend, Nsigma, "sigma", diva)
        P2.set("A", 1e-24)
        P3.set("A", np.full(P3.shape("A"), 1e-24))
        for _ in range(2 if diva else 1):   # the second DIVA update uses its lagged basal drag
            P2.update_coefficients()
            P3.update_coefficients()
        assert np.array_equal(P2.get("eta_sigma"), P3.get("eta_sigma")), diva


def test_depth_varying_rate_factor_reaches_the_column_integrals(backend):
    """test/test_rate_factor.jl:117-145: with A(ζ) = A₀ (1 + 7ζ) the layer viscosities scale as (1 + 7ζ)^(-1/3),
    η̄H = H η₀ Σ Δζ (1 + 7ζ)^(-1/3) and F₂ = H Σ wₖ (1 + 7ζ)^(1/3) / η₀ with wₖ the exact layer integrals of
    (1 - ζ)², all to 1e-13."""
    Nsigma, A0 = 8, 1e-24
    P0 = _viscosity_problem(backend, Nsigma, A0)
    P0.set("v", 0.0)
    P0.set("A", A0)
    P0.update_coefficients()
    eta0 = P0.get("eta_sigma")[0, 2, 2]
    P = _viscosity_problem(backend, Nsigma, "sigma")
    P.set("v", 0.0)
    faces, zeta = sigma_nodes(Nsigma)
    P.set("A", np.broadcast_to((A0 * (1 + 7 * zeta)).reshape(-1, 1, 1), P.shape("A")))
    P.update_coefficients()
    scale = (1 + 7 * zeta) ** (-1.0 / 3.0)
    np.testing.assert_allclose(P.get("eta_sigma")[:, 2, 2], eta0 * scale, rtol=1e-13)
    dz = np.diff(faces)
    assert abs(P.get("eta_H")[2, 2] - 1000 * eta0 * np.sum(dz * scale)) <= 1e-13 * 1000 * eta0 * np.sum(dz * scale)
    w = ((1 - faces[:-1]) ** 3 - (1 - faces[1:]) ** 3) / 3
    F2 = 1000 * np.sum(w / scale) / eta0
    assert abs(P.get("F2")[2, 2] - F2) <= 1e-13 * F2


def depth_varying_slab_error(cls, Nsigma, H0=1000.0, tau0=1e4, A0=1e-21, C=1e10):
    """depth_varying_slab_error, test/test_rate_factor.jl:11-50: the DIVA slab with A(ζ) = A₀ (1 + 3 (1 - ζ)),
    whose exact profile is u = uᵇ + U (17/20 - s⁴/4 - 3 s⁵/5), s = 1 - ζ, U = 2 A₀ τ₀³ H₀, uᵇ = τ₀ / C."""
    g = grid((4, 4), x=(0.0, 4e3), y=(0.0, 4e3), topology=("Periodic", "Periodic"))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=100),
                                   picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=300), preconditioner=None)
    P = make(cls, g, Nsigma=Nsigma, stress_balance=M.DepthIntegrated(shear=M.DIVAShear()),
             rheology=M.GlenFlowLaw(rate_factor="sigma", strain_rate_regularization=1e-16),
             friction=M.WeertmanFriction(coefficient=C, exponent=1.0), masking=None, use_effective_pressure=False,
             velocity_solver=solver)
    _, zeta = sigma_nodes(Nsigma)
    P.set("H", H0)
    P.set("phi_u", 1.0)
    P.set("phi_v", 1.0)
    P.set("A", np.broadcast_to((A0 * (1 + 3 * (1 - zeta))).reshape(-1, 1, 1), P.shape("A")))
    P.set("C", C)
    P.set("tau_u", tau0 * 1e3**2)
    st = P.picard_solve()
    P.velocity_profile()
    ub, U = tau0 / C, 2 * A0 * tau0**3 * H0
    s = 1 - zeta
    exact = ub + U * (17 / 20 - s**4 / 4 - 3 * s**5 / 5)
    us = P.get("u_sigma")[:, 0, 0]
    return dict(iterations=st.picard_iterations, profile=np.max(np.abs(us - exact)) / U,
                mean=np.max(np.abs(P.get("u") - (ub + 7 * U / 10))) / (7 * U / 10))


def test_diva_shear_follows_a_depth_varying_rate_factor(backend):
    """test/test_rate_factor.jl:147-155."""
    coarse, fine = depth_varying_slab_error(backend, 10), depth_varying_slab_error(backend, 40)
    assert 0 < fine["iterations"] < 300
    assert fine["profile"] < 1e-2
    assert fine["mean"] < 1e-2
    assert fine["profile"] < coarse["profile"] / 4


def test_sigma_grid_column_integrals(backend):
    """test/test_sigma_grid.jl:3-22: on a 7-layer σ grid (bed refinement 2) the layer thicknesses sum to 1, and a
    uniform layer viscosity η gives η̄H = η H and F₂ = H / (3η)."""
    faces, _ = sigma_nodes(7)
    assert abs(np.sum(np.diff(faces)) - 1) <= 1e-15
    g = grid((4, 3), topology=("Periodic", "Bounded"))
    P = make(backend, g, Nsigma=7, rheology=M.GlenFlowLaw(rate_factor=1e-24), masking=None)
    xc = g.centers(0)
    H = np.broadcast_to(1000 + 500 * xc, (3, 4))
    P.set("H", H)
    P.set("A", 1e-24)
    P.update_coefficients()          # u = v = 0: every layer has the same viscosity η
    eta = P.get("eta_sigma")
    assert np.all(eta == eta[0, 0, 0])
    e = eta[0, 0, 0]
    np.testing.assert_allclose(P.get("eta_H"), e * H, rtol=1e-14)
    np.testing.assert_allclose(P.get("F2"), H / (3 * e), rtol=1e-14)


# ---- the model-level velocity update (test/test_model.jl) ------------------------------------------------------

def test_model_diva_update(backend):
    """test/test_model.jl:87-111.  Without basal drag DIVA reduces to the SSA: the n = 3 ice stream to 1e-3, uᵇ = ū
    and every layer of uσ equal to ū.  With Weertman drag (C = 1e12, m = 1) on a sloped sheet DIVA flows more than
    twice as fast as the SSA, |uᵇ| ≤ |ū|, and the layer velocities average to ū within 1e-2."""
    from support import ice_sheet_model
    L, Nx, H0, delta, rho, A = 100e3, 64, 500.0, 20.0, 917.0, 1e-24
    g = grid((Nx, 4), x=(0.0, L), y=(0.0, L / Nx * 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-10, maxiter=300))
    c = M.IceSheetConstants(ice_density=rho)
    P, st = ice_sheet_model(backend, g, H=H0, bed=lambda x, y: delta * math.cos(math.pi * x / L),
                            rheology=M.GlenFlowLaw(rate_factor=A), stress_balance=M.DepthIntegrated(shear=M.DIVAShear()),
                            constants=c, velocity_solver=solver, Nsigma=4)
    U = A * (rho * c.gravitational_acceleration * delta / 2) ** 3 * L / math.pi
    xf = g.faces(0)
    ue = np.broadcast_to(U * (np.sin(np.pi * xf / L) - np.sin(np.pi * xf / L) ** 3 / 3), (4, Nx + 1))
    u = P.get("u")
    assert np.max(np.abs(u - ue)) / (2 * U / 3) < 1e-3
    assert np.array_equal(P.get("u_b"), u)
    us = P.get("u_sigma")
    for k in range(us.shape[0]):
        np.testing.assert_allclose(us[k], u, rtol=1.5e-8, atol=0)

    g2 = grid((32, 4), x=(0.0, 1e5), y=(0.0, 1.25e4))
    fr = M.WeertmanFriction(coefficient=1e12, exponent=1.0)
    rh = M.GlenFlowLaw(rate_factor=1e-24)
    ssa, _ = ice_sheet_model(backend, g2, H=lambda x, y: 1000 + x / 1e2, rheology=rh, friction=fr)
    diva, st = ice_sheet_model(backend, g2, H=lambda x, y: 1000 + x / 1e2, rheology=rh, friction=fr,
                               stress_balance=M.DepthIntegrated(shear=M.DIVAShear()))
    ubar, ub, us = diva.get("u"), diva.get("u_b"), diva.get("u_sigma")
    dz = np.diff(sigma_nodes(us.shape[0])[0]).reshape(-1, 1, 1)
    assert 0 < st.picard_iterations < 100
    assert np.max(np.abs(ubar)) > 2 * np.max(np.abs(ssa.get("u")))
    assert np.all(np.abs(ub) <= np.abs(ubar))
    assert np.max(np.abs(np.sum(us * dz, axis=0) - ubar)) < 1e-2 * np.max(np.abs(ubar))


def test_model_stress_balance_update(backend):
    """test/test_model.jl:62-85 (the parts about the velocity update and the geometry it reads; the ice stream
    itself is test_ice_stream_n3).  s = bed + H and φ = 1 without a grounding treatment; the SSA's uᵇ and every
    layer of uσ equal ū; a floating sheet (bed -2000 m, H = 100 m, SubgridGroundedFraction) has
    s = (1 - ρᵢ/ρw) H, φ = 0 and N = 0."""
    from support import ice_sheet_model
    L = 100e3
    g = grid((32, 4), x=(0.0, L), y=(0.0, L / 8))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-10, maxiter=300))
    P, st = ice_sheet_model(backend, g, H=500.0, bed=lambda x, y: 20 * math.cos(math.pi * x / L),
                            rheology=M.GlenFlowLaw(rate_factor=1e-24), constants=M.IceSheetConstants(ice_density=917.0),
                            velocity_solver=solver, Nsigma=4)
    assert 0 < st.picard_iterations < 300
    np.testing.assert_allclose(P.get("s"), P.get("bed") + P.get("H"), rtol=1e-15)
    assert np.all(P.get("phi") == 1) and np.all(P.get("phi_u") == 1)
    u = P.get("u")
    assert np.array_equal(P.get("u_b"), u)
    assert all(np.array_equal(layer, u) for layer in P.get("u_sigma"))

    box = grid((4, 4), x=(0.0, 1e4), y=(0.0, 1e4))
    F, _ = ice_sheet_model(backend, box, H=100.0, bed=-2000.0, grounding=M.SubgridGroundedFraction(), solve=False)
    c = M.IceSheetConstants()
    np.testing.assert_allclose(F.get("s"), (1 - c.ice_density / c.ocean_density) * 100, rtol=1e-14)
    assert np.all(F.get("phi") == 0) and np.all(F.get("N") == 0)


def _rate_factor_model(cls, stress_balance, T=None, A=None):
    """rate_factor_model + set!(model; H = 1000 + x / 100, T), test/test_rate_factor.jl:52-62 and :64: 16 x 4 cells
    over 160 km x 40 km, Weertman drag (C = 1e10, m = 1), ρᵢ = 910, CG 1e-12 inside Picard 1e-11, and A either from
    the temperature (Arrhenius, Clausius-Clapeyron slope 0 as in rate_factor_model) or prescribed."""
    g = grid((16, 4), x=(0.0, 1.6e5), y=(0.0, 4e4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-11, maxiter=500))
    sigma = A is None
    P = make(cls, g, stress_balance=stress_balance, friction=M.WeertmanFriction(coefficient=1e10, exponent=1.0),
             rheology=M.GlenFlowLaw(rate_factor="sigma" if sigma else A, strain_rate_regularization=1e-16),
             constants=M.IceSheetConstants(ice_density=910.0), velocity_solver=solver)
    P.set("H", np.broadcast_to(1000 + g.centers(0) / 1e2, (4, 16)))
    P.set("bed", 0.0)
    P.set("C", 1e10)
    if sigma:
        _, zeta = sigma_nodes(P.shape("A")[0])
        t = np.array([T(z) for z in zeta]) if callable(T) else np.full(zeta.shape, float(T))
        P.set("T", np.broadcast_to(t.reshape(-1, 1, 1), P.shape("T")))
        P.compute_rate_factor(clausius_clapeyron=0.0)
    else:
        P.set("A", A)
    P.compute_geometry()
    st = P.picard_solve()
    assert st.status == 0
    return P.get("u")


def test_stress_balance_feels_the_temperature(backend):
    """test/test_rate_factor.jl:186-206: the Arrhenius A of a uniform 253.15 K gives the velocities of the
    prescribed cold-branch A to 1e-9, a warmer 268.15 K flows faster (SSA and DIVA), and in DIVA a warm base
    (268.15 - 30ζ) flows faster than a warm surface (238.15 + 30ζ)."""
    for sb in (M.DepthIntegrated(), M.DepthIntegrated(shear=M.DIVAShear())):
        arrhenius = _rate_factor_model(backend, sb, T=253.15)
        prescribed = _rate_factor_model(backend, sb, A=cold_branch(253.15))
        assert np.linalg.norm(arrhenius - prescribed) <= 1e-9 * max(np.linalg.norm(arrhenius), np.linalg.norm(prescribed))
        warm = _rate_factor_model(backend, sb, T=268.15)
        assert np.max(np.abs(warm)) > np.max(np.abs(arrhenius))
    diva = M.DepthIntegrated(shear=M.DIVAShear())
    base = _rate_factor_model(backend, diva, T=lambda z: 268.15 - 30 * z)
    surface = _rate_factor_model(backend, diva, T=lambda z: 238.15 + 30 * z)
    assert np.max(np.abs(base)) > np.max(np.abs(surface))
