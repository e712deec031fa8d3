"""The reference's known answers, second part: multigrid, DIVA, grounding, calving front, ice mask.
Each test follows a testset of Nunatak.jl (file:line given) and runs on the oracle and on the GPU."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import evaluate, ice_sheet_model, isapprox, make, set_fn


def grid(size, x=(0.0, 1.0), y=(0.0, 1.0), topology=("Bounded", "Bounded"), halo=(3, 3)):
    return M.RectilinearGrid(size=size, x=x, y=y, topology=topology, halo=halo)


def corners_of(g, eta):
    """ℑxyᶠᶠᵃ(η̄H) over size(η̄Hᶠᶠ) with Oceananigans halos (wrap, or zero-gradient copy): the reference's
    _interpolate_to_corners! (src/StressBalances/stress_balance_coefficients.jl:26-29)."""
    mode = lambda d: "wrap" if g.periodic(d) else "edge"
    e = np.pad(eta, ((1, 1), (0, 0)), mode=mode(1))
    e = np.pad(e, ((0, 0), (1, 1)), mode=mode(0))
    nfx, nfy = g.face_count(0), g.face_count(1)
    out = np.empty((nfy, nfx))
    for j in range(nfy):
        for i in range(nfx):
            lo = (e[j, i] + e[j, i + 1]) / 2
            hi = (e[j + 1, i] + e[j + 1, i + 1]) / 2
            out[j, i] = (lo + hi) / 2
    return out


def holed(P, g):
    """holed_coefficients, test/test_multigrid_preconditioner.jl:16-27."""
    eta = evaluate(g, "eta_H", lambda x, y: 0.0 if (x - 0.7) ** 2 + (y - 0.4) ** 2 < 0.04 else 1 + x)
    P.set("eta_H", eta)
    P.set("eta_H_ff", corners_of(g, eta))
    P.set("beta_u", 3.0)
    P.set("beta_v", 3.0)


def smooth_vector(g, m):
    """smooth_vector, test/test_multigrid_preconditioner.jl:7-13."""
    u = evaluate(g, "u", lambda x, y: math.sin(2 * math.pi * m * x + 1) * math.cos(2 * math.pi * y + m))
    v = evaluate(g, "v", lambda x, y: math.cos(2 * math.pi * x + m) * math.sin(2 * math.pi * m * y + 2))
    return u, v


def coarse_grid(g, nx, ny):
    fx, fy = g.Nx // nx, g.Ny // ny
    xf, yf = g.faces(0)[::fx], g.faces(1)[::fy]
    return M.RectilinearGrid(size=(nx, ny), x=list(xf), y=list(yf), topology=g.topology, halo=g.halo)


def solved_dot(g, a, b):
    """solved_dot, test/test_multigrid_preconditioner.jl:4-5: sum over the Nx x Ny solved range."""
    return float(np.sum(a[0][:g.Ny, :g.Nx] * b[0][:g.Ny, :g.Nx]) + np.sum(a[1][:g.Ny, :g.Nx] * b[1][:g.Ny, :g.Nx]))


@pytest.mark.parametrize("topology", [("Bounded", "Periodic"), ("Bounded", "Bounded"), ("Periodic", "Periodic")])
@pytest.mark.parametrize("size", [(16, 8), (32, 4), (4, 32)])
def test_multigrid_transfers_and_symmetry(backend, topology, size):
    """test/test_multigrid_preconditioner.jl:39-64: restriction = prolongationᵀ, V-cycle symmetric positive."""
    g = grid(size, topology=topology, halo=(4, 4))
    P = make(backend, g, velocity_solver=M.StressBalanceSolver(preconditioner=M.StressBalanceMultigridPreconditioner()), masking=None)
    holed(P, g)
    levels = P.multigrid_levels()
    cg = coarse_grid(g, *levels[0])
    f, c = smooth_vector(g, 3), smooth_vector(cg, 2)
    Rf = P.restrict(0, *f)
    Pc = P.prolongate(0, *c)
    a, b = solved_dot(cg, Rf, c), solved_dot(g, f, Pc)
    assert abs(a - b) <= 1e-12 * max(abs(a), abs(b))

    r1, r2 = smooth_vector(g, 1), smooth_vector(g, 2)
    for smoother in (M.PointJacobi(), M.LineJacobi()):
        for walls in (M.FreeSlipWalls(), M.NoSlipWalls()):
            Q = make(backend, g, stress_balance=M.DepthIntegrated(side_walls=walls), masking=None,
                     velocity_solver=M.StressBalanceSolver(preconditioner=M.StressBalanceMultigridPreconditioner(smoother=smoother)))
            holed(Q, g)
            z1 = Q.precondition(*r1)
            z2 = Q.precondition(*r2)
            a, b = solved_dot(g, z1, r2), solved_dot(g, r1, z2)
            assert abs(a - b) <= 1e-10 * max(abs(a), abs(b))
            assert solved_dot(g, z1, r1) > 0


def ice_cap(cls, Nx=20, L=200e3, R=60e3, H0=1000.0, H_edge=0.0, masking=None, linear=None, picard=None, preconditioner=None):
    """ice_cap_model, test/test_ice_mask.jl:4-15."""
    g = grid((Nx, Nx), x=(0.0, L), y=(0.0, L), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=linear or M.Convergence(reltol=1e-10, maxiter=10_000),
                                   picard_iteration_control=picard or M.Convergence(reltol=1e-8, maxiter=200),
                                   preconditioner=preconditioner or M.StressBalanceDiagonalPreconditioner())

    def dome(x, y):
        r = math.hypot(x - L / 2, y - L / 2)
        return H0 * math.sqrt(1 - (r / R) ** 2) + H_edge if r < R else H_edge

    return ice_sheet_model(cls, g, H=dome, rheology=M.GlenFlowLaw(rate_factor=1e-24),
                           friction=M.WeertmanFriction(coefficient=3e6), masking=masking or M.SmoothIceMask(),
                           velocity_solver=solver)


def test_multigrid_cg_on_ice_cap(backend):
    """test/test_multigrid_preconditioner.jl:66-82: MG needs < 1/3 of the Jacobi iterations, same solution."""
    model, _ = ice_cap(backend, Nx=128, masking=M.SmoothIceMask(10.0, 400.0))
    g = model.grid
    fields = {k: model.get(k) for k in ("eta_H", "eta_H_ff", "beta_u", "beta_v", "tau_u", "tau_v")}
    control = M.Convergence(reltol=1e-10, maxiter=20_000)
    out = {}
    for name, pre in (("jacobi", M.StressBalanceDiagonalPreconditioner()), ("multigrid", M.StressBalanceMultigridPreconditioner())):
        P = make(backend, g, masking=None, velocity_solver=M.StressBalanceSolver(linear_iteration_control=control, preconditioner=pre))
        for k in ("eta_H", "eta_H_ff", "beta_u", "beta_v"):
            P.set(k, fields[k])
        st = P.linear_solve(fields["tau_u"], fields["tau_v"])
        out[name] = (st.linear_iterations_last, P.get("u"), P.get("v"))
    assert out["multigrid"][0] < out["jacobi"][0] / 3
    Nx, Ny = g.Nx, g.Ny
    assert isapprox(out["multigrid"][1][:Ny, :Nx], out["jacobi"][1][:Ny, :Nx], rtol=1e-7)
    assert isapprox(out["multigrid"][2][:Ny, :Nx], out["jacobi"][2][:Ny, :Nx], rtol=1e-7)


def slab_profile_error(cls, Nsigma, H0=1000.0, tau0=1e4, A=1e-21, C=1e10):
    """slab_profile_error, test/test_diva.jl:5-46."""
    g = grid((4, 4), x=(0.0, 4e3), y=(0.0, 4e3), topology=("Periodic", "Periodic"))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=100),
                                   picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=300), preconditioner=None)
    P = make(cls, g, Nsigma=Nsigma, stress_balance=M.DepthIntegrated(shear=M.DIVAShear()),
             rheology=M.GlenFlowLaw(rate_factor=A, strain_rate_regularization=1e-16),
             friction=M.WeertmanFriction(coefficient=C, exponent=1.0), masking=None, use_effective_pressure=False,
             velocity_solver=solver)
    P.set("H", H0)
    P.set("phi_u", 1.0)
    P.set("phi_v", 1.0)
    P.set("A", A)
    P.set("C", C)
    P.set("tau_u", tau0 * 1e3**2)
    st = P.picard_solve()
    P.velocity_profile()
    n = 3.0
    ub = tau0 / C
    U = 2 * A * tau0**n * H0 / (n + 1)
    f = np.array([(k / Nsigma) ** 2 for k in range(Nsigma + 1)])
    zeta = (f[1:] + f[:-1]) / 2
    exact = ub + U * (1 - (1 - zeta) ** (n + 1))
    us = P.get("u_sigma")[:, 0, 0]
    ubar = P.get("u")
    ubar_e = ub + 2 * A * tau0**n * H0 / (n + 2)
    return dict(iterations=st.picard_iterations, profile=np.max(np.abs(us - exact)) / U,
                mean=np.max(np.abs(ubar - ubar_e)) / (ubar_e - ub),
                basal=np.max(np.abs(P.get("u_b") - ub)) / ub, v=np.max(np.abs(P.get("v_sigma"))))


def test_diva_slab(backend):
    """test/test_diva.jl:48-58."""
    coarse, fine = slab_profile_error(backend, 10), slab_profile_error(backend, 40)
    assert 0 < fine["iterations"] < 300
    assert fine["profile"] < 1e-2
    assert fine["mean"] < 1e-2
    assert fine["basal"] < 1e-6
    assert fine["v"] == 0
    assert fine["profile"] < coarse["profile"] / 4


def test_grounded_fraction_and_effective_pressure(backend):
    """test/test_grounding.jl:14-67."""
    g = grid((16, 2), x=(0.0, 16.0), y=(0.0, 2.0), topology=("Bounded", "Periodic"))
    c = M.IceSheetConstants()
    ri, rw, gg, H0 = c.ice_density, c.ocean_density, c.gravitational_acceleration, 1000.0
    sub = M.SubgridGroundedFraction()
    for xgl in (3.3, 7.5, 10.9):
        P, _ = ice_sheet_model(backend, g, H=H0, bed=lambda x, y: ri / rw * (50 * (xgl - x) - H0), grounding=sub, solve=False)
        phi, phu = P.get("phi"), P.get("phi_u")
        assert abs(np.sum(phi[0]) - xgl) <= 1.5e-8 * xgl
        assert np.all((phi >= 0) & (phi <= 1))
        i = math.floor(xgl + 0.5) + 1
        assert abs(phu[0, i - 1] - (xgl + 0.5 - (i - 1))) <= 1e-12
    for b0, val in ((-800.0, 1.0), (-1000.0, 0.0)):
        P, _ = ice_sheet_model(backend, g, H=H0, bed=b0, grounding=sub, solve=False)
        assert np.all(P.get("phi") == val) and np.all(P.get("phi_u") == val) and np.all(P.get("phi_v") == val)

    box = grid((8, 8), x=(0.0, 8.0), y=(0.0, 8.0))
    unit = M.IceSheetConstants(1.0, 1.0, 9.81)
    for cc, cell, expected in ((9.0, (5, 5), 0.5), (9.0, (4, 5), 1.0), (9.3, (5, 5), 1 - 0.7**2 / 2)):
        P, _ = ice_sheet_model(backend, box, H=0.0, bed=lambda x, y: cc - x - y, constants=unit, grounding=sub, solve=False)
        assert abs(P.get("phi")[cell[1] - 1, cell[0] - 1] - expected) <= 1.5e-8

    P, _ = ice_sheet_model(backend, g, H=H0, bed=lambda x, y: 100.0 if x < 4 else (-500.0 if x < 8 else -1000.0), grounding=sub, solve=False)
    N = P.get("N")
    np.testing.assert_allclose(N[:, 0:4], ri * gg * H0, rtol=1e-14)
    np.testing.assert_allclose(N[:, 4:8], ri * gg * H0 - rw * gg * 500, rtol=1e-12)
    assert np.all(N[:, 8:16] == 0)

    fr = M.RegularizedCoulombFriction(coefficient=3e4, coulomb_coefficient=0.5)
    P, _ = ice_sheet_model(backend, g, H=H0, bed=lambda x, y: ri / rw * (50 * (7.5 - x) - H0), grounding=sub, friction=fr, solve=False)
    P.set("u", 100 / 3.15e7)
    P.set("v", 0.0)
    P.update_coefficients()
    bu = P.get("beta_u")
    assert np.all(bu[:, 1:8] > 0)
    assert np.all(bu[:, 9:16] == 0)


def test_grounding_line_split_driving_stress(backend):
    """test/test_grounding.jl:69-114."""
    ri, rw, gg, D = 918.0, 1028.0, 9.81, 1e3
    c = M.IceSheetConstants(ri, rw, gg)
    for Nx, Ny, xgl in ((16, 2, 7.3e3), (2, 16, 7.3e3)):
        g = grid((Nx, Ny), x=(0.0, Nx * D), y=(0.0, Ny * D))
        along = (lambda x, y: x) if Nx > Ny else (lambda x, y: y)
        H = lambda x, y: 1000 - 0.02 * along(x, y)
        b = lambda x, y: ri / rw * (0.05 * (xgl - along(x, y)) - 1000 + 0.02 * along(x, y))
        P0, _ = ice_sheet_model(backend, g, H=H, bed=b, masking=None, constants=c, grounding=M.SubgridGroundedFraction(), solve=False)
        P1, _ = ice_sheet_model(backend, g, H=H, bed=b, masking=None, constants=c,
                                grounding=M.SubgridGroundedFraction(driving_stress=True), solve=False)
        t0 = P0.get("tau_u" if Nx > Ny else "tau_v")
        t1 = P1.get("tau_u" if Nx > Ny else "tau_v")
        s = P1.get("s")
        face = (lambda A, n: A[0, n - 1]) if Nx > Ny else (lambda A, n: A[n - 1, 0])
        n = 8
        H1, H2 = 1000 - 0.02 * 6.5e3, 1000 - 0.02 * 7.5e3
        f1, f2 = 0.05 * (xgl - 6.5e3), 0.05 * (xgl - 7.5e3)
        th = f1 / (f1 - f2)
        Hg = H1 + th * (H2 - H1)
        s1, s2, sg = face(s, n - 1), (1 - ri / rw) * H2, (1 - ri / rw) * Hg
        expected = -D * ri * gg * ((H1 + Hg) * (sg - s1) + (Hg + H2) * (s2 - sg)) / 2
        assert abs(face(t1, n) - expected) <= 1.5e-8 * abs(expected)
        assert abs(face(t1, n) - face(t0, n)) > 1.5e-8 * abs(face(t0, n))
        others = [m for m in range(2, (Nx if Nx > Ny else Ny) + 1) if m != n]
        assert [face(t1, m) for m in others] == [face(t0, m) for m in others]

    g = grid((16, 4), x=(0.0, 16e3), y=(0.0, 4e3), halo=(4, 4))
    tau = []
    for ds in (False, True):
        P, _ = ice_sheet_model(backend, g, H=lambda x, y: 1000 - 0.02 * x, bed=lambda x, y: -600 - 0.05 * x,
                               rheology=M.GlenFlowLaw(rate_factor=1e-24), friction=M.WeertmanFriction(coefficient=1e6),
                               grounding=M.SubgridGroundedFraction(driving_stress=ds), solve=False)
        tau.append(P.get("tau_u")[1, :])
    assert list(np.nonzero(tau[0] != tau[1])[0] + 1) == [5]


def test_calving_front_force(backend):
    """test/test_calving_front.jl:3-67: front force of floating, marine and land cliffs."""
    Nx, Ny = 6, 4
    g = grid((Nx, Ny), x=(0.0, 6e3), y=(0.0, 4e3))
    ri, rw, gg, H0 = 918.0, 1028.0, 9.81, 500.0
    for b, D in ((-2000.0, ri * H0 / rw), (-300.0, 300.0), (100.0, 0.0)):
        P, _ = ice_sheet_model(backend, g, H=lambda x, y: H0 if x < 3e3 else 0.0, bed=b,
                               grounding=M.SubgridGroundedFraction(), solve=False)
        tu = P.get("tau_u")
        np.testing.assert_allclose(tu[:, 3], 1e3 * gg * (ri * H0**2 - rw * D**2) / 2, rtol=1e-12)
        assert np.all(tu[:, 4:] == 0)


def test_confined_shelf_spreading(backend):
    """test/test_calving_front.jl:23-40."""
    L, xf, H0, A, Nx = 64e3, 40e3, 500.0, 1e-24, 32
    g = grid((Nx, 4), x=(0.0, L), y=(0.0, 4 * L / Nx), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-10, maxiter=500))
    P, _ = ice_sheet_model(backend, g, H=lambda x, y: H0 if x < xf else 0.0, bed=-2000.0, u=lambda x, y: 1e-9 * x,
                           rheology=M.GlenFlowLaw(rate_factor=A), friction=M.WeertmanFriction(coefficient=1e6),
                           grounding=M.SubgridGroundedFraction(), velocity_solver=solver)
    c = M.IceSheetConstants()
    rp = c.ice_density * (1 - c.ice_density / c.ocean_density)
    e = A * (rp * c.gravitational_acceleration * H0 / 4) ** 3
    x = g.faces(0)
    u = P.get("u")[1, :]
    ice = x <= xf
    assert np.max(np.abs(u[ice] - e * x[ice])) / (e * xf) < 1e-6
    assert np.max(np.abs(P.get("v"))) < 1e-12 * e * xf


def test_steady_shelf_second_order(backend):
    """test/test_calving_front.jl:42-66."""
    L, xf, H0, A, n = 256e3, 192e3, 1e3, 1e-25, 3
    q = H0 * 1e-5
    c = M.IceSheetConstants()
    rp = c.ice_density * (1 - c.ice_density / c.ocean_density)
    k = (n + 1) * (A / q) * (rp * c.gravitational_acceleration / 4) ** n
    Hx = lambda x: (H0 ** -(n + 1) + k * x) ** (-1 / (n + 1))
    errors = []
    for Nx in (64, 128):
        g = grid((Nx, 4), x=(0.0, L), y=(0.0, 4 * L / Nx), halo=(4, 4))
        solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=20_000),
                                       picard_iteration_control=M.Convergence(reltol=1e-11, maxiter=500))
        P, _ = ice_sheet_model(backend, g, H=lambda x, y: Hx(x) if x < xf else 0.0, bed=-2000.0, u=lambda x, y: 1e-9 * x,
                               rheology=M.GlenFlowLaw(rate_factor=A), friction=M.WeertmanFriction(coefficient=1e6),
                               grounding=M.SubgridGroundedFraction(), velocity_solver=solver)
        x = g.faces(0)
        ice = x <= xf
        u = P.get("u")[1, :][ice]
        ue = q / np.array([Hx(xx) for xx in x[ice]]) - q / H0
        errors.append(np.max(np.abs(u - ue)) / np.max(ue))
    assert errors[1] < 5e-3
    assert errors[0] / errors[1] > 3


def test_smooth_ice_mask_values(backend):
    """test/test_ice_mask.jl:27-36 through compute_ice_mask!."""
    g = grid((5, 1), x=(0.0, 5.0), topology=("Bounded", "Periodic"))
    Hs = [10.0, 30.0, 20.0, 10.0 + 1e-6, 30.0 - 1e-6]
    P, _ = ice_sheet_model(backend, g, H=lambda x, y: Hs[int(x)], masking=M.SmoothIceMask(10.0, 20.0), solve=False)
    mu = P.get("ice_mask")[0]
    assert mu[0] == 0 and mu[1] == 1 and mu[2] == 0.5
    assert abs(mu[3] - 0.0) / 1e-6 < 1e-6
    assert abs(1.0 - mu[4]) / 1e-6 < 1e-6


def test_ice_free_points_decoupled(backend):
    """test/test_ice_mask.jl:38-61."""
    Nx, Ny = 8, 6
    g = grid((Nx, Ny), topology=("Bounded", "Periodic"))
    ice = lambda x, y: 1.0 if x < 0.5 else 0.0
    P = make(backend, g, masking=None)
    eta = lambda x, y: ice(x, y) * (1 + x**2)
    set_fn(P, "eta_H", eta)
    set_fn(P, "eta_H_ff", eta)
    set_fn(P, "beta_u", lambda x, y: 1 + x * y)
    set_fn(P, "beta_v", lambda x, y: 1 + x * y)
    pu, pv = evaluate(g, "u", lambda x, y: math.sin(math.pi * x) + y), evaluate(g, "v", lambda x, y: x * y**2 + 1)
    yu, yv = evaluate(g, "u", lambda x, y: math.cos(x) * y + 1), evaluate(g, "v", lambda x, y: math.sin(3 * y) + x)
    Apu, Apv = P.apply_operator(pu, pv)
    Ayu, Ayv = P.apply_operator(yu, yv)
    dot = lambda a, b, c, d: float(np.sum(a[:Ny, :Nx] * c[:Ny, :Nx]) + np.sum(b[:Ny, :Nx] * d[:Ny, :Nx]))
    a, b = dot(Apu, Apv, yu, yv), dot(pu, pv, Ayu, Ayv)
    assert abs(a - b) <= 1.5e-8 * abs(a)
    assert dot(Apu, Apv, pu, pv) > 0
    mu = P.get("eta_H")
    u_free = np.zeros((Ny, Nx + 1), bool)
    for j in range(Ny):
        for i in range(Nx + 1):
            u_free[j, i] = i == 0 or i == Nx or (mu[j, i - 1] == 0 and mu[j, i] == 0)
    v_free = np.array([[mu[(j - 1) % Ny, i] == 0 and mu[j, i] == 0 for i in range(Nx)] for j in range(Ny)])
    assert np.count_nonzero(u_free) > 2 * Ny and np.count_nonzero(v_free) > 0
    u_free[:, Nx] = False
    assert np.array_equal(Apu[u_free], pu[u_free])
    assert np.array_equal(Apv[v_free], pv[v_free])


@pytest.mark.parametrize("H_edge", [0.0, 0.5])
def test_ice_cap_with_ice_free_margins(backend, H_edge):
    """test/test_ice_mask.jl:63-79."""
    P, st = ice_cap(backend, H_edge=H_edge)
    mu = P.get("ice_mask")
    assert np.count_nonzero(mu == 0) > 0
    assert 0 < st.picard_iterations < 200
    assert np.all(P.get("eta_H")[mu == 0] == 0)
    u, v = P.get("u"), P.get("v")
    Ny, Nfx = u.shape
    Nx = Nfx - 1
    u_free = np.array([[i == 0 or i == Nx or (mu[j, i - 1] == 0 and mu[j, i] == 0) for i in range(Nx + 1)] for j in range(Ny)])
    v_free = np.array([[j == 0 or j == Ny or (mu[j - 1, i] == 0 and mu[j, i] == 0) for i in range(Nx)] for j in range(Ny + 1)])
    assert np.all(np.isfinite(u)) and np.all(np.isfinite(v))
    assert np.all(u[u_free] == 0) and np.all(v[v_free] == 0)
    assert np.max(np.abs(u)) > 0
    assert isapprox(u, -u[:, ::-1], rtol=1e-6)
