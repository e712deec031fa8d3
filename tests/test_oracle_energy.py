"""The oracle's energy step (nko_step_enthalpy: step_thermodynamics!, src/Thermodynamics/column_energy_solve.jl:26-78)
against the column testsets of test/test_thermodynamics.jl, and the library's energy step (nk_step_enthalpy,
marked gpu) against the oracle's on the same seeded inputs.

column_model (test/test_thermodynamics.jl:3-14): one Periodic column, 1 km wide, ρᵢ = 910, no velocity solve and
no thickness change, so each time step is one energy step of the same length:
- steady conduction on uniform and refined layers is linear in height, T = Tₛ + G H (1 - ζ) / k, within 1e-8 K
  after four 1e14 s steps, with no basal water (:116-128);
- surface warming by 10 K converges at second order to the Fourier series of the step response (:130-156);
- the column energy changes by Δt (G + β uᵇ² - surface flux) at every step, within 1e-11 (:158-173);
- a warm base melts at the analytic rate (G - k (T_pm - Tₛ) / H) / (ρᵢ L) within 1e-3, and once the geothermal
  flux stops, refreezes its stored water while the total energy stays balanced within 1e-10 (:175-208);
- a floating base sits at the ocean temperature, T linear from Tₒ to Tₛ, with no grounded melt (:210-222);
- an ice-free column holds the surface enthalpy (:224-231);
- a temperate layer over a wet base insulates it, so all basal heat melts (:400-412);
- temperate layers drain at the maximum rate and then down to the drainage water fraction (:414-434);
with the thickness step of the oracle as well:
- a thickening or thinning column follows the heat equation in fixed height at second order (:293-320;
  measured 0.056 / 0.014 / 0.0036 K thickening and 0.31 / 0.086 / 0.023 K thinning at 10 / 20 / 40 layers);
- a uniform enthalpy stays uniform to 1e-9 under variable thickness, shearing layer velocities, accumulation
  and melt (:322-331);
- strong accumulation over a sharp front creates no new extrema (:360-370);
- upwind transport at unit Courant number shifts each moving layer by one cell and leaves the others (:372-390);
with the velocity solve as well:
- the basal plus strain heat equals the power of the driving stress to 1e-8, SSA and DIVA (:392-398).
The library against the oracle (gpu), SSA and DIVA: a 24 x 20 sheet over a sloping bed, Bounded in x and Periodic
in y, 8 layers, the velocity state of the oracle's solve copied into the library, seeded enthalpy with cold,
temperate and draining layers, wet and dry beds, thinning and thickening columns: two energy steps agree in E,
T, ω, H_w, mᵍ, s_b, qᵍ and Φ to 1e-10 relative (FMA contraction on the GPU rounds apart by a few ulps); at
1024 x 1024 the columns of a uniform sheet at rest stay bitwise alike through three steps and match the
oracle's single column (melt, drainage and a growing basal water layer)."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import evaluate, make

K, CI, LATENT, BETA, T0, TR = 2.1, 2009.0, 3.34e5, 7.9e-8, 273.15, 223.15
RHO, GRAV = 910.0, 9.81


def enthalpy(T, omega, p):
    """enthalpy(T, ω, p, parameters), src/Thermodynamics/enthalpy_conversions.jl:49-52."""
    return CI * (np.minimum(T, T0 - BETA * p) - TR) + omega * LATENT


class Column:
    """column_model(; H₀, Nσ, bed_refinement, geothermal_flux, surface_temperature, grounding, bed) on the oracle."""

    def __init__(self, cls, H0=1000.0, Nsigma=10, bed_refinement=1.0, G=0.042, Ts=243.15, grounding=None, bed=0.0):
        g = M.RectilinearGrid(size=(1, 1), x=(0.0, 1e3), y=(0.0, 1e3), topology=("Periodic", "Periodic"), halo=(3, 3))
        self.P = make(cls, g, advection=M.UpwindBiased(order=1), Nsigma=Nsigma, bed_refinement=bed_refinement, rheology=M.GlenFlowLaw(rate_factor="sigma"),
                      constants=M.IceSheetConstants(ice_density=RHO), grounding=grounding)
        self.H0 = H0
        self.P.set("H", H0)
        self.P.set("bed", bed)
        self.P.compute_geometry()
        faces = np.array(M.sigma_faces(Nsigma, bed_refinement))
        self.faces, self.zeta = faces, (faces[1:] + faces[:-1]) / 2
        self.pressure = RHO * GRAV * H0 * (1 - self.zeta)
        for name, value in (("geothermal_flux", G), ("surface_temperature", Ts), ("ocean_temperature", 271.15),
                            ("basal_melt_rate", 0.0), ("H_previous", H0), ("Hw", 0.0)):
            self.P.energy_set(name, value)
        self.set_temperature(np.full(Nsigma, Ts))   # a new model holds the surface enthalpy
        self.set_enthalpy(np.full(Nsigma, enthalpy(Ts, 0.0, 0.0)))

    def set_temperature(self, T):
        self.set_enthalpy(enthalpy(np.asarray(T, dtype=np.float64), 0.0, self.pressure))

    def set_enthalpy(self, E):
        self.P.set("E", np.asarray(E, dtype=np.float64).reshape(-1, 1, 1))

    def step(self, dt):
        self.P.step_enthalpy(dt, grounded_melt_coupling=False)

    def column(self, name):
        return self.P.get(name)[:, 0, 0]

    def value(self, name):
        return float(self.P.energy_get(name)[0, 0])

    def energy(self):
        """ρ ∫E dz per unit area."""
        return RHO * self.H0 * float(np.sum(np.diff(self.faces) * self.column("E")))

    def surface_heat_flux(self, Ts):
        EN, Es = self.column("E")[-1], CI * (Ts - TR)
        return K / CI * (EN - Es) / (self.H0 * (1 - self.zeta[-1]))


@pytest.mark.parametrize("bed_refinement", [1.0, 2.0])
def test_steady_conduction_is_linear_in_height(oracle_cls, bed_refinement):
    H0, G, Ts = 1000.0, 0.042, 243.15
    c = Column(oracle_cls, H0=H0, G=G, Ts=Ts, bed_refinement=bed_refinement)
    for _ in range(4):
        c.step(1e14)
    exact = Ts + G * H0 * (1 - c.zeta) / K
    assert np.max(np.abs(c.column("T") - exact)) < 1e-8
    assert c.value("Hw") == 0.0


def test_surface_warming_converges_at_second_order(oracle_cls):
    H0, G, Ts, dT, t_end = 1000.0, 0.042, 243.15, 10.0, 6.3e10
    errors = []
    for Nsigma in (10, 20, 40):
        c = Column(oracle_cls, H0=H0, Nsigma=Nsigma, G=G, Ts=Ts)
        c.set_temperature(Ts + G * H0 * (1 - c.zeta) / K)
        c.P.energy_set("surface_temperature", Ts + dT)
        Nt = 4 * Nsigma ** 2
        for _ in range(Nt):
            c.step(t_end / Nt)
        kappa = K / (RHO * CI)
        z = c.zeta * H0
        steady = Ts + dT + G * (H0 - z) / K
        transient = np.zeros_like(z)
        for n in range(201):
            lam = (2 * n + 1) * math.pi / (2 * H0)
            transient += -dT * 4 / math.pi * (-1) ** n / (2 * n + 1) * np.cos(lam * z) * math.exp(-kappa * lam ** 2 * t_end)
        errors.append(float(np.max(np.abs(c.column("T") - (steady + transient)))))
    assert errors[2] < 0.01
    assert errors[0] / errors[1] > 3 and errors[1] / errors[2] > 3


def test_energy_budget_closes_with_geothermal_and_frictional_heating(oracle_cls):
    H0, G, Ts = 800.0, 0.05, 243.15
    c = Column(oracle_cls, H0=H0, G=G, Nsigma=12, bed_refinement=2.0, Ts=Ts)
    c.set_temperature(250 - 5 * c.zeta)
    beta, ub = 1e8, 1e-6
    c.P.set("beta_u", beta)
    c.P.set("u_b", ub)
    F = beta * ub ** 2
    dt = 1e9
    for _ in range(50):
        before = c.energy()
        c.step(dt)
        budget = c.energy() - before - dt * (G + F - c.surface_heat_flux(Ts))
        assert abs(budget) < 1e-11 * abs(before)


def test_warm_base_melts_at_the_analytic_rate_then_refreezes(oracle_cls):
    H0, G, Ts = 1000.0, 0.1, 263.15
    c = Column(oracle_cls, H0=H0, G=G, Ts=Ts, Nsigma=20)
    Tpm = T0 - BETA * RHO * GRAV * H0
    for _ in range(20):
        c.step(1e13)
    exact = (G - K * (Tpm - Ts) / H0) / (RHO * LATENT)
    assert exact > 0
    assert abs(c.value("grounded_melt") - exact) <= 1e-3 * exact
    assert c.value("Hw") > 0
    # too little water for one step, so the column pays back the excess latent heat itself
    c.P.energy_set("Hw", 1e-2)
    c.P.energy_set("geothermal_flux", 0.0)
    dt = 1e9

    def total():
        return c.energy() + RHO * LATENT * c.value("Hw")

    froze_out = False
    for _ in range(200):
        before = total()
        c.step(dt)
        q = K / CI * (c.column("E")[-1] - CI * (Ts - TR)) / (H0 * (1 - c.zeta[-1]))
        assert abs(total() - before + dt * q) < 1e-10 * abs(before)
        froze_out |= c.value("Hw") == 0.0
    assert froze_out
    assert c.value("grounded_melt") == 0.0


def test_floating_base_sits_at_the_ocean_temperature(oracle_cls):
    H0, Ts = 500.0, 253.15
    c = Column(oracle_cls, H0=H0, Ts=Ts, G=0.05, grounding=M.SubgridGroundedFraction(), bed=-3000.0)
    assert c.P.get("phi")[0, 0] == 0.0
    for _ in range(4):
        c.step(1e14)
    To = 271.15
    exact = To + (Ts - To) * c.zeta
    assert np.max(np.abs(c.column("T") - exact)) < 1e-8
    assert c.value("grounded_melt") == 0.0


def test_ice_free_columns_hold_the_surface_enthalpy(oracle_cls):
    Ts = 253.15
    c = Column(oracle_cls, H0=0.5, Ts=Ts)
    c.set_temperature(np.full(10, 240.0))
    c.step(1e9)
    assert np.allclose(c.column("T"), Ts, rtol=1.4901161193847656e-08, atol=0)
    assert c.value("Hw") == 0.0


def test_temperate_layer_above_the_base_insulates_it(oracle_cls):
    """test/test_thermodynamics.jl:400-412: a temperate layer (ζ < 0.2, ω = 1/50) over a wet base insulates it, so
    the basal layer is fully temperate and all the geothermal heat melts: mᵍ = G / (ρᵢ L) within 1e-12."""
    H0, G = 1000.0, 0.08
    c = Column(oracle_cls, H0=H0, G=G, Ts=263.15, Nsigma=20)
    c.P.energy_set("Hw", 1.0)
    c.set_enthalpy(np.where(c.zeta < 0.2, CI * (T0 - TR) + LATENT / 50, CI * (260 - TR)))
    c.P.compute_thermal_diagnostics(clausius_clapeyron=BETA)
    assert c.column("omega")[0] > 0
    c.P.step_enthalpy(1e8, grounded_melt_coupling=False, maximum_drainage_rate=0.0)
    assert c.value("basal_temperate_fraction") == 1.0
    assert abs(c.value("grounded_melt") - G / (RHO * LATENT)) <= 1e-12 * G / (RHO * LATENT)


def test_temperate_layers_drain_into_the_basal_water(oracle_cls):
    """test/test_thermodynamics.jl:414-434: with ω above 3 ω_d everywhere the first 1 s step drains at the maximum
    rate, Hw = H R_max Δt (1e-8); a hundred 1e9 s steps bring every layer down to ω_d and leave the water below."""
    H0, wd, Rmax = 1000.0, 0.01, 1.58443823077064e-9
    c = Column(oracle_cls, H0=H0, G=0.0, Ts=263.15, Nsigma=10)
    c.set_enthalpy(np.full(10, CI * (T0 - TR) + 5 * wd * LATENT))
    c.P.compute_thermal_diagnostics(clausius_clapeyron=BETA)
    assert np.min(c.column("omega")) > 3 * wd
    c.step(1.0)
    assert abs(c.value("Hw") - H0 * Rmax) <= 1e-8 * H0 * Rmax
    for _ in range(100):
        c.step(1e9)
    assert np.max(c.column("omega")) <= wd + 1e-12
    assert c.value("Hw") > 0.1 * H0 * wd


# ---- with the thickness step (tests/test_oracle_thickness.py): a time step is the thickness stages, then the
# energy step over the same interval (update_state! at the final stage, src/Models/ice_sheet_model_methods.jl:80-86)

@pytest.mark.parametrize("a0", [1e-8, -1e-8])
def test_thickening_or_thinning_column_follows_the_heat_equation(oracle_cls, a0):
    """test/test_thermodynamics.jl:293-320: with accumulation ±1e-8 m/s the column follows the heat equation in fixed
    height under the moving surface, T = T₀ - G z / k + B exp(-κ λ² t) cos(λ z); second-order convergence."""
    H0, G, Tb, B, lam, t_end = 1000.0, 0.04, 240.0, 5.0, math.pi / 1000, 2e10
    kappa = K / (RHO * CI)

    def exact(z, t):
        return Tb - G * z / K + B * math.exp(-kappa * lam ** 2 * t) * np.cos(lam * z)

    errors = []
    for Nsigma in (10, 20, 40):
        c = Column(oracle_cls, H0=H0, Nsigma=Nsigma, G=G)
        c.P.energy_set("surface_mass_balance", a0)
        c.set_temperature(exact(c.zeta * H0, 0.0))
        Nt = 4 * Nsigma ** 2
        dt = t_end / Nt
        for n in range(1, Nt + 1):
            c.P.energy_set("surface_temperature", float(exact(H0 + a0 * n * dt, n * dt)))
            c.P.step_thickness(dt)
            c.step(dt)
        H = float(c.P.get("H")[0, 0])
        assert abs(H - (H0 + a0 * t_end)) <= 1.4901161193847656e-08 * H
        errors.append(float(np.max(np.abs(c.column("T") - exact(c.zeta * H, t_end)))))
    assert errors[2] < 0.03
    assert errors[0] / errors[1] > 2.5 and errors[1] / errors[2] > 2.5


def test_uniform_enthalpy_stays_uniform(oracle_cls):
    """test/test_thermodynamics.jl:322-331 with patch_model (:50-63): an 8 x 8 periodic patch with variable thickness,
    layer velocities that shear with depth, accumulation and basal melt keeps a uniform enthalpy to 1e-9 while the
    thickness changes by more than 10 m."""
    L = 8e4
    g = M.RectilinearGrid(size=(8, 8), x=(0.0, L), y=(0.0, L), topology=("Periodic", "Periodic"), halo=(4, 4))
    P = make(oracle_cls, g, advection=M.UpwindBiased(order=1), Nsigma=10, bed_refinement=2.0, rheology=M.GlenFlowLaw(rate_factor="sigma"),
             constants=M.IceSheetConstants(ice_density=RHO))
    ubar = lambda x, y: 1e-6 * (1 + math.sin(2 * math.pi * y / L) / 2)
    vbar = lambda x, y: 5e-7 * math.cos(2 * math.pi * x / L)
    P.set("H", evaluate(g, "H", lambda x, y: 1000 + 200 * math.sin(2 * math.pi * x / L) * math.cos(2 * math.pi * y / L)))
    P.set("bed", 0.0)
    P.compute_geometry()
    P.set("u", evaluate(g, "u", ubar))
    P.set("v", evaluate(g, "v", vbar))
    faces = np.array(M.sigma_faces(10, 2.0))
    zeta = (faces[1:] + faces[:-1]) / 2
    P.set("u_sigma", np.stack([evaluate(g, "u", ubar) * (0.5 + z) for z in zeta]))
    P.set("v_sigma", np.stack([evaluate(g, "v", vbar) * (0.5 + z) for z in zeta]))
    H = P.get("H")
    P.set("E", np.stack([enthalpy(250.0, 0.0, RHO * GRAV * H * (1 - z)) for z in zeta]))
    for name, value in (("geothermal_flux", 0.0), ("surface_temperature", 250.0), ("ocean_temperature", 271.15),
                        ("basal_melt_rate", 2e-9), ("H_previous", H), ("Hw", 0.0),
                        ("surface_mass_balance", evaluate(g, "H", lambda x, y: 1e-8 * (1 + math.cos(2 * math.pi * x / L))))):
        P.energy_set(name, value)
    E0 = P.get("E")[0, 0, 0]
    for _ in range(20):
        P.step_thickness(1e9, grounded_melt_coupling=True)
        P.step_enthalpy(1e9, grounded_melt_coupling=True)
    assert np.max(np.abs(P.get("H") - H)) > 10
    assert np.max(np.abs(P.get("E") - E0)) < 1e-9 * E0


def test_strong_accumulation_over_a_sharp_front_creates_no_new_extrema(oracle_cls):
    """test/test_thermodynamics.jl:360-370: 2e-7 m/s of accumulation over a 230 / 260 K step keeps every layer
    within [230, 260] K for 20 steps of 1e8 s."""
    c = Column(oracle_cls, H0=1000.0, Nsigma=10, G=0.0, Ts=250.0)
    c.P.energy_set("surface_mass_balance", 2e-7)
    c.set_temperature(np.where(c.zeta < 0.5, 230.0, 260.0))
    for _ in range(20):
        c.P.step_thickness(1e8)
        c.step(1e8)
        T = c.column("T")
        assert np.min(T) >= 230 - 1e-8 and np.max(T) <= 260 + 1e-8


@pytest.mark.parametrize("direction", ["x", "y"])
def test_upwind_transport_at_unit_courant_number_shifts_each_layer(oracle_cls, direction):
    """test/test_thermodynamics.jl:372-390: on an 8-cell periodic row (Nσ = 4, conduction switched off with
    k = 1e-12), layer velocities of one cell per step above ζ = 0.5 and none below move the upper two layers'
    enthalpy by exactly one cell and leave the lower two, to 1e-10, with no vertical flux."""
    Nx, dx, dt = 8, 1e3, 1e9
    size = (Nx, 1) if direction == "x" else (1, Nx)
    g = M.RectilinearGrid(size=size, x=(0.0, size[0] * dx), y=(0.0, size[1] * dx), topology=("Periodic", "Periodic"), halo=(3, 3))
    P = make(oracle_cls, g, advection=M.UpwindBiased(order=1), Nsigma=4, bed_refinement=1.0, rheology=M.GlenFlowLaw(rate_factor="sigma"))
    P.set("H", 500.0)
    P.set("bed", 0.0)
    P.compute_geometry()
    zeta = (np.arange(4) + 0.5) / 4
    name = "u_sigma" if direction == "x" else "v_sigma"
    P.set(name, np.stack([np.full(P.shape(name)[1:], dx / dt if z > 0.5 else 0.0) for z in zeta]))
    pos = g.centers(0) if direction == "x" else g.centers(1)
    T = 250 + 10 * np.sin(2 * math.pi * pos / (Nx * dx))
    T2 = T.reshape(1, -1) if direction == "x" else T.reshape(-1, 1)
    P.set("E", np.stack([enthalpy(T2, 0.0, 918.0 * GRAV * 500.0 * (1 - z)) for z in zeta]))
    for name_, value in (("geothermal_flux", 0.0), ("surface_temperature", 243.15), ("ocean_temperature", 271.15),
                         ("basal_melt_rate", 0.0), ("H_previous", 500.0), ("Hw", 0.0), ("surface_mass_balance", 0.0)):
        P.energy_set(name_, value)
    E0 = P.get("E")
    P.step_thickness(dt)
    P.step_enthalpy(dt, thermal_conductivity=1e-12)
    E = P.get("E")
    np.testing.assert_allclose(E[:2], E0[:2], rtol=1e-10)
    axis = 2 if direction == "x" else 1
    np.testing.assert_allclose(E[2:], np.roll(E0[2:], 1, axis=axis), rtol=1e-10)


@pytest.mark.parametrize("shear", [None, M.DIVAShear()], ids=["SSA", "DIVA"])
def test_friction_and_strain_heat_account_for_the_driving_work(oracle_cls, shear):
    """test/test_thermodynamics.jl:392-398 with dissipation_mismatch (:65-95): on a 16 x 16 periodic sheet (Weertman
    m = 1, A = 1e-24) after one time step of 1e6 s with converged velocities, the basal heat qᵍ plus the strain
    heat H Σ Δζ Φ of the energy step equals the power Σ τ⋅u of the driving stress to 1e-8.  For the SSA the
    membrane heat 4 η ε̇ₑ² balances the viscous work exactly (the corner viscosity is the mean of the four
    centres); for the DIVA the shear heat τᵇ² F₂ adds the work of the vertical shear."""
    Nx, L = 16, 3.2e5
    g = M.RectilinearGrid(size=(Nx, Nx), x=(0.0, L), y=(0.0, L), topology=("Periodic", "Periodic"), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-12, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-11, maxiter=500))
    P = make(oracle_cls, g, advection=M.UpwindBiased(order=1), Nsigma=10, rheology=M.GlenFlowLaw(rate_factor=1e-24, strain_rate_regularization=1e-16),
             friction=M.WeertmanFriction(coefficient=1e10, exponent=1.0), velocity_solver=solver,
             stress_balance=M.DepthIntegrated(shear=shear), constants=M.IceSheetConstants(ice_density=RHO))
    P.set("H", evaluate(g, "H", lambda x, y: 1000 + 100 * math.sin(2 * math.pi * x / L) * math.cos(2 * math.pi * y / L)))
    P.set("bed", 0.0)
    P.set("A", 1e-24)
    P.set("C", 1e10)
    P.compute_geometry()
    assert P.picard_solve().status == 0                 # set!(model; H): the velocity solve of update_state!
    P.velocity_profile()
    for name, value in (("geothermal_flux", 0.0), ("surface_temperature", 243.15), ("ocean_temperature", 271.15),
                        ("basal_melt_rate", 0.0), ("H_previous", P.get("H")), ("Hw", 0.0), ("surface_mass_balance", 0.0)):
        P.energy_set(name, value)
    P.set("E", enthalpy(243.15, 0.0, 0.0))
    dt = 1e6
    P.step_thickness(dt)
    assert P.picard_solve().status == 0                 # the final stage's velocity update
    P.velocity_profile()
    P.step_enthalpy(dt)
    faces = np.array(M.sigma_faces(10))
    dz = np.diff(faces)[:, None, None]
    H = P.get("H")
    strain = np.sum(dz * P.energy_get("strain_heating"), axis=0)
    area = (L / Nx) ** 2
    heat = area * float(np.sum(P.energy_get("basal_heat_flux") + H * strain))
    power = float(np.sum(P.get("tau_u") * P.get("u")) + np.sum(P.get("tau_v") * P.get("v")))
    assert power > 0
    assert abs(heat - power) / power < 1e-8, (heat, power)


def seeded_energy_case(cls, shear, state=None):
    """Two energy steps of a seeded sheet on backend cls.  Without `state` the oracle solves the velocities and
    returns their state with the result; with it, that state is set instead of solving."""
    rng = np.random.default_rng(1203)
    Nx, Ny, Ns = 24, 20, 8
    g = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * 2e3), y=(0.0, Ny * 2e3), topology=("Bounded", "Periodic"), halo=(4, 4))
    P = make(cls, g, advection=M.UpwindBiased(order=1), Nsigma=Ns, rheology=M.GlenFlowLaw(rate_factor="sigma"), grounding=M.SubgridGroundedFraction(),
             friction=M.WeertmanFriction(coefficient=1e10, exponent=1.0), stress_balance=M.DepthIntegrated(shear=shear),
             constants=M.IceSheetConstants(ice_density=RHO))
    x = g.centers(0)
    H = 900 - 8 * x[None, :] / 1e3 + rng.uniform(0, 50, (Ny, Nx))
    H[rng.uniform(size=(Ny, Nx)) < 0.05] = 0.5
    P.set("H", H)
    P.set("bed", np.broadcast_to(-200 - 12 * x[None, :] / 1e3, (Ny, Nx)) + rng.uniform(-10, 10, (Ny, Nx)))
    P.set("A", 1e-24)
    P.set("C", 1e10)
    P.compute_geometry()
    names = ["u", "v", "eta_sigma", "u_sigma", "v_sigma", "u_b", "v_b"] + (["beta_b_u", "beta_b_v"] if shear else ["beta_u", "beta_v"])
    if state is None:
        assert P.picard_solve().status == 0
        P.velocity_profile()
        state = {k: P.get(k) for k in names}
    else:
        for k in names:
            P.set(k, state[k])
    zeta = np.array([(a + b) / 2 for a, b in zip(M.sigma_faces(Ns)[:-1], M.sigma_faces(Ns)[1:])])
    p = RHO * GRAV * H[None] * (1 - zeta[:, None, None])
    T = 255 + 25 * rng.uniform(size=(Ns, Ny, Nx))
    w = np.where(rng.uniform(size=(Ns, Ny, Nx)) < 0.3, rng.uniform(0, 0.04, (Ns, Ny, Nx)), 0.0)
    P.set("E", enthalpy(T, w, p))
    for name, value in (("Hw", np.where(rng.uniform(size=(Ny, Nx)) < 0.5, rng.uniform(0, 0.01, (Ny, Nx)), 0.0)),
                        ("geothermal_flux", rng.uniform(0.04, 0.08, (Ny, Nx))),
                        ("surface_temperature", rng.uniform(240, 265, (Ny, Nx))),
                        ("ocean_temperature", rng.uniform(270, 272, (Ny, Nx))),
                        ("H_previous", H * (1 + rng.uniform(-0.01, 0.01, (Ny, Nx)))),
                        ("basal_melt_rate", rng.uniform(0, 1e-8, (Ny, Nx))),
                        ("grounded_melt", rng.uniform(0, 1e-10, (Ny, Nx)))):
        P.energy_set(name, value)
    for _ in range(2):
        P.step_enthalpy(3e9)
    out = {k: P.get(k) for k in ("E", "T", "omega")}
    for k in ("Hw", "grounded_melt", "basal_temperate_fraction", "basal_heat_flux", "strain_heating", "H_previous"):
        out[k] = P.energy_get(k)
    P.close()
    return out, state


@pytest.mark.parametrize("shear", [None, M.DIVAShear()], ids=["SSA", "DIVA"])
def test_seeded_energy_case_exercises_every_branch(oracle_cls, shear):
    out, _ = seeded_energy_case(oracle_cls, shear)
    assert np.any(out["omega"] > 0.01) and np.any(out["omega"] == 0.0)        # temperate and cold layers
    assert np.any(out["Hw"] > 0) and np.any(out["Hw"] == 0.0)                  # wet and dry beds
    assert np.any(out["basal_temperate_fraction"] > 0) and np.any(out["strain_heating"] > 0)


@pytest.mark.gpu
@pytest.mark.parametrize("shear", [None, M.DIVAShear()], ids=["SSA", "DIVA"])
def test_gpu_energy_step_matches_the_oracle(oracle_cls, gpu_cls, shear):
    want, state = seeded_energy_case(oracle_cls, shear)
    got, _ = seeded_energy_case(gpu_cls, shear, state)
    for k in want:
        scale = max(1e-300, float(np.max(np.abs(want[k]))))
        np.testing.assert_allclose(got[k], want[k], rtol=1e-10, atol=1e-10 * scale, err_msg=k)


def uniform_sheet(cls, N):
    """An N x N periodic sheet at rest, every column alike: 1000 m of ice with a temperate base over a wet bed."""
    g = M.RectilinearGrid(size=(N, N), x=(0.0, N * 1e3), y=(0.0, N * 1e3), topology=("Periodic", "Periodic"), halo=(4, 4))
    Ns = 16
    P = make(cls, g, advection=M.UpwindBiased(order=1), Nsigma=Ns, rheology=M.GlenFlowLaw(rate_factor="sigma"), constants=M.IceSheetConstants(ice_density=RHO))
    P.set("H", 1000.0)
    P.set("bed", 0.0)
    P.compute_geometry()
    zeta = np.array([(a + b) / 2 for a, b in zip(M.sigma_faces(Ns)[:-1], M.sigma_faces(Ns)[1:])])
    T = np.minimum(243.15 + 35 * (1 - zeta), 300.0)
    w = np.where(zeta < 0.1, 0.02, 0.0)
    E = enthalpy(T, w, RHO * GRAV * 1000.0 * (1 - zeta))
    P.set("E", np.broadcast_to(E[:, None, None], (Ns, N, N)).copy())
    for name, value in (("Hw", 0.005), ("geothermal_flux", 0.06), ("surface_temperature", 243.15),
                        ("ocean_temperature", 271.15), ("H_previous", 1000.0)):
        P.energy_set(name, value)
    for _ in range(3):
        P.step_enthalpy(1e9)
    out = {k: P.get(k) for k in ("E", "T", "omega")}
    out["Hw"] = P.energy_get("Hw")
    out["grounded_melt"] = P.energy_get("grounded_melt")
    P.close()
    return out


@pytest.mark.gpu
def test_gpu_uniform_columns_stay_alike_at_1024(oracle_cls, gpu_cls):
    """At rest every column of a uniform sheet takes the same three energy steps: at 1024 x 1024 the library's
    columns agree bitwise with each other and with the oracle's single-column result to 1e-10."""
    want = uniform_sheet(oracle_cls, 1)
    got = uniform_sheet(gpu_cls, 1024)
    for k, a in got.items():
        first = a[..., :1, :1]
        assert np.array_equal(a, np.broadcast_to(first, a.shape)), k
        np.testing.assert_allclose(first, want[k], rtol=1e-10, atol=1e-10 * max(1e-300, float(np.max(np.abs(want[k])))), err_msg=k)


def test_uniform_sheet_melts_and_drains(oracle_cls):
    out = uniform_sheet(oracle_cls, 2)
    assert np.all(out["Hw"] > 0.005) and np.all(out["grounded_melt"] > 0)
    assert np.all(out["E"] == out["E"][:, :1, :1])
