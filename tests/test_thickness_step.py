"""The thickness step on both backends (the oracle's nko_step_thickness on the CPU, the library's nk_step_thickness
marked gpu): three split Runge-Kutta stages of the mass balance, src/Models/time_stepping.jl:15-72, with
first-order upwind fluxes, against the first-order testsets of test/test_thickness.jl, and the library against
the oracle on the same seeded inputs.

transport_model (test/test_thickness.jl:4-12): eastward flow u = U sin(πx/L) between walls on a 64 x 4 grid, a
Gaussian bump on a background thickness, velocities held:
- the volume is conserved to 1e-13 (:31-37, the upwind scheme);
- sources change it by 16 Δt (a - m) A to 1e-13 (:39-47);
- uniform flow moves the centre of mass by U t to 1e-12 (:49-58);
- the clip closes the volume budget, V = V₀ - melted + clipped, to 1e-13 (:75-89);
- basal melt acts on the floating part only, ΔH = -Δt m (1 - φ) (:91-102).
The library against the oracle (gpu): a 48 x 40 ice shelf over a sloping bed, Bounded in x and Periodic in y,
with velocities in both directions, the subgrid grounded fraction, sources, grounded melt and the clip, four
steps: H, the clipped thickness and the geometry agree to 1e-12 relative (the grounded fractions feed the
floating melt of the next stage, and the two backends may round them apart by an ulp); at 2048 x 2048 the
library conserves the volume of a periodic sheet without sources to 1e-12."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M, workloads
from support import evaluate, make


class Transport:
    def __init__(self, cls, Nx=64, L=64e3, U=1e-6, width=None, velocity=None, background=0.0, smb=0.0, melt=0.0,
                 advection=None, halo=4):
        width = L / 16 if width is None else width
        self.g = M.RectilinearGrid(size=(Nx, 4), x=(0.0, L), y=(0.0, 4 * L / Nx), topology=("Bounded", "Periodic"),
                                   halo=(halo, halo))
        self.P = make(cls, self.g, advection=advection or M.UpwindBiased(order=1), Nsigma=2, masking=M.SmoothIceMask())
        self.L, self.dx = L, L / Nx
        velocity = velocity or (lambda x, y: U * math.sin(math.pi * x / L))
        self.P.set("H", evaluate(self.g, "H", lambda x, y: background + 100 * math.exp(-((x - L / 4) / width) ** 2)))
        self.P.set("bed", 0.0)
        self.P.compute_geometry()
        self.P.set("u", evaluate(self.g, "u", velocity))
        self.P.set("v", 0.0)
        self.P.energy_set("surface_mass_balance", evaluate(self.g, "H", smb) if callable(smb) else smb)
        self.P.energy_set("basal_melt_rate", evaluate(self.g, "H", melt) if callable(melt) else melt)
        self.P.energy_set("clipped_thickness", 0.0)
        self.umax = float(np.max(np.abs(self.P.get("u"))))

    def volume(self):
        return float(np.sum(self.P.get("H"))) * self.dx * self.g.y[1] / 4

    def timescale(self):
        """cell_advection_timescale: the shortest time to cross a cell."""
        return self.dx / self.umax

    def run(self, dt, n):
        for _ in range(n):
            self.P.step_thickness(dt)


def test_upwind_conserves_volume(backend):
    t = Transport(backend, background=100.0)
    V0 = t.volume()
    t.run(0.5 * t.timescale(), 32)
    assert abs(t.volume() - V0) / V0 < 1e-13


def test_sources_change_the_volume_by_the_integrated_balance(backend):
    a, m = 3e-9, 1e-9
    t = Transport(backend, background=100.0, smb=a, melt=lambda x, y: 2 * m * x / 64e3)
    V0 = t.volume()
    dt = 0.5 * t.timescale()
    t.run(dt, 16)
    expected = V0 + 16 * dt * (a - m) * 64e3 * 4e3
    assert abs(t.volume() - expected) <= 1e-13 * expected


def test_uniform_flow_moves_the_centre_of_mass(backend):
    U, L = 1e-6, 128e3
    t = Transport(backend, U=U, L=L, Nx=128, width=2e3, velocity=lambda x, y: U if 0 < x < L else 0.0)
    x = t.g.centers(0)

    def centre():
        H = t.P.get("H")
        return float(np.sum(H * x[None, :]) / np.sum(H))

    X0 = centre()
    dt = 0.5 * t.timescale()
    assert abs(dt - 0.5 * 1e3 / U) <= 1e-12 * dt
    t.run(dt, 16)
    assert abs(centre() - (X0 + U * 16 * dt)) <= 1e-12 * (X0 + U * 16 * dt)


def test_clipped_thickness_closes_the_volume_budget(backend):
    m = 1e-7
    t = Transport(backend, width=4e3, melt=lambda x, y: m if x > 24e3 else 0.0)
    V0 = t.volume()
    dt, Nt = 0.5 * t.timescale(), 32
    t.run(dt, Nt)
    Az = t.dx * t.g.y[1] / 4
    melted = Nt * dt * float(np.sum(t.P.energy_get("basal_melt_rate"))) * Az
    clipped = float(np.sum(t.P.energy_get("clipped_thickness"))) * Az
    assert clipped > 0
    assert np.min(t.P.get("H")) == 0.0
    assert abs(t.volume() - (V0 - melted + clipped)) < 1e-13 * (V0 + melted)


def test_basal_melt_acts_on_the_floating_part_only(backend):
    Nx, L, H0, m, dt = 8, 8e3, 500.0, 1e-6, 1e3
    g = M.RectilinearGrid(size=(Nx, 1), x=(0.0, L), y=(0.0, L / Nx), topology=("Bounded", "Periodic"), halo=(4, 4))
    P = make(backend, g, advection=M.UpwindBiased(order=1), Nsigma=2, grounding=M.SubgridGroundedFraction())
    P.set("H", H0)
    P.set("bed", evaluate(g, "H", lambda x, y: -100.0 if x < L / 2 else -2000.0))
    P.compute_geometry()
    P.energy_set("basal_melt_rate", m)
    phi = P.get("phi")[0]
    P.step_thickness(dt)
    dH = P.get("H")[0] - H0
    assert phi[0] == 1.0 and phi[-1] == 0.0 and 0 < phi[Nx // 2 - 1] < 1
    np.testing.assert_allclose(dH, -dt * m * (1 - phi), rtol=1e-6)


def seeded_shelf(cls, Nx=48, Ny=40, steps=4, dt=2e8, advection=None, by_stage=False):
    """Four thickness steps of a seeded ice shelf over a sloping bed (grounded at x = 0, afloat downstream),
    Bounded in x and Periodic in y, with random velocities in both directions, the subgrid grounded fraction,
    sources, a coupled grounded melt and thin cells that the melt clips."""
    rng = np.random.default_rng(20261203)
    g = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * 1e3), y=(0.0, Ny * 1e3), topology=("Bounded", "Periodic"), halo=(4, 4))
    P = make(cls, g, advection=advection or M.UpwindBiased(order=1), Nsigma=2, grounding=M.SubgridGroundedFraction(),
             masking=M.SmoothIceMask())
    x = g.centers(0)
    H = 500 - 6 * x[None, :] / 1e3 + rng.uniform(0, 40, (Ny, Nx))
    H[rng.uniform(size=(Ny, Nx)) < 0.08] = 1.0
    P.set("H", H)
    P.set("bed", np.broadcast_to(-300 - 10 * x[None, :] / 1e3, (Ny, Nx)) + rng.uniform(-5, 5, (Ny, Nx)))
    P.compute_geometry()
    P.set("u", rng.normal(5e-7, 5e-7, P.shape("u")))
    P.set("v", rng.normal(0.0, 5e-7, P.shape("v")))
    P.energy_set("surface_mass_balance", rng.uniform(-1e-9, 3e-9, (Ny, Nx)))
    P.energy_set("basal_melt_rate", rng.uniform(0, 2e-8, (Ny, Nx)))
    P.energy_set("grounded_melt", rng.uniform(0, 1e-9, (Ny, Nx)))
    P.energy_set("clipped_thickness", 0.0)
    for _ in range(steps):
        if by_stage:
            for stage in (1, 2, 3):
                P.step_thickness_stage(dt, stage, grounded_melt_coupling=True)
        else:
            P.step_thickness(dt, grounded_melt_coupling=True)
    out = {k: P.get(k) for k in ("H", "s", "phi", "phi_u", "phi_v", "ice_mask", "N", "tau_u", "tau_v")}
    out["clipped_thickness"] = P.energy_get("clipped_thickness")
    P.close()
    return out


def test_seeded_shelf_clips_and_grounds(oracle_cls):
    """The case the library is held to exercises the clip and both grounded and floating cells."""
    out = seeded_shelf(oracle_cls)
    assert np.max(out["clipped_thickness"]) > 0 and np.min(out["H"]) == 0.0
    assert np.any(out["phi"] == 1.0) and np.any(out["phi"] == 0.0)


SCHEMES = {"upwind1": M.UpwindBiased(order=1), "upwind3": M.UpwindBiased(order=3), "weno5": M.WENO(order=5),
           "weno5_bounded": M.WENO(order=5, bounds=(0.0, 1e5))}


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", list(SCHEMES))
def test_gpu_matches_the_oracle(oracle_cls, gpu_cls, scheme):
    want, got = seeded_shelf(oracle_cls, advection=SCHEMES[scheme]), seeded_shelf(gpu_cls, advection=SCHEMES[scheme])
    for k in want:
        scale = max(1.0, float(np.max(np.abs(want[k]))))
        np.testing.assert_allclose(got[k], want[k], rtol=1e-12, atol=1e-12 * scale, err_msg=f"{scheme} {k}")


@pytest.mark.parametrize("scheme", ["upwind1", "weno5_bounded"])
def test_the_three_stages_equal_the_step(backend, scheme):
    """nk_step_thickness_stage 1, 2, 3 in order is nk_step_thickness, bit for bit."""
    want = seeded_shelf(backend, steps=2, advection=SCHEMES[scheme])
    got = seeded_shelf(backend, steps=2, advection=SCHEMES[scheme], by_stage=True)
    for k in want:
        assert np.array_equal(got[k], want[k]), (scheme, k)


def test_stage_refuses_a_stage_outside_one_to_three(backend):
    P = Transport(backend).P
    for stage in (0, 4):
        with pytest.raises(ValueError):
            P.step_thickness_stage(1e6, stage)


@pytest.mark.gpu
def test_reference_schedule_velocity_after_every_stage(oracle_cls, gpu_cls):
    """The reference's default IterationInterval(1) schedule: a velocity solve after every stage (update_state!), so
    each stage advects with the previous stage's velocities; GPU against the oracle over two steps of a marine sheet."""
    out = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-11, maxiter=5000),
                                       picard_iteration_control=M.Convergence(reltol=1e-9, maxiter=3000),
                                       preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=8))
        P = workloads.marine_sheet(32, 16, seed=3, velocity_solver=solver).problem(cls)
        P.set_thickness_advection(M.UpwindBiased(order=1))
        P.energy_set("surface_mass_balance", 1e-9)
        P.energy_set("basal_melt_rate", 2e-9)
        P.energy_set("clipped_thickness", 0.0)
        assert P.picard_solve().status == 0
        for _ in range(2):
            for stage in (1, 2, 3):
                P.step_thickness_stage(3e7, stage)
                assert P.picard_solve().status == 0
        out[key] = (P.get("H"), P.get("u"), P.get("v"))
    for a, b, name in zip(out["g"], out["o"], ("H", "u", "v")):   # two solvers converged to Picard 1e-9
        np.testing.assert_allclose(a, b, rtol=1e-6, atol=1e-6 * float(np.max(np.abs(b))), err_msg=name)


# ---- the reference's higher-order schemes (test/test_thickness.jl:29-73) ------------------------------------------
@pytest.mark.parametrize("scheme", ["upwind1", "upwind3", "weno5", "weno5_bounded_inf"])
def test_volume_is_conserved_by_every_scheme(backend, scheme):
    """test/test_thickness.jl:31-37 for UpwindBiased(order = 1), UpwindBiased(order = 3), WENO(order = 5) and
    WENO(order = 5, bounds = (0, Inf)): 32 steps at half the cell-crossing time conserve the volume to 1e-13."""
    adv = SCHEMES.get(scheme) or M.WENO(order=5, bounds=(0.0, math.inf))
    t = Transport(backend, background=100.0, advection=adv)
    V0 = t.volume()
    t.run(0.5 * t.timescale(), 32)
    assert abs(t.volume() - V0) / V0 < 1e-13


def test_bounded_weno_keeps_a_compact_bump_nonnegative_without_clipping(backend):
    """test/test_thickness.jl:60-73: a 2 km bump on no background, 64 steps at a quarter of the cell-crossing time.
    The bounded WENO stays non-negative and loses no volume to the clip (drift < 1e-12); the unbounded one
    undershoots, and the clip changes its volume by more than 1e-9."""
    drift = []
    for adv in (M.WENO(order=5, bounds=(0.0, math.inf)), M.WENO(order=5)):
        t = Transport(backend, width=2e3, advection=adv)
        V0 = t.volume()
        t.run(0.25 * t.timescale(), 64)
        assert np.min(t.P.get("H")) >= 0
        drift.append(abs(t.volume() - V0) / V0)
    assert drift[0] < 1e-12
    assert drift[1] > 1e-9


def test_bounded_weno_needs_a_halo_of_four(backend):
    """test/test_thickness.jl:70-71 (check_advection_halo, src/Models/ice_sheet_model.jl:131-135): the default bounded
    WENO(order = 5) refuses a grid whose halo is 3 (Oceananigans' default); UpwindBiased(order = 1) steps it."""
    t = Transport(backend, halo=3, advection=M.WENO(order=5, bounds=(0.0, 1e5)))
    with pytest.raises(ValueError):
        t.P.step_thickness(1.0)
    t.P.set_thickness_advection(M.UpwindBiased(order=1))
    t.P.step_thickness(1.0)


def test_default_advection_is_the_bounded_weno(backend):
    """A new problem transports the thickness with the reference's default for the SSA and the DIVA,
    WENO(order = 5, bounds = (0, 1e5)) (src/Models/ice_sheet_model.jl:123): the same result as setting it."""
    out = []
    for adv in (None, M.default_thickness_advection()):
        t = Transport(backend, width=2e3)
        if adv is None:
            t.P.close()
            t.P = make(backend, t.g, Nsigma=2, masking=M.SmoothIceMask())
            t.P.set("H", evaluate(t.g, "H", lambda x, y: 100 * math.exp(-((x - 16e3) / 2e3) ** 2)))
            t.P.set("bed", 0.0)
            t.P.compute_geometry()
            t.P.set("u", evaluate(t.g, "u", lambda x, y: 1e-6 * math.sin(math.pi * x / 64e3)))
            t.P.set("v", 0.0)
        else:
            t.P.set_thickness_advection(adv)
        t.run(0.25 * t.timescale(), 8)
        out.append(t.P.get("H"))
    assert np.array_equal(out[0], out[1])


def test_advection_schemes_are_refused_outside_the_reference(backend):
    P = Transport(backend).P
    for bad in (M.UpwindBiased(order=2), M.UpwindBiased(order=5), M.WENO(order=3), M.WENO(order=5, bounds=(1.0, 0.0))):
        with pytest.raises(ValueError):
            P.set_thickness_advection(bad)


@pytest.mark.gpu
def test_gpu_conserves_volume_at_2048(gpu_cls):
    N, L = 2048, 2048e3
    g = M.RectilinearGrid(size=(N, N), x=(0.0, L), y=(0.0, L), topology=("Periodic", "Periodic"), halo=(4, 4))
    P = make(gpu_cls, g, advection=M.UpwindBiased(order=1), Nsigma=2, masking=M.SmoothIceMask())
    P.set("H", evaluate(g, "H", lambda x, y: 800 + 200 * math.sin(2 * math.pi * x / L) * math.cos(4 * math.pi * y / L)))
    P.set("bed", 0.0)
    P.compute_geometry()
    P.set("u", evaluate(g, "u", lambda x, y: 1e-6 * math.cos(2 * math.pi * y / L)))
    P.set("v", evaluate(g, "v", lambda x, y: 1e-6 * math.sin(2 * math.pi * x / L)))
    V0 = float(np.sum(P.get("H")))
    for _ in range(3):
        P.step_thickness(2e8)
    assert abs(float(np.sum(P.get("H"))) - V0) <= 1e-12 * V0
    assert np.all(P.energy_get("clipped_thickness") == 0.0)
    P.close()
