"""The partial-cell front and calving on both backends (the oracle's nko_* on the CPU, the library's nk_* marked gpu):
the testsets of test/test_front_advance.jl and test/test_calving.jl restated, and the library against the oracle on a
seeded front with every calving law.

front_channel (test/test_front_advance.jl:4-13): a channel of full cells of thickness H₀ up to Nfull, Bounded in x,
moved by a prescribed uniform velocity U, first-order upwind transport, PartialCellFront(passes).
calving_channel (test/test_calving.jl:4-13): a floating channel of full cells up to Nfull with open ocean beyond
(bed -500 m), under prescribed velocities, PartialCellFront(calving = law).

The reference's `≈` is isapprox's default relative tolerance √eps ≈ 1.5e-8; its `==` is bitwise here too.  A model
without a flow law (`rheology = nothing`) regularises no strain rate (calving_flow_law, partial_cell_front.jl:272-274):
those channels take strain_rate_regularization = 0."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import evaluate, make

RTOL = 1.5e-8


def front_channel(cls, Nx=16, Ny=4, dx=1e3, U=1.0, H0=100.0, Nfull=4, y_topology="Periodic", advection=None, smb=0.0,
                  passes=4):
    L = Nx * dx
    g = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, L), y=(0.0, Ny * dx), topology=("Bounded", y_topology), halo=(4, 4))
    P = make(cls, g, advection=advection or M.UpwindBiased(order=1), Nsigma=2, masking=M.PartialCellFront(passes=passes),
             rheology=M.GlenFlowLaw(rate_factor=1e-24, strain_rate_regularization=0.0))
    P.set("H", evaluate(g, "H", lambda x, y: H0 if x < Nfull * dx else 0.0))
    P.set("bed", 0.0)
    P.compute_geometry()
    P.initialize_front()
    P.set("u", evaluate(g, "u", lambda x, y: U if 0 < x < L else 0.0))
    P.set("v", 0.0)
    P.energy_set("surface_mass_balance", evaluate(g, "H", smb) if callable(smb) else smb)
    P.energy_set("clipped_thickness", 0.0)
    P.area = dx * dx
    return P


def volume(P):
    return float(np.sum(P.get("H"))) * P.area


# ---- test/test_front_advance.jl ------------------------------------------------------------------------------------
def test_front_advances_one_cell_per_crossing_time(backend):
    """:21-37: a steady inflow U H₀ / Δx into the first cell moves the front one cell per Δx / U."""
    dx, U, H0, Nfull = 1e3, 1.0, 100.0, 4
    P = front_channel(backend, dx=dx, U=U, H0=H0, Nfull=Nfull, smb=lambda x, y: U * H0 / dx if x < dx else 0.0)
    mu = P.get("ice_mask")
    assert np.count_nonzero(mu[0] == 1) == Nfull
    for _ in range(20):
        P.step_thickness(dx / U / 4)
    H, mu = P.get("H"), P.get("ice_mask")
    assert np.all(mu[:, :Nfull + 5] == 1) and np.all(mu[:, Nfull + 5:] == 0)
    assert np.all(H[:, :Nfull + 5] == H0) and np.all(H[:, Nfull + 5:] == 0)


def _set_column(P, name, col, value, rows=slice(None)):
    a = P.get(name)
    a[rows, col] = value
    P.set(name, a)


def test_overfilled_front_cell_spills_and_conserves_volume(backend):
    """:39-53."""
    H0, Nfull = 100.0, 4
    P = front_channel(backend, H0=H0, Nfull=Nfull)
    _set_column(P, "H", Nfull, 2.5 * H0)
    _set_column(P, "ice_mask", Nfull, 0.0)
    V0 = volume(P)
    P.advance_front(1.0)
    H, mu = P.get("H"), P.get("ice_mask")
    np.testing.assert_allclose(H[:, :Nfull + 2], H0, rtol=RTOL)
    np.testing.assert_allclose(H[:, Nfull + 2], H0 / 2, rtol=RTOL)
    assert np.all(mu[:, :Nfull + 2] == 1) and np.all(mu[:, Nfull + 2:] == 0)
    assert math.isclose(volume(P), V0, rel_tol=RTOL)


def test_each_pass_moves_the_overflow_one_cell(backend):
    """:55-67."""
    H0, Nfull = 100.0, 4
    P = front_channel(backend, H0=H0, Nfull=Nfull, passes=1)
    _set_column(P, "H", Nfull, 3 * H0)
    _set_column(P, "ice_mask", Nfull, 0.0)
    P.advance_front(1.0)
    H = P.get("H")
    np.testing.assert_allclose(H[:, Nfull], H0, rtol=RTOL)
    np.testing.assert_allclose(H[:, Nfull + 1], 2 * H0, rtol=RTOL)
    assert np.all(P.get("ice_mask")[:, Nfull + 1] == 0)


def test_front_cell_at_a_wall_thickens(backend):
    """:69-81: a front cell at the east wall keeps its excess instead of spilling into the halo."""
    Nx, H0 = 8, 100.0
    P = front_channel(backend, Nx=Nx, H0=H0, Nfull=Nx, y_topology="Bounded")
    _set_column(P, "H", Nx - 1, 2 * H0)
    _set_column(P, "ice_mask", Nx - 1, 0.0)
    V0 = volume(P)
    P.advance_front(1.0)
    np.testing.assert_allclose(P.get("H")[:, Nx - 1], 2 * H0, rtol=RTOL)
    assert np.all(P.get("ice_mask") == 1)
    assert math.isclose(volume(P), V0, rel_tol=RTOL)


def test_drained_full_cells_become_empty(backend):
    """:83-89."""
    P = front_channel(backend, Nfull=4)
    _set_column(P, "H", 0, 0.0)
    P.advance_front(1.0)
    mu = P.get("ice_mask")
    assert np.all(mu[:, 0] == 0) and np.all(mu[:, 1:4] == 1)


def test_surface_mass_balance_thickens_a_partial_cell(backend):
    """:91-105: without changing its covered fraction."""
    H0, Nfull, a, dt = 100.0, 4, 1e-3, 1e3
    P = front_channel(backend, H0=H0, Nfull=Nfull, U=0.0, smb=a)
    _set_column(P, "H", Nfull, H0 / 4)
    _set_column(P, "front_thickness", Nfull, H0)
    V0 = volume(P)
    P.advance_front(dt)
    np.testing.assert_allclose(P.get("front_thickness")[:, Nfull], H0 + a * dt, rtol=RTOL)
    np.testing.assert_allclose(P.get("H")[:, Nfull], (H0 + a * dt) / 4, rtol=RTOL)
    assert np.all(P.get("H")[:, :Nfull] == H0)
    assert np.all(P.get("ice_mask")[:, Nfull] == 0)
    assert math.isclose(volume(P), V0 + a * dt / 4 * P.area * 4, rel_tol=RTOL)


def test_ablation_empties_a_partial_cell_and_closes_the_budget(backend):
    """:107-123."""
    H0, Nfull, dt = 100.0, 4, 1e3
    a = -2 * H0 / dt
    P = front_channel(backend, H0=H0, Nfull=Nfull, U=0.0, smb=lambda x, y: a if x > Nfull * 1e3 else 0.0)
    _set_column(P, "H", Nfull, H0 / 2)
    _set_column(P, "front_thickness", Nfull, H0)
    V0 = volume(P)
    P.advance_front(dt)
    assert np.all(P.get("H")[:, Nfull] == 0) and np.all(P.get("front_thickness")[:, Nfull] == 0)
    assert np.all(P.get("ice_mask")[:, Nfull] == 0)
    clipped = float(np.sum(P.energy_get("clipped_thickness"))) * P.area
    assert math.isclose(volume(P) - clipped, V0 + a * dt / 2 * P.area * 4, rel_tol=RTOL)


def test_a_filling_cell_is_forced_as_full_and_its_spill_as_partial(backend):
    """:125-140."""
    H0, Nfull, a, dt = 100.0, 4, 1e-3, 1e3
    P = front_channel(backend, H0=H0, Nfull=Nfull, smb=a)
    _set_column(P, "H", Nfull, 1.5 * H0)
    V0 = volume(P)
    P.advance_front(dt)
    H = P.get("H")
    np.testing.assert_allclose(H[:, Nfull], H0 + a * dt, rtol=RTOL)
    np.testing.assert_allclose(H[:, Nfull + 1], (H0 + a * dt) / 2, rtol=RTOL)
    assert np.all(P.get("front_thickness")[:, Nfull] == 0)
    np.testing.assert_allclose(P.get("front_thickness")[:, Nfull + 1], H0 + a * dt, rtol=RTOL)
    assert math.isclose(volume(P), V0 + 1.5 * a * dt * P.area * 4, rel_tol=RTOL)


def test_partial_cell_without_inflow_keeps_its_ice_thickness(backend):
    """:142-152."""
    H0, Nfull = 100.0, 4
    P = front_channel(backend, H0=H0, Nfull=Nfull, U=0.0)
    _set_column(P, "H", Nfull, H0 / 4)
    _set_column(P, "front_thickness", Nfull, 3 * H0)
    P.advance_front(1.0)
    assert np.all(P.get("front_thickness")[:, Nfull] == 3 * H0)
    assert np.all(P.get("H")[:, Nfull] == H0 / 4)


def test_ice_without_inflow_takes_thickness_from_neighbours_or_fills(backend):
    """:154-167."""
    H0, Nfull, a, dt = 100.0, 4, 1e-3, 1e3
    P = front_channel(backend, H0=H0, Nfull=Nfull, U=0.0, smb=a)
    _set_column(P, "H", Nfull, H0 / 4)
    _set_column(P, "H", Nfull + 3, H0 / 4)
    P.advance_front(dt)
    np.testing.assert_allclose(P.get("front_thickness")[:, Nfull], H0 + a * dt, rtol=RTOL)
    np.testing.assert_allclose(P.get("H")[:, Nfull], (H0 + a * dt) / 4, rtol=RTOL)
    assert np.all(P.get("ice_mask")[:, Nfull + 3] == 1)
    np.testing.assert_allclose(P.get("H")[:, Nfull + 3], H0 / 4 + a * dt, rtol=RTOL)


def test_overflow_across_a_periodic_boundary(backend):
    """:169-180: the spill sees the spilling cell's new thickness across the periodic boundary in y."""
    H0, Nfull = 100.0, 4
    P = front_channel(backend, H0=H0, Nfull=Nfull)
    _set_column(P, "H", Nfull, 0.0)
    _set_column(P, "H", Nfull, 2.5 * H0, rows=slice(0, 1))
    _set_column(P, "ice_mask", Nfull, 0.0)
    P.advance_front(1.0)
    Hr = P.get("front_thickness")
    assert Hr[1, Nfull] == H0 and Hr[3, Nfull] == H0


def test_bounded_weno_conserves_volume_through_the_moving_front(backend):
    """:182-199."""
    dx, U, H0, Nfull = 1e3, 1.0, 100.0, 4
    P = front_channel(backend, dx=dx, U=U, H0=H0, Nfull=Nfull, advection=M.WENO(order=5, bounds=(0.0, 1e5)),
                      smb=lambda x, y: U * H0 / dx if x < dx else 0.0)
    V0 = volume(P)
    Nt, dt = 20, dx / U / 4
    for _ in range(Nt):
        P.step_thickness(dt)
    supplied = Nt * dt * U * H0 * 4 * dx
    clipped = float(np.sum(P.energy_get("clipped_thickness"))) * dx * dx
    assert math.isclose(volume(P) - clipped, V0 + supplied, rel_tol=1e-12)
    assert np.count_nonzero(P.get("ice_mask")[0] == 1) >= Nfull + 4
    assert np.all(P.get("H") >= 0)


def test_spreading_floating_shelf_advances_its_front(backend):
    """:201-218, with a converged velocity solve after every thickness step (the reference solves at every stage of
    update_state!): the volume is conserved to 1e-12, the front advances, the rows stay alike, velocities finite."""
    L, x_front, H0, A, Nx = 64e3, 40e3, 500.0, 1e-24, 32
    g = M.RectilinearGrid(size=(Nx, 4), x=(0.0, L), y=(0.0, 4 * L / Nx), topology=("Bounded", "Periodic"), halo=(4, 4))
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-8, maxiter=200))
    P = make(backend, g, advection=M.default_thickness_advection(), Nsigma=2, masking=M.PartialCellFront(),
             rheology=M.GlenFlowLaw(rate_factor=A), friction=M.WeertmanFriction(coefficient=1e6),
             grounding=M.SubgridGroundedFraction(), velocity_solver=solver)
    P.set("H", evaluate(g, "H", lambda x, y: H0 if x < x_front else 0.0))
    P.set("bed", -2000.0)
    P.set("A", A)
    P.set("C", 1e6)
    P.compute_geometry()
    P.initialize_front()
    P.compute_geometry()
    P.set("u", evaluate(g, "u", lambda x, y: 1e-9 * x))
    P.set("v", 0.0)
    P.energy_set("clipped_thickness", 0.0)
    P.picard_solve()
    area = (L / Nx) ** 2
    V0 = float(np.sum(P.get("H"))) * area
    full0 = np.count_nonzero(P.get("ice_mask")[0] == 1)
    for _ in range(10):
        P.step_thickness(5e6)
        P.picard_solve()
    mu = P.get("ice_mask")
    clipped = float(np.sum(P.energy_get("clipped_thickness"))) * area
    assert math.isclose(float(np.sum(P.get("H"))) * area - clipped, V0, rel_tol=1e-12)
    assert np.count_nonzero(mu[0] == 1) > full0
    assert np.all(mu[0] == mu[2])
    assert np.all(np.isfinite(P.get("u")))


# ---- test/test_calving.jl ------------------------------------------------------------------------------------------
def calving_channel(cls, calving, Nx=12, Ny=4, dx=1e3, H0=100.0, Nfull=4, bed=-500.0, y_topology="Periodic", u=0.0, v=0.0,
                    rheology=None, grounding=None):
    g = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * dx), y=(0.0, Ny * dx), topology=("Bounded", y_topology), halo=(4, 4))
    rheology = rheology or M.GlenFlowLaw(rate_factor=1e-24, strain_rate_regularization=0.0)
    P = make(cls, g, Nsigma=2, masking=M.PartialCellFront(calving=calving), rheology=rheology, grounding=grounding)
    P.set("H", evaluate(g, "H", lambda x, y: H0 if x < Nfull * dx else 0.0))
    P.set("bed", bed)
    P.compute_geometry()
    P.initialize_front()
    P.compute_geometry()
    P.set("u", evaluate(g, "u", u) if callable(u) else u)
    P.set("v", evaluate(g, "v", v) if callable(v) else v)
    P.area = dx * dx
    return P


def calved_volume(P):
    return float(np.sum(P.get("calved_thickness"))) * P.area


def test_thickness_threshold_removes_the_marine_front_column(backend):
    """test/test_calving.jl:20-33."""
    H0, Nfull = 100.0, 4
    P = calving_channel(backend, M.ThicknessThresholdCalving(thickness=2 * H0), H0=H0, Nfull=Nfull)
    V0 = volume(P)
    P.advance_front(1.0)
    H, mu = P.get("H"), P.get("ice_mask")
    assert np.all(H[:, :Nfull - 1] == H0) and np.all(mu[:, :Nfull - 1] == 1)
    assert np.all(H[:, Nfull - 1:] == 0) and np.all(mu[:, Nfull - 1:] == 0)
    assert np.all(P.get("calved_thickness")[:, Nfull - 1] == H0)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)


@pytest.mark.parametrize("thickness,bed", [(50.0, -500.0), (200.0, 100.0)])
def test_thick_ice_and_land_fronts_do_not_calve(backend, thickness, bed):
    """:35-43."""
    P = calving_channel(backend, M.ThicknessThresholdCalving(thickness=thickness), bed=bed)
    H0 = P.get("H")
    P.advance_front(1.0)
    assert np.array_equal(P.get("H"), H0)
    assert np.all(P.get("calved_thickness") == 0)


def test_thin_partial_cell_calves_and_leaves_the_full_cells(backend):
    """:45-57."""
    H0, Nfull = 100.0, 4
    P = calving_channel(backend, M.ThicknessThresholdCalving(thickness=2 * H0), H0=H0, Nfull=Nfull)
    _set_column(P, "H", Nfull, H0 / 2)
    _set_column(P, "front_thickness", Nfull, H0)
    P.advance_front(1.0)
    assert np.all(P.get("H")[:, Nfull] == 0)
    assert np.all(P.get("H")[:, :Nfull] == H0) and np.all(P.get("ice_mask")[:, :Nfull] == 1)
    np.testing.assert_allclose(P.get("calved_thickness")[:, Nfull], H0 / 2, rtol=RTOL)


def test_time_stepping_calves_one_column_per_step(backend):
    """:59-69."""
    H0, Nfull = 100.0, 4
    P = calving_channel(backend, M.ThicknessThresholdCalving(thickness=2 * H0), H0=H0, Nfull=Nfull)
    P.set_thickness_advection(M.default_thickness_advection())
    P.energy_set("clipped_thickness", 0.0)
    V0 = volume(P)
    for n in range(1, Nfull + 1):
        P.step_thickness(1.0)
        assert np.all(P.get("ice_mask")[:, :Nfull - n] == 1)
        assert np.all(P.get("H")[:, Nfull - n:] == 0)
    assert math.isclose(calved_volume(P), V0, rel_tol=RTOL)


def test_eigencalving_retreat_under_biaxial_spreading(backend):
    """:71-100."""
    H0, Nfull, dx, Ny, a, b, K, dt = 100.0, 4, 1e3, 6, 1e-9, 1e-9, 1e13, 1e7
    P = calving_channel(backend, M.EigenCalving(coefficient=K), H0=H0, Nfull=Nfull, dx=dx, Ny=Ny, y_topology="Bounded",
                        u=lambda x, y: a * x, v=lambda x, y: b * y, rheology=M.GlenFlowLaw(rate_factor=1e-24))
    V0 = volume(P)
    P.advance_front(dt)
    e0 = 1e-13
    rows = range(1, Ny - 1)
    f = []
    for j in rows:
        y = (j - 0.5) * dx
        exy = -b * y / (4 * dx)
        r = math.sqrt(((a - b) / 2) ** 2 + exy ** 2 + e0 ** 2)
        c = K * max((a + b) / 2 + r, 0) * max((a + b) / 2 - r, 0)
        ub, vb = a * (Nfull - 0.5) * dx, b * y
        f.append(min(1, c * dt * ub / math.sqrt(ub ** 2 + vb ** 2) / dx))
    f = np.array(f)
    H = P.get("H")
    assert np.all((0 < f) & (f < 1))
    np.testing.assert_allclose(H[[j - 1 for j in rows], Nfull - 1], H0 * (1 - f), rtol=RTOL)
    assert list(H[Ny - 2:, Nfull - 1]) == [H0, H0]
    assert np.all(P.get("ice_mask")[[j - 1 for j in rows], Nfull - 1] == 0)
    np.testing.assert_allclose(P.get("front_thickness")[[j - 1 for j in rows], Nfull - 1], H0, rtol=RTOL)
    assert np.all(H[:, :Nfull - 1] == H0)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)


def test_von_mises_retreat_of_a_full_cell_and_its_partial_successor(backend):
    """:102-130."""
    H0, Nfull, dx, a, eta, smax, dt = 100.0, 4, 1e3, 1e-9, 1e14, 3e5, 1e7
    P = calving_channel(backend, M.VonMisesCalving(stress_threshold=smax), H0=H0, Nfull=Nfull, dx=dx, u=lambda x, y: a * x,
                        rheology=M.GlenFlowLaw(rate_factor=1e-24))
    P.set("eta_H", evaluate(P.grid, "eta_H", lambda x, y: eta * H0 if x < Nfull * dx else 0.0))
    n, e0 = 3.0, 1e-13
    e1 = a / 2 + math.sqrt(a ** 2 / 4 + e0 ** 2)
    et2 = e1 ** 2 / 2
    B = 2 * eta * (a ** 2 + e0 ** 2) ** ((n - 1) / (2 * n))
    sig = math.sqrt(3) * B * et2 * (et2 + e0 ** 2) ** ((1 - 2 * n) / (2 * n))

    def speed(ub):
        return math.sqrt(ub ** 2 + (e0 * dx) ** 2)

    f = speed(Nfull * a * dx) * sig / smax * dt / dx
    V0 = volume(P)
    P.advance_front(dt)
    assert 0 < f < 1
    np.testing.assert_allclose(P.get("H")[:, Nfull - 1], H0 * (1 - f), rtol=RTOL)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)
    f2 = speed((Nfull - 1) * a * dx) * sig / smax * dt / dx
    P.advance_front(dt)
    np.testing.assert_allclose(P.get("H")[:, Nfull - 1], H0 * (1 - f - f2), rtol=RTOL)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)


@pytest.mark.parametrize("w", [0.0, -2e-6])
def test_front_velocity_calving_moves_the_front_at_the_set_velocity(backend, w):
    """:132-146."""
    H0, Nfull, dx, U, dt = 100.0, 4, 1e3, 1e-6, 1e8
    P = calving_channel(backend, M.FrontVelocityCalving(front_velocity=w), H0=H0, Nfull=Nfull, dx=dx, u=U,
                        grounding=M.SubgridGroundedFraction())
    V0 = volume(P)
    P.advance_front(dt)
    f = (U - w) * dt / dx
    np.testing.assert_allclose(P.get("H")[:, Nfull - 1], H0 * (1 - f), rtol=RTOL)
    assert np.all(P.get("ice_mask")[:, Nfull - 1] == 0)
    assert np.all(P.get("H")[:, :Nfull - 1] == H0)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)


def test_front_velocity_calving_passes_residual_retreat_behind(backend):
    """:148-167."""
    H0, Nfull, dx, U, dt, w = 100.0, 4, 1e3, 1e-6, 1e8, -5e-6
    P = calving_channel(backend, M.FrontVelocityCalving(front_velocity=w), H0=H0, Nfull=Nfull, dx=dx, u=U,
                        grounding=M.SubgridGroundedFraction())
    _set_column(P, "H", Nfull, H0 / 4)
    _set_column(P, "front_thickness", Nfull, H0)
    V0 = volume(P)
    P.advance_front(dt)
    f = (U - w) * dt / dx
    assert 0.25 < f < 1
    assert np.all(P.get("H")[:, Nfull] == 0)
    np.testing.assert_allclose(P.get("H")[:, Nfull - 1], H0 * (1 - (f - 0.25)), rtol=RTOL)
    assert np.all(P.get("ice_mask")[:, Nfull - 1] == 0)
    assert np.all(P.get("H")[:, :Nfull - 1] == H0)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)


def test_maximum_extent_calving_keeps_the_ice_inside(backend):
    """:169-180."""
    H0, Nfull, dx = 100.0, 4, 1e3
    g_extent = lambda x, y: (Nfull - 1) * dx - x   # noqa: E731
    P = calving_channel(backend, M.MaximumExtentCalving(), H0=H0, Nfull=Nfull, dx=dx)
    P.set("calving_extent", evaluate(P.grid, "H", g_extent))
    V0 = volume(P)
    for _ in range(2):
        P.advance_front(1.0)
        assert np.all(P.get("H")[:, Nfull - 1:] == 0)
        assert np.all(P.get("H")[:, :Nfull - 1] == H0) and np.all(P.get("ice_mask")[:, :Nfull - 1] == 1)
    assert math.isclose(volume(P) + calved_volume(P), V0, rel_tol=RTOL)


# ---- the library against the oracle ---------------------------------------------------------------------------------
LAWS = {"none": None, "threshold": M.ThicknessThresholdCalving(thickness=300.0), "eigen": M.EigenCalving(coefficient=1e14),
        "von_mises": M.VonMisesCalving(stress_threshold=1e6, floating_stress_threshold=2e5),
        "front_velocity": M.FrontVelocityCalving(front_velocity=-2e-7), "extent": M.MaximumExtentCalving()}


def seeded_front(cls, law, steps=4):
    """A 40 x 24 floating shelf with a ragged front over a deepening bed, Bounded x Periodic, seeded thickness, 2-D
    velocities, sources and melt, bounded WENO transport, four steps with the calving law."""
    rng = np.random.default_rng(20261204)
    Nx, Ny, dx = 40, 24, 2e3
    g = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * dx), y=(0.0, Ny * dx), topology=("Bounded", "Periodic"), halo=(4, 4))
    P = make(cls, g, advection=M.default_thickness_advection(), Nsigma=2, masking=M.PartialCellFront(calving=LAWS[law]),
             rheology=M.GlenFlowLaw(rate_factor=1e-24), grounding=M.SubgridGroundedFraction())
    x = g.centers(0)
    front = 50e3 + 8e3 * np.sin(2 * np.pi * g.centers(1) / (Ny * dx))
    H = np.where(x[None, :] < front[:, None], 400.0 - 3e-3 * x[None, :] + rng.uniform(0, 20, (Ny, Nx)), 0.0)
    P.set("H", H)
    P.set("bed", np.broadcast_to(-200.0 - 8e-3 * x[None, :], (Ny, Nx)) + rng.uniform(-5, 5, (Ny, Nx)))
    P.compute_geometry()
    P.initialize_front()
    P.compute_geometry()
    P.set("u", 3e-6 + rng.normal(0, 1e-7, P.shape("u")))
    P.set("v", rng.normal(0.0, 3e-7, P.shape("v")))
    P.set("eta_H", 1e14 * np.maximum(H, 1.0))
    P.set("calving_extent", np.where(x[None, :] < 48e3, 1.0, -1.0) * np.ones((Ny, 1)))
    P.energy_set("surface_mass_balance", rng.uniform(-1e-9, 3e-9, (Ny, Nx)))
    P.energy_set("basal_melt_rate", rng.uniform(0, 1e-8, (Ny, Nx)))
    P.energy_set("clipped_thickness", 0.0)
    for _ in range(steps):
        P.step_thickness(3e5)
    out = {k: P.get(k) for k in ("H", "ice_mask", "front_thickness", "calved_thickness", "s", "phi", "tau_u", "tau_v")}
    out["clipped_thickness"] = P.energy_get("clipped_thickness")
    P.close()
    return out


@pytest.mark.parametrize("law", list(LAWS))
def test_seeded_front_moves_and_calves(oracle_cls, law):
    """The case the library is held to advances and (except without a law) calves."""
    out = seeded_front(oracle_cls, law)
    assert np.all(out["H"] >= 0)
    if law == "none":
        assert np.any((out["front_thickness"] > 0) & (out["ice_mask"] == 0))
    else:
        assert np.max(out["calved_thickness"]) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("law", list(LAWS))
def test_gpu_front_matches_the_oracle(oracle_cls, gpu_cls, law):
    want, got = seeded_front(oracle_cls, law), seeded_front(gpu_cls, law)
    for k in want:
        scale = max(1.0, float(np.max(np.abs(want[k]))))
        np.testing.assert_allclose(got[k], want[k], rtol=1e-10, atol=1e-10 * scale, err_msg=f"{law} {k}")
