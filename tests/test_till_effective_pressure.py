"""TillEffectivePressure (src/Thermodynamics/till_effective_pressure.jl) through nk_set_till / nko_set_till: the
testsets of test/test_till_effective_pressure.jl on the oracle (CPU) and the library (GPU).

- dry, partly wet, saturated and floating till: N is the ocean-connected value where the dry till would carry more,
  the till's own value between, δ P₀ once saturated (and beyond), zero where the ice floats;
- ice-free cells have zero effective pressure;
- one time step of a two-column sheet at rest (Nσ = 10, ρᵢ = 910, no geothermal heat): the till drains the basal
  water by Δt times its rate and caps it at its maximum, the grounded melt rate is that of the water balance before
  the drainage, the geometry diagnosed before the energy step sees the old water and the next one the new;
- the library's N and energy step equal the oracle's on a seeded sheet."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import make

RHO_DEFAULT, RHO, GRAV = 918.0, 910.0, 9.81
CI, TR, T0, BETA = 2009.0, 223.15, 273.15, 7.9e-8


def till_effective_pressure(law, P0, Hw):
    """The testset's own closed form (test/test_till_effective_pressure.jl:3-9)."""
    s = np.clip(np.asarray(Hw, dtype=np.float64) / law.maximum_water_thickness, 0, 1)
    Nt = law.reference_effective_pressure * (law.overburden_fraction * P0 / law.reference_effective_pressure) ** s * \
        10 ** (law.reference_void_ratio / law.compressibility * (1 - s))
    return np.minimum(Nt, P0)


def test_dry_partly_wet_saturated_and_floating_till(backend):
    g = M.RectilinearGrid(size=(5, 1), x=(0.0, 5.0), y=(0.0, 1.0), topology=("Bounded", "Periodic"), halo=(3, 3))
    law = M.TillEffectivePressure()
    P = make(backend, g, Nsigma=2)
    P.set_till(law)
    H0, Hws = 1000.0, np.array([0, 1.5, 2, 3, 1.0])
    P.set("H", H0)
    P.set("bed", np.array([[0.0, 0.0, 0.0, 0.0, -2000.0]]))
    P.energy_set("Hw", Hws[None, :])
    P.compute_geometry()
    P0 = RHO_DEFAULT * GRAV * H0
    N = P.get("N")[0]
    assert math.isclose(N[0], P0, rel_tol=1e-12)
    assert math.isclose(N[1], till_effective_pressure(law, P0, 1.5), rel_tol=1e-12) and N[1] < P0
    assert math.isclose(N[2], law.overburden_fraction * P0, rel_tol=1e-12)
    assert math.isclose(N[3], law.overburden_fraction * P0, rel_tol=1e-12)
    assert N[4] == 0
    assert N[0] > N[1] > N[2]
    P.set_till(None)   # back to the ocean-connected law
    P.compute_geometry()
    assert np.allclose(P.get("N")[0, :4], P0, rtol=1e-14, atol=0)


def test_ice_free_cells_have_zero_effective_pressure(backend):
    g = M.RectilinearGrid(size=(2, 1), x=(0.0, 2.0), y=(0.0, 1.0), topology=("Bounded", "Periodic"), halo=(3, 3))
    P = make(backend, g, Nsigma=2)
    P.set_till(M.TillEffectivePressure())
    P.set("H", np.array([[0.0, 100.0]]))
    P.set("bed", 0.0)
    P.energy_set("Hw", 1.0)
    P.compute_geometry()
    N = P.get("N")[0]
    assert N[0] == 0 and N[1] > 0


def till_column(cls, till, Hw=(1.5, 3.0), H0=1000.0):
    """till_column_model: two periodic columns at rest, Nσ = 10, ρᵢ = 910, no geothermal heat, first-order upwinding,
    the cold surface enthalpy throughout, basal water Hw per column."""
    g = M.RectilinearGrid(size=(2, 1), x=(0.0, 2e3), y=(0.0, 1e3), topology=("Periodic", "Periodic"), halo=(3, 3))
    P = make(cls, g, advection=M.UpwindBiased(order=1), Nsigma=10, rheology=M.GlenFlowLaw(rate_factor="sigma"),
             constants=M.IceSheetConstants(ice_density=RHO))
    if till is not None:
        P.set_till(till)
    P.set("H", H0)
    P.set("bed", 0.0)
    P.set("u", 0.0)
    P.set("v", 0.0)
    for name, value in (("geothermal_flux", 0.0), ("surface_temperature", 253.15), ("ocean_temperature", 271.15),
                        ("basal_melt_rate", 0.0), ("surface_mass_balance", 0.0), ("clipped_thickness", 0.0),
                        ("H_previous", H0), ("Hw", np.array([list(Hw)]))):
        P.energy_set(name, value)
    P.set("E", np.full((10, 1, 2), CI * (253.15 - TR)))
    P.compute_geometry()
    return P


def time_step(P, dt):
    """time_step! of a model without a velocity solver: the three thickness stages, then the energy step."""
    P.step_thickness(dt)
    P.step_enthalpy(dt, grounded_melt_coupling=True)


def test_the_till_drains_and_is_capped_and_the_model_sees_it(backend):
    dt = 365.25 * 86400
    law = M.TillEffectivePressure()
    ref, till = till_column(backend, None), till_column(backend, law)
    time_step(ref, dt)
    time_step(till, dt)
    Hw_r, Hw_t = ref.energy_get("Hw")[0], till.energy_get("Hw")[0]
    assert math.isclose(Hw_t[0], Hw_r[0] - dt * law.drainage_rate, rel_tol=1e-12)
    assert Hw_t[1] == law.maximum_water_thickness
    assert Hw_r[1] > law.maximum_water_thickness
    assert np.array_equal(till.energy_get("grounded_melt"), ref.energy_get("grounded_melt"))
    P0 = RHO * GRAV * till.get("H")[0]
    # the geometry, and so N, is diagnosed before the energy step updates the water
    assert np.allclose(till.get("N")[0], till_effective_pressure(law, P0, [1.5, 3.0]), rtol=1e-12, atol=0)
    till.compute_geometry()
    assert np.allclose(till.get("N")[0], till_effective_pressure(law, P0, Hw_t), rtol=1e-12, atol=0)
    assert np.allclose(ref.get("N")[0], P0, rtol=1e-12, atol=0)


def test_till_rejects_bad_parameters(backend):
    g = M.RectilinearGrid(size=(2, 1), x=(0.0, 2.0), y=(0.0, 1.0), topology=("Bounded", "Periodic"), halo=(3, 3))
    P = make(backend, g, Nsigma=2)
    for bad in (M.TillEffectivePressure(maximum_water_thickness=0.0), M.TillEffectivePressure(compressibility=-1.0),
                M.TillEffectivePressure(drainage_rate=-1e-9)):
        with pytest.raises(Exception):
            P.set_till(bad)


def seeded_till_sheet(cls):
    """A 24 x 16 sheet over a bed dipping below the sea, seeded thickness, basal water from dry to beyond saturation and
    enthalpy, under a till: N after the geometry, Hw after each of two energy steps, then the grounded melt and N."""
    rng = np.random.default_rng(1204)
    Nx, Ny, Ns = 24, 16, 6
    g = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * 2e3), y=(0.0, Ny * 2e3), topology=("Bounded", "Periodic"), halo=(4, 4))
    P = make(cls, g, advection=M.UpwindBiased(order=1), Nsigma=Ns, rheology=M.GlenFlowLaw(rate_factor="sigma"),
             grounding=M.SubgridGroundedFraction(), constants=M.IceSheetConstants(ice_density=RHO))
    P.set_till(M.TillEffectivePressure(drainage_rate=1e-9))
    x = g.centers(0)
    H = 800 - 10 * x[None, :] / 1e3 + rng.uniform(0, 40, (Ny, Nx))
    H[rng.uniform(size=(Ny, Nx)) < 0.05] = 0.0
    P.set("H", H)
    P.set("bed", np.broadcast_to(100 - 25 * x[None, :] / 1e3, (Ny, Nx)) + rng.uniform(-10, 10, (Ny, Nx)))
    P.set("u", 0.0)
    P.set("v", 0.0)
    zeta = np.array([(a + b) / 2 for a, b in zip(M.sigma_faces(Ns)[:-1], M.sigma_faces(Ns)[1:])])
    p = RHO * GRAV * H[None] * (1 - zeta[:, None, None])
    T = 250 + 25 * rng.uniform(size=(Ns, Ny, Nx))
    P.set("E", CI * (np.minimum(T, T0 - BETA * p) - TR))
    for name, value in (("Hw", rng.uniform(0, 4, (Ny, Nx))), ("geothermal_flux", rng.uniform(0.04, 0.12, (Ny, Nx))),
                        ("surface_temperature", rng.uniform(240, 265, (Ny, Nx))),
                        ("ocean_temperature", rng.uniform(270, 272, (Ny, Nx))), ("H_previous", H),
                        ("basal_melt_rate", 0.0)):
        P.energy_set(name, value)
    P.compute_geometry()
    out = {"N0": P.get("N")}
    for n in range(2):
        P.step_enthalpy(3e7)
        out[f"Hw{n + 1}"] = P.energy_get("Hw")
    P.compute_geometry()
    out.update(N1=P.get("N"), Hw=P.energy_get("Hw"), grounded_melt=P.energy_get("grounded_melt"), E=P.get("E"))
    P.close()
    return out


def test_seeded_till_sheet_exercises_every_branch(oracle_cls):
    out = seeded_till_sheet(oracle_cls)
    Hw1, Hw = out["Hw1"], out["Hw"]   # after the first step (capped cells) and the second (refrozen towards dry)
    assert np.any(Hw1 == M.TillEffectivePressure().maximum_water_thickness)
    assert np.any(Hw == 0.0) and np.any((Hw > 0) & (Hw < 2))
    assert np.any(out["N0"] == 0) and np.any(out["N0"] > 0)


@pytest.mark.gpu
def test_gpu_till_matches_the_oracle(oracle_cls, gpu_cls):
    want, got = seeded_till_sheet(oracle_cls), seeded_till_sheet(gpu_cls)
    for k in want:
        scale = max(1e-300, float(np.max(np.abs(want[k]))))
        np.testing.assert_allclose(got[k], want[k], rtol=1e-10, atol=1e-10 * scale, err_msg=k)
