"""The rate factor from the enthalpy (nk_compute_thermal_diagnostics: update_thermal_diagnostics! with an
ArrheniusRateFactor, src/Thermodynamics/column_energy_solve.jl:85-110), on both backends (the oracle on the CPU,
the GPU library marked gpu), against the reference's own known answers:
- the enthalpy doctest (src/Thermodynamics/enthalpy_conversions.jl:20-33): the enthalpy of 263.15 K ice at 1 MPa
  gives back T = 263.15 K and ω = 0;
- "Enthalpy conversions round trip" (test/test_thermodynamics.jl:99-114): cold ice at three pressures gives back
  its temperature with ω = 0; temperate ice with ω = 0.01 at 10 MPa sits at T_pm = 273.15 - 7.9e-8 p with
  ω = 0.01;
- "Model diagnoses A from the enthalpy" (test/test_rate_factor.jl:157-184): the surface enthalpy of a new model
  (243.15 K, no ice) gives A = cold_branch(243.15); on the
  16 x 4 grid of rate_factor_model (ρᵢ = 910, H = 1000 m, Nσ = 10, Clausius-Clapeyron 7.9e-8), the enthalpy
  E_pm(p) + 0.005 L gives A = warm_branch(273.15) (1 + 181.25 × 0.005) on every layer (rtol 1e-9), and
  E_pm(p) + 0.05 L the capped softening (1 + 181.25 × 0.01).
The enthalpy of a temperature is restated here from enthalpy_conversions.jl:49-52 to build the inputs."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from support import julia_value, make, reference_doctest

HEAT_CAPACITY, LATENT_HEAT, BETA, T0, TR = 2009.0, 3.34e5, 7.9e-8, 273.15, 223.15


def pressure_melting_temperature(p):
    return T0 - BETA * p


def pressure_melting_enthalpy(p):
    return HEAT_CAPACITY * (pressure_melting_temperature(p) - TR)


def enthalpy(T, omega, p):
    """enthalpy(T, ω, p, parameters), src/Thermodynamics/enthalpy_conversions.jl:49-52."""
    return HEAT_CAPACITY * (min(T, pressure_melting_temperature(p)) - TR) + omega * LATENT_HEAT


def warm_branch(t):
    return 1.73e3 * math.exp(-13.9e4 / (8.31441 * t))


def columns(cls, H, Nsigma=1, ice_density=918.0, bed_refinement=2.0):
    """A row of len(H) columns with thicknesses H and the σ-grid rate factor."""
    g = M.RectilinearGrid(size=(len(H), 1), x=(0.0, float(len(H))), y=(0.0, 1.0), topology=("Bounded", "Periodic"), halo=(3, 3))
    P = make(cls, g, Nsigma=Nsigma, bed_refinement=bed_refinement, rheology=M.GlenFlowLaw(rate_factor="sigma"),
             constants=M.IceSheetConstants(ice_density=ice_density), masking=None)
    P.set("H", np.array([H], dtype=np.float64))
    return P


def test_enthalpy_doctest(backend):
    """src/Thermodynamics/enthalpy_conversions.jl:20-33."""
    zeta = 0.5                  # one layer with faces 0 and 1: its centre
    p = 1e6
    P = columns(backend, [p / (918.0 * 9.81 * (1 - zeta))])
    P.set("E", enthalpy(263.15, 0.0, p))
    P.compute_thermal_diagnostics()
    T_doc, w_doc = julia_value(reference_doctest("src/Thermodynamics/enthalpy_conversions.jl", 20)[0])
    assert abs(P.get("T")[0, 0, 0] - T_doc) <= 1e-12 * T_doc
    assert P.get("omega")[0, 0, 0] == w_doc == 0.0


def test_enthalpy_conversions_round_trip(backend):
    """test/test_thermodynamics.jl:99-114."""
    cases = [(243.15, 0.0), (263.15, 5e6), (270.0, 1e7)]
    rhog = 918.0 * 9.81 * 0.5
    P = columns(backend, [p / rhog for _, p in cases])
    P.set("E", np.array([[[enthalpy(T, 0.0, p) for T, p in cases]]]))
    P.compute_thermal_diagnostics()
    T, w = P.get("T")[0, 0], P.get("omega")[0, 0]
    for k, (Tk, _) in enumerate(cases):
        assert abs(T[k] - Tk) <= 1.4901161193847656e-08 * Tk
        assert w[k] == 0.0
    Pa = 1e7
    assert abs(pressure_melting_temperature(Pa) - (273.15 - 7.9e-8 * Pa)) <= 1e-12
    assert abs(enthalpy(300.0, 0.0, Pa) - pressure_melting_enthalpy(Pa)) <= 1e-9
    P = columns(backend, [Pa / rhog])
    P.set("E", enthalpy(pressure_melting_temperature(Pa), 0.01, Pa))
    P.compute_thermal_diagnostics()
    assert abs(P.get("omega")[0, 0, 0] - 0.01) <= 1.4901161193847656e-08 * 0.01
    assert abs(P.get("T")[0, 0, 0] - pressure_melting_temperature(Pa)) <= 1.4901161193847656e-08 * 273.15


def cold_branch(t):
    return 3.61e-13 * math.exp(-6.0e4 / (8.31441 * t))


def test_rate_factor_of_the_surface_enthalpy(backend):
    """test/test_rate_factor.jl:162-165: a new model holds the surface enthalpy enthalpy(243.15, 0, 0) on every layer
    and no ice yet (H = 0, so p = 0), which gives A = cold_branch(243.15)."""
    g = M.RectilinearGrid(size=(16, 4), x=(0.0, 1.6e5), y=(0.0, 4e4), topology=("Bounded", "Bounded"), halo=(4, 4))
    P = make(backend, g, Nsigma=10, rheology=M.GlenFlowLaw(rate_factor="sigma"), constants=M.IceSheetConstants(ice_density=910.0))
    P.set("H", 0.0)
    P.set("E", enthalpy(243.15, 0.0, 0.0))
    P.compute_thermal_diagnostics()
    np.testing.assert_allclose(P.get("A"), cold_branch(243.15), rtol=1.4901161193847656e-08)
    assert np.all(P.get("omega") == 0.0)


@pytest.mark.parametrize("excess,omega_eff", [(0.005, 0.005), (0.05, 0.01)])
def test_rate_factor_of_temperate_ice(backend, excess, omega_eff):
    """test/test_rate_factor.jl:176-184: temperate ice has T′ = T₀ and the water softening, up to the cap."""
    g = M.RectilinearGrid(size=(16, 4), x=(0.0, 1.6e5), y=(0.0, 4e4), topology=("Bounded", "Bounded"), halo=(4, 4))
    P = make(backend, g, Nsigma=10, rheology=M.GlenFlowLaw(rate_factor="sigma"),
             constants=M.IceSheetConstants(ice_density=910.0))
    P.set("H", 1000.0)
    faces = np.array(M.sigma_faces(10))
    zeta = (faces[1:] + faces[:-1]) / 2
    rhog = 910.0 * 9.81
    E = np.array([pressure_melting_enthalpy(rhog * 1000.0 * (1 - z)) + excess * LATENT_HEAT for z in zeta])
    P.set("E", np.broadcast_to(E[:, None, None], (10, 4, 16)).copy())
    P.compute_thermal_diagnostics(clausius_clapeyron=7.9e-8)
    A = P.get("A")
    expected = warm_branch(273.15) * (1 + 181.25 * omega_eff)
    np.testing.assert_allclose(A, expected, rtol=1e-9)
    np.testing.assert_allclose(P.get("omega"), np.broadcast_to(np.full(10, excess)[:, None, None], (10, 4, 16)), rtol=1e-9)


def test_thermal_diagnostics_need_the_sigma_layout(backend):
    g = M.RectilinearGrid(size=(4, 4), x=(0.0, 1.0), y=(0.0, 1.0), halo=(3, 3))
    P = make(backend, g, Nsigma=2, rheology=M.GlenFlowLaw(rate_factor=1e-24))
    with pytest.raises(ValueError):
        P.compute_thermal_diagnostics()
    with pytest.raises(ValueError):
        columns(backend, [100.0]).compute_thermal_diagnostics(heat_capacity=0.0)
