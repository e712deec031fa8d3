"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the FP64 CPU oracle (oracle/_build/libnunatak_oracle.so).

Used by tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the checker.  The
oracle has the same entry points as the GPU library (nko_* for nk_*), so `OracleProblem` reuses the
argument marshalling of nunatak_gb300.Problem with the oracle's library in place of the GPU one.
"""
import ctypes as C
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG_PARENT = os.path.join(ROOT, "nunatak.jl_gb300")
if PKG_PARENT not in sys.path:
    sys.path.insert(0, PKG_PARENT)

import numpy as np  # noqa: E402

from nunatak_gb300 import abi  # noqa: E402
from nunatak_gb300.problem import Problem, _check, _dptr  # noqa: E402

sys.path.insert(0, HERE)
import build as _oracle_build  # noqa: E402

_LIB = None


def load():
    global _LIB
    if _LIB is None:
        path = _oracle_build.build()
        lib = C.CDLL(path)
        vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
        sig = {
            "nko_problem_create": [C.POINTER(abi.GridDesc), C.POINTER(abi.PhysicsDesc), C.POINTER(abi.SolverDesc), C.POINTER(vp)],
            "nko_problem_destroy": [vp],
            "nko_problem_field_size": [vp, i32],
            "nko_problem_set_field": [vp, i32, dp, i64],
            "nko_problem_get_field": [vp, i32, dp, i64],
            "nko_compute_geometry": [vp],
            "nko_compute_rate_factor": [vp] + [C.c_double] * 9,
            "nko_update_coefficients": [vp],
            "nko_apply_operator": [vp, dp, dp, dp, dp],
            "nko_precondition": [vp, dp, dp, dp, dp],
            "nko_linear_solve": [vp, dp, dp, C.POINTER(abi.SolveStats)],
            "nko_picard_solve": [vp, C.POINTER(abi.SolveStats)],
            "nko_velocity_profile": [vp],
            "nko_compute_thermal_diagnostics": [vp, C.POINTER(abi.ThermalParams)],
            "nko_energy_field": [vp, C.c_int32, dp, i64, C.c_int32],
            "nko_step_enthalpy": [vp, dp, C.c_double],
            "nko_step_thickness": [vp, C.c_double, C.c_int32],
            "nko_step_thickness_stage": [vp, C.c_double, C.c_int32, C.c_int32],
            "nko_set_thickness_advection": [vp, C.POINTER(abi.AdvectionDesc)],
            "nko_set_front": [vp, C.POINTER(abi.FrontDesc)],
            "nko_set_till": [vp, C.POINTER(abi.TillDesc)],
            "nko_initialize_front": [vp],
            "nko_advance_front": [vp, C.c_double],
            "nko_picard_adjoint": [vp, dp, dp, C.POINTER(abi.IterationControl), dp, dp, dp, dp, C.POINTER(abi.SolveStats)],
            "nko_multigrid_levels": [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), i32],
            "nko_multigrid_restrict": [vp, i32, dp, dp, dp, dp],
            "nko_multigrid_prolongate": [vp, i32, dp, dp, dp, dp],
            "nko_grid_metrics": [vp, i32, dp],
            "nko_set_threads": [C.c_int],
            "nko_checkpointed_gradient": [vp, C.POINTER(abi.TimeGradientDesc), abi.COST_FN, vp, C.POINTER(abi.TimeGradient),
                                          C.POINTER(abi.TimeGradientStats)],
        }
        for name, args in sig.items():
            f = getattr(lib, name)
            f.argtypes = args
            f.restype = C.c_int64 if name == "nko_problem_field_size" else C.c_int32
        _LIB = lib
    return _LIB


def set_threads(n):
    return load().nko_set_threads(n)


class OracleProblem(Problem):
    """The oracle's FP64 CPU restatement behind the same methods as nunatak_gb300.Problem."""

    prefix = "nko_"

    def _load(self):
        return load()

    def _create(self):
        st = self._lib.nko_problem_create(C.byref(self.desc.grid), C.byref(self.desc.physics),
                                          C.byref(self.desc.solver), C.byref(self._h))
        _check(st, "oracle problem_create")

    def adjoint_solve(self, bu, bv):
        return self.linear_solve(bu, bv)

    # ---- the energy step (test infrastructure for EnthalpyThermodynamics; no library counterpart yet) ----
    ENERGY_FIELDS = {"Hw": 0, "grounded_melt": 1, "geothermal_flux": 2, "surface_temperature": 3,
                     "ocean_temperature": 4, "basal_melt_rate": 5, "H_previous": 6, "strain_heating": 7,
                     "basal_temperate_fraction": 8, "surface_mass_balance": 9, "clipped_thickness": 10,
                     "basal_heat_flux": 11}

    def _energy_shape(self, name):
        return (self.Nsigma, self.grid.Ny, self.grid.Nx) if name == "strain_heating" else (self.grid.Ny, self.grid.Nx)

    def energy_set(self, name, value):
        a = np.ascontiguousarray(np.broadcast_to(np.asarray(value, dtype=np.float64), self._energy_shape(name)))
        _check(self._lib.nko_energy_field(self._h, self.ENERGY_FIELDS[name], a.ctypes.data_as(_dptr), a.size, 1), "energy_set")

    def energy_get(self, name):
        a = np.empty(self._energy_shape(name))
        _check(self._lib.nko_energy_field(self._h, self.ENERGY_FIELDS[name], a.ctypes.data_as(_dptr), a.size, 0), "energy_get")
        return a

    def step_enthalpy(self, dt, thermal_conductivity=2.1, heat_capacity=2009.0, latent_heat=3.34e5, clausius_clapeyron=7.9e-8,
                      melting_temperature=273.15, reference_temperature=223.15, temperate_diffusivity_ratio=1e-3,
                      enthalpy_blend_width=1.0, water_layer_blend_thickness=1e-3, minimum_thickness=1.0,
                      drainage_water_fraction=0.01, maximum_drainage_rate=1.58443823077064e-9, grounded_melt_coupling=True):
        """One energy step of length dt (step_thermodynamics!); defaults: EnthalpyThermodynamics'."""
        prm = np.array([thermal_conductivity, heat_capacity, latent_heat, clausius_clapeyron, melting_temperature,
                        reference_temperature, temperate_diffusivity_ratio, enthalpy_blend_width, water_layer_blend_thickness,
                        minimum_thickness, drainage_water_fraction, maximum_drainage_rate, float(grounded_melt_coupling)])
        _check(self._lib.nko_step_enthalpy(self._h, prm.ctypes.data_as(_dptr), float(dt)), "step_enthalpy")

    def step_thickness(self, dt, grounded_melt_coupling=False):
        """One ice time step of the thickness with the velocities held (time_step! without a velocity solve)."""
        _check(self._lib.nko_step_thickness(self._h, float(dt), int(grounded_melt_coupling)), "step_thickness")

    def step_thickness_stage(self, dt, stage, grounded_melt_coupling=False):
        """One stage (1, 2, 3) of step_thickness."""
        _check(self._lib.nko_step_thickness_stage(self._h, float(dt), int(stage), int(grounded_melt_coupling)), "step_thickness_stage")

    def grid_metrics(self, which):
        n = (self.grid.Nx if which in (0,) else self.grid.Nx + 1 if which == 1 else self.grid.Ny if which == 2 else self.grid.Ny + 1)
        out = np.empty(n)
        _check(self._lib.nko_grid_metrics(self._h, which, out.ctypes.data_as(_dptr)), "grid_metrics")
        return out
