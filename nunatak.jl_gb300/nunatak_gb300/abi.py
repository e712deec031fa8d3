"""ctypes mirror of include/nunatak_gb300.h: constants and descriptor structs of the C ABI."""
import ctypes as C

NK_API_VERSION = 1

NK_OK = 0
NK_NOT_CONVERGED = 1
NK_NONFINITE = 2
NK_BREAKDOWN = 3
NK_OOM = 4
NK_BAD_ARGUMENT = 5
NK_TIMEOUT = 6
NK_CUDA_ERROR = 7
NK_BUSY = 8

STATUS_NAMES = {0: "OK", 1: "NOT_CONVERGED", 2: "NONFINITE", 3: "BREAKDOWN", 4: "OOM",
                5: "BAD_ARGUMENT", 6: "TIMEOUT", 7: "CUDA_ERROR", 8: "BUSY"}

NK_BOUNDED, NK_PERIODIC = 0, 1
NK_FREE_SLIP, NK_NO_SLIP = 0, 1
NK_SSA, NK_DIVA = 0, 1
NK_FRICTION_NONE, NK_WEERTMAN, NK_REGULARIZED_COULOMB = 0, 1, 2
NK_RATE_FACTOR_2D, NK_RATE_FACTOR_SIGMA = 0, 1
NK_PRECONDITIONER_NONE, NK_PRECONDITIONER_DIAGONAL, NK_PRECONDITIONER_MULTIGRID = 0, 1, 2
NK_SMOOTHER_POINT_JACOBI, NK_SMOOTHER_LINE_JACOBI = 0, 1
NK_PRECISION_FP64, NK_PRECISION_MIXED = 0, 1
NK_CONVERGENCE, NK_FIXED_ITERATIONS, NK_VISCOSITY_CONVERGENCE = 0, 1, 2

FIELD_IDS = {
    "u": 0, "v": 1, "H": 2, "bed": 3, "s": 4, "ice_mask": 5, "phi": 6, "phi_u": 7, "phi_v": 8,
    "N": 9, "tau_u": 10, "tau_v": 11, "A": 12, "C": 13, "eta_H": 14, "eta_H_ff": 15,
    "beta_u": 16, "beta_v": 17, "eta_sigma": 18, "F2": 19, "beta_b_u": 20, "beta_b_v": 21,
    "u_b": 22, "v_b": 23, "u_sigma": 24, "v_sigma": 25, "T": 26,
    "u_prescribed": 27, "v_prescribed": 28, "E": 29, "omega": 30,
    "surface_mass_balance": 31, "basal_melt_rate": 32, "grounded_melt": 33, "clipped_thickness": 34,
    "Hw": 35, "geothermal_flux": 36, "surface_temperature": 37, "ocean_temperature": 38, "H_previous": 39,
    "basal_temperate_fraction": 40, "basal_heat_flux": 41, "strain_heating": 42,
    "front_thickness": 43, "calved_thickness": 44, "calving_extent": 45,
}

# (location x, location y, on the sigma grid) of each field: "c" Center, "f" Face.
FIELD_LOCATIONS = {
    "u": ("f", "c", False), "v": ("c", "f", False), "H": ("c", "c", False), "bed": ("c", "c", False),
    "s": ("c", "c", False), "ice_mask": ("c", "c", False), "phi": ("c", "c", False),
    "phi_u": ("f", "c", False), "phi_v": ("c", "f", False), "N": ("c", "c", False),
    "tau_u": ("f", "c", False), "tau_v": ("c", "f", False), "A": ("c", "c", None),
    "C": ("c", "c", False), "eta_H": ("c", "c", False), "eta_H_ff": ("f", "f", False),
    "beta_u": ("f", "c", False), "beta_v": ("c", "f", False), "eta_sigma": ("c", "c", True),
    "F2": ("c", "c", False), "beta_b_u": ("f", "c", False), "beta_b_v": ("c", "f", False),
    "u_b": ("f", "c", False), "v_b": ("c", "f", False), "u_sigma": ("f", "c", True),
    "v_sigma": ("c", "f", True), "T": ("c", "c", True),
    "u_prescribed": ("f", "c", False), "v_prescribed": ("c", "f", False),
    "E": ("c", "c", True), "omega": ("c", "c", True),
    "surface_mass_balance": ("c", "c", False), "basal_melt_rate": ("c", "c", False),
    "grounded_melt": ("c", "c", False), "clipped_thickness": ("c", "c", False),
    "Hw": ("c", "c", False), "geothermal_flux": ("c", "c", False), "surface_temperature": ("c", "c", False),
    "ocean_temperature": ("c", "c", False), "H_previous": ("c", "c", False),
    "basal_temperate_fraction": ("c", "c", False), "basal_heat_flux": ("c", "c", False),
    "strain_heating": ("c", "c", True),
    "front_thickness": ("c", "c", False), "calved_thickness": ("c", "c", False), "calving_extent": ("c", "c", False),
}


class EnergyParams(C.Structure):
    """nk_energy_params: the EnthalpyThermodynamics constants of nk_step_enthalpy."""
    _fields_ = [(n, C.c_double) for n in (
        "thermal_conductivity", "heat_capacity", "latent_heat", "clausius_clapeyron", "melting_temperature",
        "reference_temperature", "temperate_diffusivity_ratio", "enthalpy_blend_width", "water_layer_blend_thickness",
        "minimum_thickness", "drainage_water_fraction", "maximum_drainage_rate")] + \
        [("grounded_melt_coupling", C.c_int32), ("reserved", C.c_int32)]


NK_ADVECTION_UPWIND, NK_ADVECTION_WENO = 0, 1
(NK_CALVING_NONE, NK_CALVING_THICKNESS_THRESHOLD, NK_CALVING_EIGEN, NK_CALVING_VON_MISES, NK_CALVING_FRONT_VELOCITY,
 NK_CALVING_MAXIMUM_EXTENT) = range(6)


class FrontDesc(C.Structure):
    """nk_front_desc: a PartialCellFront and its calving law."""
    _fields_ = [("enabled", C.c_int32), ("passes", C.c_int32), ("calving", C.c_int32), ("reserved", C.c_int32),
                ("thickness", C.c_double), ("coefficient", C.c_double), ("stress_threshold", C.c_double),
                ("floating_stress_threshold", C.c_double), ("front_velocity", C.c_double)]


class TillDesc(C.Structure):
    """nk_till_desc: a TillEffectivePressure (the effective pressure from the basal water, and its drainage)."""
    _fields_ = [("enabled", C.c_int32), ("reserved", C.c_int32), ("reference_effective_pressure", C.c_double),
                ("overburden_fraction", C.c_double), ("reference_void_ratio", C.c_double), ("compressibility", C.c_double),
                ("maximum_water_thickness", C.c_double), ("drainage_rate", C.c_double)]


class AdvectionDesc(C.Structure):
    """nk_advection_desc: the thickness advection scheme of nk_step_thickness."""
    _fields_ = [("scheme", C.c_int32), ("order", C.c_int32), ("bounded", C.c_int32), ("reserved", C.c_int32),
                ("lower", C.c_double), ("upper", C.c_double)]


class IterationControl(C.Structure):
    _fields_ = [("kind", C.c_int32), ("iterations", C.c_int32), ("maxiter", C.c_int32),
                ("reserved", C.c_int32), ("reltol", C.c_double), ("abstol", C.c_double)]


class GridDesc(C.Structure):
    _fields_ = [("Nx", C.c_int32), ("Ny", C.c_int32), ("topology_x", C.c_int32), ("topology_y", C.c_int32),
                ("halo_x", C.c_int32), ("halo_y", C.c_int32), ("Nsigma", C.c_int32), ("reserved", C.c_int32),
                ("x_faces", C.POINTER(C.c_double)), ("y_faces", C.POINTER(C.c_double)),
                ("x0", C.c_double), ("Lx", C.c_double), ("y0", C.c_double), ("Ly", C.c_double),
                ("sigma_faces", C.POINTER(C.c_double)), ("bed_refinement", C.c_double)]


class ThermalParams(C.Structure):
    """nk_thermal_params: ArrheniusParameters and the enthalpy constants the conversions read."""
    _fields_ = [(name, C.c_double) for name in (
        "cold_prefactor", "warm_prefactor", "cold_activation_energy", "warm_activation_energy", "transition_temperature",
        "transition_width", "gas_constant", "water_softening_coefficient", "maximum_water_fraction", "heat_capacity",
        "latent_heat", "clausius_clapeyron", "melting_temperature", "reference_temperature")]


class PhysicsDesc(C.Structure):
    _fields_ = [("stress_balance", C.c_int32), ("side_walls", C.c_int32), ("rate_factor_layout", C.c_int32),
                ("friction", C.c_int32), ("glen_exponent", C.c_double), ("strain_rate_regularization", C.c_double),
                ("friction_exponent", C.c_double), ("coulomb_coefficient", C.c_double),
                ("velocity_regularization", C.c_double), ("ice_density", C.c_double),
                ("ocean_density", C.c_double), ("gravitational_acceleration", C.c_double),
                ("use_ice_mask", C.c_int32), ("grounding", C.c_int32),
                ("grounding_line_driving_stress", C.c_int32), ("use_effective_pressure", C.c_int32),
                ("mask_minimum_thickness", C.c_double), ("mask_transition_thickness", C.c_double)]


class SolverDesc(C.Structure):
    _fields_ = [("precision", C.c_int32), ("preconditioner", C.c_int32), ("smoother", C.c_int32),
                ("smoothing_sweeps", C.c_int32), ("coarsest_sweeps", C.c_int32), ("minimum_coarse_size", C.c_int32),
                ("linear", IterationControl), ("picard", IterationControl), ("flags", C.c_int32), ("reserved", C.c_int32)]


NK_SOLVER_HOST_LOOP = 1


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("picard_iterations", C.c_int32), ("linear_iterations_last", C.c_int32),
                ("linear_iterations_total", C.c_int32), ("residual_norm", C.c_double),
                ("initial_residual_norm", C.c_double), ("picard_change", C.c_double),
                ("picard_norm", C.c_double), ("device_ms", C.c_double),
                ("device_start_ms", C.c_double), ("device_end_ms", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class ServerDesc(C.Structure):
    _fields_ = [("max_in_flight", C.c_int32), ("flags", C.c_int32), ("memory_cap_bytes", C.c_int64), ("batch_slots", C.c_int32),
                ("reserved", C.c_int32)]


NK_SERVER_ADMISSION_THREAD = 1


class Request(C.Structure):
    _fields_ = [("grid", GridDesc), ("physics", PhysicsDesc), ("solver", SolverDesc),
                ("H", C.POINTER(C.c_double)), ("bed", C.POINTER(C.c_double)),
                ("friction_coefficient", C.POINTER(C.c_double)), ("rate_factor", C.POINTER(C.c_double)),
                ("u_init", C.POINTER(C.c_double)), ("v_init", C.POINTER(C.c_double)),
                ("u_out", C.POINTER(C.c_double)), ("v_out", C.POINTER(C.c_double))]


# ---- the gradient through time steps (nk_checkpointed_gradient) ----
class CostState(C.Structure):
    """nk_cost_state: the host copies of the state after `step` steps that the cost callback reads."""
    _fields_ = [("step", C.c_int32), ("steps", C.c_int32), ("H", C.POINTER(C.c_double)), ("u", C.POINTER(C.c_double)),
                ("v", C.POINTER(C.c_double)), ("ice_mask", C.POINTER(C.c_double))]


COST_FN = C.CFUNCTYPE(C.c_int32, C.c_void_p, C.POINTER(CostState), C.POINTER(C.c_double), C.POINTER(C.c_double),
                      C.POINTER(C.c_double), C.POINTER(C.c_double))


class TimeGradientDesc(C.Structure):
    _fields_ = [("dt", C.c_double), ("steps", C.c_int32), ("checkpoint_interval", C.c_int32),
                ("velocity_solves", C.c_int32), ("reserved", C.c_int32), ("melt_weights", C.POINTER(C.c_double)),
                ("adjoint_control", C.POINTER(IterationControl))]


class TimeGradient(C.Structure):
    _fields_ = [(n, C.POINTER(C.c_double)) for n in ("grad_H", "grad_u", "grad_v", "grad_smb", "grad_melt", "grad_log_C",
                                                      "grad_log_A")]


class TimeGradientStats(C.Structure):
    _fields_ = [("J", C.c_double), ("segments", C.c_int32), ("picard_solves", C.c_int32), ("picard_adjoints", C.c_int32),
                ("adjoint_iterations", C.c_int32), ("worst_solve_status", C.c_int32), ("reserved", C.c_int32),
                ("elapsed_ms", C.c_double)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}
