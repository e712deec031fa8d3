"""Host-side mirror of the reference's solver API over the C ABI of libnunatak_gb300.so.

`Problem` holds one nk_problem: a grid, its fields and coefficients, the solver state and the multigrid
hierarchy, resident on the GPU.  Its methods are the reference's entry points for this path:

  set! / interior(field)            -> Problem.set / Problem.get
  update_geometry! + driving stress -> Problem.compute_geometry   (src/Models/ice_sheet_model_methods.jl:103-111, :126)
  update_stress_balance_coefficients! / update_diva_coefficients!
                                    -> Problem.update_coefficients (stress_balance_coefficients.jl:10-20, diva.jl:61-75)
  ssa_operator!(q, p, ...)          -> Problem.apply_operator      (src/StressBalances/ssa_operator.jl:47-52)
  precondition!(z, P, r, ...)       -> Problem.precondition
  solve!(x, solver, b, ...)         -> Problem.linear_solve        (src/Solvers/conjugate_gradient.jl:128-129)
  adjoint_solve!(λ, solver, b, ...) -> Problem.adjoint_solve       (src/Solvers/conjugate_gradient.jl:155-156)
  picard_solve!(x, picard, ...)     -> Problem.picard_solve        (src/Solvers/picard.jl:63-90)
  compute_velocity_profile! / extend_depth_average! -> Problem.velocity_profile

Errors map the reference's behaviour: a bad argument raises ValueError (ArgumentError), a solve that
stops at maxiter returns its iteration count with stats.status == NOT_CONVERGED (the reference stops
silently), a non-finite result raises FloatingPointError.
"""
import ctypes as C
import warnings

import numpy as np

from . import abi
from .model import Descriptors, field_shape

_dptr = C.POINTER(C.c_double)


class NunatakError(RuntimeError):
    pass


def _warn_unconverged(stats):
    """The reverse rule's warning when maxiter ended the Picard adjoint (ext/NunatakEnzymeExt.jl:222)."""
    if stats.status == abi.NK_NOT_CONVERGED:
        warnings.warn(f"Picard adjoint did not converge in {stats.picard_iterations} iterations: "
                      f"‖Δλ‖ = {stats.picard_change}, ‖λ‖ = {stats.picard_norm}", RuntimeWarning, stacklevel=3)


def _check(status, what, message=""):
    if status == abi.NK_OK:
        return
    name = abi.STATUS_NAMES.get(status, str(status))
    if status == abi.NK_BAD_ARGUMENT:
        raise ValueError(f"{what}: {name} {message}".strip())
    if status == abi.NK_NONFINITE:
        raise FloatingPointError(f"{what}: {name} {message}".strip())
    raise NunatakError(f"{what}: {name} {message}".strip())


def _as_f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Problem:
    """One grid's velocity solve on the GPU (nk_problem)."""

    prefix = "nk_"

    def __init__(self, grid, desc: Descriptors, context=None):
        from . import library
        self.grid = grid
        self.desc = desc
        self.Nsigma = desc.grid.Nsigma
        self.sigma_rate = desc.physics.rate_factor_layout == abi.NK_RATE_FACTOR_SIGMA
        self._lib = self._load()
        self._ctx = context if context is not None else (library.default_context() if self.prefix == "nk_" else None)
        self._h = C.c_void_p()
        self._create()
        if getattr(desc, "front", None) is not None:
            self.set_front(desc.front)

    # -- library plumbing ------------------------------------------------------------------------
    def _load(self):
        from . import library
        return library.load()

    def _fn(self, name):
        return getattr(self._lib, self.prefix + name)

    def _create(self):
        st = self._fn("problem_create")(self._ctx.handle, C.byref(self.desc.grid), C.byref(self.desc.physics),
                                         C.byref(self.desc.solver), C.byref(self._h))
        _check(st, "problem_create", self._ctx.last_error())

    def _err(self):
        return self._ctx.last_error() if self._ctx is not None else ""

    def close(self):
        if self._h:
            self._fn("problem_destroy")(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- fields ----------------------------------------------------------------------------------------
    def shape(self, name):
        return field_shape(self.grid, name, self.Nsigma, self.sigma_rate)

    def set(self, name, value):
        """set!(field, value): a number, or an array in interior layout of shape self.shape(name)."""
        shp = self.shape(name)
        a = np.broadcast_to(np.asarray(value, dtype=np.float64), shp)
        a = _as_f64(a)
        st = self._fn("problem_set_field")(self._h, abi.FIELD_IDS[name], a.ctypes.data_as(_dptr), C.c_int64(a.size))
        _check(st, f"set {name}", self._err())

    def set_device(self, name, address):
        """set!(field, array) from a contiguous float64 array in device memory (its address, e.g. a CUDA
        tensor's data_ptr()) in interior layout of shape self.shape(name)."""
        n = int(np.prod(self.shape(name)))
        st = self._fn("problem_set_field")(self._h, abi.FIELD_IDS[name], C.cast(C.c_void_p(int(address)), _dptr), C.c_int64(n))
        _check(st, f"set {name}", self._err())

    def parent_shape(self, name, halo):
        """Shape of the field's Oceananigans parent array for halo = (hx, hy) or (hx, hy, hz): the interior shape with
        2 hx, 2 hy (and 2 hz levels on the sigma grid) added; C order, x fastest."""
        hx, hy, hz = (tuple(halo) + (0,))[:3]
        shp = self.shape(name)
        if len(shp) == 2:
            return (shp[0] + 2 * hy, shp[1] + 2 * hx)
        return (shp[0] + 2 * hz, shp[1] + 2 * hy, shp[2] + 2 * hx)

    def set_parent(self, name, parent, halo):
        """set! from the field's parent array (interior points read, halos ignored)."""
        hx, hy, hz = (tuple(halo) + (0,))[:3]
        a = _as_f64(np.asarray(parent, dtype=np.float64))
        if a.shape != self.parent_shape(name, halo):
            raise ValueError(f"set_parent {name}: shape {a.shape}, expected {self.parent_shape(name, halo)}")
        st = self._fn("problem_set_field_parent")(self._h, abi.FIELD_IDS[name], a.ctypes.data_as(_dptr), hx, hy, hz, C.c_int64(a.size))
        _check(st, f"set_parent {name}", self._err())

    def get_parent(self, name, parent, halo):
        """Write the field into the interior of `parent` (a C-contiguous float64 array of parent_shape), halos kept."""
        hx, hy, hz = (tuple(halo) + (0,))[:3]
        if parent.dtype != np.float64 or not parent.flags.c_contiguous or parent.shape != self.parent_shape(name, halo):
            raise ValueError(f"get_parent {name}: needs a C-contiguous float64 array of shape {self.parent_shape(name, halo)}")
        st = self._fn("problem_get_field_parent")(self._h, abi.FIELD_IDS[name], parent.ctypes.data_as(_dptr), hx, hy, hz,
                                                  C.c_int64(parent.size))
        _check(st, f"get_parent {name}", self._err())
        return parent

    def get(self, name):
        out = np.empty(self.shape(name), dtype=np.float64)
        st = self._fn("problem_get_field")(self._h, abi.FIELD_IDS[name], out.ctypes.data_as(_dptr), C.c_int64(out.size))
        _check(st, f"get {name}", self._err())
        return out

    # -- the solve --------------------------------------------------------------------------------------
    def compute_geometry(self):
        _check(self._fn("compute_geometry")(self._h), "compute_geometry", self._err())

    def compute_rate_factor(self, cold_prefactor=3.61e-13, warm_prefactor=1.73e3, cold_activation_energy=6.0e4,
                            warm_activation_energy=13.9e4, transition_temperature=263.15, transition_width=1.0,
                            gas_constant=8.31441, clausius_clapeyron=7.9e-8, melting_temperature=273.15):
        """ArrheniusRateFactor defaults (src/Rheologies/arrhenius_rate_factor.jl:60-69) and
        EnthalpyThermodynamics' clausius_clapeyron / melting_temperature (enthalpy_thermodynamics.jl:99-100)."""
        st = self._fn("compute_rate_factor")(self._h, *[C.c_double(v) for v in (
            cold_prefactor, warm_prefactor, cold_activation_energy, warm_activation_energy, transition_temperature,
            transition_width, gas_constant, clausius_clapeyron, melting_temperature)])
        _check(st, "compute_rate_factor", self._err())

    def compute_thermal_diagnostics(self, cold_prefactor=3.61e-13, warm_prefactor=1.73e3, cold_activation_energy=6.0e4,
                                    warm_activation_energy=13.9e4, transition_temperature=263.15, transition_width=1.0,
                                    gas_constant=8.31441, water_softening_coefficient=181.25, maximum_water_fraction=0.01,
                                    heat_capacity=2009.0, latent_heat=3.34e5, clausius_clapeyron=7.9e-8,
                                    melting_temperature=273.15, reference_temperature=223.15):
        """update_thermal_diagnostics! with an ArrheniusRateFactor: T and the water fraction from the enthalpy field
        "E", then the σ-grid rate factor with the water softening.  Defaults: ArrheniusRateFactor
        (src/Rheologies/arrhenius_rate_factor.jl:60-69) and EnthalpyThermodynamics
        (src/Thermodynamics/enthalpy_thermodynamics.jl:92-104)."""
        prm = abi.ThermalParams(cold_prefactor, warm_prefactor, cold_activation_energy, warm_activation_energy,
                                transition_temperature, transition_width, gas_constant, water_softening_coefficient,
                                maximum_water_fraction, heat_capacity, latent_heat, clausius_clapeyron,
                                melting_temperature, reference_temperature)
        _check(self._fn("compute_thermal_diagnostics")(self._h, C.byref(prm)), "compute_thermal_diagnostics", self._err())

    # the thickness and energy steps' sources, state and diagnostics
    TRANSPORT_FIELDS = ("surface_mass_balance", "basal_melt_rate", "grounded_melt", "clipped_thickness", "Hw",
                        "geothermal_flux", "surface_temperature", "ocean_temperature", "H_previous",
                        "basal_temperate_fraction", "basal_heat_flux", "strain_heating")

    def energy_set(self, name, value):
        if name not in self.TRANSPORT_FIELDS:
            raise KeyError(f"the library holds no energy-step field {name!r}")
        self.set(name, value)

    def energy_get(self, name):
        if name not in self.TRANSPORT_FIELDS:
            raise KeyError(f"the library holds no energy-step field {name!r}")
        return self.get(name)

    def step_enthalpy(self, dt, thermal_conductivity=2.1, heat_capacity=2009.0, latent_heat=3.34e5, clausius_clapeyron=7.9e-8,
                      melting_temperature=273.15, reference_temperature=223.15, temperate_diffusivity_ratio=1e-3,
                      enthalpy_blend_width=1.0, water_layer_blend_thickness=1e-3, minimum_thickness=1.0,
                      drainage_water_fraction=0.01, maximum_drainage_rate=1.58443823077064e-9, grounded_melt_coupling=True,
                      rate_factor=None):
        """One energy step of length dt (step_thermodynamics!, src/Thermodynamics/column_energy_solve.jl:26-78) from
        the velocities and viscosity of the last solve (velocity_profile first); defaults: EnthalpyThermodynamics'
        (src/Thermodynamics/enthalpy_thermodynamics.jl:92-104).  The step leaves the rate factor as it was; with
        `rate_factor` (a dict of compute_thermal_diagnostics' keywords, {} for the ArrheniusRateFactor defaults) the
        rate factor follows the new enthalpy, as advance_enthalpy! ends with update_thermal_diagnostics! (:85-97)."""
        prm = abi.EnergyParams(thermal_conductivity, heat_capacity, latent_heat, clausius_clapeyron, melting_temperature,
                               reference_temperature, temperate_diffusivity_ratio, enthalpy_blend_width,
                               water_layer_blend_thickness, minimum_thickness, drainage_water_fraction, maximum_drainage_rate,
                               int(grounded_melt_coupling), 0)
        _check(self._fn("step_enthalpy")(self._h, C.byref(prm), float(dt)), "step_enthalpy", self._err())
        if rate_factor is not None:
            self.compute_thermal_diagnostics(**dict(dict(heat_capacity=heat_capacity, latent_heat=latent_heat,
                                                         clausius_clapeyron=clausius_clapeyron,
                                                         melting_temperature=melting_temperature,
                                                         reference_temperature=reference_temperature), **rate_factor))

    def set_front(self, front):
        """The masking becomes a PartialCellFront (src/Models/partial_cell_front.jl): its 0/1 flag of full cells is the
        ice mask, the thickness step advances the front and calves it under `front.calving`."""
        d = front.desc()
        _check(self._fn("set_front")(self._h, C.byref(d)), "set_front", self._err())
        if getattr(front.calving, "extent", None) is not None:
            self.set("calving_extent", front.calving.extent)

    def set_till(self, till):
        """EnthalpyThermodynamics' effective_pressure: a TillEffectivePressure makes the geometry's N follow the basal
        water (the "Hw" energy field) and the energy step drain it; None restores the ocean-connected N."""
        d = abi.TillDesc() if till is None else till.desc()
        _check(self._fn("set_till")(self._h, C.byref(d)), "set_till", self._err())

    def initialize_front(self):
        """initialize_front!: every cell holding ice is full, none partial (what set!(model; H) does)."""
        _check(self._fn("initialize_front")(self._h), "initialize_front", self._err())

    def advance_front(self, dt):
        """advance_front!(front, model, dt) alone, then the geometry."""
        _check(self._fn("advance_front")(self._h, float(dt)), "advance_front", self._err())

    def set_thickness_advection(self, advection):
        """The thickness advection scheme of step_thickness (IceSheetModel's `advection`): an UpwindBiased(order = 1 or 3)
        or a WENO(order = 5, bounds = None or (lower, upper)); a new problem has WENO(order = 5, bounds = (0, 1e5))."""
        d = advection.desc()
        _check(self._fn("set_thickness_advection")(self._h, C.byref(d)), "set_thickness_advection", self._err())

    def step_thickness(self, dt, grounded_melt_coupling=False):
        """One ice time step of the thickness with the velocities held (the three rk_substep! stages of time_step!,
        src/Models/time_stepping.jl:15-72, with the problem's advection scheme, the geometry after every stage)."""
        _check(self._fn("step_thickness")(self._h, float(dt), int(grounded_melt_coupling)), "step_thickness", self._err())

    def step_thickness_stage(self, dt, stage, grounded_melt_coupling=False):
        """One stage (1, 2 or 3) of step_thickness (nk_step_thickness_stage): a host that solves the velocity after
        every stage, as the reference's default IterationInterval(1) schedule does, calls stage, picard_solve, ..."""
        _check(self._fn("step_thickness_stage")(self._h, float(dt), int(stage), int(grounded_melt_coupling)),
               "step_thickness_stage", self._err())

    def update_coefficients(self):
        _check(self._fn("update_coefficients")(self._h), "update_coefficients", self._err())

    def _vec_in(self, u, v):
        return _as_f64(np.broadcast_to(np.asarray(u, dtype=np.float64), self.shape("u"))), \
               _as_f64(np.broadcast_to(np.asarray(v, dtype=np.float64), self.shape("v")))

    def apply_operator(self, pu, pv, qu=None, qv=None):
        """q = A p (ssa_operator!).  Entries of q outside the Nx x Ny range keep the values passed in."""
        pu, pv = self._vec_in(pu, pv)
        qu = np.zeros(self.shape("u")) if qu is None else _as_f64(qu).copy()
        qv = np.zeros(self.shape("v")) if qv is None else _as_f64(qv).copy()
        st = self._fn("apply_operator")(self._h, pu.ctypes.data_as(_dptr), pv.ctypes.data_as(_dptr),
                                        qu.ctypes.data_as(_dptr), qv.ctypes.data_as(_dptr))
        _check(st, "apply_operator", self._err())
        return qu, qv

    def precondition(self, ru, rv, zu=None, zv=None):
        ru, rv = self._vec_in(ru, rv)
        zu = np.zeros(self.shape("u")) if zu is None else _as_f64(zu).copy()
        zv = np.zeros(self.shape("v")) if zv is None else _as_f64(zv).copy()
        st = self._fn("precondition")(self._h, ru.ctypes.data_as(_dptr), rv.ctypes.data_as(_dptr),
                                      zu.ctypes.data_as(_dptr), zv.ctypes.data_as(_dptr))
        _check(st, "precondition", self._err())
        return zu, zv

    def linear_solve(self, bu, bv):
        """solve!(x, solver, b, coefficients...) from the warm start in fields u, v; returns stats."""
        bu, bv = self._vec_in(bu, bv)
        stats = abi.SolveStats()
        st = self._fn("linear_solve")(self._h, bu.ctypes.data_as(_dptr), bv.ctypes.data_as(_dptr), C.byref(stats))
        _check(st, "linear_solve", self._err())
        return stats

    def adjoint_solve(self, bu, bv):
        """adjoint_solve!(λ, solver, b, ...): λ in fields u, v."""
        bu, bv = self._vec_in(bu, bv)
        stats = abi.SolveStats()
        st = self._fn("adjoint_solve")(self._h, bu.ctypes.data_as(_dptr), bv.ctypes.data_as(_dptr), C.byref(stats))
        _check(st, "adjoint_solve", self._err())
        return stats

    def picard_solve(self):
        """picard_solve!(x, picard, linear_solver, update!, tau, coefficients...): returns stats
        (stats.picard_iterations is the reference's return value)."""
        stats = abi.SolveStats()
        st = self._fn("picard_solve")(self._h, C.byref(stats))
        _check(st, "picard_solve", self._err())
        return stats

    def picard_solve_async(self):
        """Enqueue picard_solve! on this problem's stream and return at once (see wait())."""
        _check(self._fn("picard_solve_async")(self._h), "picard_solve_async", self._err())

    def picard_adjoint(self, ubar, vbar, control=None, thickness=False):
        """Fixed-point adjoint of the converged picard_solve! (the reverse rule of ext/NunatakEnzymeExt.jl:167-240)
        for x̄ = (ubar, vbar) = ∂J/∂(u, v): returns (λu, λv, ∂J/∂log C per cell, ∂J/∂log A in the layout of the rate
        factor, stats), λ being ∂J/∂τ.  `control` is a Convergence / FixedIterations (default: the solver's
        adjoint_iteration_control, which itself defaults to the Picard control).  thickness=True: also ∂J/∂H per
        cell, the total derivative with the geometry and the driving stress recomputed from H
        (nk_picard_adjoint_gradients), returned before the stats."""
        if control is None:
            control = getattr(self.desc, "adjoint_control", None)
        ub, vb = self._vec_in(ubar, vbar)
        lu, lv = np.empty(self.shape("u")), np.empty(self.shape("v"))
        grad = np.empty((self.grid.Ny, self.grid.Nx))
        grad_a = np.empty(self.shape("A"))
        stats = abi.SolveStats()
        ctl = C.byref(control.desc()) if control is not None else None
        if thickness:
            grad_h = np.empty((self.grid.Ny, self.grid.Nx))
            st = self._fn("picard_adjoint_gradients")(self._h, ub.ctypes.data_as(_dptr), vb.ctypes.data_as(_dptr), ctl,
                                                      lu.ctypes.data_as(_dptr), lv.ctypes.data_as(_dptr),
                                                      grad.ctypes.data_as(_dptr), grad_a.ctypes.data_as(_dptr),
                                                      grad_h.ctypes.data_as(_dptr), C.byref(stats))
            _check(st, "picard_adjoint_gradients", self._err())
            _warn_unconverged(stats)
            return lu, lv, grad, grad_a, grad_h, stats
        st = self._fn("picard_adjoint")(self._h, ub.ctypes.data_as(_dptr), vb.ctypes.data_as(_dptr), ctl,
                                        lu.ctypes.data_as(_dptr), lv.ctypes.data_as(_dptr), grad.ctypes.data_as(_dptr),
                                        grad_a.ctypes.data_as(_dptr), C.byref(stats))
        _check(st, "picard_adjoint", self._err())
        _warn_unconverged(stats)
        return lu, lv, grad, grad_a, stats

    def checkpointed_gradient(self, cost, dt, steps, checkpoint_interval=None, velocity_solves=True, melt_weights=None,
                              adjoint_control=None):
        """checkpointed_gradient!(dmodel, cost, model, Δt, Nt; checkpoint_interval) (ext/NunatakEnzymeExt.jl:245-263)
        on the device (nk_checkpointed_gradient): `steps` time steps of dt from the problem's state, each the three
        thickness stages with a Picard solve after every stage (velocity_solves) or with the velocities held.
        cost(step, H, u, v, ice_mask) is called on the state after each step (1..steps) and returns None (no cost
        there) or (J, ∂J/∂H, ∂J/∂u, ∂J/∂v), None for a zero part; the reference's cost of the final model is the one
        returned at step == steps.  melt_weights: a factor of the basal melt rate per step.  Returns a dict: J, the
        gradients "H", "u", "v" (of the initial thickness and velocities), "smb", "melt", "log_C", "log_A" (with
        velocity solves), and "stats".  The problem is left at the final state."""
        errors = []
        shp = {n: self.shape(n) for n in ("H", "u", "v", "ice_mask")}

        def callback(user, state_p, J_p, dH_p, du_p, dv_p):
            try:
                s = state_p.contents
                arrays = [np.ctypeslib.as_array(getattr(s, n), shape=shp[n]).copy() for n in ("H", "u", "v", "ice_mask")]
                r = cost(int(s.step), *arrays)
                J_p[0] = 0.0
                if r is None:
                    return 0
                J, dH, du, dv = r
                J_p[0] = float(J)
                for ptr, arr, n in ((dH_p, dH, "H"), (du_p, du, "u"), (dv_p, dv, "v")):
                    if arr is not None:
                        np.ctypeslib.as_array(ptr, shape=shp[n])[...] = arr
                return 0
            except Exception as e:   # the library stops the gradient; the exception is raised below
                errors.append(e)
                return 1

        cb = abi.COST_FN(callback)
        keep = []
        desc = abi.TimeGradientDesc()
        desc.dt = float(dt)
        desc.steps = int(steps)
        desc.checkpoint_interval = int(checkpoint_interval or 0)
        desc.velocity_solves = int(bool(velocity_solves))
        if melt_weights is not None:
            w = _as_f64(np.asarray(melt_weights, dtype=np.float64).ravel())
            if w.size != steps:
                raise ValueError("melt_weights needs one factor per step")
            keep.append(w)
            desc.melt_weights = w.ctypes.data_as(_dptr)
        if adjoint_control is None:
            adjoint_control = getattr(self.desc, "adjoint_control", None)
        if adjoint_control is not None:
            ctl = adjoint_control.desc()
            keep.append(ctl)
            desc.adjoint_control = C.pointer(ctl)
        grads = {"H": np.zeros(shp["H"]), "u": np.zeros(shp["u"]), "v": np.zeros(shp["v"]), "smb": np.zeros(shp["H"]),
                 "melt": np.zeros(shp["H"]), "log_C": np.zeros(shp["H"]), "log_A": np.zeros(self.shape("A"))}
        out = abi.TimeGradient(*(grads[n].ctypes.data_as(_dptr) for n in ("H", "u", "v", "smb", "melt", "log_C", "log_A")))
        stats = abi.TimeGradientStats()
        st = self._fn("checkpointed_gradient")(self._h, C.byref(desc), cb, None, C.byref(out), C.byref(stats))
        if errors:
            raise errors[0]
        _check(st, "checkpointed_gradient", self._err())
        grads["J"] = stats.J
        grads["stats"] = stats.as_dict()
        return grads

    def query(self):
        """True once the asynchronous solve has finished (wait() then returns at once)."""
        d = C.c_int32()
        _check(self._fn("problem_query")(self._h, C.byref(d)), "problem_query", self._err())
        return bool(d.value)

    def wait(self):
        """Block until the asynchronous solve has finished; returns its stats."""
        stats = abi.SolveStats()
        _check(self._fn("problem_wait")(self._h, C.byref(stats)), "problem_wait", self._err())
        return stats

    def velocity_profile(self):
        _check(self._fn("velocity_profile")(self._h), "velocity_profile", self._err())

    def multigrid_levels(self):
        cap = 64
        nx = (C.c_int32 * cap)()
        ny = (C.c_int32 * cap)()
        count = C.c_int32()
        _check(self._fn("multigrid_levels")(self._h, C.byref(count), nx, ny, cap), "multigrid_levels", self._err())
        return [(nx[i], ny[i]) for i in range(count.value)]

    # -- multigrid transfers -------------------------------------------------------------------------------
    def _level_shape(self, level, comp):
        """(ny, nx) of component comp of a vector on multigrid level `level` (-1 = the finest grid)."""
        nx, ny = (self.grid.Nx, self.grid.Ny) if level < 0 else self.multigrid_levels()[level]
        fx = nx if self.grid.periodic(0) else nx + 1
        fy = ny if self.grid.periodic(1) else ny + 1
        return (ny, fx) if comp == "u" else (fy, nx)

    def restrict(self, level, fu, fv):
        """restrict!: coarse = R fine between level - 1 and coarse level `level` (0 = first coarse level)."""
        fu, fv = _as_f64(fu), _as_f64(fv)
        cu, cv = np.zeros(self._level_shape(level, "u")), np.zeros(self._level_shape(level, "v"))
        st = self._fn("multigrid_restrict")(self._h, level, fu.ctypes.data_as(_dptr), fv.ctypes.data_as(_dptr),
                                            cu.ctypes.data_as(_dptr), cv.ctypes.data_as(_dptr))
        _check(st, "multigrid_restrict", self._err())
        return cu, cv

    def prolongate(self, level, cu, cv, fu=None, fv=None):
        """prolongate!: fine += P coarse (fine starts at zero unless given)."""
        cu, cv = _as_f64(cu), _as_f64(cv)
        fu = np.zeros(self._level_shape(level - 1, "u")) if fu is None else _as_f64(fu).copy()
        fv = np.zeros(self._level_shape(level - 1, "v")) if fv is None else _as_f64(fv).copy()
        st = self._fn("multigrid_prolongate")(self._h, level, cu.ctypes.data_as(_dptr), cv.ctypes.data_as(_dptr),
                                              fu.ctypes.data_as(_dptr), fv.ctypes.data_as(_dptr))
        _check(st, "multigrid_prolongate", self._err())
        return fu, fv

    # -- measurement ---------------------------------------------------------------------------------------
    KERNELS = {"operator_fp64": 0, "smoother": 1, "cg_update": 2, "thickness_stage": 3, "thickness_limiter": 4,
               "step_enthalpy": 5, "thickness_faces": 6}

    def time_kernel(self, kernel, repeats=20, flush_bytes=0):
        """Mean CUDA-event duration (ms) of one launch of a hot kernel and its algorithmic bytes
        (nk_time_kernel); flush_bytes > 0 overwrites a buffer of that size before each launch."""
        ms, by = C.c_double(), C.c_double()
        st = self._fn("time_kernel")(self._h, self.KERNELS[kernel], repeats, C.c_int64(flush_bytes), C.byref(ms), C.byref(by))
        _check(st, "time_kernel", self._err())
        return ms.value, by.value
