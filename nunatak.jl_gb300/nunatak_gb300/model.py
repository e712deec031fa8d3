"""Configuration objects with the reference's names and defaults, and their translation into the C-ABI
descriptors (include/nunatak_gb300.h).  Nothing here touches a device.

Reference constructors mirrored (file:line in Nunatak.jl):
  RectilinearGrid (Oceananigans; halo default 3), SigmaGrid                 src/Grids/sigma_grid.jl:43-62
  Convergence / FixedIterations                                             src/Solvers/iteration_controls.jl:18-43
  GlenFlowLaw(grid; rate_factor, exponent = 3, strain_rate_regularization = 1e-13)   src/Rheologies/glen_flow_law.jl:36-40
  WeertmanFriction(grid; coefficient, exponent = 1/3, velocity_regularization = 1e-8) src/Frictions/frictions.jl:34-37
  RegularizedCoulombFriction(grid; coefficient, coulomb_coefficient, ...)   src/Frictions/frictions.jl:65-71
  DepthIntegrated(; shear = nothing, side_walls = FreeSlipWalls())          src/StressBalances/depth_integrated.jl:29
  SubgridGroundedFraction(; driving_stress = false)                         src/Groundings/subgrid_grounded_fraction.jl:23
  SmoothIceMask(grid; minimum_thickness = 1, transition_thickness = 1)      src/Models/smooth_ice_mask.jl:41-45
  IceSheetConstants(grid; 918, 1028, 9.81)                                  src/Models/ice_sheet_constants.jl:33-36
  StressBalanceMultigridPreconditioner(grid; smoother = PointJacobi(), smoothing_sweeps = 2,
                                       coarsest_sweeps = 20, minimum_coarse_size = 2)   src/StressBalances/multigrid_preconditioner.jl:57
  StressBalanceSolver(grid; linear_iteration_control = Convergence(reltol = 1e-8, maxiter = 10_000),
                      picard_iteration_control = Convergence(reltol = 1e-6, maxiter = 100),
                      adjoint_iteration_control = picard_iteration_control,
                      preconditioner = StressBalanceDiagonalPreconditioner())     src/StressBalances/stress_balance_solver.jl:43-52
"""
import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence, Tuple, Union

import numpy as np

from . import abi

YEAR = 31556926.0   # seconds, benchmarks/multigrid_scaling.jl:8


# ---- grid ---------------------------------------------------------------------------------------
@dataclass
class RectilinearGrid:
    """Horizontal grid, Flat in z.  `x`/`y` are a (start, end) tuple (regular) or a sequence of N+1 faces."""
    size: Tuple[int, int]
    x: Union[Tuple[float, float], Sequence[float]] = (0.0, 1.0)
    y: Union[Tuple[float, float], Sequence[float]] = (0.0, 1.0)
    topology: Tuple[str, str] = ("Bounded", "Bounded")
    halo: Tuple[int, int] = (3, 3)

    @property
    def Nx(self):
        return int(self.size[0])

    @property
    def Ny(self):
        return int(self.size[1])

    def periodic(self, d):
        return self.topology[d] == "Periodic"

    def face_count(self, d):
        n = self.size[d]
        return n if self.periodic(d) else n + 1

    def regular(self, d):
        """A (start, end) tuple is a regular axis; a list or array holds the N + 1 faces."""
        return isinstance(self.x if d == 0 else self.y, tuple)

    def faces(self, d):
        c = self.x if d == 0 else self.y
        n = self.size[d]
        if self.regular(d):
            a, b = float(c[0]), float(c[1])
            return np.array([a + ((i) * (b - a)) / n for i in range(n + 1)])
        return np.asarray(c, dtype=np.float64)

    def centers(self, d):
        f = self.faces(d)
        return (f[1:] + f[:-1]) / 2

    def field_shape(self, location):
        """(nx, ny) of the interior of a field at ('c'|'f', 'c'|'f')."""
        nx = self.face_count(0) if location[0] == "f" else self.Nx
        ny = self.face_count(1) if location[1] == "f" else self.Ny
        return nx, ny


def sigma_faces(Nsigma, bed_refinement=2):
    """sigma_faces(Nσ; bed_refinement = 2) (src/Grids/sigma_grid.jl:20-22): the Nσ + 1 faces (k / Nσ)^bed_refinement
    of the normalised height above the bed, the rule nk_problem_create applies when nk_grid_desc.sigma_faces is
    NULL."""
    return [(k / Nsigma) ** bed_refinement for k in range(Nsigma + 1)]


# ---- iteration controls ---------------------------------------------------------------------------
@dataclass
class Convergence:
    reltol: float = float(np.sqrt(np.finfo(np.float64).eps))
    abstol: float = 0.0
    maxiter: int = 1000

    def desc(self):
        return abi.IterationControl(abi.NK_CONVERGENCE, 0, self.maxiter, 0, self.reltol, self.abstol)


@dataclass
class FixedIterations:
    iterations: int

    def desc(self):
        return abi.IterationControl(abi.NK_FIXED_ITERATIONS, self.iterations, self.iterations, 0, 0.0, 0.0)


@dataclass
class ViscosityConvergence:
    """Picard stopping rule on the relative change of the depth-integrated viscosity between consecutive
    coefficient updates (an extension; the reference's Convergence tests the velocity change)."""
    reltol: float = 1e-6
    abstol: float = 0.0
    maxiter: int = 100

    def desc(self):
        return abi.IterationControl(abi.NK_VISCOSITY_CONVERGENCE, 0, self.maxiter, 0, self.reltol, self.abstol)


# ---- physics ----------------------------------------------------------------------------------------
@dataclass
class FreeSlipWalls:
    code: int = abi.NK_FREE_SLIP


@dataclass
class NoSlipWalls:
    code: int = abi.NK_NO_SLIP


@dataclass
class DIVAShear:
    pass


@dataclass
class DepthIntegrated:
    shear: Optional[DIVAShear] = None
    side_walls: Union[FreeSlipWalls, NoSlipWalls] = field(default_factory=FreeSlipWalls)


@dataclass
class GlenFlowLaw:
    rate_factor: object = None          # number, (Nx, Ny) array, or (Nx, Ny, Nsigma) array on the sigma grid
    exponent: float = 3.0
    strain_rate_regularization: float = 1e-13


@dataclass
class WeertmanFriction:
    coefficient: object = None
    exponent: float = 1.0 / 3
    velocity_regularization: float = 1e-8


@dataclass
class RegularizedCoulombFriction:
    coefficient: object = None
    coulomb_coefficient: float = 0.5
    exponent: float = 1.0 / 3
    velocity_regularization: float = 1e-8


@dataclass
class SubgridGroundedFraction:
    driving_stress: bool = False


@dataclass
class SmoothIceMask:
    minimum_thickness: float = 1.0
    transition_thickness: float = 1.0


# ---- partial-cell front and calving (src/Models/partial_cell_front.jl, src/Models/calving.jl) ----------------------
@dataclass
class ThicknessThresholdCalving:
    thickness: float
    code: int = abi.NK_CALVING_THICKNESS_THRESHOLD


@dataclass
class EigenCalving:
    coefficient: float
    code: int = abi.NK_CALVING_EIGEN


@dataclass
class VonMisesCalving:
    stress_threshold: float
    floating_stress_threshold: Optional[float] = None
    code: int = abi.NK_CALVING_VON_MISES


@dataclass
class FrontVelocityCalving:
    """front_velocity w (m/s) as a number; a time-dependent w(t) is set before each step (Problem.set_front)."""
    front_velocity: float = 0.0
    code: int = abi.NK_CALVING_FRONT_VELOCITY


@dataclass
class MaximumExtentCalving:
    """The region the ice may cover, positive inside: an (Ny, Nx) array or a number, set as the "calving_extent" field."""
    extent: object = None
    code: int = abi.NK_CALVING_MAXIMUM_EXTENT


@dataclass
class TillEffectivePressure:
    """TillEffectivePressure(grid; ...) (src/Thermodynamics/till_effective_pressure.jl:44-57): the effective pressure of
    a saturated till from the basal water (Bueler and van Pelt 2015), capped by the ocean-connected one, and the till's
    drainage of 1 mm per year up to its maximum water thickness."""
    reference_effective_pressure: float = 1000.0
    overburden_fraction: float = 0.02
    reference_void_ratio: float = 0.69
    compressibility: float = 0.12
    maximum_water_thickness: float = 2.0
    drainage_rate: float = 1e-3 / (365.25 * 86400)

    def desc(self):
        return abi.TillDesc(1, 0, float(self.reference_effective_pressure), float(self.overburden_fraction),
                            float(self.reference_void_ratio), float(self.compressibility),
                            float(self.maximum_water_thickness), float(self.drainage_rate))


@dataclass
class PartialCellFront:
    """PartialCellFront(grid; passes = 4, calving = nothing) (src/Models/partial_cell_front.jl:49-54)."""
    passes: int = 4
    calving: object = None

    def desc(self):
        c = self.calving
        d = abi.FrontDesc()
        d.enabled, d.passes = 1, int(self.passes)
        d.calving = abi.NK_CALVING_NONE if c is None else c.code
        if isinstance(c, ThicknessThresholdCalving):
            d.thickness = float(c.thickness)
        elif isinstance(c, EigenCalving):
            d.coefficient = float(c.coefficient)
        elif isinstance(c, VonMisesCalving):
            d.stress_threshold = float(c.stress_threshold)
            d.floating_stress_threshold = float(c.stress_threshold if c.floating_stress_threshold is None else c.floating_stress_threshold)
        elif isinstance(c, FrontVelocityCalving):
            d.front_velocity = float(c.front_velocity)
        return d


@dataclass
class IceSheetConstants:
    ice_density: float = 918.0
    ocean_density: float = 1028.0
    gravitational_acceleration: float = 9.81


# ---- thickness advection ----------------------------------------------------------------------------------
@dataclass
class UpwindBiased:
    """UpwindBiased(order = 1 or 3), Oceananigans' upwind-biased advection of the thickness."""
    order: int = 1

    def desc(self):
        return abi.AdvectionDesc(abi.NK_ADVECTION_UPWIND, int(self.order), 0, 0, 0.0, 0.0)


@dataclass
class WENO:
    """WENO(order = 5), and with `bounds = (lower, upper)` its bounds-preserving form.  The reference's default thickness
    advection for the SSA and the DIVA is WENO(order = 5, bounds = (0, 1e5)) (src/Models/ice_sheet_model.jl:123)."""
    order: int = 5
    bounds: Optional[Tuple[float, float]] = None

    def desc(self):
        lo, hi = self.bounds if self.bounds is not None else (0.0, 0.0)
        return abi.AdvectionDesc(abi.NK_ADVECTION_WENO, int(self.order), 1 if self.bounds is not None else 0, 0, float(lo), float(hi))


def default_thickness_advection():
    """default_thickness_advection(grid, stress_balance) of the SSA and the DIVA (src/Models/ice_sheet_model.jl:123)."""
    return WENO(order=5, bounds=(0.0, 1e5))


# ---- solver -------------------------------------------------------------------------------------------
@dataclass
class PointJacobi:
    code: int = abi.NK_SMOOTHER_POINT_JACOBI


@dataclass
class LineJacobi:
    code: int = abi.NK_SMOOTHER_LINE_JACOBI


@dataclass
class StressBalanceDiagonalPreconditioner:
    code: int = abi.NK_PRECONDITIONER_DIAGONAL


@dataclass
class StressBalanceMultigridPreconditioner:
    smoother: Union[PointJacobi, LineJacobi] = field(default_factory=PointJacobi)
    smoothing_sweeps: int = 2
    coarsest_sweeps: int = 20
    minimum_coarse_size: int = 2
    code: int = abi.NK_PRECONDITIONER_MULTIGRID


@dataclass
class StressBalanceSolver:
    linear_iteration_control: object = field(default_factory=lambda: Convergence(reltol=1e-8, maxiter=10_000))
    picard_iteration_control: object = field(default_factory=lambda: Convergence(reltol=1e-6, maxiter=100))
    preconditioner: object = field(default_factory=StressBalanceDiagonalPreconditioner)   # None = no preconditioner
    precision: str = "fp64"             # "fp64" or "mixed" (FP32 multigrid under FP64 outer iterations)
    adjoint_iteration_control: object = None   # stops the fixed-point adjoint; None = picard_iteration_control
    host_loop: bool = False             # issue the kernels from a host loop instead of one CUDA graph (NK_SOLVER_HOST_LOOP)

    @property
    def adjoint_control(self):
        """The control of the fixed-point adjoint of converged Picard iterations; like the reference's
        `adjoint_iteration_control = picard_iteration_control` default it falls back to the Picard control."""
        c = self.adjoint_iteration_control
        return self.picard_iteration_control if c is None else c


# ---- descriptors ------------------------------------------------------------------------------------
class Descriptors:
    """C descriptors plus the arrays their pointers refer to (kept alive with the object).  `adjoint_control`
    is the StressBalanceSolver's adjoint iteration control, the default of Problem.picard_adjoint."""

    def __init__(self, grid, physics, solver, keep, adjoint_control=None, front=None):
        self.grid, self.physics, self.solver, self._keep = grid, physics, solver, keep
        self.adjoint_control = adjoint_control
        self.front = front                  # a PartialCellFront, applied when the problem is created


def _as_ptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_descriptors(grid: RectilinearGrid, Nsigma=10, bed_refinement=2.0, sigma_faces=None,
                     stress_balance: DepthIntegrated = None, rheology: GlenFlowLaw = None, friction=None,
                     grounding=None, masking="default", constants: IceSheetConstants = None,
                     velocity_solver: StressBalanceSolver = None, use_effective_pressure=True):
    """Translate the configuration objects into (nk_grid_desc, nk_physics_desc, nk_solver_desc).

    masking: "default" -> SmoothIceMask(), None -> no mask (the reference's `nothing`), or a PartialCellFront."""
    stress_balance = stress_balance or DepthIntegrated()
    rheology = rheology or GlenFlowLaw(rate_factor=1e-24)
    constants = constants or IceSheetConstants()
    velocity_solver = velocity_solver or StressBalanceSolver()
    if masking == "default":
        masking = SmoothIceMask()
    keep = []
    g = abi.GridDesc()
    g.Nx, g.Ny = grid.Nx, grid.Ny
    g.topology_x = abi.NK_PERIODIC if grid.periodic(0) else abi.NK_BOUNDED
    g.topology_y = abi.NK_PERIODIC if grid.periodic(1) else abi.NK_BOUNDED
    g.halo_x, g.halo_y = int(grid.halo[0]), int(grid.halo[1])
    g.Nsigma = int(Nsigma)
    for d, (pname, o, L) in enumerate((("x_faces", "x0", "Lx"), ("y_faces", "y0", "Ly"))):
        c = grid.x if d == 0 else grid.y
        if grid.regular(d):
            setattr(g, o, float(c[0]))
            setattr(g, L, float(c[1]) - float(c[0]))
        else:
            arr = np.ascontiguousarray(np.asarray(c, dtype=np.float64))
            if arr.size != grid.size[d] + 1:
                raise ValueError("a face vector needs N + 1 entries")
            keep.append(arr)
            setattr(g, pname, _as_ptr(arr))
            setattr(g, o, float(arr[0]))
            setattr(g, L, float(arr[-1] - arr[0]))
    if sigma_faces is not None:
        sf = np.ascontiguousarray(np.asarray(sigma_faces, dtype=np.float64))
        keep.append(sf)
        g.sigma_faces = _as_ptr(sf)
    g.bed_refinement = float(bed_refinement)

    p = abi.PhysicsDesc()
    p.stress_balance = abi.NK_DIVA if isinstance(stress_balance.shear, DIVAShear) else abi.NK_SSA
    p.side_walls = stress_balance.side_walls.code
    A = rheology.rate_factor
    sigma_rate = (isinstance(A, np.ndarray) and A.ndim == 3) or (isinstance(A, str) and A == "sigma")
    p.rate_factor_layout = abi.NK_RATE_FACTOR_SIGMA if sigma_rate else abi.NK_RATE_FACTOR_2D
    p.glen_exponent = float(rheology.exponent)
    p.strain_rate_regularization = float(rheology.strain_rate_regularization)
    if friction is None:
        p.friction = abi.NK_FRICTION_NONE
        p.friction_exponent, p.coulomb_coefficient, p.velocity_regularization = 1.0 / 3, 0.0, 1e-8
    elif isinstance(friction, WeertmanFriction):
        p.friction = abi.NK_WEERTMAN
        p.friction_exponent, p.coulomb_coefficient, p.velocity_regularization = friction.exponent, 0.0, friction.velocity_regularization
    else:
        p.friction = abi.NK_REGULARIZED_COULOMB
        p.friction_exponent = friction.exponent
        p.coulomb_coefficient = friction.coulomb_coefficient
        p.velocity_regularization = friction.velocity_regularization
    p.ice_density = constants.ice_density
    p.ocean_density = constants.ocean_density
    p.gravitational_acceleration = constants.gravitational_acceleration
    front = masking if isinstance(masking, PartialCellFront) else None
    if front is not None:
        masking = SmoothIceMask()           # its thickness parameters are unused: the front's flag is the mask
    p.use_ice_mask = 1 if masking is not None else 0
    p.grounding = 1 if isinstance(grounding, SubgridGroundedFraction) else 0
    p.grounding_line_driving_stress = 1 if (isinstance(grounding, SubgridGroundedFraction) and grounding.driving_stress) else 0
    p.use_effective_pressure = 1 if use_effective_pressure else 0
    m = masking or SmoothIceMask()
    p.mask_minimum_thickness = m.minimum_thickness
    p.mask_transition_thickness = m.transition_thickness

    s = abi.SolverDesc()
    if velocity_solver.precision not in ("fp64", "mixed"):
        raise ValueError(f"precision {velocity_solver.precision!r}: 'fp64' or 'mixed'")
    s.precision = abi.NK_PRECISION_MIXED if velocity_solver.precision == "mixed" else abi.NK_PRECISION_FP64
    P = velocity_solver.preconditioner
    if P is None:
        s.preconditioner = abi.NK_PRECONDITIONER_NONE
        s.smoother, s.smoothing_sweeps, s.coarsest_sweeps, s.minimum_coarse_size = 0, 2, 20, 2
    elif isinstance(P, StressBalanceMultigridPreconditioner):
        s.preconditioner = abi.NK_PRECONDITIONER_MULTIGRID
        s.smoother = P.smoother.code
        s.smoothing_sweeps, s.coarsest_sweeps, s.minimum_coarse_size = P.smoothing_sweeps, P.coarsest_sweeps, P.minimum_coarse_size
    else:
        s.preconditioner = abi.NK_PRECONDITIONER_DIAGONAL
        s.smoother, s.smoothing_sweeps, s.coarsest_sweeps, s.minimum_coarse_size = 0, 2, 20, 2
    s.linear = velocity_solver.linear_iteration_control.desc()
    s.picard = velocity_solver.picard_iteration_control.desc()
    s.flags = abi.NK_SOLVER_HOST_LOOP if velocity_solver.host_loop else 0
    return Descriptors(g, p, s, keep, velocity_solver.adjoint_control, front)


def field_shape(grid: RectilinearGrid, name: str, Nsigma: int, rate_layout_sigma=False):
    """numpy shape (Nsigma?, ny, nx) of a field in interior layout (x fastest)."""
    lx, ly, sig = abi.FIELD_LOCATIONS[name]
    if sig is None:
        sig = rate_layout_sigma
    nx, ny = grid.field_shape((lx, ly))
    return (Nsigma, ny, nx) if sig else (ny, nx)
