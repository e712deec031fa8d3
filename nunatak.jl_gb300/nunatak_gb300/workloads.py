"""Seeded synthetic workloads of the velocity solve (no dataset involved).

  channel_shelf   floating shelf in a channel, 80 km long, no-slip walls, calving front at 80 km
  marine_sheet    marine ice sheet on a random bed, Weertman friction with a random coefficient
  serving_stream  Poisson stream of marine_sheet requests of four sizes on one 512 km x 256 km domain
  diva_sheet      DIVA marine sheet with an Arrhenius rate factor from a seeded temperature field

Random fields are standard normal draws from numpy.random.default_rng(seed), Gaussian-filtered
(reflect mode) to the stated correlation length and renormalised to zero mean and unit deviation.
Units are SI with a year of 31556926 s."""
from dataclasses import dataclass, field
from typing import Callable, Dict, Optional

import functools

import numpy as np

from . import model as M

YEAR = M.YEAR


def _gaussian_reflect(a, sigma, truncate=4.0):
    """Gaussian filter of a 2-D array with reflected edges (scipy.ndimage.gaussian_filter, mode "reflect", the
    same truncated kernel) evaluated as two FFT convolutions of the padded array."""
    from scipy.signal import fftconvolve
    r = int(truncate * float(sigma) + 0.5)
    x = np.arange(-r, r + 1, dtype=np.float64)
    k = np.exp(-0.5 * (x / sigma) ** 2)
    k /= k.sum()
    p = np.pad(a, r, mode="symmetric")
    p = fftconvolve(p, k[None, :], mode="valid", axes=1)
    return fftconvolve(p, k[:, None], mode="valid", axes=0)


def random_field(shape, seed, correlation_cells):
    """Smoothed, renormalised standard normal field of shape (ny, nx)."""
    g = np.random.default_rng(seed).standard_normal(shape)
    g = _gaussian_reflect(g, correlation_cells)
    g = g - g.mean()
    s = g.std()
    return g / s if s > 0 else g


@dataclass
class Case:
    """A grid, the configuration objects and the input fields of one velocity solve."""
    name: str
    grid: M.RectilinearGrid
    config: Dict
    fields: Dict[str, np.ndarray]
    initial: Dict[str, np.ndarray] = field(default_factory=dict)
    temperature: Optional[np.ndarray] = None

    def descriptors(self):
        return M.make_descriptors(self.grid, **self.config)

    def problem(self, cls, context=None):
        """Problem of class `cls` with the fields set and the geometry and driving stress computed."""
        P = cls(self.grid, self.descriptors()) if context is None else cls(self.grid, self.descriptors(), context=context)
        for k, v in self.fields.items():
            P.set(k, v)
        if self.temperature is not None:
            P.set("T", self.temperature)
            P.compute_rate_factor()
        P.compute_geometry()
        for k, v in self.initial.items():
            P.set(k, v)
        return P

    @property
    def cells(self):
        return self.grid.Nx * self.grid.Ny


@functools.lru_cache(maxsize=16)
def _bed_field(ny, nx, seed, correlation_cells):
    """random_field of the bed, shared by every case of one grid and seed (read-only)."""
    g = random_field((ny, nx), seed, correlation_cells)
    g.setflags(write=False)
    return g


def _centers(grid):
    return np.meshgrid(grid.centers(0), grid.centers(1))


def west_inflow(grid, speed):
    """u_prescribed with `speed` m/yr (stored in m/s) on the faces at the west edge (i = 0) and NaN (free) on every
    other face."""
    u = np.full((grid.Ny, grid.face_count(0)), np.nan)
    u[:, 0] = speed / YEAR
    return u


def channel_shelf(Nx=84, Ny=40, dx=1e3, velocity_solver=None, inflow=None):
    """Floating shelf in a channel: H = 600 - 400 x / 80 km up to the calving front at x = 80 km (ice free
    beyond), bed -1000 m (all floating), Glen n = 3, A = 3.17e-24, no-slip side walls, no friction,
    Jacobi-PCG to 1e-10 inside Picard to 1e-6.  The west wall is impenetrable (u = 0), or, with `inflow` (m/yr),
    its faces hold that prescribed velocity."""
    grid = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * dx), y=(0.0, Ny * dx), halo=(4, 4))
    X, _ = _centers(grid)
    H = np.where(X < 80e3, 600.0 - 400.0 * X / 80e3, 0.0)
    solver = velocity_solver or M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=10_000),
                                                      picard_iteration_control=M.Convergence(reltol=1e-6, maxiter=100),
                                                      preconditioner=M.StressBalanceDiagonalPreconditioner())
    cfg = dict(Nsigma=10, stress_balance=M.DepthIntegrated(side_walls=M.NoSlipWalls()),
               rheology=M.GlenFlowLaw(rate_factor=3.17e-24, strain_rate_regularization=1e-13), friction=None,
               grounding=M.SubgridGroundedFraction(), velocity_solver=solver)
    fields = {"H": H, "bed": np.full_like(H, -1000.0), "A": np.full_like(H, 3.17e-24)}
    if inflow is not None:
        fields["u_prescribed"] = west_inflow(grid, inflow)
    return Case("channel_shelf" if inflow is None else "channel_shelf_inflow", grid, cfg, fields)


def marine_sheet(Nx=256, Ny=128, seed=1, seed_friction=None, Lx=512e3, Ly=256e3, velocity_solver=None,
                 minimum_coarse_size=32, precision="fp64"):
    """Marine ice sheet on a Lx x Ly domain: bed -100 - 600 x / 512 km + 50 m g (g a 20 km random field),
    H = 2000 sqrt(max(0, 1 - (x / 420 km)²)), Weertman m = 1/3 with C = 10^(6.5 + 0.3 ξ) Pa (m/yr)^(-1/3)
    (ξ a 20 km random field), Glen n = 3, A = 3.17e-24, free-slip walls, subgrid grounded fraction,
    multigrid PCG (2 + 2 point sweeps, coarsening stops at 32 cells)."""
    grid = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Lx), y=(0.0, Ly), halo=(4, 4))
    dx = Lx / Nx
    X, _ = _centers(grid)
    g = _bed_field(Ny, Nx, seed, 20e3 / dx)
    xi = random_field((Ny, Nx), seed + 7919 if seed_friction is None else seed_friction, 20e3 / dx)
    bed = -100.0 - 600.0 * X / 512e3 + 50.0 * g
    H = 2000.0 * np.sqrt(np.maximum(0.0, 1.0 - (X / 420e3) ** 2))
    C = 10.0 ** (6.5 + 0.3 * xi) * YEAR ** (1.0 / 3.0)
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=minimum_coarse_size)
    solver = velocity_solver or M.StressBalanceSolver(preconditioner=mg, precision=precision)
    cfg = dict(Nsigma=10, stress_balance=M.DepthIntegrated(side_walls=M.FreeSlipWalls()),
               rheology=M.GlenFlowLaw(rate_factor=3.17e-24, strain_rate_regularization=1e-13),
               friction=M.WeertmanFriction(coefficient=None, exponent=1.0 / 3.0), grounding=M.SubgridGroundedFraction(),
               velocity_solver=solver)
    return Case("marine_sheet", grid, cfg, {"H": H, "bed": bed, "C": C, "A": np.full_like(H, 3.17e-24)})


SERVING_SIZES = ((128, 64), (256, 128), (512, 256), (1024, 512))


def serving_stream(n_requests=512, rate=200.0, seed=11, base_seed=1000):
    """Request list of the serving workload: arrival times from a Poisson process at `rate` requests/s and
    grid sizes drawn uniformly from 128x64 ... 1024x512, all on the 512 km x 256 km marine-sheet domain,
    request k carrying friction seed base_seed + k."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, n_requests)
    arrivals = np.cumsum(gaps) - gaps[0]
    sizes = rng.integers(len(SERVING_SIZES), size=n_requests)
    return [dict(index=k, arrival=float(arrivals[k]), size=SERVING_SIZES[int(sizes[k])], seed_friction=base_seed + k)
            for k in range(n_requests)]


def serving_case(request, precision="mixed"):
    """The marine-sheet Case of one serving_stream request."""
    nx, ny = request["size"]
    return marine_sheet(nx, ny, seed=1, seed_friction=request["seed_friction"], precision=precision)


def diva_sheet(Nx=2048, Ny=1024, seed=3, dx=1e3, velocity_solver=None, precision="fp64", Nsigma=10):
    """DIVA marine sheet on a 2048 km x 1024 km domain (marine-sheet geometry stretched by 4), calving front
    at x = 1900 km, Arrhenius rate factor from T(ζ) = 270 - 17 ζ + 3 K × (30 km random field),
    regularised Coulomb friction (m = 1/3, α² = 0.5) with the ocean-connected effective pressure."""
    Lx, Ly = Nx * dx, Ny * dx
    grid = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Lx), y=(0.0, Ly), halo=(4, 4))
    X, _ = _centers(grid)
    s = Lx / 512e3
    g = random_field((Ny, Nx), seed, 20e3 * s / dx)
    xi = random_field((Ny, Nx), seed + 7919, 20e3 * s / dx)
    dT = random_field((Ny, Nx), seed + 104729, 30e3 / dx)
    bed = -100.0 - 600.0 * X / Lx + 50.0 * g
    H = np.where(X < 1900e3, 2000.0 * np.sqrt(np.maximum(0.0, 1.0 - (X / (420e3 * s)) ** 2)), 0.0)
    C = 10.0 ** (6.5 + 0.3 * xi) * YEAR ** (1.0 / 3.0)
    faces = np.array([(k / Nsigma) ** 2 for k in range(Nsigma + 1)])
    zeta = (faces[1:] + faces[:-1]) / 2
    T = np.stack([270.0 - 17.0 * z + 3.0 * dT for z in zeta])
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=32)
    solver = velocity_solver or M.StressBalanceSolver(preconditioner=mg, precision=precision)
    cfg = dict(Nsigma=Nsigma, stress_balance=M.DepthIntegrated(shear=M.DIVAShear(), side_walls=M.FreeSlipWalls()),
               rheology=M.GlenFlowLaw(rate_factor="sigma", strain_rate_regularization=1e-13),
               friction=M.RegularizedCoulombFriction(coefficient=None, coulomb_coefficient=0.5, exponent=1.0 / 3.0),
               grounding=M.SubgridGroundedFraction(), velocity_solver=solver)
    return Case("diva_sheet", grid, cfg, {"H": H, "bed": bed, "C": C}, temperature=T)


def mismip_stream(dx, velocity_solver=None):
    """The MISMIP+-like marine ice stream of the reference's multigrid scaling benchmark
    (benchmarks/multigrid_scaling.jl:10-34): a 640 km x 80 km channel with Bounded free-slip walls, the MISMIP+
    polynomial bed with side walls (Asay-Davis et al. 2016, the benchmark's constants), the prescribed thickness
    1500 sqrt(1 - x / 650 km) up to a calving front at 600 km, Glen A = 2.0392e-17 / yr with ε̇₀ = 1e-5 / yr,
    regularised Coulomb drag (C = 1e4 yr^(1/3), α² = 0.5, m = 1/3, u₀ = 1e-5 / yr), the subgrid grounded
    fraction, the smooth ice mask and Nσ = 10; grid spacing dx (m), halo 4.  The benchmark's velocity solver
    (multigrid PCG to 1e-6, five Picard iterations) is the default."""
    Lx, Ly = 640e3, 80e3
    nx, ny = int(round(Lx / dx)), int(round(Ly / dx))
    grid = M.RectilinearGrid(size=(nx, ny), x=(0.0, Lx), y=(0.0, Ly), halo=(4, 4))
    X, Y = _centers(grid)
    B0, B2, B4, B6, xbar = -150.0, -728.8, 343.91, -50.57, 300e3
    fc, dc, wc, z_deep = 4e3, 500.0, 24e3, -720.0
    along = B0 + B2 * (X / xbar) ** 2 + B4 * (X / xbar) ** 4 + B6 * (X / xbar) ** 6
    across = dc / (1 + np.exp(-2 * (Y - Ly / 2 - wc) / fc)) + dc / (1 + np.exp(2 * (Y - Ly / 2 + wc) / fc))
    bed = np.maximum(along + across, z_deep)
    H = np.where(X < 600e3, 1500.0 * np.sqrt(np.maximum(0.0, 1 - X / 650e3)), 0.0)
    solver = velocity_solver or M.StressBalanceSolver(
        preconditioner=M.StressBalanceMultigridPreconditioner(),
        linear_iteration_control=M.Convergence(reltol=1e-6, maxiter=50_000),
        picard_iteration_control=M.FixedIterations(5))
    A = 2.0392e-17 / YEAR
    cfg = dict(Nsigma=10, stress_balance=M.DepthIntegrated(side_walls=M.FreeSlipWalls()),
               rheology=M.GlenFlowLaw(rate_factor=A, strain_rate_regularization=1e-5 / YEAR),
               friction=M.RegularizedCoulombFriction(coefficient=None, coulomb_coefficient=0.5, exponent=1.0 / 3.0,
                                                     velocity_regularization=1e-5 / YEAR),
               grounding=M.SubgridGroundedFraction(), velocity_solver=solver)
    C = np.full_like(H, 1e4 * YEAR ** (1.0 / 3.0))
    return Case("mismip_stream", grid, cfg, {"H": H, "bed": bed, "A": np.full_like(H, A), "C": C})


def halfpipe_streamice(spec, Nsigma=10, velocity_solver=None):
    """MITgcm STREAMICE's verification experiment halfpipe_streamice as Nunatak.jl sets it up
    (benchmarks/halfpipe_streamice.jl:1-37, benchmarks/halfpipe_streamice_adjoint.jl:17-32): a mostly floating shelf
    in a half-pipe channel of `Nx` x `Ny` cells of `dx_km`, fed through its west column by a mass source inflow / Δx,
    with DIVA stress balance, no-slip side walls, the subgrid grounded fraction, a partial-cell front without overflow
    passes, Glen A = (B²)^(-n) / yr and Weertman drag C² yr |u|⁰ u (ε̇₀ and u₀ 1e-12 / yr), and STREAMICE's analytic
    initial shelf: 300 m beyond 50 km, thickening quadratically upstream, ice free beyond 70 km.  `spec` holds the
    experiment's values (the densities, B, C, n, the grid, the inflow and the bed profile across the channel).  The
    year is Oceananigans' 365 days.  Returns (Case, surface mass balance in m/s, seconds per year)."""
    year = 365 * 86400.0
    dx = spec["dx_km"] * 1e3
    Nx, Ny = int(spec["Nx"]), int(spec["Ny"])
    grid = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, Nx * dx), y=(0.0, Ny * dx), halo=(4, 4))
    B, C, n = spec["B"], spec["C"], spec["n"]
    solver = velocity_solver or M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=10_000),
                                                      picard_iteration_control=M.Convergence(reltol=1e-8, maxiter=500))
    cfg = dict(Nsigma=Nsigma, stress_balance=M.DepthIntegrated(shear=M.DIVAShear(), side_walls=M.NoSlipWalls()),
               rheology=M.GlenFlowLaw(rate_factor=(B ** 2) ** (-n) / year, exponent=n, strain_rate_regularization=1e-12 / year),
               friction=M.WeertmanFriction(coefficient=None, exponent=1.0, velocity_regularization=1e-12 / year),
               grounding=M.SubgridGroundedFraction(), masking=M.PartialCellFront(passes=0),
               constants=M.IceSheetConstants(ice_density=spec["ice_density"], ocean_density=spec["ocean_density"],
                                             gravitational_acceleration=spec["gravitational_acceleration"]),
               velocity_solver=solver)
    X, _ = _centers(grid)
    H = np.where(X < 70e3, 300.0 + 1000.0 * np.minimum(1.0, (np.maximum(50e3 - X, 0.0) / 62e3) ** 2), 0.0)
    bed = np.repeat(np.asarray(spec["bed_profile"], dtype=np.float64)[:, None], Nx, axis=1)
    fields = {"H": H, "bed": bed, "C": np.full_like(H, C ** 2 * year), "A": np.full_like(H, (B ** 2) ** (-n) / year)}
    smb = np.where(X < dx, spec["inflow_m2_per_year"] / year / dx, 0.0)
    return Case("halfpipe_streamice", grid, cfg, fields), smb, year


def halfpipe_problem(cls, spec, velocity_solver=None, context=None):
    """set!(model, H = initial_thickness) of the halfpipe (src/Models/ice_sheet_model_methods.jl:11-20): the fields, the
    front flagged from H, the geometry, the inflow as the west column's surface mass balance, no melt, and a Picard
    solve.  Returns (problem, seconds per year, solve stats)."""
    case, smb, year = halfpipe_streamice(spec, velocity_solver=velocity_solver)
    P = cls(case.grid, case.descriptors()) if context is None else cls(case.grid, case.descriptors(), context=context)
    for k, v in case.fields.items():
        P.set(k, v)
    P.initialize_front()
    P.compute_geometry()
    P.energy_set("surface_mass_balance", smb)
    P.energy_set("basal_melt_rate", 0.0)
    P.energy_set("clipped_thickness", 0.0)
    return P, year, P.picard_solve()


def halfpipe_velocity_cost(u, v, mask, year):
    """velocity_cost of the halfpipe adjoint (benchmarks/halfpipe_streamice_adjoint.jl:35-45): Σ over the full cells
    (mask 1) of uᶜ² + vᶜ², uᶜ = (u[i, j-1] + u[i, j]) / 2 (0 in the first row) and vᶜ = (v[i-1, j] + v[i, j]) / 2 (0 in
    the first column) in m/yr, with its gradient in the interior layouts of u and v."""
    Ny, Nx = mask.shape
    full = mask == 1
    uc = np.zeros((Ny, Nx))
    vc = np.zeros((Ny, Nx))
    uc[1:, :] = (u[:Ny - 1, :Nx] + u[1:Ny, :Nx]) / 2 * year
    vc[:, 1:] = (v[:Ny, :Nx - 1] + v[:Ny, 1:Nx]) / 2 * year
    J = float(np.sum(np.where(full, uc * uc + vc * vc, 0.0)))
    gu, gv = np.zeros_like(u), np.zeros_like(v)
    wu = np.where(full, uc, 0.0) * year   # ∂(uᶜ²)/∂u of each of its two faces
    wv = np.where(full, vc, 0.0) * year
    gu[:Ny - 1, :Nx] += wu[1:, :]
    gu[1:Ny, :Nx] += wu[1:, :]
    gv[:Ny, :Nx - 1] += wv[:, 1:]
    gv[:Ny, 1:Nx] += wv[:, 1:]
    return J, gu, gv


def halfpipe_cost(year):
    """The halfpipe adjoint's cost as the callback of Problem.checkpointed_gradient (:47-64): the velocity cost of the
    state after step 2 (STREAMICE solves the velocity at the start of each step) and Σ H² over the full cells after
    step 3."""
    def cost(step, H, u, v, mask):
        if step == 2:
            J, gu, gv = halfpipe_velocity_cost(u, v, mask, year)
            return J, None, gu, gv
        if step == 3:
            full = mask == 1
            return float(np.sum(np.where(full, H * H, 0.0))), np.where(full, 2 * H, 0.0), None, None
        return None
    return cost


def halfpipe_forward_cost(P, year, weights, control=None):
    """The same cost from the forward steps alone (adjoint_cost, :47-64), the control xx (m/yr) scaled per step."""
    Ny, Nx = P.get("H").shape
    base = np.zeros((Ny, Nx)) if control is None else control / year
    J = 0.0
    dt = 0.2 * year
    for n, w in enumerate(weights):
        P.energy_set("basal_melt_rate", w * base)
        if n == 2:
            J += halfpipe_velocity_cost(P.get("u"), P.get("v"), P.get("ice_mask"), year)[0]
        for stage in (1, 2, 3):
            P.step_thickness_stage(dt, stage)
            st = P.picard_solve()
            if st.status == 2:
                raise RuntimeError("non-finite Picard solve")
    H, mask = P.get("H"), P.get("ice_mask")
    return J + float(np.sum(np.where(mask == 1, H * H, 0.0)))
