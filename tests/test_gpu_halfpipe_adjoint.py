"""The STREAMICE halfpipe adjoint (benchmarks/halfpipe_streamice_adjoint.jl of Nunatak.jl; MITgcm
verification/halfpipe_streamice, input_ad) through nk_checkpointed_gradient on the GPU.

The experiment (workloads.halfpipe_streamice, its values in tests/golden/halfpipe_streamice.json): a 39 x 19 shelf in
a half-pipe channel, DIVA with no-slip walls, the subgrid grounded fraction and a partial-cell front without overflow
passes; three steps of 0.2 yr with a Picard solve after every stage; the basal melt rate is the control xx (m/yr),
scaled by 0.5, 1 and 0.5 over the steps; J = Σ (u² + v²) of the corner velocities in m/yr over the full cells after
step 2 plus Σ H² over the full cells after step 3 (:35-64).  The gradient ∂J/∂xx at the four centreline cells of the
benchmark is held to centred differences of the library's own forward steps (ε = 0.1 m/yr, as the benchmark's) with
the solves converged past the benchmark's tolerances (Picard 1e-12, CG 1e-13), to 1e-4.  STREAMICE's cost and
gradient are another model's (their ratio to the library's is reported by bench.py --halfpipe-adjoint)."""
import json
import os

import numpy as np
import pytest

from nunatak_gb300 import model as M, workloads

pytestmark = pytest.mark.gpu

SPEC = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "halfpipe_streamice.json")))
WEIGHTS = tuple(SPEC["control_weights"])
CELLS = [(j - 1, i - 1) for i, j in SPEC["check_cells_julia"]]
TIGHT = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                              picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=2000),
                              adjoint_iteration_control=M.Convergence(reltol=1e-12, maxiter=2000))


def halfpipe(cls, solver=None):
    """set!(model, H = initial_thickness) of the benchmark: the thickness, the front flagged from it, the geometry and a
    Picard solve; the inflow as the surface mass balance of the west column."""
    case, smb, year = workloads.halfpipe_streamice(SPEC, velocity_solver=solver)
    P = cls(case.grid, case.descriptors())
    for k, v in case.fields.items():
        P.set(k, v)
    P.initialize_front()
    P.compute_geometry()
    P.energy_set("surface_mass_balance", smb)
    P.energy_set("basal_melt_rate", 0.0)
    P.energy_set("clipped_thickness", 0.0)
    assert P.picard_solve().status == 0
    return P, year


def velocity_cost(u, v, mask, year):
    """velocity_cost (:35-45): Σ over the full cells of uᶜ² + vᶜ² with uᶜ = (u[i, j-1] + u[i, j]) / 2 (0 in the first
    row) and vᶜ = (v[i-1, j] + v[i, j]) / 2 (0 in the first column) in m/yr; and its gradient in u, v."""
    Ny, Nx = mask.shape
    full = mask == 1
    uc = np.zeros((Ny, Nx))
    vc = np.zeros((Ny, Nx))
    uc[1:, :] = (u[:-1, :Nx][:Ny - 1] + u[1:Ny, :Nx]) / 2 * year
    vc[:, 1:] = (v[:Ny, :Nx - 1] + v[:Ny, 1:Nx]) / 2 * year
    J = float(np.sum(np.where(full, uc * uc + vc * vc, 0.0)))
    gu, gv = np.zeros_like(u), np.zeros_like(v)
    wu = np.where(full, uc, 0.0) * year   # ∂/∂u of uᶜ² is uᶜ year for each of its two faces
    wv = np.where(full, vc, 0.0) * year
    gu[:Ny - 1, :Nx] += wu[1:, :]
    gu[1:Ny, :Nx] += wu[1:, :]
    gv[:Ny, :Nx - 1] += wv[:, 1:]
    gv[:Ny, 1:Nx] += wv[:, 1:]
    return J, gu, gv


def cost(year):
    def f(step, H, u, v, mask):
        if step == 2:
            J, gu, gv = velocity_cost(u, v, mask, year)
            return J, None, gu, gv
        if step == 3:
            full = mask == 1
            return float(np.sum(np.where(full, H * H, 0.0))), np.where(full, 2 * H, 0.0), None, None
        return None
    return f


def forward_cost(cls, solver, cell=None, eps=0.0):
    """adjoint_cost (:47-64) of the library's forward steps with xx = eps (m/yr) at `cell`."""
    P, year = halfpipe(cls, solver)
    base = np.zeros((SPEC["Ny"], SPEC["Nx"]))
    if cell is not None:
        base[cell] = eps / year
    J = 0.0
    dt = 0.2 * year
    for n, w in enumerate(WEIGHTS):
        P.energy_set("basal_melt_rate", w * base)
        if n == 2:
            J += velocity_cost(P.get("u"), P.get("v"), P.get("ice_mask"), year)[0]
        for stage in (1, 2, 3):
            P.step_thickness_stage(dt, stage)
            assert P.picard_solve().status == 0
    H, mask = P.get("H"), P.get("ice_mask")
    return J + float(np.sum(np.where(mask == 1, H * H, 0.0)))


def test_halfpipe_gradient_matches_differences(gpu_cls):
    P, year = halfpipe(gpu_cls, TIGHT)
    g = P.checkpointed_gradient(cost(year), 0.2 * year, 3, melt_weights=WEIGHTS)
    assert g["stats"]["worst_solve_status"] == 0
    J0 = forward_cost(gpu_cls, TIGHT)
    assert abs(g["J"] - J0) <= 1e-12 * J0
    for cell in CELLS:
        ad = g["melt"][cell] / year      # ∂J/∂xx with m = w xx / yr
        fd = (forward_cost(gpu_cls, TIGHT, cell, 0.1) - forward_cost(gpu_cls, TIGHT, cell, -0.1)) / 0.2
        assert ad < 0 and abs(ad - fd) <= 1e-4 * abs(fd), (cell, ad, fd)
