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


def forward_cost(cls, solver, cell=None, eps=0.0):
    P, year, st = workloads.halfpipe_problem(cls, SPEC, solver)
    assert st.status == 0
    control = None
    if cell is not None:
        control = np.zeros((SPEC["Ny"], SPEC["Nx"]))
        control[cell] = eps
    return workloads.halfpipe_forward_cost(P, year, WEIGHTS, control)


def test_halfpipe_gradient_matches_differences(gpu_cls):
    P, year, st = workloads.halfpipe_problem(gpu_cls, SPEC, TIGHT)
    assert st.status == 0
    g = P.checkpointed_gradient(workloads.halfpipe_cost(year), 0.2 * year, 3, melt_weights=WEIGHTS)
    assert g["stats"]["worst_solve_status"] == 0
    J0 = forward_cost(gpu_cls, TIGHT)
    assert abs(g["J"] - J0) <= 1e-12 * J0
    for cell in CELLS:
        ad = g["melt"][cell] / year      # ∂J/∂xx with m = w xx / yr
        fd = (forward_cost(gpu_cls, TIGHT, cell, 0.1) - forward_cost(gpu_cls, TIGHT, cell, -0.1)) / 0.2
        assert ad < 0 and abs(ad - fd) <= 1e-4 * abs(fd), (cell, ad, fd)
