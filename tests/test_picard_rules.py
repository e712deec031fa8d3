"""Picard stopping rules: the reference's velocity change (Convergence, picard.jl:79-85) and the viscosity-change
rule offered as an extension (ViscosityConvergence: ‖η̄H_k − η̄H_(k−1)‖ ≤ max(reltol ‖η̄H_k‖, abstol)).

On both backends (oracle on the CPU, GPU marked gpu), on the 84 x 40 channel shelf with Jacobi-PCG to 1e-10:
- the viscosity rule stops with picard_change ≤ reltol · picard_norm, and the first iteration never stops it;
- at reltol 1e-6 its solution agrees with the velocity rule's to 1e-5 (relative L2), and a looser reltol stops
  earlier.
GPU against the oracle: the same iteration count and velocities within 1e-10 (relative L2).  The linear control
and the adjoint control refuse the viscosity rule."""
import math

import numpy as np
import pytest

from nunatak_gb300 import model as M
from nunatak_gb300 import workloads


def rel_l2(ua, va, ub, vb):
    return math.sqrt(np.sum((ua - ub) ** 2) + np.sum((va - vb) ** 2)) / math.sqrt(np.sum(ub ** 2) + np.sum(vb ** 2))


def _solver(picard):
    return M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=10_000), picard_iteration_control=picard,
                                 preconditioner=M.StressBalanceDiagonalPreconditioner())


def _solve(cls, picard, inflow=None):
    P = workloads.channel_shelf(velocity_solver=_solver(picard), inflow=inflow).problem(cls)
    st = P.picard_solve()
    return P.get("u"), P.get("v"), st


def test_viscosity_rule_stops_on_the_viscosity_change(backend):
    u, v, st = _solve(backend, M.ViscosityConvergence(reltol=1e-6, maxiter=100))
    assert st.status == 0 and st.picard_iterations > 2
    assert st.picard_change <= 1e-6 * st.picard_norm
    u0, v0, st0 = _solve(backend, M.Convergence(reltol=1e-6, maxiter=100))
    assert rel_l2(u, v, u0, v0) < 1e-5
    _, _, loose = _solve(backend, M.ViscosityConvergence(reltol=1e-4, maxiter=100))
    assert loose.status == 0 and loose.picard_iterations < st.picard_iterations


def test_viscosity_rule_never_stops_at_the_first_iteration(backend):
    """Even a huge tolerance runs two iterations: the first has no previous viscosity to compare with."""
    _, _, st = _solve(backend, M.ViscosityConvergence(reltol=1e3, maxiter=100))
    assert st.status == 0 and st.picard_iterations == 2
    _, _, one = _solve(backend, M.ViscosityConvergence(reltol=1e3, maxiter=1))
    assert one.picard_iterations == 1 and math.isinf(one.picard_change)


@pytest.mark.gpu
@pytest.mark.parametrize("inflow", [None, 100.0])
def test_viscosity_rule_matches_oracle(oracle_cls, gpu_cls, inflow):
    ug, vg, sg = _solve(gpu_cls, M.ViscosityConvergence(reltol=1e-6, maxiter=100), inflow)
    uo, vo, so = _solve(oracle_cls, M.ViscosityConvergence(reltol=1e-6, maxiter=100), inflow)
    assert sg.status == 0 and so.status == 0
    assert sg.picard_iterations == so.picard_iterations
    assert rel_l2(ug, vg, uo, vo) < 1e-10
    assert abs(sg.picard_change - so.picard_change) <= 1e-6 * so.picard_change


@pytest.mark.gpu
def test_viscosity_rule_mixed_precision(gpu_cls):
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)
    solver = M.StressBalanceSolver(precision="mixed", linear_iteration_control=M.Convergence(reltol=1e-8, maxiter=2000),
                                   picard_iteration_control=M.ViscosityConvergence(reltol=1e-6, maxiter=200), preconditioner=mg)
    P = workloads.marine_sheet(64, 32, seed=2, velocity_solver=solver).problem(gpu_cls)
    st = P.picard_solve()
    assert st.status == 0 and st.picard_change <= 1e-6 * st.picard_norm


@pytest.mark.gpu
def test_viscosity_rule_is_picard_only(gpu_cls):
    bad = M.StressBalanceSolver(linear_iteration_control=M.ViscosityConvergence(reltol=1e-8))
    with pytest.raises(ValueError):
        workloads.channel_shelf(velocity_solver=bad).problem(gpu_cls)
    P = workloads.channel_shelf().problem(gpu_cls)
    P.picard_solve()
    u, v = P.get("u"), P.get("v")
    with pytest.raises(ValueError):
        P.picard_adjoint(u, v, M.ViscosityConvergence(reltol=1e-8, maxiter=10))
