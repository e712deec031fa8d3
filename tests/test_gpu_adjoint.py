"""The fixed-point Picard adjoint (nk_picard_adjoint; the reverse rule of ext/NunatakEnzymeExt.jl:167-240) against
centred finite differences, following the checks of test/test_enzyme.jl:221-381.

J = ½ Σ (u - u_obs)² + (v - v_obs)² over the velocity points of a marine sheet, with u_obs from a solve with
another friction seed.  ∂J/∂log C and ∂J/∂log A from the adjoint must match (J(p e^ε) - J(p e^-ε)) / 2ε of converged
solves (Picard 1e-12, CG 1e-13) at seeded grounded cells:
- on the GPU forward solve for three configurations (bounded / periodic x, free-slip / no-slip walls, Weertman /
  regularised Coulomb friction);
- for one layer of a σ-grid rate factor;
- on the oracle's forward solve at one cell.
Tolerance: 1e-4 relative to the largest gradient entry."""
import math

import numpy as np
import pytest

import nunatak_gb300 as nk
from nunatak_gb300 import model as M, workloads

pytestmark = pytest.mark.gpu

EPS = 1e-3
RTOL = 1e-4


def _solver():
    return M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                 picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=500),
                                 preconditioner=M.StressBalanceDiagonalPreconditioner())


def _case(kind, seed_friction, nx=40, ny=20):
    base = workloads.marine_sheet(nx, ny, seed=2, seed_friction=seed_friction, velocity_solver=_solver())
    cfg = dict(base.config)
    grid = base.grid
    if kind == "periodic_x":
        grid = M.RectilinearGrid(size=(nx, ny), x=(0.0, 512e3), y=(0.0, 256e3), halo=(4, 4), topology=("Periodic", "Bounded"))
    if kind == "no_slip_coulomb":
        cfg["stress_balance"] = M.DepthIntegrated(side_walls=M.NoSlipWalls())
        cfg["friction"] = M.RegularizedCoulombFriction(coefficient=None, coulomb_coefficient=0.5, exponent=1.0 / 3.0)
    return workloads.Case(f"marine_sheet_{kind}", grid, cfg, base.fields)


def _cost(P, uo, vo):
    u, v = P.get("u"), P.get("v")
    return 0.5 * (np.sum((u - uo) ** 2) + np.sum((v - vo) ** 2)), u - uo, v - vo


def _fd(P, case, cell, xs, uo, vo, name="C"):
    """Centred difference of J in log `name` at `cell` (an index of that field) from converged solves warm-started
    at x*."""
    J = []
    for s in (1.0, -1.0):
        p = case.fields[name].copy()
        p[cell] *= math.exp(s * EPS)
        P.set(name, p)
        P.set("u", xs[0])
        P.set("v", xs[1])
        P.picard_solve()
        J.append(_cost(P, uo, vo)[0])
    P.set(name, case.fields[name])
    return (J[0] - J[1]) / (2 * EPS)


def _cells(P, n, seed):
    phi, H = P.get("phi"), P.get("H")
    cand = np.argwhere((phi > 0.5) & (H > 200.0))
    rng = np.random.default_rng(seed)
    return [tuple(cand[k]) for k in rng.choice(len(cand), size=n, replace=False)]


def _adjoint(cls, kind):
    case = _case(kind, 1100)
    obs = _case(kind, 1200).problem(cls)
    obs.picard_solve()
    uo, vo = obs.get("u"), obs.get("v")
    P = case.problem(cls)
    P.picard_solve()
    J0, ub, vb = _cost(P, uo, vo)
    return case, P, uo, vo, ub, vb


@pytest.mark.parametrize("kind", ["bounded", "periodic_x", "no_slip_coulomb"])
def test_picard_adjoint_matches_finite_differences(gpu_cls, kind):
    case, P, uo, vo, ub, vb = _adjoint(gpu_cls, kind)
    xs = (P.get("u"), P.get("v"))
    lu, lv, grad, grad_a, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500))
    assert st.status == 0 and st.picard_iterations > 1
    assert np.array_equal(P.get("u"), xs[0])              # the forward state is left at x*
    scale, scale_a = np.max(np.abs(grad)), np.max(np.abs(grad_a))
    assert scale > 0 and scale_a > 0
    for n, cell in enumerate(_cells(P, 4, 7)):
        fd = _fd(P, case, cell, xs, uo, vo)
        assert abs(fd - grad[cell]) <= RTOL * scale, (kind, cell, fd, grad[cell], scale)
        if n < 2:
            fd = _fd(P, case, cell, xs, uo, vo, "A")
            assert abs(fd - grad_a[cell]) <= RTOL * scale_a, (kind, "A", cell, fd, grad_a[cell], scale_a)


def test_picard_adjoint_rate_factor_on_the_sigma_grid(gpu_cls):
    """∂J/∂log A for a σ-grid rate factor: one layer of one cell against a centred difference."""
    base = _case("bounded", 1100)
    cfg = dict(base.config)
    cfg["rheology"] = M.GlenFlowLaw(rate_factor="sigma", strain_rate_regularization=1e-13)
    A2 = base.fields["A"]
    ns = cfg["Nsigma"]
    fields = dict(base.fields)
    fields["A"] = np.stack([A2 * (1.0 + 0.5 * k / ns) for k in range(ns)])
    case = workloads.Case("marine_sheet_sigma_A", base.grid, cfg, fields)
    obs = workloads.Case("obs", base.grid, cfg, dict(_case("bounded", 1200).fields, A=fields["A"])).problem(gpu_cls)
    obs.picard_solve()
    uo, vo = obs.get("u"), obs.get("v")
    P = case.problem(gpu_cls)
    P.picard_solve()
    _, ub, vb = _cost(P, uo, vo)
    xs = (P.get("u"), P.get("v"))
    _, _, _, grad_a, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500))
    assert st.status == 0 and grad_a.shape == (ns,) + A2.shape
    cell = _cells(P, 1, 3)[0]
    for layer in (1, ns - 2):
        idx = (layer,) + cell
        fd = _fd(P, case, idx, xs, uo, vo, "A")
        assert abs(fd - grad_a[idx]) <= RTOL * np.max(np.abs(grad_a)), (layer, cell, fd, grad_a[idx])


def test_picard_adjoint_matches_oracle_finite_difference(gpu_cls, oracle_cls):
    """The adjoint gradient of the GPU library against a centred difference of the oracle's forward solve."""
    case, P, uo, vo, ub, vb = _adjoint(gpu_cls, "bounded")
    _, _, grad, _, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=500))
    assert st.status == 0
    O = case.problem(oracle_cls)
    O.picard_solve()
    xs = (O.get("u"), O.get("v"))
    cell = _cells(P, 1, 11)[0]
    fd = _fd(O, case, cell, xs, uo, vo)
    assert abs(fd - grad[cell]) <= RTOL * np.max(np.abs(grad)), (cell, fd, grad[cell])
