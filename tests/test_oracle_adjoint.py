"""The oracle's fixed-point Picard adjoint (nko_picard_adjoint; the reverse rule of ext/NunatakEnzymeExt.jl:159-240
for the SSA) against centred differences of the oracle's own forward solves, and the GPU library's adjoint against
the oracle's.

J = ½ Σ (u - u_obs)² + (v - v_obs)² on the 40 x 20 marine sheet with u_obs from a solve with another friction
seed (the cases of tests/test_gpu_adjoint.py: bounded with free-slip walls and Weertman drag, periodic in x, and
no-slip walls with regularised Coulomb drag), converged solves (Picard 1e-14, CG 1e-15):
- ∂J/∂log C against (J(C e^ε) - J(C e^-ε)) / 2ε, ε = 1e-3, within 1e-4 of the cell's own gradient, at seeded cells
  whose gradient is at least 1e-3 of the largest entry and at the largest-gradient cells of the rows beside the
  south and north walls (J(+) - J(-) formed from the two solves' velocities, not as a difference of two costs);
- ∂J/∂log A along a seeded random direction d against the Richardson extrapolation of centred differences with
  ε = 4e-5 and 2e-5, within 1e-4 of Σ|gᵢdᵢ| (the third derivative along d is large for the Coulomb case: a plain
  centred difference with ε = 1e-4 is 0.8 % off, and its error falls as ε²);
- the DIVA adjoint, which sweeps the adjoint of the step's lagged state (βᵇ, F₂, ησ) along with λ, on a 24 x 12
  DIVA sheet with Weertman and regularised Coulomb drag, log C and σ-grid log A along directions;
- GPU (marked gpu): λ, ∂J/∂log C and ∂J/∂log A of nk_picard_adjoint against the oracle's, within 1e-6 of each
  one's largest entry, for the three SSA cases and the two DIVA ones.
The oracle refuses problems with prescribed velocities, as the library does.  An adjoint stopped by its maxiter warns
on both backends (test/test_enzyme.jl:383-389)."""
import math
import warnings

import numpy as np
import pytest

from nunatak_gb300 import abi, model as M, workloads

CONTROL = M.Convergence(reltol=1e-12, maxiter=500)
KINDS = ["bounded", "periodic_x", "no_slip_coulomb"]


def _solver():
    """Converged to Picard 1e-14 and CG 1e-15: the per-cell differences below resolve 1e-6 of a cell's gradient only
    when the perturbed solves leave no more than that (at 1e-12 / 1e-13 a cell at 1 % of the largest gradient
    carried 2e-4 of solver noise, growing as 1/ε)."""
    return M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-15, maxiter=20_000),
                                 picard_iteration_control=M.Convergence(reltol=1e-14, maxiter=2000),
                                 preconditioner=M.StressBalanceDiagonalPreconditioner())


def _case(kind, seed_friction):
    base = workloads.marine_sheet(40, 20, seed=2, seed_friction=seed_friction, velocity_solver=_solver())
    cfg, grid = dict(base.config), base.grid
    if kind == "periodic_x":
        grid = M.RectilinearGrid(size=(40, 20), x=(0.0, 512e3), y=(0.0, 256e3), halo=(4, 4), topology=("Periodic", "Bounded"))
    if kind == "no_slip_coulomb":
        cfg["stress_balance"] = M.DepthIntegrated(side_walls=M.NoSlipWalls())
        cfg["friction"] = M.RegularizedCoulombFriction(coefficient=None, coulomb_coefficient=0.5, exponent=1.0 / 3.0)
    return workloads.Case(f"marine_sheet_{kind}", grid, cfg, base.fields)


def _setup(cls, kind):
    obs = _case(kind, 1200).problem(cls)
    obs.picard_solve()
    uo, vo = obs.get("u"), obs.get("v")
    P = _case(kind, 1100).problem(cls)
    assert P.picard_solve().status == 0
    return P, uo, vo


def _cost(P, uo, vo):
    return 0.5 * (np.sum((P.get("u") - uo) ** 2) + np.sum((P.get("v") - vo) ** 2))


def _centred(P, name, factor_plus, factor_minus, xs, uo, vo, eps):
    """(J(p f₊) - J(p f₋)) / 2ε from converged solves warm-started at x*, with J(+) - J(-) formed as
    ½ Σ (x₊ - x₋)(x₊ + x₋ - 2 x_obs): subtracting two rounded costs would bury weakly sensitive cells."""
    p0 = P.get(name)
    vel = []
    for factor in (factor_plus, factor_minus):
        P.set(name, p0 * factor)
        P.set("u", xs[0])
        P.set("v", xs[1])
        P.picard_solve()
        vel.append((P.get("u"), P.get("v")))
    P.set(name, p0)
    (up, vp), (um, vm) = vel
    dJ = 0.5 * (float(np.sum((up - um) * (up + um - 2 * uo))) + float(np.sum((vp - vm) * (vp + vm - 2 * vo))))
    return dJ / (2 * eps)


def _check_cells(grad, ny):
    """Seeded cells whose gradient is at least 1e-3 of the largest, plus the largest-gradient cell of the first and
    the last row (next to the south and north walls)."""
    floor = 1e-3 * np.max(np.abs(grad))
    cand = np.argwhere(np.abs(grad) >= floor)
    cells = [tuple(cand[k]) for k in np.random.default_rng(7).choice(len(cand), size=min(3, len(cand)), replace=False)]
    for j in (0, ny - 1):
        i = int(np.argmax(np.abs(grad[j])))
        if abs(grad[j, i]) >= floor:
            cells.append((j, i))
    return cells


@pytest.mark.parametrize("kind", KINDS)
def test_oracle_adjoint_matches_finite_differences(oracle_cls, kind):
    P, uo, vo = _setup(oracle_cls, kind)
    xs = (P.get("u"), P.get("v"))
    lu, lv, grad, grad_a, st = P.picard_adjoint(xs[0] - uo, xs[1] - vo, CONTROL)
    assert st.status == 0 and st.picard_iterations > 1 and st.picard_change <= 1e-12 * st.picard_norm
    assert np.array_equal(P.get("u"), xs[0])          # the forward state is left at x*
    scale = np.max(np.abs(grad))
    assert scale > 0
    for cell in _check_cells(grad, grad.shape[0]):
        e = np.ones_like(grad)
        e[cell] = math.exp(1e-3)
        fd = _centred(P, "C", e, 1 / e, xs, uo, vo, 1e-3)
        assert abs(fd - grad[cell]) <= 1e-4 * abs(grad[cell]), (kind, cell, fd, grad[cell], scale)
    d = np.random.default_rng(3).standard_normal(grad_a.shape)
    eps = 4e-5
    fd1 = _centred(P, "A", np.exp(eps * d), np.exp(-eps * d), xs, uo, vo, eps)
    fd2 = _centred(P, "A", np.exp(eps / 2 * d), np.exp(-eps / 2 * d), xs, uo, vo, eps / 2)
    fd = (4 * fd2 - fd1) / 3                                 # Richardson: the ε² term cancels
    ad = float(np.sum(grad_a * d))
    assert abs(fd - ad) <= 1e-4 * float(np.sum(np.abs(grad_a * d))), (kind, fd, ad)


def test_oracle_adjoint_refuses_prescribed_faces(oracle_cls):
    inflow = workloads.channel_shelf(inflow=100.0).problem(oracle_cls)
    with pytest.raises(ValueError):
        inflow.picard_adjoint(np.zeros(inflow.shape("u")), np.zeros(inflow.shape("v")), CONTROL)


def test_unconverged_adjoint_warns(backend):
    """test/test_enzyme.jl:383-389: an adjoint whose control stops it at one iteration warns, and its stats say so;
    a converged one does not."""
    P, uo, vo = _setup(backend, "bounded")
    ub, vb = P.get("u") - uo, P.get("v") - vo
    with pytest.warns(RuntimeWarning, match="Picard adjoint did not converge"):
        *_, st = P.picard_adjoint(ub, vb, M.Convergence(reltol=1e-12, maxiter=1))
    assert st.status == abi.NK_NOT_CONVERGED and st.picard_iterations == 1
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        *_, st = P.picard_adjoint(ub, vb, CONTROL)
    assert st.status == abi.NK_OK


# ---- DIVA: the step also maps its lagged state (βᵇ, F₂, ησ), whose adjoint is swept along with λ --------------
# The stopping test watches λ (as the reference's does); the state adjoint settles more slowly, so 1e-14.
DIVA_CONTROL = M.Convergence(reltol=1e-14, maxiter=3000)


def _diva(friction, obs=False):
    """24 x 12 DIVA sheet (64 km cells, Nσ = 4, Arrhenius rate factor on the σ grid); the observations come from
    other friction coefficients and a 3 % thinner sheet, so the misfit dominates J's second-order terms."""
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-13, maxiter=1000),
                                   preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4))
    case = workloads.diva_sheet(24, 12, dx=64e3, velocity_solver=solver, Nsigma=4)
    cfg = dict(case.config)
    if friction == "weertman":
        cfg["friction"] = M.WeertmanFriction(coefficient=None, exponent=1.0 / 3.0)
    fields = dict(case.fields)
    if obs:
        fields["C"] = fields["C"] * np.exp(0.3 * np.random.default_rng(5).standard_normal(fields["C"].shape))
        fields["H"] = 0.97 * fields["H"]
    return workloads.Case(f"diva_{friction}", case.grid, cfg, fields, temperature=case.temperature)


def _diva_setup(cls, friction):
    obs = _diva(friction, obs=True).problem(cls)
    assert obs.picard_solve().status == 0
    uo, vo = obs.get("u"), obs.get("v")
    P = _diva(friction).problem(cls)
    assert P.picard_solve().status == 0
    return P, uo, vo


@pytest.mark.parametrize("friction", ["weertman", "coulomb"])
def test_oracle_diva_adjoint_matches_finite_differences(oracle_cls, friction):
    """⟨∂J/∂log C, d⟩ and ⟨∂J/∂log A, d⟩ (σ-grid A) along seeded random directions against centred differences:
    ε = 1e-3 and 1e-4 within 1e-4 of Σ|gᵢdᵢ| (measured 1.3e-6 and 4e-9 with Weertman drag).  The Coulomb cap
    leaves J nearly insensitive to C, so its C difference takes ε = 1e-2 and is resolved to 1e-3 (measured 4e-4)."""
    P, uo, vo = _diva_setup(oracle_cls, friction)
    xs = (P.get("u"), P.get("v"))
    lu, lv, grad, grad_a, st = P.picard_adjoint(xs[0] - uo, xs[1] - vo, DIVA_CONTROL)
    assert st.status == 0 and st.picard_iterations > 1
    assert grad_a.shape == P.get("A").shape
    rng = np.random.default_rng(17)
    coulomb = friction == "coulomb"
    for name, g, eps, tol in (("C", grad, 1e-2 if coulomb else 1e-3, 1e-3 if coulomb else 1e-4), ("A", grad_a, 1e-4, 1e-4)):
        d = rng.standard_normal(g.shape)
        fd = _centred(P, name, np.exp(eps * d), np.exp(-eps * d), xs, uo, vo, eps)
        ad = float(np.sum(g * d))
        assert abs(fd - ad) <= tol * float(np.sum(np.abs(g * d))), (friction, name, fd, ad)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", KINDS)
def test_gpu_adjoint_matches_oracle_adjoint(oracle_cls, gpu_cls, kind):
    out = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P, uo, vo = _setup(cls, kind)
        ub, vb = P.get("u") - uo, P.get("v") - vo
        out[key] = P.picard_adjoint(ub, vb, CONTROL)
        assert out[key][4].status == 0
    for idx, name in ((0, "lambda_u"), (1, "lambda_v"), (2, "grad_log_C"), (3, "grad_log_A")):
        g, o = out["g"][idx], out["o"][idx]
        assert g.shape == o.shape, name
        assert np.max(np.abs(g - o)) <= 1e-6 * np.max(np.abs(o)), (kind, name)


@pytest.mark.gpu
@pytest.mark.parametrize("friction", ["weertman", "coulomb"])
def test_gpu_diva_adjoint_matches_oracle_adjoint(oracle_cls, gpu_cls, friction):
    out = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P, uo, vo = _diva_setup(cls, friction)
        out[key] = P.picard_adjoint(P.get("u") - uo, P.get("v") - vo, DIVA_CONTROL)
        assert out[key][4].status == 0
    for idx, name in ((0, "lambda_u"), (1, "lambda_v"), (2, "grad_log_C"), (3, "grad_log_A")):
        g, o = out["g"][idx], out["o"][idx]
        assert g.shape == o.shape, name
        assert np.max(np.abs(g - o)) <= 1e-6 * np.max(np.abs(o)), (friction, name)
