"""GPU library vs the FP64 CPU oracle on the same seeded inputs (all marked gpu).

Tolerances (relative, stated per test): single kernels ≤ 1e-12 (the GPU fuses multiply-adds and
multiplies by precomputed reciprocals, so results differ from the oracle in the last bits); solves with
identical fixed iteration counts ≤ 1e-10 relative L2 velocity difference; converged solves at tight
tolerances ≤ 1e-10; the mixed-precision solve ≤ 1e-6 against the FP64 oracle."""
import math

import numpy as np
import pytest

import nunatak_gb300 as nk
from nunatak_gb300 import model as M
from nunatak_gb300 import workloads
from support import evaluate, make, set_fn

pytestmark = pytest.mark.gpu


def rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    d = np.linalg.norm((a - b).ravel())
    n = np.linalg.norm(b.ravel())
    return d / n if n > 0 else d


def rel_l2(ua, va, ub, vb):
    return math.sqrt(np.sum((ua - ub) ** 2) + np.sum((va - vb) ** 2)) / math.sqrt(np.sum(ub ** 2) + np.sum(vb ** 2))


def random_coefficients(P, g, seed, holes=True):
    rng = np.random.default_rng(seed)
    eta = 1.0 + rng.random(P.shape("eta_H"))
    if holes:
        eta[rng.random(eta.shape) < 0.1] = 0.0
    P.set("eta_H", eta)
    P.set("eta_H_ff", 1.0 + rng.random(P.shape("eta_H_ff")))
    P.set("beta_u", rng.random(P.shape("beta_u")))
    P.set("beta_v", rng.random(P.shape("beta_v")))


GRIDS = [
    ("bounded", dict(size=(37, 23), x=(0.0, 3.0), y=(0.0, 2.0), topology=("Bounded", "Bounded"))),
    ("periodic", dict(size=(32, 16), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Periodic", "Periodic"))),
    ("mixed", dict(size=(20, 30), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Periodic", "Bounded"))),
    ("stretched", dict(size=(24, 12), x=list(np.linspace(0, 1, 25) ** 1.3), y=(0.0, 1.0), topology=("Bounded", "Bounded"))),
    # edge shapes of the column-marching kernels: one cell, a sliver narrower than a warp, and ragged sizes whose
    # last 30-column strip and last row walk are partial
    ("one_cell", dict(size=(1, 1), x=(0.0, 1.0), y=(0.0, 1.0), topology=("Bounded", "Bounded"))),
    ("sliver_periodic", dict(size=(2, 5), x=(0.0, 1.0), y=(0.0, 2.0), topology=("Periodic", "Bounded"))),
    ("ragged", dict(size=(61, 33), x=(0.0, 6.1), y=(0.0, 3.3), topology=("Bounded", "Bounded"))),
    ("ragged_periodic", dict(size=(45, 17), x=(0.0, 4.5), y=(0.0, 1.7), topology=("Periodic", "Periodic"))),
]


@pytest.mark.parametrize("walls", [M.FreeSlipWalls(), M.NoSlipWalls()])
@pytest.mark.parametrize("name,gk", GRIDS)
def test_operator_and_preconditioners_match_oracle(oracle_cls, gpu_cls, name, gk, walls):
    g = M.RectilinearGrid(halo=(3, 3), **gk)
    rng = np.random.default_rng(5)
    out = {}
    for pre in (M.StressBalanceDiagonalPreconditioner(), M.StressBalanceMultigridPreconditioner()):
        for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
            P = make(cls, g, stress_balance=M.DepthIntegrated(side_walls=walls), masking=None,
                     velocity_solver=M.StressBalanceSolver(preconditioner=pre))
            random_coefficients(P, g, 3)
            pu = np.random.default_rng(7).standard_normal(P.shape("u"))
            pv = np.random.default_rng(8).standard_normal(P.shape("v"))
            out[(type(pre).__name__, key)] = P.apply_operator(pu, pv) + P.precondition(pu, pv)
    for pre in ("StressBalanceDiagonalPreconditioner", "StressBalanceMultigridPreconditioner"):
        o, gg = out[(pre, "o")], out[(pre, "g")]
        assert rel(gg[0], o[0]) < 1e-13 and rel(gg[1], o[1]) < 1e-13, "operator"
        assert rel(gg[2], o[2]) < 1e-12 and rel(gg[3], o[3]) < 1e-12, pre


@pytest.mark.parametrize("smoother", [M.PointJacobi(), M.LineJacobi()])
def test_multigrid_transfers_match_oracle(oracle_cls, gpu_cls, smoother):
    g = M.RectilinearGrid(size=(32, 16), x=(0.0, 2.0), y=(0.0, 1.0), halo=(4, 4))
    res = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P = make(cls, g, masking=None, velocity_solver=M.StressBalanceSolver(
            preconditioner=M.StressBalanceMultigridPreconditioner(smoother=smoother)))
        random_coefficients(P, g, 11)
        levels = P.multigrid_levels()
        fu = np.random.default_rng(1).standard_normal(P.shape("u"))
        fv = np.random.default_rng(2).standard_normal(P.shape("v"))
        cu, cv = P.restrict(0, fu, fv)
        pu, pv = P.prolongate(0, np.ones_like(cu), np.ones_like(cv))
        zu, zv = P.precondition(fu, fv)
        res[key] = (levels, cu, cv, pu, pv, zu, zv)
    assert res["o"][0] == res["g"][0]
    for a, b in zip(res["g"][1:], res["o"][1:]):
        assert rel(a, b) < 1e-12


@pytest.mark.parametrize("diva", [False, True])
def test_coefficient_update_matches_oracle(oracle_cls, gpu_cls, diva):
    case = workloads.marine_sheet(48, 24, seed=4)
    cfg = dict(case.config)
    if diva:
        cfg["stress_balance"] = M.DepthIntegrated(shear=M.DIVAShear())
    out = {}
    rng = np.random.default_rng(9)
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P = cls(case.grid, M.make_descriptors(case.grid, **cfg))
        for k, v in case.fields.items():
            P.set(k, v)
        P.compute_geometry()
        P.set("u", 100 / M.YEAR * np.random.default_rng(1).random(P.shape("u")))
        P.set("v", 10 / M.YEAR * np.random.default_rng(2).standard_normal(P.shape("v")))
        for _ in range(2):   # the second DIVA update uses the lagged viscosity and drag
            P.update_coefficients()
        out[key] = {k: P.get(k) for k in ("eta_H", "eta_H_ff", "beta_u", "beta_v", "eta_sigma", "F2", "tau_u", "tau_v",
                                          "s", "N", "phi", "phi_u", "phi_v", "ice_mask")}
        if diva:
            out[key].update({k: P.get(k) for k in ("beta_b_u", "beta_b_v", "u_b", "v_b")})
    for k in out["o"]:
        assert rel(out["g"][k], out["o"][k]) < 1e-12, k


def solve_both(oracle_cls, gpu_cls, case):
    res = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P = case.problem(cls)
        st = P.picard_solve()
        res[key] = (P.get("u"), P.get("v"), st)
    return res


def test_channel_shelf_fixed_iterations(oracle_cls, gpu_cls):
    """Floating channel shelf (84 x 40, Jacobi): identical Picard(3) x CG(40) iteration counts.  (Longer
    unconverged runs amplify the last-bit differences: 4 x 200 iterations differ by 2e-8 while the converged
    solves below agree to 1e-10.)"""
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(40), picard_iteration_control=M.FixedIterations(3))
    r = solve_both(oracle_cls, gpu_cls, workloads.channel_shelf(velocity_solver=solver))
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10


def test_channel_shelf_converged(oracle_cls, gpu_cls):
    """Floating channel shelf at the workload tolerances tightened to CG 1e-13, Picard 1e-12."""
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=300))
    r = solve_both(oracle_cls, gpu_cls, workloads.channel_shelf(velocity_solver=solver))
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10
    assert abs(r["g"][2].picard_iterations - r["o"][2].picard_iterations) <= 1


def test_marine_sheet_multigrid_fp64_fixed(oracle_cls, gpu_cls):
    """Marine sheet 64 x 32 with the FP64 multigrid: Picard(3) x CG(25)."""
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(25), picard_iteration_control=M.FixedIterations(3),
                                   preconditioner=mg)
    r = solve_both(oracle_cls, gpu_cls, workloads.marine_sheet(64, 32, seed=2, velocity_solver=solver))
    assert rel_l2(r["g"][0], r["g"][1], r["o"][0], r["o"][1]) < 1e-10


def test_marine_sheet_mixed_precision_vs_fp64_oracle(oracle_cls, gpu_cls):
    """The FP32-multigrid mixed solve converged tightly agrees with the FP64 oracle to 1e-6."""
    mg = M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4)
    tight = dict(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=2000),
                 picard_iteration_control=M.Convergence(reltol=1e-9, maxiter=300), preconditioner=mg)
    ref = workloads.marine_sheet(64, 32, seed=2, velocity_solver=M.StressBalanceSolver(**tight)).problem(oracle_cls)
    ref.picard_solve()
    P = workloads.marine_sheet(64, 32, seed=2, velocity_solver=M.StressBalanceSolver(precision="mixed", **tight)).problem(gpu_cls)
    st = P.picard_solve()
    assert st.status == 0
    assert rel_l2(P.get("u"), P.get("v"), ref.get("u"), ref.get("v")) < 1e-6


def test_diva_fixed_iterations(oracle_cls, gpu_cls):
    """DIVA sheet 64 x 32 (Nσ = 6, Arrhenius rate factor, regularised Coulomb): Picard(3) x CG(30), then the profile."""
    solver = M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(30), picard_iteration_control=M.FixedIterations(3),
                                   preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=4))
    case = workloads.diva_sheet(64, 32, dx=32e3, velocity_solver=solver, Nsigma=6)
    res = {}
    for key, cls in (("o", oracle_cls), ("g", gpu_cls)):
        P = case.problem(cls)
        P.picard_solve()
        P.velocity_profile()
        res[key] = {k: P.get(k) for k in ("u", "v", "A", "eta_sigma", "u_sigma", "v_sigma", "u_b", "v_b")}
    assert rel_l2(res["g"]["u"], res["g"]["v"], res["o"]["u"], res["o"]["v"]) < 1e-10
    for k in ("A", "eta_sigma", "u_sigma", "v_sigma", "u_b", "v_b"):
        assert rel(res["g"][k], res["o"][k]) < 1e-10, k


def test_solve_is_deterministic(gpu_cls):
    """Two runs of the same solve give bitwise identical velocities (fixed-order reductions)."""
    case = workloads.marine_sheet(64, 32, seed=5)
    runs = []
    for _ in range(2):
        P = case.problem(gpu_cls)
        P.picard_solve()
        runs.append((P.get("u"), P.get("v")))
    assert np.array_equal(runs[0][0], runs[1][0]) and np.array_equal(runs[0][1], runs[1][1])


def test_solve_velocities_host_entry_point(gpu_cls):
    """nk_solve_velocities (host u, v in and out) equals nk_picard_solve on resident fields."""
    import ctypes as C
    case = workloads.channel_shelf(velocity_solver=M.StressBalanceSolver(
        linear_iteration_control=M.FixedIterations(50), picard_iteration_control=M.FixedIterations(2)))
    P = case.problem(gpu_cls)
    u = np.zeros(P.shape("u"))
    v = np.zeros(P.shape("v"))
    st = nk.abi.SolveStats()
    dp = C.POINTER(C.c_double)
    assert P._lib.nk_solve_velocities(P._h, u.ctypes.data_as(dp), v.ctypes.data_as(dp), C.byref(st)) == 0
    Q = case.problem(gpu_cls)
    Q.picard_solve()
    assert np.array_equal(u, Q.get("u")) and np.array_equal(v, Q.get("v"))
