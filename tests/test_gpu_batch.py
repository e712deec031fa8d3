"""Batched solves (nk_batch): each slot of a batch gives the same bits, iteration counts and statistics as its problem
solved alone, whatever the other slots hold and whichever slots are solved; slots left out are not touched."""
import numpy as np
import pytest

import nunatak_gb300 as nk
from nunatak_gb300 import library, model as M, workloads

pytestmark = pytest.mark.gpu

SLOTS = 5


def marine(seed, precision="mixed", solver=None, nx=64, ny=32):
    return workloads.marine_sheet(nx, ny, seed=1, seed_friction=300 + seed, precision=precision, minimum_coarse_size=8,
                                  velocity_solver=solver)


def line_jacobi_solver():
    mg = M.StressBalanceMultigridPreconditioner(smoother=M.LineJacobi(), smoothing_sweeps=3, coarsest_sweeps=7,
                                                minimum_coarse_size=8)
    return M.StressBalanceSolver(preconditioner=mg, precision="fp64")


def jacobi_solver():
    return M.StressBalanceSolver(preconditioner=M.StressBalanceDiagonalPreconditioner(),
                                 linear_iteration_control=M.Convergence(reltol=1e-8, maxiter=2000))


def odd_sweeps_solver():
    mg = M.StressBalanceMultigridPreconditioner(smoothing_sweeps=3, coarsest_sweeps=9, minimum_coarse_size=8)
    return M.StressBalanceSolver(preconditioner=mg, precision="mixed")


CONFIGS = {
    "ssa_mixed_multigrid": lambda k: marine(k, "mixed"),
    "ssa_fp64_multigrid": lambda k: marine(k, "fp64"),
    "ssa_jacobi": lambda k: marine(k, solver=jacobi_solver()),
    "ssa_line_jacobi_odd_sweeps": lambda k: marine(k, solver=line_jacobi_solver()),
    "ssa_point_jacobi_odd_sweeps": lambda k: marine(k, solver=odd_sweeps_solver()),
    "diva_mixed": lambda k: workloads.diva_sheet(64, 32, seed=5 + k, dx=8e3, precision="mixed", Nsigma=6),
}


def alone(case):
    """u, v, stats and kernel launches of the case solved by a problem of its own (one solve from the state that
    Case.problem leaves: the DIVA's lagged basal state carries over from one solve to the next)."""
    P = case.problem(nk.Problem)
    n0 = library.launch_count()
    st = P.picard_solve()
    out = P.get("u"), P.get("v"), st, library.launch_count() - n0
    P.close()
    return out


def load(B, k, case):
    """The case's inputs into slot k, as Case.problem does for a problem of its own."""
    P = B.problem(k)
    for name, v in case.fields.items():
        P.set(name, v)
    if case.temperature is not None:
        P.set("T", case.temperature)
        P.compute_rate_factor()
    P.compute_geometry()
    for name, v in case.initial.items():
        P.set(name, v)
    P.set("u", 0.0)
    P.set("v", 0.0)
    return P


@pytest.mark.parametrize("config", sorted(CONFIGS))
def test_batched_slots_equal_solves_alone(config):
    cases = [CONFIGS[config](k) for k in range(SLOTS)]
    ref = [alone(c) for c in cases]
    with nk.Batch(cases[0].grid, cases[0].descriptors(), SLOTS) as B:
        for k, c in enumerate(cases):
            load(B, k, c)
        n0 = library.launch_count()
        stats = B.picard_solve()
        launches = library.launch_count() - n0
        for k, (ur, vr, sr, _) in enumerate(ref):
            st = stats[k]
            assert st.status == sr.status
            assert st.picard_iterations == sr.picard_iterations
            assert st.linear_iterations_total == sr.linear_iterations_total
            assert st.picard_change == sr.picard_change and st.residual_norm == sr.residual_norm
            P = B.problem(k)
            assert np.array_equal(P.get("u"), ur) and np.array_equal(P.get("v"), vr), f"slot {k}"
    # one launch per kernel for all slots: about the launches of the slowest slot alone, plus one small kernel per loop
    # body that takes the loop decision over the slots
    solo = [r[3] for r in ref]
    assert max(solo) <= launches < 1.5 * max(solo), (launches, solo)


def test_chosen_slots_only_and_a_second_solve():
    cases = [marine(k) for k in range(SLOTS)]
    ref = [alone(c) for c in cases]
    with nk.Batch(cases[0].grid, cases[0].descriptors(), SLOTS) as B:
        for k, c in enumerate(cases):
            load(B, k, c)
        marker = {k: (np.full(B.problem(k).shape("u"), 7.0 + k), np.full(B.problem(k).shape("v"), -3.0 - k)) for k in (1, 3)}
        for k, (mu, mv) in marker.items():
            B.problem(k).set("u", mu)
            B.problem(k).set("v", mv)
        stats = B.picard_solve([0, 2, 4])
        assert stats[1] is None and stats[3] is None
        for k in (0, 2, 4):
            assert stats[k].picard_iterations == ref[k][2].picard_iterations
            assert np.array_equal(B.problem(k).get("u"), ref[k][0])
        for k, (mu, mv) in marker.items():
            assert np.array_equal(B.problem(k).get("u"), mu) and np.array_equal(B.problem(k).get("v"), mv)
        # the other slots next, from zero, then every slot again from zero: the same bits each time
        for k in (1, 3):
            B.problem(k).set("u", 0.0)
            B.problem(k).set("v", 0.0)
        B.picard_solve(np.array([False, True, False, True, False]))
        for k in (1, 3):
            assert np.array_equal(B.problem(k).get("u"), ref[k][0])
        for k in range(SLOTS):
            B.problem(k).set("u", 0.0)
            B.problem(k).set("v", 0.0)
        B.picard_solve_async()
        while not B.query():
            pass
        stats = B.wait()
        for k in range(SLOTS):
            assert stats[k].linear_iterations_total == ref[k][2].linear_iterations_total
            assert np.array_equal(B.problem(k).get("u"), ref[k][0]) and np.array_equal(B.problem(k).get("v"), ref[k][1])


def test_slot_problem_solves_alone_too():
    cases = [marine(k) for k in range(2)]
    ref = alone(cases[1])
    with nk.Batch(cases[0].grid, cases[0].descriptors(), 2) as B:
        P = load(B, 1, cases[1])
        st = P.picard_solve()
        assert st.picard_iterations == ref[2].picard_iterations
        assert np.array_equal(P.get("u"), ref[0])


def test_batches_refuse_what_they_cannot_run():
    case = marine(0)
    solver = M.StressBalanceSolver(preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=8),
                                   precision="mixed", host_loop=True)
    host = workloads.marine_sheet(64, 32, seed=1, velocity_solver=solver)
    with pytest.raises(ValueError):
        nk.Batch(host.grid, host.descriptors(), 2)
    with pytest.raises(ValueError):
        nk.Batch(case.grid, case.descriptors(), 0)
    with nk.Batch(case.grid, case.descriptors(), 2) as B:
        load(B, 0, case)
        load(B, 1, case)
        u = workloads.west_inflow(case.grid, 100.0)
        B.problem(1).set("u_prescribed", u)
        with pytest.raises(ValueError):
            B.picard_solve()
        stats = B.picard_solve([0])   # the slot with prescribed velocities left out
        assert stats[0].status == 0
