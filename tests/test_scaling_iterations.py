"""The reference's published multigrid scaling benchmark, restated: the conjugate-gradient iteration counts of
docs/src/model/numerics.md:42-49 (tests/golden/reference_scaling.json, extracted by
tests/golden/make_reference_scaling.py), produced by benchmarks/multigrid_scaling.jl.

The benchmark (workloads.mismip_stream) sets the MISMIP+-like ice stream at a grid spacing, which runs five Picard
iterations of multigrid PCG to 1e-6 from rest (the model's velocity update), and then solves the SSA system of
the last coefficients once more from zero to a relative residual of 1e-8, with the diagonal and with the
multigrid preconditioner.  These counts depend on every part of the solve path: the geometry (subgrid grounded
fraction, effective pressure, ice mask, calving front), the driving stress, the regularised Coulomb drag, the
Glen viscosity and column integrals, the operator with its masks, both preconditioners (coarsening, smoothing,
transfers) and the CG stopping rule.
- The oracle reproduces all five published rows up to 0.5 km exactly (42/14, 91/18, 188/20, 392/22, 817/24).
- The GPU library (marked gpu), FP64: all six rows (also 0.25 km, 1769/27) within 2 % (at least one iteration)
  of the published count: a long CG run can end an iteration or two apart under different rounding."""
import json
import os

import pytest

from nunatak_gb300 import model as M, workloads

with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_scaling.json"), encoding="utf-8") as f:
    ROWS = json.load(f)["rows"]


def scaling_iterations(cls, dx):
    """(diagonal, multigrid) CG iterations of the benchmark's timed solve at spacing dx."""
    case = workloads.mismip_stream(dx)
    P = case.problem(cls)
    assert P.picard_solve().status == 0
    coefficients = {k: P.get(k) for k in ("eta_H", "eta_H_ff", "beta_u", "beta_v")}
    tau = P.get("tau_u"), P.get("tau_v")
    P.close()
    counts = []
    for pre in (M.StressBalanceDiagonalPreconditioner(), M.StressBalanceMultigridPreconditioner()):
        solver = M.StressBalanceSolver(preconditioner=pre, linear_iteration_control=M.Convergence(reltol=1e-8, maxiter=100_000),
                                       picard_iteration_control=M.FixedIterations(1))
        Q = workloads.Case("mismip_stream", case.grid, dict(case.config, velocity_solver=solver), case.fields).problem(cls)
        for k, value in coefficients.items():
            Q.set(k, value)
        Q.set("u", 0.0)
        Q.set("v", 0.0)
        st = Q.linear_solve(*tau)
        assert st.status == 0
        counts.append(st.linear_iterations_last)
        Q.close()
    return tuple(counts)


def test_table_holds_six_spacings():
    assert [r["dx_m"] for r in ROWS] == [8e3, 4e3, 2e3, 1e3, 500.0, 250.0]
    for r in ROWS:
        assert (r["nx"], r["ny"]) == (round(640e3 / r["dx_m"]), round(80e3 / r["dx_m"]))


@pytest.mark.parametrize("row", [r for r in ROWS if r["dx_m"] >= 500.0], ids=lambda r: f"{r['dx_m']:g}m")
def test_oracle_reproduces_the_published_iterations(oracle_cls, row):
    assert scaling_iterations(oracle_cls, row["dx_m"]) == (row["diagonal_iterations"], row["multigrid_iterations"])


@pytest.mark.gpu
@pytest.mark.parametrize("row", ROWS, ids=lambda r: f"{r['dx_m']:g}m")
def test_gpu_reproduces_the_published_iterations(gpu_cls, row):
    got = scaling_iterations(gpu_cls, row["dx_m"])
    for n, want in zip(got, (row["diagonal_iterations"], row["multigrid_iterations"])):
        assert abs(n - want) <= max(1, round(0.02 * want)), (row["dx_m"], got)
