"""GPU solves against the FP64 oracle at the workloads' own sizes and physics.

- The marine sheet of the 256 x 128 (2 km) workload, multigrid PCG (coarsening stops at 32 cells), converged to
  tight tolerances (Picard 1e-12, CG 1e-13) from rest: the FP64 library within 1e-10 and the mixed-precision library
  (FP32 multigrid under FP64 flexible CG) within 1e-6 of the oracle (relative L2 over u and v).
- The serving stream: the first request of every grid size (128 x 64 to 1024 x 512 on the 512 x 256 km domain, each
  with its own friction seed) solved by the mixed-precision library with the stream's tolerances (Picard 1e-6, CG
  1e-8) within 1e-6 of the oracle's FP64 solve of the same request.
- The DIVA sheet's physics (Nσ = 10 levels with faces (k/10)², Arrhenius rate factor from the seeded temperature
  field, regularised Coulomb drag with the ocean-connected effective pressure, calving front at x = 1900 km) on a
  reduced 128 x 64 grid of 16 km cells over the same 2048 x 1024 km domain, tight tolerances: FP64 within 1e-10,
  mixed within 1e-6.
The oracle's solves of the large stream requests take a minute on the host cores; they run once per module."""
import functools

import numpy as np
import pytest

from nunatak_gb300 import model as M, workloads


def _rel(a, b):
    (u, v), (ur, vr) = a, b
    return float(np.sqrt(np.sum((u - ur) ** 2) + np.sum((v - vr) ** 2)) / np.sqrt(np.sum(ur ** 2) + np.sum(vr ** 2)))


def _solve(case, cls):
    P = case.problem(cls)
    st = P.picard_solve()
    out = (P.get("u"), P.get("v")), st
    P.close()
    return out


def _tight(precision):
    return M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                 picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=1000),
                                 preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=32),
                                 precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_marine_sheet_256x128_against_oracle(gpu_cls, oracle_cls, precision, tol):
    want, sto = _oracle_marine()
    got, st = _solve(workloads.marine_sheet(256, 128, seed=1, velocity_solver=_tight(precision)), gpu_cls)
    assert st.status == 0 and sto.status == 0
    err = _rel(got, want)
    assert err <= tol, (precision, err, st.picard_iterations, sto.picard_iterations)


@functools.lru_cache(maxsize=1)
def _oracle_marine():
    import nunatak_oracle
    return _solve(workloads.marine_sheet(256, 128, seed=1, velocity_solver=_tight("fp64")), nunatak_oracle.OracleProblem)


def _first_of_each_size():
    seen = {}
    for r in workloads.serving_stream():
        seen.setdefault(r["size"], r)
    return [seen[s] for s in workloads.SERVING_SIZES]


@functools.lru_cache(maxsize=4)
def _oracle_request(index):
    import nunatak_oracle
    r = workloads.serving_stream()[index]
    return _solve(workloads.serving_case(r, "fp64"), nunatak_oracle.OracleProblem)


@pytest.mark.gpu
@pytest.mark.parametrize("request_", _first_of_each_size(), ids=lambda r: "%dx%d" % r["size"])
def test_stream_request_mixed_against_oracle(gpu_cls, request_):
    want, sto = _oracle_request(request_["index"])
    got, st = _solve(workloads.serving_case(request_, "mixed"), gpu_cls)
    assert st.status == 0 and sto.status == 0
    err = _rel(got, want)
    assert err <= 1e-6, (request_["size"], err, st.picard_iterations, sto.picard_iterations)


def _diva(precision):
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-13, maxiter=20_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-12, maxiter=1000),
                                   preconditioner=M.StressBalanceMultigridPreconditioner(minimum_coarse_size=32),
                                   precision=precision)
    return workloads.diva_sheet(128, 64, dx=16e3, velocity_solver=solver)


@functools.lru_cache(maxsize=1)
def _oracle_diva():
    import nunatak_oracle
    return _solve(_diva("fp64"), nunatak_oracle.OracleProblem)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_diva_sheet_physics_against_oracle(gpu_cls, precision, tol):
    want, sto = _oracle_diva()
    got, st = _solve(_diva(precision), gpu_cls)
    assert st.status == 0 and sto.status == 0
    err = _rel(got, want)
    assert err <= tol, (precision, err, st.picard_iterations, sto.picard_iterations)


def test_diva_case_has_the_workload_physics():
    """The reduced DIVA case keeps the workload's physics: σ levels, Arrhenius A from T, regularised Coulomb drag,
    no ice beyond x = 1900 km (the sheet's profile 2000 m sqrt(1 - (x / 1680 km)²) reaches zero before it)."""
    case = _diva("fp64")
    cfg = case.config
    assert cfg["Nsigma"] == 10 and isinstance(cfg["stress_balance"].shear, M.DIVAShear)
    assert isinstance(cfg["friction"], M.RegularizedCoulombFriction) and cfg["friction"].coulomb_coefficient == 0.5
    assert case.temperature.shape == (10, 64, 128)
    x = case.grid.centers(0)
    assert np.all(case.fields["H"][:, x > 1900e3] == 0) and np.all(case.fields["H"][:, x < 1600e3] > 0)
