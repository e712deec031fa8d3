"""Parity against the committed golden fixtures tests/golden/oracle_solves.npz (written by
tests/golden/make_oracle_solves.py from the FP64 oracle; cases in tests/golden_cases.py).

- The oracle reproduces every fixture bit for bit (it is deterministic: row sums in a fixed order, no
  floating-point contraction), so a change of the oracle cannot go unnoticed.
- The GPU library reproduces every fixture: each case runs Picard and CG with fixed iteration counts, so the two
  differ by rounding only.  Velocities within 1e-10 relative L2 over each velocity pair ((u, v) and
  (u_sigma, v_sigma), the measure of the fixed-count parity tests) and u_b on its own; the coefficients of the
  last Picard update (η̄H, β, ησ) within 1e-9 per field."""
import os

import numpy as np
import pytest

import golden_cases

FIXTURES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_solves.npz")
RTOL_VELOCITY = 1e-10
RTOL_COEFFICIENT = 1e-9
PAIRS = {"u": ("u", "v"), "v": ("u", "v"), "u_sigma": ("u_sigma", "v_sigma"), "v_sigma": ("u_sigma", "v_sigma")}


def _fixture(name):
    with np.load(FIXTURES) as d:
        return {k.split("/", 1)[1]: d[k] for k in d.files if k.split("/", 1)[0] == name}


def test_fixture_file_holds_every_case():
    with np.load(FIXTURES) as d:
        stored = {k.split("/", 1)[0] for k in d.files}
    assert stored == set(golden_cases.CASES)
    for name, (_, fields) in golden_cases.CASES.items():
        assert set(_fixture(name)) == set(fields), name


@pytest.mark.parametrize("name", sorted(golden_cases.CASES))
def test_oracle_reproduces_golden_solves(oracle_cls, name):
    got, want = golden_cases.solve(name, oracle_cls), _fixture(name)
    for k, w in want.items():
        assert got[k].shape == w.shape and np.array_equal(got[k], w), (name, k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(golden_cases.CASES))
def test_gpu_matches_golden_solves(gpu_cls, name):
    got, want = golden_cases.solve(name, gpu_cls), _fixture(name)
    for k, w in want.items():
        assert got[k].shape == w.shape, (name, k)
        group = PAIRS.get(k, (k,))
        scale = np.sqrt(sum(np.sum(want[m] ** 2) for m in group))
        err = np.linalg.norm((got[k] - w).ravel()) / scale
        tol = RTOL_VELOCITY if k in PAIRS or k == "u_b" else RTOL_COEFFICIENT
        assert err <= tol, (name, k, err)
