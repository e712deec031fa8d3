"""The strip autotuner (nk_problem.cu, opt-in with NK_AUTOTUNE=1) picks the walk length of the FP64 multigrid
sweeps and residuals by timing.  Those kernels write one value per cell with no reduction; a different walk
length only changes how the compiler contracts multiply-adds, so results move in the last bits.  Checked in
separate processes: one V-cycle with every walk length forced (NK_STRIP_ROWS) agrees to 1e-12, and mixed and
FP64 solves with and without the autotuner agree to 1e-6 (the CG tolerance bounds the difference)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys, numpy as np
sys.path[:0] = [sys.argv[1], sys.argv[1] + "/nunatak.jl_gb300"]
import nunatak_gb300 as nk
from nunatak_gb300 import workloads
out = []
for precision in ("mixed", "fp64"):
    P = workloads.marine_sheet(192, 96, seed=1, seed_friction=1003, precision=precision).problem(nk.Problem)
    P.picard_solve()
    out += [P.get("u").ravel(), P.get("v").ravel()]
    r = np.random.default_rng(2)
    ru, rv = r.standard_normal(P.shape("u")), r.standard_normal(P.shape("v"))
    zu, zv = P.precondition(ru, rv)             # one V-cycle: sweeps, residuals and transfers only
    out += [zu.ravel(), zv.ravel()]
np.save(sys.argv[2], np.concatenate(out))
"""


def _run(tmp_path, name, env_extra):
    path = tmp_path / f"{name}.npy"
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "-c", SCRIPT, ROOT, str(path)], env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    return np.load(path)


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def _vcycle_parts(a):
    """The V-cycle outputs (zu, zv) of both precisions: each precision's block is u, v, zu, zv of one grid, so its
    second half."""
    half = a.size // 2
    return np.concatenate([blk[blk.size // 2:] for blk in (a[:half], a[half:])])


def _solve_parts(a):
    half = a.size // 2
    return np.concatenate([blk[:blk.size // 2] for blk in (a[:half], a[half:])])


def test_autotuned_walks_agree_with_the_fixed_rule(tmp_path):
    tuned = _run(tmp_path, "tuned", {"NK_AUTOTUNE": "1"})
    fixed = _run(tmp_path, "fixed", {"NK_AUTOTUNE": "0"})
    assert _rel(_vcycle_parts(tuned), _vcycle_parts(fixed)) < 1e-12
    assert _rel(_solve_parts(tuned), _solve_parts(fixed)) < 1e-6


def test_preconditioner_depends_on_the_walk_length_in_the_last_bits_only(tmp_path):
    base, *others = [_vcycle_parts(_run(tmp_path, f"rows{r}", {"NK_STRIP_ROWS": str(r)})) for r in (1, 2, 4)]
    for other in others:
        assert _rel(other, base) < 1e-12
