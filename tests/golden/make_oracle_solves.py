"""Write oracle_solves.npz: the FP64 CPU oracle's velocity solves of small seeded workloads, with fixed iteration
counts, as golden fixtures for the parity tests (tests/test_golden_solves.py).

The oracle restates the reference's algorithm and is pinned on the reference's own known answers; these fixtures
freeze its outputs so the GPU library is checked against committed numbers, and any later change of the oracle
shows up as a mismatch.  The cases are defined in tests/golden_cases.py (shared with the test).

Usage: python tests/golden/make_oracle_solves.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(ROOT, "nunatak.jl_gb300"), os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    sys.path.insert(0, p)

import numpy as np  # noqa: E402

import golden_cases  # noqa: E402
import nunatak_oracle  # noqa: E402


def main():
    arrays = {}
    for name in golden_cases.CASES:
        for key, value in golden_cases.solve(name, nunatak_oracle.OracleProblem).items():
            arrays[f"{name}/{key}"] = value
    path = os.path.join(HERE, "oracle_solves.npz")
    np.savez_compressed(path, **arrays)
    print(f"{len(arrays)} arrays, {os.path.getsize(path)} bytes -> {path}")


if __name__ == "__main__":
    main()
