"""Extract the jldoctest blocks of the reference's velocity-solve sources into reference_doctests.json.

The reference (Nunatak.jl, Julia) cannot run in this environment, so its doctests are its golden vectors: each
block is a sequence of `julia>` inputs, some followed by the printed result.  This script reads the sources as
text and records, per block, the file, the line of its opening fence and the (input, output) steps.  The tests
read the expected outputs from the JSON (support.reference_doctest); nothing at test time reads the reference.

Usage: python tests/golden/make_reference_doctests.py <path to the Nunatak.jl checkout>
"""
import json
import os
import sys

# The reference files of the velocity solve and its inputs whose doctests pin the restatement.
FILES = [
    "src/Solvers/velocity_vector.jl",
    "src/Solvers/iteration_controls.jl",
    "src/Solvers/conjugate_gradient.jl",
    "src/Solvers/picard.jl",
    "src/StressBalances/ssa_operator.jl",
    "src/StressBalances/depth_integrated.jl",
    "src/StressBalances/driving_stress.jl",
    "src/StressBalances/multigrid_preconditioner.jl",
    "src/StressBalances/stress_balance_solver.jl",
    "src/Rheologies/glen_flow_law.jl",
    "src/Rheologies/arrhenius_rate_factor.jl",
    "src/Frictions/frictions.jl",
    "src/Groundings/subgrid_grounded_fraction.jl",
    "src/Models/smooth_ice_mask.jl",
    "src/Models/ice_sheet_constants.jl",
    "src/Grids/sigma_grid.jl",
    "src/Thermodynamics/enthalpy_conversions.jl",
]


def blocks(lines):
    """(first line number, body lines) of every ```jldoctest ... ``` block, 1-based."""
    out, start, body = [], None, []
    for n, line in enumerate(lines, 1):
        s = line.strip()
        if start is None and s.startswith("```jldoctest"):
            start, body = n, []
        elif start is not None and s == "```":
            out.append((start, n, body))
            start = None
        elif start is not None:
            body.append(line.rstrip("\n"))
    return out


def steps(body):
    """Split a block into (input, output) steps; continuation lines of an input start with spaces."""
    out = []
    for line in body:
        if line.startswith("julia> "):
            out.append({"input": line[len("julia> "):], "output": []})
        elif out and not out[-1]["output"] and line.startswith("       "):
            out[-1]["input"] += "\n" + line.strip()
        elif out and line.strip():
            out[-1]["output"].append(line)
    for s in out:
        s["output"] = "\n".join(s["output"])
    return out


def main(root):
    entries = []
    for rel in FILES:
        with open(os.path.join(root, rel), encoding="utf-8") as f:
            lines = f.readlines()
        for start, end, body in blocks(lines):
            entries.append({"file": rel, "lines": [start, end], "steps": steps(body)})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_doctests.json")
    with open(path, "w", encoding="utf-8") as f:
        json.dump({"source": "Nunatak.jl doctests (jldoctest blocks), extracted as text", "doctests": entries},
                  f, indent=1, ensure_ascii=False)
        f.write("\n")
    print(f"{len(entries)} doctests -> {path}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])
