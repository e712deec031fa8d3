"""Extract the reference's published multigrid scaling table into reference_scaling.json.

docs/src/model/numerics.md of Nunatak.jl lists, for its MISMIP+-like ice stream (benchmarks/multigrid_scaling.jl),
the conjugate-gradient iterations of one SSA solve from zero to a relative residual of 1e-8 with the diagonal and
the multigrid preconditioner at six grid spacings, with their CPU and GPU times.  This script reads the table as
text and records, per row, the spacing, the grid and the iteration counts (the times are kept as printed).
tests/test_scaling_iterations.py checks the restated solve against the counts; nothing at test time reads the
reference.

Usage: python tests/golden/make_reference_scaling.py <path to the Nunatak.jl checkout>
"""
import json
import os
import re
import sys

SOURCE = "docs/src/model/numerics.md"


def main(root):
    rows = []
    with open(os.path.join(root, SOURCE), encoding="utf-8") as f:
        lines = f.readlines()
    row = re.compile(r"^\|\s*([\d.]+) km\s*\|\s*(\d+) × (\d+)\s*\|\s*(\d+), ([^|]+)\|\s*(\d+), ([^|]+)\|\s*$")
    for n, line in enumerate(lines, 1):
        m = row.match(line.strip())
        if m:
            rows.append({"line": n, "dx_m": float(m.group(1)) * 1e3, "nx": int(m.group(2)), "ny": int(m.group(3)),
                         "diagonal_iterations": int(m.group(4)), "diagonal_cpu_gpu_s": m.group(5).strip(),
                         "multigrid_iterations": int(m.group(6)), "multigrid_cpu_gpu_s": m.group(7).strip()})
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_scaling.json")
    with open(path, "w", encoding="utf-8") as f:
        json.dump({"source": SOURCE, "benchmark": "benchmarks/multigrid_scaling.jl",
                   "solve": "one SSA solve from zero to a relative residual of 1e-8 after five Picard iterations",
                   "rows": rows}, f, indent=1, ensure_ascii=False)
        f.write("\n")
    print(f"{len(rows)} rows -> {path}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    main(sys.argv[1])
