"""Extract the STREAMICE halfpipe adjoint's configuration and published results into halfpipe_streamice.json.

benchmarks/halfpipe_streamice.jl and benchmarks/halfpipe_streamice_adjoint.jl of Nunatak.jl set up MITgcm's
verification experiment halfpipe_streamice (a mostly floating shelf in a half-pipe channel with a partial-cell front)
and its adjoint variant (input_ad): three 0.2-year steps, the cost of the velocities after step 2 and of the thickness
after step 3, the basal melt control at four centreline cells with records weighted 0.5, 1, 0.5 over the steps, and
STREAMICE's cost, adjoint gradient and finite differences (from its output_adm.txt).  This script reads those values as
text; tests/test_gpu_halfpipe_adjoint.py and bench.py --halfpipe-adjoint compare the library's gradient with them.
Nothing at test time reads the reference.

Usage: python tests/golden/make_halfpipe_reference.py <path to the Nunatak.jl checkout>
"""
import json
import os
import re
import sys

FORWARD = "benchmarks/halfpipe_streamice.jl"
ADJOINT = "benchmarks/halfpipe_streamice_adjoint.jl"


def numbers(text):
    return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?(?:e-?\d+)?", text)]


def main(root):
    fwd = open(os.path.join(root, FORWARD), encoding="utf-8").read()
    adj = open(os.path.join(root, ADJOINT), encoding="utf-8").read()

    def scalar(src, name):
        m = re.search(rf"^{re.escape(name)} = (.+)$", src, flags=re.M)
        return m.group(1).strip()

    def tuple_of(src, name):
        m = re.search(rf"^{re.escape(name)} = \((.*?)\)\s*$", src, flags=re.M | re.S)
        return numbers(m.group(1))

    rho = numbers(scalar(fwd, "ρᵢ, ρw, g"))
    B, C, n = numbers(scalar(fwd, "B, C, n"))
    Nx, Ny = (int(v) for v in numbers(scalar(fwd, "Nx, Ny")))
    bed = numbers(re.search(r"bed_profile = \[(.*?)\]", fwd, flags=re.S).group(1))
    cells = [[int(a), int(b)] for a, b in re.findall(r"\((\d+), (\d+)\)", scalar(adj, "check_cells"))]
    out = {
        "source": [FORWARD, ADJOINT],
        "ice_density": rho[0], "ocean_density": rho[1], "gravitational_acceleration": rho[2],
        "B": B, "C": C, "n": n, "Nx": Nx, "Ny": Ny,
        "dx_km": numbers(scalar(fwd, "Δx"))[0],
        "inflow_m2_per_year": numbers(scalar(fwd, "inflow"))[0],
        "bed_profile": bed,
        "control_weights": tuple_of(adj, "control_weights"),
        "check_cells_julia": cells,
        "streamice_cost": numbers(scalar(adj, "streamice_cost"))[0],
        "streamice_adjoint_gradient": tuple_of(adj, "streamice_adjoint_gradient"),
        "streamice_finite_difference": tuple_of(adj, "streamice_finite_difference"),
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "halfpipe_streamice.json")
    with open(path, "w", encoding="utf-8") as f:
        json.dump(out, f, indent=1, ensure_ascii=False)
        f.write("\n")
    print(f"-> {path}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else ".")
