"""The Julia binding (nunatak.jl_gb300/julia/NunatakGB300.jl) against the C header it binds.

Julia cannot run here, so the binding is held to the header as text: each descriptor struct mirrors its C struct
field for field, in order, with matching widths (Int32 / Float64 / Ptr), every `ccall` names a function the header
declares, and the field ids it uses are the header's."""
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "nunatak_gb300.h")
JULIA = os.path.join(ROOT, "nunatak.jl_gb300", "julia", "NunatakGB300.jl")

C_TYPES = {"int32_t": "Int32", "double": "Float64", "const double*": "Ptr{Float64}", "double*": "Ptr{Float64}",
           "const nk_iteration_control*": "Ptr{IterationControl}"}


def c_structs():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \w+;", text, flags=re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            mt = re.match(r"(const double\*|double\*|int32_t|double|int64_t|const nk_iteration_control\*|"
                          r"nk_iteration_control|nk_grid_desc|"
                          r"nk_physics_desc|nk_solver_desc|const double \*)\s*(.*)", decl)
            assert mt, decl
            typ = mt.group(1).replace(" *", "*")
            for name in mt.group(2).split(","):
                name = name.strip()
                if name.startswith("*"):
                    typ, name = typ + "*", name[1:]
                fields.append((name, C_TYPES.get(typ, typ)))
        out[m.group(1)] = fields
    return out


def julia_structs():
    text = open(JULIA).read()
    out = {}
    for m in re.finditer(r"(?:mutable )?struct (\w+)\n(.*?)\nend", text, flags=re.S):
        fields = []
        for line in m.group(2).splitlines():
            if "=" in line and "::" not in line.split("=")[0]:
                continue
            for decl in line.split(";"):
                decl = decl.strip()
                mt = re.match(r"^(\w+)::([\w{}]+)$", decl)
                if mt:
                    fields.append((mt.group(1), mt.group(2)))
        out[m.group(1)] = fields
    return out


PAIRS = {"IterationControl": "nk_iteration_control", "GridDesc": "nk_grid_desc", "PhysicsDesc": "nk_physics_desc",
         "SolverDesc": "nk_solver_desc", "SolveStats": "nk_solve_stats", "AdvectionDesc": "nk_advection_desc",
         "CostState": "nk_cost_state", "TimeGradientDesc": "nk_time_gradient_desc", "TimeGradient": "nk_time_gradient",
         "TimeGradientStats": "nk_time_gradient_stats"}


def test_descriptor_mirrors_match_the_header():
    c, j = c_structs(), julia_structs()
    for jl, cn in PAIRS.items():
        want = [(n, "IterationControl" if t == "nk_iteration_control" else t) for n, t in c[cn]]
        assert j[jl] == want, (jl, j[jl], want)


def test_every_ccall_is_declared():
    header = open(HEADER).read()
    declared = set(re.findall(r"\b(nk_\w+)\s*\(", header))
    called = set(re.findall(r"ccall\(\(:(nk_\w+), libnk\)", open(JULIA).read()))
    assert called and called <= declared, called - declared
    # the drop-in covers the entry points of the boundary's Julia-side methods
    for name in ("nk_problem_create", "nk_picard_solve", "nk_linear_solve", "nk_adjoint_solve", "nk_precondition",
                 "nk_picard_adjoint", "nk_problem_set_field_parent", "nk_problem_get_field_parent",
                 "nk_checkpointed_gradient"):
        assert name in called, name


def test_field_ids_match_the_header():
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    ids = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+NK_FIELD_(\w+)\s+(\d+)", text)}
    jl = open(JULIA).read()
    table = re.search(r"const FIELD = \((.*?)\)\n", jl, flags=re.S).group(1)
    got = {k.strip(): int(v) for k, v in re.findall(r"(\S+?) = (\d+)", table)}
    names = {"u": "U", "v": "V", "H": "H", "bed": "BED", "s": "SURFACE", "ice_mask": "ICE_MASK", "φ": "PHI",
             "φᵘ": "PHI_U", "φᵛ": "PHI_V", "N": "EFFECTIVE_PRESSURE", "τᵘ": "TAU_U", "τᵛ": "TAU_V", "A": "RATE_FACTOR",
             "C": "FRICTION_COEFFICIENT", "η̄H": "ETA_H", "η̄Hᶠᶠ": "ETA_H_FF", "βᵘ": "BETA_U", "βᵛ": "BETA_V",
             "ησ": "ETA_SIGMA", "F₂": "F2", "βᵇᵘ": "BETA_B_U", "βᵇᵛ": "BETA_B_V", "uᵇ": "U_B", "vᵇ": "V_B",
             "uσ": "U_SIGMA", "vσ": "V_SIGMA", "T": "TEMPERATURE", "a": "SURFACE_MASS_BALANCE", "m": "BASAL_MELT_RATE"}
    assert set(got) == set(names)
    for k, v in got.items():
        assert ids[names[k]] == v, (k, v, ids[names[k]])
