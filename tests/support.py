"""Test helpers: build the reference's test scenarios on a backend (the CPU oracle or the GPU library).

`cls` is nunatak_oracle.OracleProblem or nunatak_gb300.Problem; both take (grid, descriptors) and offer
the same methods, so every scenario runs unchanged on either."""
import numpy as np

from nunatak_gb300 import model as M
from nunatak_gb300.abi import FIELD_LOCATIONS


def coords(grid, d, loc):
    """Node coordinates along direction d of a field located at loc ('c' or 'f'), interior points only."""
    if loc == "c":
        return grid.centers(d)
    f = grid.faces(d)
    return f[:-1] if grid.periodic(d) else f


def evaluate(grid, name, f, Nsigma=None):
    """f(x, y) (or a number) evaluated at the interior points of field `name`, shape (ny, nx)."""
    lx, ly, _ = FIELD_LOCATIONS[name]
    x = coords(grid, 0, lx)
    y = coords(grid, 1, ly)
    if callable(f):
        X, Y = np.meshgrid(x, y)
        return np.asarray(np.vectorize(f)(X, Y), dtype=np.float64)
    return np.full((y.size, x.size), float(f))


def make(cls, grid, advection=None, **kw):
    """A problem of class `cls`; `advection` (an UpwindBiased or a WENO) sets its thickness advection scheme, which is
    otherwise the reference's default WENO(order = 5, bounds = (0, 1e5))."""
    P = cls(grid, M.make_descriptors(grid, **kw))
    if advection is not None:
        P.set_thickness_advection(advection)
    return P


def set_fn(P, name, f):
    P.set(name, evaluate(P.grid, name, f))


def vector_dot(grid, au, av, bu, bv):
    """Dot product over the Nx x Ny range of each component (vector_dot!, src/Solvers/velocity_vector.jl:125-133)."""
    Nx, Ny = grid.Nx, grid.Ny
    return float(np.sum(au[:Ny, :Nx] * bu[:Ny, :Nx]) + np.sum(av[:Ny, :Nx] * bv[:Ny, :Nx]))


def ice_sheet_model(cls, grid, H, bed=0.0, u=None, v=None, rheology=None, friction=None, grounding=None,
                    masking="default", stress_balance=None, velocity_solver=None, Nsigma=10, constants=None,
                    solve=True):
    """IceSheetModel(grid; ...) followed by set!(model; H, u, v) (src/Models/ice_sheet_model.jl:79-120,
    src/Models/ice_sheet_model_methods.jl:11-20): geometry, driving stress, Picard solve, profile."""
    rheology = rheology or M.GlenFlowLaw(rate_factor=1e-24)
    P = make(cls, grid, Nsigma=Nsigma, stress_balance=stress_balance, rheology=rheology, friction=friction,
             grounding=grounding, masking=masking, constants=constants, velocity_solver=velocity_solver)
    set_fn(P, "H", H)
    set_fn(P, "bed", bed)
    A = rheology.rate_factor
    P.set("A", A if isinstance(A, np.ndarray) else (A if not callable(A) else evaluate(grid, "H", A)))
    if friction is not None:
        Cc = friction.coefficient
        P.set("C", evaluate(grid, "C", Cc) if callable(Cc) else Cc)
    P.compute_geometry()
    if u is not None:
        set_fn(P, "u", u)
    if v is not None:
        set_fn(P, "v", v)
    stats = P.picard_solve() if solve else None
    if solve:
        P.velocity_profile()
    return P, stats


def isapprox(a, b, rtol=1.4901161193847656e-08, atol=0.0):
    """Julia's isapprox for arrays: norm(a - b) <= max(atol, rtol * max(norm(a), norm(b)))."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    d = np.linalg.norm((a - b).ravel())
    return d <= max(atol, rtol * max(np.linalg.norm(a.ravel()), np.linalg.norm(b.ravel())))


# ---- the reference's doctests as golden values (tests/golden/reference_doctests.json) -------------------------

_DOCTESTS = None


def reference_doctests():
    """Every doctest block of the reference's velocity-solve sources, as extracted from its text by
    tests/golden/make_reference_doctests.py: [{"file", "lines": [first, last], "steps": [{"input", "output"}]}]."""
    global _DOCTESTS
    if _DOCTESTS is None:
        import json
        import os
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_doctests.json")
        with open(path, encoding="utf-8") as f:
            _DOCTESTS = json.load(f)["doctests"]
    return _DOCTESTS


def reference_doctest(file, first_line):
    """The printed outputs, in order, of the doctest whose opening fence is at file:first_line."""
    for d in reference_doctests():
        if d["file"] == file and d["lines"][0] == first_line:
            return [s["output"] for s in d["steps"] if s["output"]]
    raise KeyError(f"no doctest at {file}:{first_line}")


def julia_value(text):
    """A value as Julia prints it: a number, a tuple (nested tuples of numbers) or an `n-element Vector{T}:`
    listing, as Python floats, tuples and lists."""
    import ast
    text = text.strip()
    if "-element Vector" in text:
        return [float(line) for line in text.split("\n")[1:]]
    value = ast.literal_eval(text)
    if isinstance(value, tuple):
        return tuple(julia_value(repr(v)) if isinstance(v, tuple) else float(v) for v in value)
    return float(value)
