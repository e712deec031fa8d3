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


def make(cls, grid, **kw):
    return cls(grid, M.make_descriptors(grid, **kw))


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
