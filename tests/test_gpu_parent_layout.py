"""Field copies with Oceananigans parent arrays (nk_problem_set_field_parent / nk_problem_get_field_parent).

The Julia call site holds fields as halo-padded parent arrays (x fastest, then y, then the sigma level with a
z halo of 1, src/Grids/sigma_grid.jl:57).  Setting from a parent must equal setting the interior, whatever the
halos hold (NaN here, so a halo read would show); getting into a parent must write the interior and leave every
halo value as it was.  Checked for Center-Center, Face-Center (Bounded and Periodic x), Center-Face and sigma
fields, on host and device parents, and for the prescribed-velocity field."""
import ctypes as C

import numpy as np
import pytest

from nunatak_gb300 import model as M, workloads

pytestmark = pytest.mark.gpu


def _pad(a, halo, fill=np.nan):
    hx, hy, hz = (tuple(halo) + (0,))[:3]
    if a.ndim == 2:
        return np.pad(a, ((hy, hy), (hx, hx)), constant_values=fill)
    return np.pad(a, ((hz, hz), (hy, hy), (hx, hx)), constant_values=fill)


def _interior(p, halo, ndim):
    hx, hy, hz = (tuple(halo) + (0,))[:3]
    if ndim == 2:
        return p[hy:p.shape[0] - hy, hx:p.shape[1] - hx]
    return p[hz:p.shape[0] - hz, hy:p.shape[1] - hy, hx:p.shape[2] - hx]


@pytest.mark.parametrize("topology", [("Bounded", "Bounded"), ("Periodic", "Bounded")])
def test_set_and_get_through_parent_arrays(gpu_cls, topology):
    base = workloads.diva_sheet(24, 12, dx=32e3, Nsigma=4)
    grid = M.RectilinearGrid(size=(24, 12), x=base.grid.x, y=base.grid.y, halo=(4, 4), topology=topology)
    P = workloads.Case("parent", grid, base.config, base.fields, temperature=base.temperature).problem(gpu_cls)
    rng = np.random.default_rng(3)
    for name, halo in (("H", (4, 4)), ("u", (4, 4)), ("v", (3, 2)), ("C", (0, 0)), ("A", (4, 4, 1)), ("eta_sigma", (2, 3, 1))):
        a = rng.random(P.shape(name)) + 1.0
        P.set_parent(name, _pad(a, halo), halo)
        assert np.array_equal(P.get(name), a), name
        out = _pad(np.zeros_like(a), halo, fill=-7.0)
        P.get_parent(name, out, halo)
        assert np.array_equal(_interior(out, halo, a.ndim), a), name
        inner = np.zeros(out.shape, bool)
        _interior(inner, halo, a.ndim)[...] = True
        assert np.all(out[~inner] == -7.0), name


def test_parent_arrays_in_device_memory_and_prescribed_field(gpu_cls):
    torch = pytest.importorskip("torch")
    P = workloads.channel_shelf().problem(gpu_cls)
    halo = (4, 4)
    ud = np.full(P.shape("u_prescribed"), np.nan)
    ud[:, 0] = 100.0 / M.YEAR
    t = torch.from_numpy(_pad(ud, halo, fill=5.0)).cuda()
    ptr = C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    assert P._fn("problem_set_field_parent")(P._h, 27, ptr, 4, 4, 0, t.numel()) == 0
    got = P.get("u_prescribed")
    assert np.array_equal(np.isnan(got), np.isnan(ud)) and np.array_equal(got[:, 0], ud[:, 0])
    assert np.all(P.get("tau_u")[:, 0] == 100.0 / M.YEAR)
    with pytest.raises(ValueError):
        P.set_parent("H", np.zeros((3, 3)), halo)
