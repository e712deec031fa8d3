"""Error behaviour of the C ABI: invalid arguments are refused with NK_BAD_ARGUMENT and a message (no kernel
runs), and the problem stays usable afterwards.  All checks are host-side validations."""
import ctypes as C

import numpy as np
import pytest

import nunatak_gb300 as nk
from nunatak_gb300 import abi, library, model as M, workloads

pytestmark = pytest.mark.gpu


def test_empty_grid_is_refused():
    g = M.RectilinearGrid(size=(4, 4), x=(0.0, 1.0), y=(0.0, 1.0), halo=(3, 3))
    desc = workloads.marine_sheet(8, 4).descriptors()
    desc.grid.Nx = 0
    h = C.c_void_p()
    lib = library.load()
    ctx = library.default_context()
    st = lib.nk_problem_create(ctx.handle, C.byref(desc.grid), C.byref(desc.physics), C.byref(desc.solver), C.byref(h))
    assert st == abi.NK_BAD_ARGUMENT
    assert "grid size" in ctx.last_error()


def test_field_size_mismatch_and_unknown_field_are_refused():
    P = workloads.marine_sheet(16, 8).problem(nk.Problem)
    lib = library.load()
    H = np.ones(16 * 8 + 1)
    ptr = H.ctypes.data_as(C.POINTER(C.c_double))
    assert lib.nk_problem_set_field(P._h, abi.FIELD_IDS["H"], ptr, H.size) == abi.NK_BAD_ARGUMENT
    assert "size mismatch" in P._err()
    assert lib.nk_problem_set_field(P._h, 999, ptr, 16 * 8) == abi.NK_BAD_ARGUMENT
    assert "unknown field" in P._err()
    P.picard_solve()                                   # still usable
    assert np.all(np.isfinite(P.get("u")))


def test_wait_without_a_pending_solve_is_refused():
    P = workloads.marine_sheet(16, 8).problem(nk.Problem)
    with pytest.raises(ValueError, match="no asynchronous solve pending"):
        P.wait()


def test_picard_adjoint_refuses_prescribed_velocities():
    P = workloads.channel_shelf(inflow=100.0).problem(nk.Problem)
    P.picard_solve()
    u, v = P.get("u"), P.get("v")
    with pytest.raises(ValueError, match="prescribed velocities"):
        P.picard_adjoint(np.zeros_like(u), np.zeros_like(v))


def test_picard_adjoint_of_zero_misfit_is_zero():
    """DIVA: x̄ = 0 gives λ = 0 and zero gradients (the lagged-state sweep adds nothing from nothing)."""
    P = workloads.diva_sheet(32, 16, precision="fp64").problem(nk.Problem)
    P.picard_solve()
    u, v = P.get("u"), P.get("v")
    lu, lv, grad, grad_a, st = P.picard_adjoint(np.zeros_like(u), np.zeros_like(v))
    assert st.status == 0
    assert not lu.any() and not lv.any() and not grad.any() and not grad_a.any()
