"""The C ABI on a machine without a CUDA device: no CPU fallback, and no crash.

- nk_context_create reports NK_CUDA_ERROR and writes no handle; the Python layer raises instead of solving
  anywhere else (so a product path without the GPU library fails loudly).
- Every entry point that takes a handle refuses a NULL one with NK_BAD_ARGUMENT before any CUDA call (the
  destroy functions accept NULL as a no-op, like free), and the query helpers return their neutral values.
These run only where no device is visible; on a GPU machine they are skipped."""
import ctypes as C

import pytest

from nunatak_gb300 import abi


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    from nunatak_gb300 import library
    L = library.load()
    h = C.c_void_p()
    if L.nk_context_create(0, C.byref(h)) == abi.NK_OK:
        L.nk_context_destroy(h)
        pytest.skip("a CUDA device is present")
    return L


def test_context_creation_fails_without_a_device(lib):
    h = C.c_void_p()
    assert lib.nk_context_create(0, C.byref(h)) == abi.NK_CUDA_ERROR
    assert not h.value
    assert lib.nk_context_create(0, None) == abi.NK_BAD_ARGUMENT
    assert lib.nk_last_error(None) == b"no context"


def test_python_layer_raises_without_a_device(lib):
    from nunatak_gb300 import library, model as M
    import nunatak_gb300
    with pytest.raises(RuntimeError, match="nk_context_create"):
        library.Context(0)
    g = M.RectilinearGrid(size=(4, 4), x=(0.0, 1.0), y=(0.0, 1.0))
    with pytest.raises(RuntimeError):
        nunatak_gb300.Problem(g, M.make_descriptors(g))


def test_null_handles_are_refused(lib):
    null, d = None, C.cast(None, C.POINTER(C.c_double))
    i32 = C.c_int32()
    bad = abi.NK_BAD_ARGUMENT
    calls = {
        "nk_problem_create": lambda: lib.nk_problem_create(null, null, null, null, null),
        "nk_problem_set_field": lambda: lib.nk_problem_set_field(null, 0, d, 0),
        "nk_problem_get_field": lambda: lib.nk_problem_get_field(null, 0, d, 0),
        "nk_problem_set_field_parent": lambda: lib.nk_problem_set_field_parent(null, 0, d, 0, 0, 0, 0),
        "nk_problem_get_field_parent": lambda: lib.nk_problem_get_field_parent(null, 0, d, 0, 0, 0, 0),
        "nk_compute_geometry": lambda: lib.nk_compute_geometry(null),
        "nk_compute_rate_factor": lambda: lib.nk_compute_rate_factor(null, *([0.0] * 9)),
        "nk_compute_thermal_diagnostics": lambda: lib.nk_compute_thermal_diagnostics(null, null),
        "nk_step_thickness": lambda: lib.nk_step_thickness(null, 1.0, 0),
        "nk_step_enthalpy": lambda: lib.nk_step_enthalpy(null, null, 1.0),
        "nk_update_coefficients": lambda: lib.nk_update_coefficients(null),
        "nk_apply_operator": lambda: lib.nk_apply_operator(null, d, d, d, d),
        "nk_precondition": lambda: lib.nk_precondition(null, d, d, d, d),
        "nk_linear_solve": lambda: lib.nk_linear_solve(null, d, d, null),
        "nk_adjoint_solve": lambda: lib.nk_adjoint_solve(null, d, d, null),
        "nk_picard_solve": lambda: lib.nk_picard_solve(null, null),
        "nk_picard_solve_async": lambda: lib.nk_picard_solve_async(null),
        "nk_picard_adjoint": lambda: lib.nk_picard_adjoint(null, d, d, null, d, d, d, d, null),
        "nk_picard_adjoint_gradients": lambda: lib.nk_picard_adjoint_gradients(null, d, d, null, d, d, d, d, d, null),
        "nk_problem_query": lambda: lib.nk_problem_query(null, C.byref(i32)),
        "nk_problem_wait": lambda: lib.nk_problem_wait(null, null),
        "nk_solve_velocities": lambda: lib.nk_solve_velocities(null, d, d, null),
        "nk_velocity_profile": lambda: lib.nk_velocity_profile(null),
        "nk_multigrid_levels": lambda: lib.nk_multigrid_levels(null, C.byref(i32), None, None, 0),
        "nk_multigrid_restrict": lambda: lib.nk_multigrid_restrict(null, 0, d, d, d, d),
        "nk_multigrid_prolongate": lambda: lib.nk_multigrid_prolongate(null, 0, d, d, d, d),
        "nk_time_kernel": lambda: lib.nk_time_kernel(null, 0, 1, 0, d, d),
        "nk_server_create": lambda: lib.nk_server_create(null, null, null),
        "nk_server_submit": lambda: lib.nk_server_submit(null, null, null),
        "nk_server_progress": lambda: lib.nk_server_progress(null, None),
        "nk_server_wait": lambda: lib.nk_server_wait(null, 0, null, d, d, d),
        "nk_server_wait_all": lambda: lib.nk_server_wait_all(null),
        "nk_server_info": lambda: lib.nk_server_info(null, None, None, None),
        "nk_picard_change_noalloc": lambda: lib.nk_picard_change_noalloc(null, null, null, null, null, null, null, null),
        "nk_batch_create": lambda: lib.nk_batch_create(null, null, null, null, 2, null),
        "nk_batch_picard_solve_async": lambda: lib.nk_batch_picard_solve_async(null, None),
        "nk_batch_query": lambda: lib.nk_batch_query(null, C.byref(i32)),
        "nk_batch_wait": lambda: lib.nk_batch_wait(null, null),
        "nk_checkpointed_gradient": lambda: lib.nk_checkpointed_gradient(null, null, abi.COST_FN(), null, null, null),
        "nk_set_till": lambda: lib.nk_set_till(null, C.byref(abi.TillDesc())),
        "nk_set_front": lambda: lib.nk_set_front(null, C.byref(abi.FrontDesc())),
    }
    got = {name: f() for name, f in calls.items()}
    assert got == {name: bad for name in calls}
    assert lib.nk_problem_destroy(null) == abi.NK_OK
    assert lib.nk_server_destroy(null) == abi.NK_OK
    assert lib.nk_context_destroy(null) == abi.NK_OK
    assert lib.nk_problem_field_size(null, 0) == 0
    assert lib.nk_server_clock(null) == 0.0
    assert lib.nk_batch_destroy(null) == abi.NK_OK
    assert lib.nk_batch_slots(null) == 0
    assert lib.nk_batch_problem(null, 0) is None
