"""nk_picard_change_noalloc, the velocity-change measure for callers that cannot allocate device memory.

Such callers are a model whose framework already pools the whole device, where another cudaMalloc fails,
and a coupled time loop that cannot take the device synchronisation of a cudaFree.  The entry point works
in a fixed scratch array inside the library.  Here it is called through the C ABI on device buffers. Two
calls in a row must give the picard_change and picard_norm that nk_picard_solve reports for the same two
velocity iterates.  The first call uses a larger grid, so the second one runs over scratch that still holds
the first call's block sums.  Sizes beyond the scratch must be refused with a message."""
import ctypes as C

import numpy as np
import pytest

import nunatak_gb300
from nunatak_gb300 import abi, library, model as M, workloads

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _entry():
    lib = library.load()
    f = lib.nk_picard_change_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(abi.GridDesc)] + [C.c_void_p] * 6
    f.restype = C.c_int32
    return f


def _solver():
    return M.StressBalanceSolver(linear_iteration_control=M.FixedIterations(40),
                                 picard_iteration_control=M.FixedIterations(1),
                                 preconditioner=M.StressBalanceDiagonalPreconditioner())


def _two_iterates(case):
    """Velocities before and after one Picard iteration, and that iteration's stats."""
    P = case.problem(nunatak_gb300.Problem)
    P.picard_solve()
    u_prev, v_prev = P.get("u"), P.get("v")
    stats = P.picard_solve()
    u, v = P.get("u"), P.get("v")
    grid_desc = case.descriptors().grid
    P.close()
    return grid_desc, (u, v, u_prev, v_prev), (stats.picard_change, stats.picard_norm)


def _periodic_x(Nx, Ny):
    base = workloads.marine_sheet(Nx, Ny, seed=5, velocity_solver=_solver())
    grid = M.RectilinearGrid(size=(Nx, Ny), x=(0.0, 512e3), y=(0.0, 256e3), halo=(4, 4),
                             topology=("Periodic", "Bounded"))
    return workloads.Case("marine_sheet_periodic_x", grid, base.config, base.fields)


def _call(f, grid_desc, arrays, out, stream):
    import torch
    dev = [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]
    st = f(library.default_context().handle, C.byref(grid_desc), *[d.data_ptr() for d in dev], out.data_ptr(), stream)
    return st, dev   # keep the inputs alive until the stream has run the kernel


def test_noalloc_change_matches_picard_solve_twice_in_a_row():
    import torch
    f = _entry()
    bounded = _two_iterates(workloads.marine_sheet(96, 48, seed=3, velocity_solver=_solver()))
    periodic = _two_iterates(_periodic_x(64, 24))
    stream = torch.cuda.current_stream().cuda_stream
    outs = [torch.full((2,), float("nan"), dtype=torch.float64, device="cuda") for _ in range(2)]
    keep = []
    for (grid_desc, arrays, _), out in zip((bounded, periodic), outs):
        st, dev = _call(f, grid_desc, arrays, out, stream)
        assert st == abi.NK_OK, library.default_context().last_error()
        keep.append(dev)
    torch.cuda.synchronize()
    for (_, _, expected), out in zip((bounded, periodic), outs):
        got = out.cpu().numpy()
        assert expected[0] > 0 and expected[1] > 0
        np.testing.assert_allclose(got, np.array(expected), rtol=RTOL, atol=0)


def test_noalloc_change_at_the_maximum_size():
    """2048 x 2048 cells fill the scratch exactly (16384 blocks); checked against a float64 numpy norm."""
    import torch
    f = _entry()
    Nx = Ny = 2048
    grid_desc = abi.GridDesc(Nx=Nx, Ny=Ny, topology_x=abi.NK_BOUNDED, topology_y=abi.NK_BOUNDED)
    rng = np.random.default_rng(11)
    u, u_prev = rng.standard_normal((2, Ny, Nx + 1))
    v, v_prev = rng.standard_normal((2, Ny + 1, Nx))
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    st, keep = _call(f, grid_desc, (u, v, u_prev, v_prev), out, torch.cuda.current_stream().cuda_stream)
    assert st == abi.NK_OK, library.default_context().last_error()
    torch.cuda.synchronize()
    du, dv = (u_prev - u)[:, :Nx], (v_prev - v)[:Ny, :]
    expected = [np.sqrt(np.sum(du * du) + np.sum(dv * dv)),
                np.sqrt(np.sum(u[:, :Nx] ** 2) + np.sum(v[:Ny, :] ** 2))]
    np.testing.assert_allclose(out.cpu().numpy(), expected, rtol=RTOL, atol=0)


def test_noalloc_refuses_grids_beyond_the_scratch():
    import torch
    f = _entry()
    grid_desc = abi.GridDesc(Nx=2048, Ny=2056, topology_x=abi.NK_BOUNDED, topology_y=abi.NK_BOUNDED)
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    small = torch.zeros(8, dtype=torch.float64, device="cuda")
    st = f(library.default_context().handle, C.byref(grid_desc), *[small.data_ptr()] * 4, out.data_ptr(),
           torch.cuda.current_stream().cuda_stream)
    assert st == abi.NK_BAD_ARGUMENT
    msg = library.default_context().last_error()
    assert "16448" in msg and "16384" in msg
