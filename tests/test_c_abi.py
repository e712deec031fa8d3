"""The C ABI from a plain C caller (tests/c_abi_client.c): the header compiles as C11 and the client links against
libnunatak_gb300.so on any machine; on a GPU the client's picard_solve! of the channel shelf equals the Python
binding's solve of the same inputs bit for bit (the same library and arithmetic)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _compile(tmp_path):
    import __graft_entry__ as g
    g.build()
    from nunatak_gb300 import library
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "c_abi_client")
    lib = library.LIB_PATH
    cmd = [cc, "-std=c11", "-O2", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c_abi_client.c"), lib, "-Wl,-rpath," + os.path.dirname(lib), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_is_c_and_the_client_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_c_client_solve_equals_python_solve(tmp_path, gpu_cls):
    from nunatak_gb300 import model as M, workloads
    exe = _compile(tmp_path)
    solver = M.StressBalanceSolver(linear_iteration_control=M.Convergence(reltol=1e-10, maxiter=10_000),
                                   picard_iteration_control=M.Convergence(reltol=1e-6, maxiter=100),
                                   preconditioner=M.StressBalanceDiagonalPreconditioner())
    case = workloads.channel_shelf(velocity_solver=solver)
    desc = case.descriptors()
    for name, s in (("grid", desc.grid), ("physics", desc.physics), ("solver", desc.solver)):
        (tmp_path / f"{name}.bin").write_bytes(bytes(s))
    for name in ("H", "bed", "A"):
        (tmp_path / f"{name}.bin").write_bytes(np.ascontiguousarray(case.fields[name], dtype=np.float64).tobytes())
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    P = case.problem(gpu_cls)
    st = P.picard_solve()
    assert f"picard_iterations {st.picard_iterations} " in r.stdout
    u = np.frombuffer((tmp_path / "u.bin").read_bytes(), dtype=np.float64).reshape(P.shape("u"))
    v = np.frombuffer((tmp_path / "v.bin").read_bytes(), dtype=np.float64).reshape(P.shape("v"))
    assert np.array_equal(u, P.get("u")) and np.array_equal(v, P.get("v"))
