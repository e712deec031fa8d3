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


LAYOUT_PROGRAM = r"""
#include <stddef.h>
#include <stdio.h>
#include "nunatak_gb300.h"
#define F(T, m) printf("%s.%s %zu %zu\n", #T, #m, offsetof(T, m), sizeof(((T*)0)->m));
#define S(T) printf("%s %zu\n", #T, sizeof(T));
int main(void) {
    S(nk_iteration_control) F(nk_iteration_control, kind) F(nk_iteration_control, reltol) F(nk_iteration_control, abstol)
    S(nk_grid_desc) F(nk_grid_desc, Nsigma) F(nk_grid_desc, x_faces) F(nk_grid_desc, x0) F(nk_grid_desc, sigma_faces)
    F(nk_grid_desc, bed_refinement)
    S(nk_physics_desc) F(nk_physics_desc, glen_exponent) F(nk_physics_desc, use_ice_mask) F(nk_physics_desc, mask_transition_thickness)
    S(nk_solver_desc) F(nk_solver_desc, linear) F(nk_solver_desc, picard)
    S(nk_solve_stats) F(nk_solve_stats, residual_norm) F(nk_solve_stats, device_end_ms)
    S(nk_server_desc) F(nk_server_desc, flags) F(nk_server_desc, memory_cap_bytes)
    S(nk_request) F(nk_request, physics) F(nk_request, solver) F(nk_request, H) F(nk_request, v_out)
    S(nk_thermal_params) F(nk_thermal_params, water_softening_coefficient) F(nk_thermal_params, reference_temperature)
    S(nk_energy_params) F(nk_energy_params, maximum_drainage_rate) F(nk_energy_params, grounded_melt_coupling) F(nk_energy_params, reserved)
    S(nk_cost_state) F(nk_cost_state, H) F(nk_cost_state, ice_mask)
    S(nk_time_gradient_desc) F(nk_time_gradient_desc, steps) F(nk_time_gradient_desc, melt_weights) F(nk_time_gradient_desc, adjoint_control)
    S(nk_time_gradient) F(nk_time_gradient, grad_log_A)
    S(nk_time_gradient_stats) F(nk_time_gradient_stats, worst_solve_status) F(nk_time_gradient_stats, elapsed_ms)
    S(nk_till_desc) F(nk_till_desc, reference_effective_pressure) F(nk_till_desc, drainage_rate)
    S(nk_front_desc) F(nk_front_desc, calving) F(nk_front_desc, front_velocity)
    return 0;
}
"""


def test_ctypes_mirrors_match_the_c_layout(tmp_path):
    """Sizes and field offsets of every descriptor, as the C compiler lays them out, against the ctypes mirrors."""
    import ctypes
    from nunatak_gb300 import abi
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "layout.c"
    src.write_text(LAYOUT_PROGRAM)
    exe = str(tmp_path / "layout")
    r = subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split("\n")
    mirrors = {"nk_iteration_control": abi.IterationControl, "nk_grid_desc": abi.GridDesc, "nk_physics_desc": abi.PhysicsDesc,
               "nk_solver_desc": abi.SolverDesc, "nk_solve_stats": abi.SolveStats, "nk_server_desc": abi.ServerDesc,
               "nk_request": abi.Request, "nk_thermal_params": abi.ThermalParams,
               "nk_energy_params": abi.EnergyParams, "nk_cost_state": abi.CostState, "nk_time_gradient_desc": abi.TimeGradientDesc,
               "nk_time_gradient": abi.TimeGradient, "nk_time_gradient_stats": abi.TimeGradientStats,
               "nk_till_desc": abi.TillDesc, "nk_front_desc": abi.FrontDesc}
    checked = 0
    for line in filter(None, out):
        parts = line.split()
        if "." in parts[0]:
            struct, field = parts[0].split(".")
            off, size = int(parts[1]), int(parts[2])
            m = getattr(mirrors[struct], field)
            assert (m.offset, m.size) == (off, size), (struct, field, m.offset, m.size, off, size)
        else:
            assert ctypes.sizeof(mirrors[parts[0]]) == int(parts[1]), parts
        checked += 1
    assert checked == 53
