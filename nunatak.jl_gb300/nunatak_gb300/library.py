"""Loader of libnunatak_gb300.so (built in-tree by nunatak.jl_gb300/build.py) and the device context.

There is no CPU fallback: if the shared library is missing or no CUDA device is present, loading
raises.  Every solve in this package runs in the library's CUDA kernels."""
import ctypes as C
import os

from . import abi

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libnunatak_gb300.so")

_LIB = None
_CTX = None


def _declare(lib):
    vp, i32, i64, dp = C.c_void_p, C.c_int32, C.c_int64, C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int32)
    sig = {
        "nk_api_version": ([], i32),
        "nk_launch_count": ([], i64),
        "nk_context_create": ([i32, C.POINTER(vp)], i32),
        "nk_context_destroy": ([vp], i32),
        "nk_last_error": ([vp], C.c_char_p),
        "nk_problem_create": ([vp, C.POINTER(abi.GridDesc), C.POINTER(abi.PhysicsDesc), C.POINTER(abi.SolverDesc), C.POINTER(vp)], i32),
        "nk_problem_destroy": ([vp], i32),
        "nk_problem_set_field": ([vp, i32, dp, i64], i32),
        "nk_problem_get_field": ([vp, i32, dp, i64], i32),
        "nk_problem_field_size": ([vp, i32], i64),
        "nk_problem_set_field_parent": ([vp, i32, dp, i32, i32, i32, i64], i32),
        "nk_problem_get_field_parent": ([vp, i32, dp, i32, i32, i32, i64], i32),
        "nk_compute_geometry": ([vp], i32),
        "nk_compute_rate_factor": ([vp] + [C.c_double] * 9, i32),
        "nk_compute_thermal_diagnostics": ([vp, C.POINTER(abi.ThermalParams)], i32),
        "nk_step_thickness": ([vp, C.c_double, i32], i32),
        "nk_step_thickness_stage": ([vp, C.c_double, i32, i32], i32),
        "nk_set_thickness_advection": ([vp, C.POINTER(abi.AdvectionDesc)], i32),
        "nk_set_front": ([vp, C.POINTER(abi.FrontDesc)], i32),
        "nk_set_till": ([vp, C.POINTER(abi.TillDesc)], i32),
        "nk_initialize_front": ([vp], i32),
        "nk_advance_front": ([vp, C.c_double], i32),
        "nk_step_enthalpy": ([vp, C.POINTER(abi.EnergyParams), C.c_double], i32),
        "nk_update_coefficients": ([vp], i32),
        "nk_apply_operator": ([vp, dp, dp, dp, dp], i32),
        "nk_precondition": ([vp, dp, dp, dp, dp], i32),
        "nk_linear_solve": ([vp, dp, dp, C.POINTER(abi.SolveStats)], i32),
        "nk_adjoint_solve": ([vp, dp, dp, C.POINTER(abi.SolveStats)], i32),
        "nk_picard_solve": ([vp, C.POINTER(abi.SolveStats)], i32),
        "nk_picard_solve_async": ([vp], i32),
        "nk_problem_wait": ([vp, C.POINTER(abi.SolveStats)], i32),
        "nk_problem_query": ([vp, ip], i32),
        "nk_picard_adjoint": ([vp, dp, dp, C.POINTER(abi.IterationControl), dp, dp, dp, dp, C.POINTER(abi.SolveStats)], i32),
        "nk_picard_adjoint_gradients": ([vp, dp, dp, C.POINTER(abi.IterationControl), dp, dp, dp, dp, dp, C.POINTER(abi.SolveStats)], i32),
        "nk_solve_velocities": ([vp, dp, dp, C.POINTER(abi.SolveStats)], i32),
        "nk_velocity_profile": ([vp], i32),
        "nk_multigrid_levels": ([vp, ip, ip, ip, i32], i32),
        "nk_multigrid_restrict": ([vp, i32, dp, dp, dp, dp], i32),
        "nk_time_kernel": ([vp, i32, i32, i64, dp, dp], i32),
        "nk_server_create": ([vp, C.POINTER(abi.ServerDesc), C.POINTER(vp)], i32),
        "nk_server_destroy": ([vp], i32),
        "nk_server_submit": ([vp, C.POINTER(abi.Request), C.POINTER(i64)], i32),
        "nk_server_progress": ([vp, ip], i32),
        "nk_server_wait": ([vp, i64, C.POINTER(abi.SolveStats), dp, dp, dp], i32),
        "nk_server_wait_all": ([vp], i32),
        "nk_server_clock": ([vp], C.c_double),
        "nk_server_info": ([vp, ip, C.POINTER(i64), ip], i32),
        "nk_multigrid_prolongate": ([vp, i32, dp, dp, dp, dp], i32),
        "nk_batch_create": ([vp, C.POINTER(abi.GridDesc), C.POINTER(abi.PhysicsDesc), C.POINTER(abi.SolverDesc), i32, C.POINTER(vp)], i32),
        "nk_batch_destroy": ([vp], i32),
        "nk_batch_slots": ([vp], i32),
        "nk_batch_problem": ([vp, i32], vp),
        "nk_batch_picard_solve_async": ([vp, C.POINTER(C.c_uint8)], i32),
        "nk_batch_query": ([vp, ip], i32),
        "nk_batch_wait": ([vp, C.POINTER(abi.SolveStats)], i32),
        "nk_checkpointed_gradient": ([vp, C.POINTER(abi.TimeGradientDesc), abi.COST_FN, vp, C.POINTER(abi.TimeGradient),
                                      C.POINTER(abi.TimeGradientStats)], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


def load():
    """Load the CUDA library; raises OSError when it has not been built."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"libnunatak_gb300.so not built at {LIB_PATH}: run nunatak.jl_gb300/build.py "
                          "(there is no CPU fallback)")
        _LIB = _declare(C.CDLL(LIB_PATH))
        if _LIB.nk_api_version() != abi.NK_API_VERSION:
            raise OSError("libnunatak_gb300.so API version mismatch")
    return _LIB


class Context:
    """nk_context on one CUDA device."""

    def __init__(self, device=0):
        self.lib = load()
        self.handle = C.c_void_p()
        st = self.lib.nk_context_create(device, C.byref(self.handle))
        if st != abi.NK_OK:
            raise RuntimeError(f"nk_context_create(device={device}) failed: {abi.STATUS_NAMES.get(st, st)}")

    def last_error(self):
        msg = self.lib.nk_last_error(self.handle)
        return msg.decode() if msg else ""

    def close(self):
        if self.handle:
            self.lib.nk_context_destroy(self.handle)
            self.handle = C.c_void_p()


def default_context():
    global _CTX
    if _CTX is None:
        _CTX = Context(0)
    return _CTX


def launch_count():
    """Kernels launched by libnunatak_gb300 in this process so far."""
    return int(load().nk_launch_count())
