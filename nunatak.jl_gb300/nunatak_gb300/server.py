"""Serving: many independent velocity solves through the library's request loop (nk_server_*).

Each request is one workloads.Case (grid, configuration and input fields H, bed, C, A); the server keeps
solved problems resident on the GPU, reuses one for the next request of the same shape, and runs up to
`max_in_flight` requests at once on separate streams."""
import ctypes as C

import numpy as np

from . import abi, library
from .problem import _check

_dptr = C.POINTER(C.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dptr) if a is not None else None


class Server:
    def __init__(self, max_in_flight=16, memory_cap_bytes=16 << 30, context=None, admission_thread=False, batch_slots=0):
        """`admission_thread`: the library's own host thread admits and retires requests (NK_SERVER_ADMISSION_THREAD);
        otherwise submit / progress / wait drive the loop.  `batch_slots` > 1: queued requests of one shape are
        solved together, up to batch_slots per solve, by one batched graph (nk_batch)."""
        self.ctx = context or library.default_context()
        self.lib = library.load()
        self.h = C.c_void_p()
        d = abi.ServerDesc(max_in_flight, abi.NK_SERVER_ADMISSION_THREAD if admission_thread else 0, int(memory_cap_bytes),
                           int(batch_slots), 0)
        _check(self.lib.nk_server_create(self.ctx.handle, C.byref(d), C.byref(self.h)), "server_create", self.ctx.last_error())
        self._keep = {}

    def close(self):
        if self.h:
            self.lib.nk_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, case, u_init=None, v_init=None):
        """Queue the velocity solve of `case`; returns its ticket."""
        desc = case.descriptors()
        g = case.grid
        nfx, nfy = g.face_count(0), g.face_count(1)
        f = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in case.fields.items()}
        u = np.zeros((g.Ny, nfx))
        v = np.zeros((nfy, g.Nx))
        r = abi.Request()
        r.grid, r.physics, r.solver = desc.grid, desc.physics, desc.solver
        r.H, r.bed = _ptr(f["H"]), _ptr(f["bed"])
        r.friction_coefficient = _ptr(f.get("C"))
        r.rate_factor = _ptr(f["A"])
        ui = None if u_init is None else np.ascontiguousarray(u_init, dtype=np.float64)
        vi = None if v_init is None else np.ascontiguousarray(v_init, dtype=np.float64)
        r.u_init, r.v_init = _ptr(ui), _ptr(vi)
        r.u_out, r.v_out = _ptr(u), _ptr(v)
        t = C.c_int64()
        _check(self.lib.nk_server_submit(self.h, C.byref(r), C.byref(t)), "server_submit", self.ctx.last_error())
        self._keep[t.value] = (u, v)
        return t.value

    def progress(self):
        n = C.c_int32()
        _check(self.lib.nk_server_progress(self.h, C.byref(n)), "server_progress", self.ctx.last_error())
        return n.value

    def wait(self, ticket):
        """(u, v, stats, (t_submit, t_admit, t_done)) of a request, blocking until it is done."""
        st = abi.SolveStats()
        ts, ta, td = C.c_double(), C.c_double(), C.c_double()
        rc = self.lib.nk_server_wait(self.h, ticket, C.byref(st), C.byref(ts), C.byref(ta), C.byref(td))
        _check(rc, "server_wait", self.ctx.last_error())
        u, v = self._keep.pop(ticket)
        return u, v, st, (ts.value, ta.value, td.value)

    def wait_all(self):
        _check(self.lib.nk_server_wait_all(self.h), "server_wait_all", self.ctx.last_error())

    def clock(self):
        return self.lib.nk_server_clock(self.h)

    def info(self):
        n, b, p = C.c_int32(), C.c_int64(), C.c_int32()
        _check(self.lib.nk_server_info(self.h, C.byref(n), C.byref(b), C.byref(p)), "server_info")
        return {"resident": n.value, "device_bytes": b.value, "peak_in_flight": p.value}
