"""Batched solves (nk_batch): `slots` problems of one configuration solved together by one CUDA graph.

Every kernel launch of a batched solve covers all slots, so S small solves cost the launches of the slowest one
instead of S times as many; each slot's result is that of its problem solved alone.  The reference has no
counterpart (it solves one grid per picard_solve!, src/Solvers/picard.jl:63-90); a batch serves many independent
solves of one grid, such as ensemble members or the requests of one size in a serving stream.

    B = Batch(grid, desc, slots=8)
    for k, case in enumerate(cases):
        P = B.problem(k)                  # a Problem: set fields, compute_geometry, get results
        ...
    stats = B.picard_solve(active)        # one stats per slot (None for the slots not solved)
"""
import ctypes as C

import numpy as np

from . import abi
from .problem import Problem, _check


class SlotProblem(Problem):
    """The problem of one batch slot: a Problem over a handle the batch owns (closing it only drops the handle)."""

    def __init__(self, grid, desc, handle, context):
        self._slot_handle = handle
        super().__init__(grid, desc, context=context)

    def _create(self):
        self._h = C.c_void_p(self._slot_handle)

    def close(self):
        self._h = C.c_void_p()


class Batch:
    """nk_batch: `slots` problems of `desc` on `grid` in one device allocation, solved by one graph."""

    def __init__(self, grid, desc, slots, context=None):
        from . import library
        self._lib = library.load()
        self._ctx = context if context is not None else library.default_context()
        self.grid, self.desc, self.slots = grid, desc, int(slots)
        self._h = C.c_void_p()
        st = self._lib.nk_batch_create(self._ctx.handle, C.byref(desc.grid), C.byref(desc.physics), C.byref(desc.solver),
                                       self.slots, C.byref(self._h))
        _check(st, "batch_create", self._ctx.last_error())
        self.problems = [SlotProblem(grid, desc, self._lib.nk_batch_problem(self._h, k), self._ctx) for k in range(self.slots)]
        self._active = None

    def problem(self, k):
        return self.problems[k]

    def close(self):
        if self._h:
            for P in self.problems:
                P.close()
            self._lib.nk_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _mask(self, active):
        if active is None:
            return None
        a = np.zeros(self.slots, dtype=np.uint8)
        idx = np.asarray(active)
        if idx.dtype == bool:
            a[: len(idx)] = idx
        else:
            a[idx.astype(int)] = 1
        return a

    def picard_solve_async(self, active=None):
        """Enqueue picard_solve! of the chosen slots (indices or a boolean mask; all when None) and return."""
        a = self._mask(active)
        self._active = a
        ptr = a.ctypes.data_as(C.POINTER(C.c_uint8)) if a is not None else None
        _check(self._lib.nk_batch_picard_solve_async(self._h, ptr), "batch_picard_solve_async", self._ctx.last_error())

    def query(self):
        d = C.c_int32()
        _check(self._lib.nk_batch_query(self._h, C.byref(d)), "batch_query", self._ctx.last_error())
        return bool(d.value)

    def wait(self):
        """Block until the batched solve has finished: one SolveStats per slot, None for a slot not solved."""
        stats = (abi.SolveStats * self.slots)()
        st = self._lib.nk_batch_wait(self._h, stats)
        active = self._active if self._active is not None else np.ones(self.slots, dtype=np.uint8)
        _check(st, "batch_wait", self._ctx.last_error())
        return [stats[k] if active[k] else None for k in range(self.slots)]

    def picard_solve(self, active=None):
        self.picard_solve_async(active)
        return self.wait()
