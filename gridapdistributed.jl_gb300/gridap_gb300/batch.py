"""Batched assembly and solve of many independent problems (``gd_batch_*``).

No counterpart in the reference, which assembles one problem per
``assemble_matrix_and_vector`` call.  A batch takes assemblers (any order 1..3)
with their bilinear and linear forms; ``assemble()`` fills every problem's
PSparseMatrix and PVector in one persistent kernel launch (replayed from a CUDA
graph after the first, autotuned call) and ``solve()`` runs Jacobi-PCG in FP64 on
all problems at once.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .distributed import PSparseMatrix, PVector


class BatchedAssembler:
    """problems: a sequence of (assembler, a, l) with a = integral_grad_grad(...) and
    l = integral_source(...), as for AffineFEOperator."""

    def __init__(self, problems):
        self.problems = list(problems)
        n = len(self.problems)
        if n == 0:
            raise ValueError("empty batch")
        self._keep = []
        coeffs = (L.gd_coeffs * n)()
        handles = (C.c_void_p * n)()
        for i, (assem, a, l) in enumerate(self.problems):
            assem.symbolic()
            handles[i] = assem.handle.value if isinstance(assem.handle, C.c_void_p) else assem.handle
            c = coeffs[i]
            if a.kappa is not None:
                kap = np.ascontiguousarray(a.kappa, dtype=np.float64)
                self._keep.append(kap)
                c.kappa = kap.ctypes.data
            else:
                c.kappa = None
            f = l.f if l is not None else 0.0
            if np.isscalar(f):
                c.f_nodal = None
                c.f_const = float(f)
            else:
                fa = np.ascontiguousarray(f, dtype=np.float64)
                self._keep.append(fa)
                c.f_nodal = fa.ctypes.data
                c.f_const = 0.0
            c.degree = int(a.measure.degree if a.measure is not None else 2 * assem.V.order)
            c.where = L.GD_HOST
        h = C.c_void_p()
        L.call("gd_batch_create", C.cast(handles, C.c_void_p), C.cast(coeffs, C.c_void_p), n, C.byref(h))
        self.handle = h
        self.matrices = [PSparseMatrix(assem) for assem, _, _ in self.problems]
        self.vectors = [PVector(assem, m) for (assem, _, _), m in zip(self.problems, self.matrices)]

    def __len__(self):
        return len(self.problems)

    def assemble(self, sync: bool = True):
        L.call("gd_batch_assemble" if sync else "gd_batch_assemble_async", self.handle)
        for m in self.matrices:
            m._parts = None   # host copies are stale

    def counts(self):
        n, rows, nnz = C.c_int32(), C.c_int64(), C.c_int64()
        L.call("gd_batch_counts", self.handle, C.byref(n), C.byref(rows), C.byref(nnz))
        return {"problems": n.value, "rows": rows.value, "nnz_owned": nnz.value}

    def tuning(self):
        shape, rows, per_sm, ns = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        ms = (C.c_float * 16)()
        L.call("gd_batch_tuning", self.handle, C.byref(shape), C.byref(rows), C.byref(per_sm), ms, C.byref(ns))
        return {"shape": shape.value, "rows_per_task": rows.value, "ctas_per_sm": per_sm.value,
                "ms_per_shape": [float(ms[i]) for i in range(ns.value)]}

    def solve(self, rtol=1e-8, maxit=100000):
        """Jacobi-PCG (FP64) of every problem; returns the per-problem gd_solve_stats."""
        stats = (L.gd_solve_stats * len(self))()
        L.call("gd_batch_solve", self.handle, float(rtol), int(maxit), C.cast(stats, C.c_void_p))
        return list(stats)

    def solution(self, p: int) -> np.ndarray:
        x = np.zeros(self.matrices[p].n_global)
        L.call("gd_batch_solution", self.handle, int(p), L.vptr(x), L.GD_HOST)
        return x

    def close(self):
        if getattr(self, "handle", None):
            L.load().gd_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
