"""Learned preconditioner: training, persistence and the learned flexible-CG solve.

The network and all of its arithmetic live in libgdgpu.so (``gd_learned_*``); this
module drives it: it generates (residual, error) pairs with the solver itself,
trains on the GPU with the library's forward/backward kernels, saves and loads the
parameters in a versioned binary file, and solves with the learned flexible CG.

Training pairs for one coefficient field: the converged solution x* of A x = b
(mixed-precision refinement to 1e-10), then the iterates x_k the same solver reaches
after k inner iterations; each pair is (r_k = b - A x_k, e_k = x* - x_k), scaled to
unit residual norm.  The loss is the relative A-norm error ||M(r) - e||_A^2 / ||e||_A^2.
"""
from __future__ import annotations

import ctypes as C
import struct
import zlib
from pathlib import Path

import numpy as np

from . import _lib as L

MAGIC = b"GDLP"
# header: magic, version, levels, flags, parameter count, CRC32 of the float32 payload
# (version 2 files have no flags word: flags 0)
FORMAT_VERSION = 3
COARSE_START = 1   # gd_learned flag: network on the once-restricted lattice


def _torch():
    import torch
    return torch


class LearnedPreconditioner:
    """The L-level (default 3), 8-channel network bound to one assembler (one problem
    size), applied as z = D^-1 r + D^-1/2 S^T S D^-1/2 r (symmetric positive definite);
    with coarse_start the network runs on the once-restricted lattice,
    z = D^-1 r + D^-1/2 R^T S^T S R D^-1/2 r."""

    def __init__(self, matrix, seed: int = 0, levels: int = 3, coarse_start: bool = False):
        self.matrix = matrix
        self.assem = matrix.assem
        self.levels = int(levels)
        self.flags = COARSE_START if coarse_start else 0
        h = C.c_void_p()
        L.call("gd_learned_create", self.assem.handle, self.levels, self.flags, C.c_uint64(seed), C.byref(h))
        self.handle = h
        n = C.c_int64()
        L.call("gd_learned_num_params", self.handle, C.byref(n))
        self.num_params = n.value

    # ---- parameters --------------------------------------------------------------------
    def get_params(self) -> np.ndarray:
        p = np.zeros(self.num_params, dtype=np.float32)
        L.call("gd_learned_get_params", self.handle, p.ctypes.data_as(C.POINTER(C.c_float)))
        return p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, dtype=np.float32)
        if p.size != self.num_params:
            raise ValueError(f"expected {self.num_params} parameters, got {p.size}")
        L.call("gd_learned_set_params", self.handle, p.ctypes.data_as(C.POINTER(C.c_float)))

    def save(self, path):
        """Versioned little-endian file: magic, format version, levels, flags, parameter
        count, CRC32, float32 params.  The parameters do not depend on the mesh size."""
        p = self.get_params()
        blob = p.tobytes()
        Path(path).write_bytes(MAGIC + struct.pack("<IIIII", FORMAT_VERSION, self.levels, self.flags, p.size,
                                                   zlib.crc32(blob)) + blob)

    @staticmethod
    def _header(data, path):
        if data[:4] != MAGIC:
            raise ValueError(f"{path}: not a learned-preconditioner file")
        version, = struct.unpack("<I", data[4:8])
        if version == 2:
            levels, count, crc = struct.unpack("<III", data[8:20])
            return levels, 0, count, crc, 20
        if version != FORMAT_VERSION:
            raise ValueError(f"{path}: format version {version}, expected {FORMAT_VERSION}")
        levels, flags, count, crc = struct.unpack("<IIII", data[8:24])
        return levels, flags, count, crc, 24

    @staticmethod
    def file_spec(path):
        """(levels, coarse_start) stored in a parameter file, to construct a matching net."""
        levels, flags, _, _, _ = LearnedPreconditioner._header(Path(path).read_bytes()[:24], path)
        return levels, bool(flags & COARSE_START)

    @staticmethod
    def file_levels(path) -> int:
        return LearnedPreconditioner.file_spec(path)[0]

    def load(self, path):
        data = Path(path).read_bytes()
        levels, flags, count, crc, start = self._header(data, path)
        if levels != self.levels or flags != self.flags:
            raise ValueError(f"{path}: network ({levels} levels, flags {flags}) differs from this one "
                             f"({self.levels} levels, flags {self.flags})")
        blob = data[start:]
        if count != self.num_params or len(blob) != 4 * count or zlib.crc32(blob) != crc:
            raise ValueError(f"{path}: parameter count or checksum mismatch")
        self.set_params(np.frombuffer(blob, dtype=np.float32))

    # ---- network ------------------------------------------------------------------------
    def apply(self, r):
        """z = M(r) for FP32 device tensors in gid order."""
        torch = _torch()
        z = torch.empty_like(r)
        L.call("gd_learned_apply", self.handle, C.c_void_p(r.data_ptr()), C.c_void_p(z.data_ptr()))
        return z

    def gradient(self, r, e):
        """Mean loss and summed parameter gradients for a batch [B, n] of pairs."""
        torch = _torch()
        r = r.contiguous()
        e = e.contiguous()
        g = np.zeros(self.num_params, dtype=np.float32)
        loss = C.c_double()
        L.call("gd_learned_gradient", self.handle, C.c_void_p(r.data_ptr()), C.c_void_p(e.data_ptr()),
               int(r.shape[0]), C.byref(loss), g.ctypes.data_as(C.POINTER(C.c_float)))
        return loss.value, g

    def train_step(self, r, e, lr: float) -> float:
        loss = C.c_double()
        L.call("gd_learned_train_step", self.handle, C.c_void_p(r.data_ptr()), C.c_void_p(e.data_ptr()),
               int(r.shape[0]), C.c_float(lr), C.byref(loss))
        return loss.value

    def solve(self, rtol=1e-8, maxit=100000):
        """x = A \\ b with the learned flexible CG; Jacobi fallback when the learned
        iteration stagnates.  Returns (x, stats, fallback_used)."""
        x = np.zeros(self.matrix.n_global)
        st = L.gd_solve_stats()
        fb = C.c_int32()
        L.call("gd_solve_learned", self.assem.handle, self.handle, float(rtol), int(maxit), L.vptr(x), L.GD_HOST,
               C.byref(st), C.byref(fb))
        return x, st, bool(fb.value)

    def close(self):
        if getattr(self, "handle", None):
            L.load().gd_learned_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- solver-generated training pairs ---------------------------------------------------------
def solve_rhs(matrix, b, method="mixed_ir", rtol=1e-10, maxit=100000, allow_unconverged=False):
    """x = A \\ b for a device FP64 tensor b (gid order); returns (x, stats)."""
    torch = _torch()
    codes = {"jacobi_pcg": L.GD_SOLVE_JACOBI_PCG, "mixed_ir": L.GD_SOLVE_MIXED_IR}
    x = torch.empty_like(b)
    st = L.gd_solve_stats()
    rc = L.load().gd_solve_rhs(matrix.assem.handle, codes[method], float(rtol), int(maxit), C.c_void_p(b.data_ptr()),
                               C.c_void_p(x.data_ptr()), L.GD_DEVICE, C.byref(st))
    if rc != 0 and not (allow_unconverged and rc in (5, 9)):
        L.check(rc)
    return x, st


def spmv(matrix, x):
    torch = _torch()
    y = torch.empty_like(x)
    L.call("gd_spmv", matrix.assem.handle, C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), L.GD_DEVICE)
    return y


def solver_pairs(matrix, b, ks=(4, 16, 64, 256)):
    """(r_k, e_k) pairs from the solver's own iterates on A x = b, unit residual norm."""
    torch = _torch()
    xs, _ = solve_rhs(matrix, b, rtol=1e-10)
    rs, es = [], []
    for k in ks:
        xk, _ = solve_rhs(matrix, b, rtol=1e-30, maxit=k, allow_unconverged=True)
        rk = b - spmv(matrix, xk)
        ek = xs - xk
        s = torch.linalg.vector_norm(rk)
        if s > 0:
            rs.append((rk / s).float())
            es.append((ek / s).float())
    return torch.stack(rs), torch.stack(es)
