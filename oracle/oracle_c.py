"""ctypes wrapper of the oracle's C core (oracle_core.c).  Test infrastructure only."""
import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


class orc_problem(C.Structure):
    _fields_ = [("dim", C.c_int), ("n", C.c_int64 * 3), ("np", C.c_int32 * 3), ("domain", C.c_double * 6),
                ("dsides", C.c_int32 * 6), ("kappa", C.c_void_p), ("f_const", C.c_double), ("degree", C.c_int)]


class orc_system(C.Structure):
    _fields_ = [("nparts", C.c_int), ("ngdofs", C.c_int64), ("nrows", C.POINTER(C.c_int64)),
                ("ncols", C.POINTER(C.c_int64)), ("nnz", C.POINTER(C.c_int64)),
                ("rowptr", C.POINTER(C.POINTER(C.c_int64))), ("colidx", C.POINTER(C.POINTER(C.c_int64))),
                ("vals", C.POINTER(C.POINTER(C.c_double))), ("b", C.POINTER(C.POINTER(C.c_double))),
                ("row_ghost_gid", C.POINTER(C.POINTER(C.c_int64))),
                ("col_ghost_gid", C.POINTER(C.POINTER(C.c_int64))),
                ("n_ghost_rows", C.POINTER(C.c_int64)), ("n_ghost_cols", C.POINTER(C.c_int64))]


_lib = None


def lib():
    global _lib
    if _lib is None:
        import build_oracle
        path = build_oracle.build()
        _lib = C.CDLL(str(path))
        _lib.orc_assemble.argtypes = [C.POINTER(orc_problem), C.c_int, C.c_int, C.POINTER(C.POINTER(orc_system)),
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _lib.orc_free.argtypes = [C.POINTER(orc_system)]
        _lib.orc_pcg.argtypes = [C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_double, C.c_int,
                                 C.c_int, C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)]
    return _lib


def assemble(dim, n, parts, domain, sides, kappa, f_const, degree, strategy="sub", threads=0, keep=True):
    """Runs the C restatement; returns (parts list or None, t_setup, t_assembly)."""
    L = lib()
    pb = orc_problem()
    pb.dim = dim
    for d in range(3):
        pb.n[d] = n[d] if d < dim else 1
        pb.np[d] = parts[d] if d < dim else 1
    for i in range(6):
        pb.domain[i] = domain[i] if i < 2 * dim else (0.0 if i % 2 == 0 else 1.0)
        pb.dsides[i] = int(sides[i]) if i < 2 * dim else 0
    kap = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    pb.kappa = None if kap is None else kap.ctypes.data
    pb.f_const = f_const
    pb.degree = degree
    out = C.POINTER(orc_system)()
    ts, ta = C.c_double(), C.c_double()
    L.orc_assemble(C.byref(pb), 0 if strategy == "sub" else 1, threads, C.byref(out), C.byref(ts), C.byref(ta))
    S = out.contents
    res = None
    if keep:
        res = []
        for p in range(S.nparts):
            nr, nz = S.nrows[p], S.nnz[p]
            res.append(dict(
                rowptr=np.ctypeslib.as_array(S.rowptr[p], (nr + 1,)).copy(),
                colidx=np.ctypeslib.as_array(S.colidx[p], (max(nz, 1),))[:nz].copy(),
                vals=np.ctypeslib.as_array(S.vals[p], (max(nz, 1),))[:nz].copy(),
                b=np.ctypeslib.as_array(S.b[p], (max(nr, 1),))[:nr].copy(),
                row_ghost_gids=np.ctypeslib.as_array(S.row_ghost_gid[p], (max(S.n_ghost_rows[p], 1),))[
                    :S.n_ghost_rows[p]].copy(),
                col_ghost_gids=np.ctypeslib.as_array(S.col_ghost_gid[p], (max(S.n_ghost_cols[p], 1),))[
                    :S.n_ghost_cols[p]].copy()))
    L.orc_free(out)
    return res, ts.value, ta.value
