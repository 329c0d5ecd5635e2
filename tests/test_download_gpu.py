"""gd_assemble_download: the numeric assembly with the download of the rhs and the
owned-row values overlapped (the Q1 kernel runs over 8 ranges of owned rows, each range
copied to the host on a second stream while the next one is assembled).

It must give exactly what gd_assemble_numeric followed by gd_system_download gives (the
same kernels compute every row; only the launches are split): bit-identical values and
rhs, on the cube Q1 path, the general Q1 path (non-cube cells, partial Dirichlet sides),
2D Q1, with nodal sources and Dirichlet values (the kernel's fused rhs variants), and on a
path without the row-range launches (3D Q2: assemble, then download).  Either host
pointer may be NULL, repeated calls agree, and a non-finite coefficient is reported as
GD_ERR_NUMERIC with the assembler still usable afterwards.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import gpu_system, make_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def _coeffs(pb, kappa=None):
    from gridap_gb300 import _lib as L
    c = L.gd_coeffs()
    k = pb.kappa if kappa is None else kappa
    keep = []
    if k is not None:
        k = np.ascontiguousarray(k, dtype=np.float64)
        keep.append(k)
        c.kappa = k.ctypes.data
    else:
        c.kappa = None
    if pb.f_nodal is not None:
        f = np.ascontiguousarray(pb.f_nodal, dtype=np.float64)
        keep.append(f)
        c.f_nodal = f.ctypes.data
        c.f_const = 0.0
    else:
        c.f_nodal = None
        c.f_const = float(pb.f_const)
    c.degree = int(pb.degree)
    c.where = L.GD_HOST
    return c, keep


def _sizes(handle):
    from gridap_gb300 import _lib as L
    n, nnz, tot, kern = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
    L.call("gd_assembler_counts", handle, C.byref(n), C.byref(nnz), C.byref(tot), C.byref(kern))
    return n.value, nnz.value


def _sequential(handle, c, n, nnz):
    from gridap_gb300 import _lib as L
    rhs, vals = np.full(n, np.nan), np.full(nnz, np.nan)
    L.call("gd_assemble_numeric", handle, C.byref(c))
    L.call("gd_system_download", handle, L.ptr(rhs, C.c_double), L.ptr(vals, C.c_double))
    return rhs, vals


def _overlapped(handle, c, n, nnz, want_rhs=True, want_vals=True):
    from gridap_gb300 import _lib as L
    rhs, vals = np.full(n, np.nan), np.full(nnz, np.nan)
    L.call("gd_assemble_download", handle, C.byref(c), L.ptr(rhs, C.c_double) if want_rhs else None,
           L.ptr(vals, C.c_double) if want_vals else None)
    return rhs, vals


CASES = [
    dict(dim=3, n=(40, 40, 40), parts=(2, 2, 2), order=1, seed=71),                          # cube Q1
    dict(dim=3, n=(37, 29, 33), parts=(2, 2, 2), order=1, seed=72, sides=(1, 0, 1, 1, 0, 1),
         domain=(0, 1.0, 0, 0.7, 0, 1.2)),                                                   # general Q1
    dict(dim=2, n=(300, 210), parts=(2, 2), order=1, seed=73),                               # 2D Q1
    dict(dim=3, n=(24, 24, 24), parts=(2, 2, 1), order=1, seed=74, f_nodal=True,
         u=lambda x, y, z: 1.0 + x - y * z),                                                 # fused rhs variants
    dict(dim=3, n=(10, 9, 8), parts=(2, 1, 2), order=2, seed=75),                            # Q2: no row ranges
]


@pytest.mark.parametrize("case", CASES, ids=["cube_q1", "noncube_q1", "2d_q1", "fn_ud", "q2"])
def test_overlapped_download_matches_assemble_then_download(backend, case):
    pb = make_problem(**case)
    _, V, U, op = gpu_system(backend, pb, "sub")
    h = op.matrix.assem.handle
    n, nnz = _sizes(h)
    c, keep = _coeffs(pb)
    rhs_a, vals_a = _sequential(h, c, n, nnz)
    assert np.isfinite(rhs_a).all() and np.isfinite(vals_a).all()
    for _ in range(2):
        rhs_b, vals_b = _overlapped(h, c, n, nnz)
        assert np.array_equal(rhs_a, rhs_b)
        assert np.array_equal(vals_a, vals_b)
    rhs_c, vals_c = _overlapped(h, c, n, nnz, want_vals=False)
    assert np.array_equal(rhs_a, rhs_c) and np.isnan(vals_c).all()
    rhs_d, vals_d = _overlapped(h, c, n, nnz, want_rhs=False)
    assert np.array_equal(vals_a, vals_d) and np.isnan(rhs_d).all()


def test_overlapped_download_reports_bad_coefficient_and_recovers(backend):
    from gridap_gb300 import _lib as L
    pb = make_problem(3, (20, 20, 20), (2, 2, 2), 1, seed=76)
    _, V, U, op = gpu_system(backend, pb, "sub")
    h = op.matrix.assem.handle
    n, nnz = _sizes(h)
    c, keep = _coeffs(pb)
    rhs_a, vals_a = _sequential(h, c, n, nnz)
    bad_kappa = pb.kappa.copy()
    bad_kappa[137] = np.nan
    cb, keep_b = _coeffs(pb, bad_kappa)
    rhs, vals = np.zeros(n), np.zeros(nnz)
    st = L.load().gd_assemble_download(h, C.byref(cb), L.ptr(rhs, C.c_double), L.ptr(vals, C.c_double))
    assert st == 8, L.load().gd_last_error()   # GD_ERR_NUMERIC
    rhs_b, vals_b = _overlapped(h, c, n, nnz)
    assert np.array_equal(rhs_a, rhs_b) and np.array_equal(vals_a, vals_b)
