"""Parity of the Q1 numeric kernel at the benchmarked size, for every launch shape.

The Q1 kernel (k_numeric_q1) has several launch shapes (64, 128 or 256 rows per chunk,
one or two staging buffers); the autotuner keeps the fastest, so without a way to force
a shape only the one it happened to pick would ever be checked.  gd_assembler_set_shape
fixes the shape, and every shape is compared with the oracle at sizes with many chunks
per CTA: the prefetch pipeline, the bulk stores across chunk boundaries with their
unaligned first and last entries, and the staging-buffer wrap-around all run.

* 128^3 Q1, parts (2,2,2), kappa = exp(GRF) of the bench workload, SubAssembledRows --
  the bench's own configuration, against the oracle's C restatement (oracle_core.c,
  pinned to the Python oracle by tests/test_oracle_c_vs_py.py);
* non-cube boxes (the general class-sum path), partial Dirichlet sides, both strategies;
* 2D Q1;
* nodal sources and non-zero Dirichlet values (the kernel's fused rhs variants), cube
  and non-cube, against the Python oracle.

Patterns, ghost rows and ghost columns bit-exact; values within 1e-12 x max|row|; rhs
within 1e-12 x max|b|.
"""
import os

import numpy as np
import pytest

import gridap_oracle as go
import oracle_c
from helpers import export_part, gpu_system, make_problem, row_scaled_error_fast

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def _nshapes(handle):
    import ctypes as C
    import gridap_gb300 as G
    sh, rows, nbuf, nsh = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
    ms = (C.c_float * 8)()
    G._lib.call("gd_assembler_tuning", handle, C.byref(sh), C.byref(rows), C.byref(nbuf), ms, C.byref(nsh))
    return nsh.value


def _check_parts(handle, ref, nparts, label):
    for p in range(nparts):
        got = export_part(handle, p)
        M = ref[p]
        rp = M["rowptr"] if isinstance(M, dict) else M.rowptr
        get = (lambda k: M[k]) if isinstance(M, dict) else (lambda k: getattr(M, k))
        assert np.array_equal(got["rowptr"], rp), f"{label} part {p}: rowptr"
        assert np.array_equal(got["colidx"], get("colidx")), f"{label} part {p}: colidx"
        assert np.array_equal(got["row_ghost_gids"], get("row_ghost_gids")), f"{label} part {p}: ghost rows"
        assert np.array_equal(got["col_ghost_gids"], get("col_ghost_gids")), f"{label} part {p}: ghost cols"
        err = row_scaled_error_fast(got["vals"], get("vals"), rp)
        assert err <= VAL_TOL, f"{label} part {p}: values {err}"
        b = get("b")
        scale = max(np.abs(b).max(initial=0.0), 1e-300)
        assert np.abs(got["b"] - b).max(initial=0.0) <= VAL_TOL * scale, f"{label} part {p}: rhs"


def _every_shape(op, ref, nparts):
    """Re-assemble with each forced launch shape and compare all parts."""
    import gridap_gb300 as G
    assem = op.matrix.assem
    n = _nshapes(assem.handle)
    assert n >= 5
    a, l = op.a, op.l
    for shape in range(n):
        G._lib.call("gd_assembler_set_shape", assem.handle, shape)
        assem.numeric(a, l)
        _check_parts(assem.handle, ref, nparts, f"shape {shape}")
    G._lib.call("gd_assembler_set_shape", assem.handle, -1)


def test_c2_bench_workload_every_shape(backend):
    from gridap_gb300.synthetic import POISSON3D_128, lognormal_kappa
    w = POISSON3D_128
    kappa = lognormal_kappa(w["cells"], w["sigma"], w["corr_len"], w["seed"])
    threads = min(8, os.cpu_count() or 1)
    ref, _, _ = oracle_c.assemble(3, w["cells"], w["parts"], w["domain"], (1,) * 6, kappa, w["f"], w["degree"],
                                  "sub", threads, keep=True)
    pb = go.Problem(np=w["parts"], n=w["cells"], domain=w["domain"], order=1, degree=w["degree"],
                    dirichlet_sides=None, kappa=kappa, f_const=w["f"])
    _, V, U, op = gpu_system(backend, pb, "sub")
    _check_parts(op.matrix.assem.handle, ref, 8, "autotuned")
    _every_shape(op, ref, 8)


LARGE = [
    # non-cube boxes, partial Dirichlet sides (general class-sum rows)
    dict(dim=3, n=(81, 73, 67), parts=(2, 2, 2), order=1, sides=(1, 1, 0, 1, 1, 0), seed=31,
         domain=(0, 1.0, 0, 1.3, 0, 0.8)),
    # cube cells, odd sizes, uneven parts
    dict(dim=3, n=(75, 69, 63), parts=(3, 2, 2), order=1, seed=32, domain=(0, 1.5, 0, 1.38, 0, 1.26)),
    # 2D
    dict(dim=2, n=(420, 350), parts=(2, 2), order=1, seed=33),
]


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("case", LARGE, ids=["3d_noncube", "3d_cube_odd", "2d"])
def test_large_q1_every_shape_against_oracle_c(backend, case, strategy):
    pb = make_problem(**case)
    sides = pb.dirichlet_sides if pb.dirichlet_sides is not None else (1,) * (2 * pb.dim)
    threads = min(8, os.cpu_count() or 1)
    ref, _, _ = oracle_c.assemble(pb.dim, pb.n, pb.np, pb.domain, sides, pb.kappa, pb.f_const, pb.degree,
                                  strategy, threads, keep=True)
    _, V, U, op = gpu_system(backend, pb, strategy)
    _every_shape(op, ref, int(np.prod(pb.np)))


FUSED = [
    # nodal source + non-zero Dirichlet values on cube cells
    dict(dim=3, n=(56, 56, 56), parts=(2, 2, 2), order=1, sides=(1, 1, 1, 0, 1, 1), seed=41, f_nodal=True,
         u=lambda x, y, z: 1.0 + x - 2 * y + z * z),
    # the same on non-cube boxes
    dict(dim=3, n=(52, 44, 40), parts=(2, 2, 1), order=1, sides=(1, 0, 1, 1, 0, 1), seed=42, f_nodal=True,
         u=lambda x, y, z: x * y - z, domain=(0, 1.0, 0, 0.7, 0, 1.2)),
    # Dirichlet values only (no nodal source)
    dict(dim=3, n=(48, 48, 48), parts=(2, 2, 2), order=1, seed=43, u=lambda x, y, z: 2.0 + x + y),
]


@pytest.mark.parametrize("case", FUSED, ids=["cube_fn_ud", "noncube_fn_ud", "cube_ud"])
def test_fused_rhs_variants_every_shape(backend, case):
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, "sub")
    _, V, U, op = gpu_system(backend, pb, "sub")
    _every_shape(op, ref, int(np.prod(pb.np)))
