"""The allocation-free solve entry point, through the C ABI.

gd_solve_noalloc serves callers that cannot allocate device memory while they run
(their device memory is owned by their own pool allocator, or a cudaMalloc inside
their loop is not acceptable).  It runs the Jacobi-PCG iteration of gd_solve (one
shared body: the same steps, restarts and stopping rule) on the CSR matrix kernel,
where gd_solve reads a sliced-ELL copy for short rows and lane groups for long ones,
so the two agree to the solve tolerance, not bit for bit.  It must match the oracle's
gathered sparse LU (the reference's own `\\`) on repeated calls (the shared static
scratch keeps the previous call's contents), on Q1 and Q2 rows, reach tight
tolerances, report the exact iteration count, handle a system with no free DOFs, and
reject systems above its fixed size limit with an error status.

This file is named so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem

pytestmark = pytest.mark.gpu

LU_TOL = 1e-8       # relative difference to the oracle's gathered LU (the reference's `\`)
SOLVE_TOL = 1e-8    # relative difference to gd_solve (same iteration, other SpMV kernel)
NOALLOC_MAX_DOFS = 1 << 18


def _assembled(be, pb):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, pb.order), dirichlet_tags="boundary")
    U = G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    op = G.AffineFEOperator(G.integral_grad_grad(pb.kappa, dO), G.integral_source(pb.f_const, dO), U, V)
    return model, V, U, op


def _noalloc(L, lib, op, n, rtol):
    x = np.full(n, np.nan)
    st = L.gd_solve_stats()
    rc = lib.gd_solve_noalloc(op.matrix.assem.handle, rtol, 100000, L.vptr(x), L.GD_HOST, C.byref(st))
    assert rc == 0, lib.gd_last_error().decode()
    return x, st


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("dim,n,parts,order", [
    (3, (16, 14, 12), (2, 2, 2), 1),
    (3, (8, 7, 6), (2, 2, 1), 2),
    (2, (40, 36), (2, 2), 2),
])
def test_noalloc_solve_matches_lu_and_solve_on_repeated_calls(dim, n, parts, order):
    import gridap_gb300 as G
    L = G._lib
    lib = L.load()
    pb = make_problem(dim, n, parts, order, seed=21)
    fe = go.build_fespace(pb)
    x_lu = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    be = G.GB300Backend(0)
    try:
        model, V, U, op = _assembled(be, pb)
        nd = V.num_free_dofs()
        assert nd <= NOALLOC_MAX_DOFS
        x_solve = op.matrix.solve(rtol=1e-12)
        for call in range(2):
            x, st = _noalloc(L, lib, op, nd, 1e-12)
            assert st.converged and st.rel_residual <= 1e-12
            assert _rel(x, x_lu) <= LU_TOL, f"call {call}: vs LU {_rel(x, x_lu)}"
            assert _rel(x, x_solve) <= SOLVE_TOL, f"call {call}: vs gd_solve {_rel(x, x_solve)}"
    finally:
        be.close()


def test_noalloc_tight_tolerance_and_exact_iteration_count():
    """rtol 1e-13 needs the restart from the true FP64 residual; the iteration count is
    the step at which the recursive residual met the tolerance, as in the oracle's own
    Jacobi-PCG on the gathered matrix (a few steps apart at most: other rounding)."""
    import gridap_gb300 as G
    L = G._lib
    lib = L.load()
    pb = make_problem(3, (16, 14, 12), (2, 2, 2), 1, seed=23)
    fe = go.build_fespace(pb)
    ngd = fe.dofs[0].ngdofs
    A, b = go.gather_global(go.assemble(pb, fe, "sub"), ngd)
    _, it_oracle = go.pcg_jacobi(A.tocsr(), b, rtol=1e-10)
    be = G.GB300Backend(0)
    try:
        model, V, U, op = _assembled(be, pb)
        x, st = _noalloc(L, lib, op, ngd, 1e-13)
        assert st.converged and st.rel_residual <= 1e-13
        assert np.linalg.norm(b - A @ x) <= 1e-12 * np.linalg.norm(b)
        x, st = _noalloc(L, lib, op, ngd, 1e-10)
        assert abs(st.iterations - it_oracle) <= 3, (st.iterations, it_oracle)
    finally:
        be.close()


def test_noalloc_system_without_free_dofs():
    """One Q1 cell with Dirichlet values on the whole boundary: no free DOFs."""
    import gridap_gb300 as G
    L = G._lib
    lib = L.load()
    be = G.GB300Backend(0)
    try:
        pb = make_problem(2, (1, 1), (1, 1), 1, seed=24)
        model, V, U, op = _assembled(be, pb)
        assert V.num_free_dofs() == 0
        x = np.zeros(1)
        st = L.gd_solve_stats()
        rc = lib.gd_solve_noalloc(op.matrix.assem.handle, 1e-8, 10, L.vptr(x), L.GD_HOST, C.byref(st))
        assert rc == 0, lib.gd_last_error().decode()
        assert st.converged and st.iterations == 0
    finally:
        be.close()


def test_noalloc_rejects_systems_above_its_limit():
    import gridap_gb300 as G
    L = G._lib
    lib = L.load()
    be = G.GB300Backend(0)
    try:
        pb = make_problem(3, (66, 66, 66), (2, 2, 2), 1, seed=22)   # 65^3 = 274,625 DOFs
        model, V, U, op = _assembled(be, pb)
        assert V.num_free_dofs() > NOALLOC_MAX_DOFS
        x = np.zeros(V.num_free_dofs())
        st = L.gd_solve_stats()
        rc = lib.gd_solve_noalloc(op.matrix.assem.handle, 1e-8, 10, L.vptr(x), L.GD_HOST, C.byref(st))
        assert rc == 1   # GD_ERR_ARG
        assert "limit" in lib.gd_last_error().decode()
    finally:
        be.close()
