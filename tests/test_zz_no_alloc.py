"""The allocation-free solve entry point, through the C ABI.

gd_solve_noalloc serves callers that cannot allocate device memory while they run
(their device memory is owned by their own pool allocator, or a cudaMalloc inside
their loop is not acceptable).  It must give the same solution as gd_solve, on
repeated calls (the shared static scratch keeps the previous call's contents), and
must reject systems above its fixed size limit with an error status.

This file is named so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import make_problem

pytestmark = pytest.mark.gpu

SOL_TOL = 1e-12     # same algorithm, same kernels: relative difference to gd_solve
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


def test_noalloc_solve_matches_solve_on_repeated_calls():
    import gridap_gb300 as G
    L = G._lib
    lib = L.load()
    be = G.GB300Backend(0)
    try:
        pb = make_problem(3, (16, 14, 12), (2, 2, 2), 1, seed=21)
        model, V, U, op = _assembled(be, pb)
        n = V.num_free_dofs()
        x_ref = op.matrix.solve(rtol=1e-10)
        for call in range(2):
            x = np.full(n, np.nan)
            st = L.gd_solve_stats()
            rc = lib.gd_solve_noalloc(op.matrix.assem.handle, 1e-10, 100000, L.vptr(x), L.GD_HOST, C.byref(st))
            assert rc == 0, lib.gd_last_error().decode()
            assert st.converged
            err = np.abs(x - x_ref).max() / np.abs(x_ref).max()
            assert err <= SOL_TOL, f"call {call}: relative difference {err}"
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
