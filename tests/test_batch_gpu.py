"""Batched assembly (one persistent launch for all problems) and batched Jacobi-PCG:
every problem of an uneven batch against the oracle and against its own
single-problem assembly."""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem, row_scaled_error

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
SOL_TOL = 1e-8

BATCH = [
    dict(dim=3, n=(6, 5, 4), parts=(2, 2, 1), order=1, seed=50),
    dict(dim=3, n=(4, 3, 5), parts=(2, 2, 1), order=2, seed=51),
    dict(dim=3, n=(3, 4, 3), parts=(2, 2, 1), order=3, seed=52),
    dict(dim=2, n=(7, 5), parts=(2, 2), order=2, seed=53, f_nodal=True),
    dict(dim=3, n=(5, 5, 5), parts=(2, 2, 1), order=2, sides=(1, 0, 1, 1, 0, 1), seed=54),
    dict(dim=2, n=(6, 6), parts=(2, 1), order=3, seed=55, u=lambda x, y: 1.0 + x * y),
    dict(dim=3, n=(8, 7, 6), parts=(2, 2, 1), order=1, sides=(1, 1, 0, 1, 1, 0), seed=56, f_nodal=True,
         u=lambda x, y, z: x + 2 * y + z * z),
]


def build(be, pb):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    tags = ["left", "right", "bottom", "top", "back", "front"]
    sides = [t for t, s in zip(tags, pb.dirichlet_sides) if s]
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, pb.order), dirichlet_tags=sides)
    U = G.TrialFESpace(pb.u_dir, V) if pb.u_dir is not None else G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    a = G.integral_grad_grad(pb.kappa, dO)
    l = G.integral_source(pb.f_nodal if pb.f_nodal is not None else pb.f_const, dO)
    assem = G.SparseMatrixAssembler(U, V, G.SubAssembledRows())
    return model, V, U, assem, a, l


@pytest.fixture(scope="module")
def batch_setup():
    import gridap_gb300 as G
    from gridap_gb300.batch import BatchedAssembler
    be = G.GB300Backend(0)
    pbs = [make_problem(**c) for c in BATCH]
    built = [build(be, pb) for pb in pbs]
    B = BatchedAssembler([(assem, a, l) for (_, _, _, assem, a, l) in built])
    B.assemble()
    yield be, pbs, built, B
    B.close()
    be.close()


def test_batch_matches_oracle(batch_setup):
    be, pbs, built, B = batch_setup
    for pb, (model, V, U, assem, a, l), M, vec in zip(pbs, built, B.matrices, B.vectors):
        fe = go.build_fespace(pb)
        parts = go.assemble(pb, fe, "sub")
        b_parts = vec.partition
        for p, (rp, ci, vv) in enumerate(M.csr_parts()):
            O = parts[p]
            assert np.array_equal(rp, O.rowptr) and np.array_equal(ci, O.colidx)
            assert row_scaled_error(vv, O.vals, O.rowptr) <= VAL_TOL
            scale = max(np.abs(O.b).max(), 1e-300)
            assert np.abs(b_parts[p] - O.b).max() <= VAL_TOL * scale


def test_batch_matches_single_problem_assembly(batch_setup):
    """Orders 2 and 3 run the same row bodies as the single-problem kernel with the cells'
    terms summed one by one (the 2D class sums switched off): values bit-exact; the rhs
    bit-exact in 3D and within 1e-14 x max|b| in 2D, where the single-problem kernel adds
    the halves of a row's cells formed by two lanes."""
    import gridap_gb300 as G
    be, pbs, built, B = batch_setup
    for pb, M, vec in zip(pbs, B.matrices, B.vectors):
        if pb.order == 1:
            continue   # the single-problem Q1 path is a different (class-based) kernel
        _, V, U, assem, a, l = build(be, pb)
        G._lib.call("gd_assembler_set_class_sums", assem.handle, 0)
        op = G.AffineFEOperator(a, l, U, V, assem)
        for (rp, ci, vv), (rp2, ci2, vv2) in zip(M.csr_parts(), op.matrix.csr_parts()):
            assert np.array_equal(vv, vv2)
        for b1, b2 in zip(vec.partition, op.vector.partition):
            if pb.dim == 3:
                assert np.array_equal(b1, b2)
            else:
                assert np.abs(b1 - b2).max(initial=0.0) <= 1e-14 * max(np.abs(b2).max(initial=0.0), 1e-300)


def test_batch_tuning_and_graph_replay_are_stable(batch_setup):
    be, pbs, built, B = batch_setup
    t = B.tuning()
    assert t["shape"] >= 0 and t["rows_per_task"] > 0 and t["ctas_per_sm"] > 0
    assert len(t["ms_per_shape"]) == 8 and all(ms > 0 for ms in t["ms_per_shape"])
    before = [[vv.copy() for (_, _, vv) in M.csr_parts()] for M in B.matrices]
    B.assemble()   # graph replay
    for M, ref in zip(B.matrices, before):
        for (_, _, vv), v0 in zip(M.csr_parts(), ref):
            assert np.array_equal(vv, v0)
    c = B.counts()
    assert c["problems"] == len(BATCH)
    assert c["rows"] == sum(M.n_global for M in B.matrices)
    assert c["nnz_owned"] > c["rows"]


def test_batch_solve_matches_gathered_lu(batch_setup):
    be, pbs, built, B = batch_setup
    stats = B.solve(rtol=1e-12)
    for p, pb in enumerate(pbs):
        assert stats[p].converged and stats[p].rel_residual <= 1e-11
        fe = go.build_fespace(pb)
        x_ref = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
        x = B.solution(p)
        assert np.abs(x - x_ref).max() / np.abs(x_ref).max() <= SOL_TOL
