"""Multi-field block assembly on the GPU against the oracle, on the configuration of
test/BlockSparseMatrixAssemblersTests.jl:98-120: 8x8 Q1 on the unit square, Dirichlet
on the boundary with u = x + y, biform2/liform2 and biform3/liform3, styles
ConsecutiveMultiFieldStyle, BlockMultiFieldStyle() and BlockMultiFieldStyle(2, (1, n-1)),
FullyAssembledRows (the strategy the test passes) and SubAssembledRows (the default of its
AffineFEOperator(biform, liform, X, Y) calls), parts (2,2), (2,1), (1,2).

Bit-exact: row/column index sets (local CSR pattern, ghost row and ghost column gids and
owners; under SubAssembledRows the zeroed ghost rows and first-appearance columns of the
oracle's loop restatement) and the multi-field gids.  FP64 values: |gpu - oracle| <= 1e-12 * (max |oracle| in the row);
right-hand sides <= 1e-12 * max |b|.  Block vs monolithic (the reference's own check):
mul! with all-ones inputs and the right-hand sides agree field by field to 1e-10.
"""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem, row_scaled_error
from test_oracle_multifield import FORMS

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
PARTS = [(2, 2), (2, 1), (1, 2)]


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def styles(nf):
    import gridap_gb300 as G
    return {"consecutive": G.ConsecutiveMultiFieldStyle(), "block": G.BlockMultiFieldStyle(),
            "block_1_rest": G.BlockMultiFieldStyle(2, (1, nf - 1))}


def gpu_system(backend, parts, nf, style, stiff=None, mass=None, src=None, strategy="full"):
    import gridap_gb300 as G
    ranks = backend.distribute(range(int(np.prod(parts))))
    model = G.CartesianDiscreteModel(ranks, parts, (0, 1, 0, 1), (8, 8))
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
    U = G.TrialFESpace(lambda x, y: x + y, V)
    dO = G.Measure(G.Triangulation(model), 2)
    Y = G.MultiFieldFESpace([V] * nf, style=style)
    X = G.MultiFieldFESpace([U] * nf, style=style)
    st, ms, sr = FORMS[nf]
    a = G.integral_multifield(st if stiff is None else stiff, ms if mass is None else mass, dO)
    l = G.integral_multifield_source(sr if src is None else src, dO)
    if strategy == "default":   # AffineFEOperator(biform, liform, X, Y): the default assembler
        op = G.AffineFEOperator(a, l, X, Y)
        return model, V, op.assem, op
    assem = G.SparseMatrixAssembler(X, Y, G.FullyAssembledRows() if strategy == "full" else G.SubAssembledRows())
    op = G.AffineFEOperator(a, l, X, Y, assem)
    return model, V, assem, op


def oracle(parts):
    pb = make_problem(2, (8, 8), parts, 1, f=0.0, u=lambda x, y: x + y)
    return pb, go.build_fespace(pb)


def check_matrix(mat, ref):
    for p, (M, (rp, ci, vv), rows, cols, b) in enumerate(zip(ref, mat.csr_parts(), mat.row_partition,
                                                              mat.col_partition, mat.rhs_parts())):
        assert np.array_equal(rp, M.rowptr), f"rowptr part {p}"
        assert np.array_equal(ci, M.colidx), f"colidx part {p}"
        assert np.array_equal(rows.ghost_to_global, M.row_ghost_gids), f"ghost rows part {p}"
        assert np.array_equal(rows.ghost_to_owner, M.row_ghost_owner)
        assert np.array_equal(cols.own_to_global, M.col_own_gids)
        assert np.array_equal(cols.ghost_to_global, M.col_ghost_gids), f"ghost cols part {p}"
        assert np.array_equal(cols.ghost_to_owner, M.col_ghost_owner)
        assert row_scaled_error(vv, M.vals, M.rowptr) <= VAL_TOL
        scale = max(np.abs(M.b).max(), 1e-300)
        assert np.abs(b - M.b).max() <= VAL_TOL * scale


@pytest.mark.parametrize("strategy", ["full", "sub", "default"])
@pytest.mark.parametrize("parts", PARTS)
@pytest.mark.parametrize("nf", [2, 3])
@pytest.mark.parametrize("style", ["consecutive", "block", "block_1_rest"])
def test_multifield_matches_oracle(backend, parts, nf, style, strategy):
    import gridap_gb300 as G
    _, V, assem, op = gpu_system(backend, parts, nf, styles(nf)[style], strategy=strategy)
    pb, fe = oracle(parts)
    st, ms, sr = FORMS[nf]
    groups = op.assem.Y.groups()
    strat = "full" if strategy == "full" else "sub"
    if style == "consecutive":
        assert isinstance(op.matrix, G.multifield.MultiFieldMatrix)
        check_matrix(op.matrix, go.assemble_multifield(pb, fe, st, ms, sr, groups[0], groups[0], strategy=strat))
    else:
        assert isinstance(op.matrix, G.BlockPMatrix)
        for I, gI in enumerate(groups):
            for J, gJ in enumerate(groups):
                check_matrix(op.matrix.blocks[I][J],
                             go.assemble_multifield(pb, fe, st, ms, sr, gI, gJ, strategy=strat))


@pytest.mark.parametrize("strategy", ["full", "default"])
@pytest.mark.parametrize("parts", PARTS)
@pytest.mark.parametrize("nf", [2, 3])
def test_block_equals_monolithic(backend, parts, nf, strategy):
    """is_same_matrix / is_same_vector of test/BlockSparseMatrixAssemblersTests.jl:17-39
    (with its explicit FullyAssembledRows assemblers and its default-assembler
    AffineFEOperator calls)."""
    import gridap_gb300 as G
    _, V, _, mono = gpu_system(backend, parts, nf, G.ConsecutiveMultiFieldStyle(), strategy=strategy)
    Y = mono.assem.Y
    n = V.num_free_dofs()
    y_mono = mono.matrix.mul(np.ones(nf * n))
    b_mono = mono.vector.global_values()
    for style in ("block", "block_1_rest"):
        _, _, _, blk = gpu_system(backend, parts, nf, styles(nf)[style], strategy=strategy)
        Yb = blk.assem.Y
        groups = Yb.groups()
        ys = blk.matrix.mul([np.ones(len(g) * n) for g in groups])
        bs = blk.vector.global_values()
        for I, g in enumerate(groups):
            for f in g:
                yi = G.restrict_to_field(Yb, ys[I], f)
                bi = G.restrict_to_field(Yb, bs[I], f)
                assert np.abs(yi - G.restrict_to_field(Y, y_mono, f)).max() < 1e-10
                assert np.abs(bi - G.restrict_to_field(Y, b_mono, f)).max() < 1e-10


@pytest.mark.parametrize("parts", [(2, 2), (3, 1)])
def test_multifield_gids_match_oracle(backend, parts):
    import gridap_gb300 as G
    _, V, assem, _ = gpu_system(backend, parts, 3, G.ConsecutiveMultiFieldStyle())
    pb, fe = oracle(parts)
    for fields in ([0], [0, 1], [0, 1, 2], [1, 2]):
        ref = go.multifield_gids(fe, len(fields))
        got = assem.gids(fields).partition()
        for p, (a, b) in enumerate(zip(got, ref)):
            assert np.array_equal(a.local_to_global, b.ldof_to_gdof), f"gids part {p}"
            assert np.array_equal(a.local_to_owner, b.ldof_to_owner), f"owners part {p}"


def test_reassembly_refreshes_values(backend):
    """assemble_matrix! semantics: a second assembly with other coefficients on the same
    touched blocks updates every matrix built from the field set."""
    import gridap_gb300 as G
    parts = (2, 2)
    _, V, assem, op = gpu_system(backend, parts, 2, G.BlockMultiFieldStyle())
    st2, ms2, sr2 = [[2.5, 0], [0, 0]], [[0, 0], [0.5, 3.0]], [0.25, -1.0]
    dO = G.Measure(G.Triangulation(V.model), 2)
    assem.numeric(G.integral_multifield(st2, ms2, dO), G.integral_multifield_source(sr2, dO))
    pb, fe = oracle(parts)
    for I in range(2):
        for J in range(2):
            check_matrix(op.matrix.blocks[I][J], go.assemble_multifield(pb, fe, st2, ms2, sr2, [I], [J]))
    with pytest.raises(RuntimeError):   # a block the pattern does not hold
        assem.numeric(G.integral_multifield([[1, 1], [0, 0]], [[0, 0], [1, 1]], dO), None)


@pytest.mark.parametrize("strategy", ["full", "sub"])
def test_untouched_block_is_empty(backend, strategy):
    import gridap_gb300 as G
    _, V, _, op = gpu_system(backend, (2, 2), 2, G.BlockMultiFieldStyle(), strategy=strategy)
    assert all(len(vv) == 0 for _, _, vv in op.matrix.blocks[0][1].csr_parts())   # u2 never meets v1
