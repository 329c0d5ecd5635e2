"""Multi-field systems in the oracle (CPU): the checks of
test/BlockSparseMatrixAssemblersTests.jl:41-93 restated on the oracle's assembly.

- block assembly (BlockMultiFieldStyle(), BlockMultiFieldStyle(2, (1, n-1))) equals the
  monolithic ConsecutiveMultiFieldStyle assembly: mul! with all-ones inputs and the
  right-hand sides agree field by field (is_same_matrix / is_same_vector, 1e-10);
- a single-field block of the multi-field assembly is the single-field assembly of its
  form (the path pinned to the reference's KATs), pattern bit-exact, values equal;
- the multi-field gids are a part-contiguous bijection numbered field by field.
"""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem

# biform2 / liform2 and biform3 / liform3 (test/BlockSparseMatrixAssemblersTests.jl:111-114):
# stiff[i][j] multiplies grad(u_j).grad(v_i), mass[i][j] multiplies u_j v_i
FORMS = {
    2: ([[1, 0], [0, 0]], [[0, 0], [1, 1]], [1.0, 1.0]),
    3: ([[1, 0, 0], [0, 0, 0], [0, 0, 0]], [[0, 0, 0], [1, 1, 1], [0, 1, 0]], [1.0, 1.0, 1.0]),
}


def reference_problem(parts):
    return make_problem(2, (8, 8), parts, 1, f=0.0, u=lambda x, y: x + y)


def group_gid(fe, ngroup, jj, g):
    """gid in the multi-field numbering of a group of ngroup fields of the scalar dof g
    seen as field jj of the group."""
    first = fe.first_gdof
    q = int(np.searchsorted(first, g, side="right") - 1)
    nown = fe.dofs[q].n_own
    return ngroup * int(first[q]) + jj * nown + (int(g) - int(first[q]))


def global_mul(mats, x):
    y = {}
    for M in mats:
        cols = np.concatenate([M.col_own_gids, M.col_ghost_gids])
        for r in range(M.nrows):
            s = 0.0
            for e in range(M.rowptr[r], M.rowptr[r + 1]):
                s += M.vals[e] * x[cols[M.colidx[e]]]
            y[int(M.row_own_gids[r])] = s
    return y


def rhs_map(mats):
    return {int(g): float(b) for M in mats for g, b in zip(M.row_own_gids, M.b)}


@pytest.mark.parametrize("parts", [(2, 2), (2, 1), (1, 2), (1, 1)])
@pytest.mark.parametrize("nf", [2, 3])
def test_block_equals_monolithic(parts, nf):
    pb = reference_problem(parts)
    fe = go.build_fespace(pb)
    stiff, mass, src = FORMS[nf]
    allf = list(range(nf))
    mono = go.assemble_multifield(pb, fe, stiff, mass, src, allf, allf)
    n = fe.dofs[0].ngdofs
    y_mono = global_mul(mono, np.ones(nf * n))
    b_mono = rhs_map(mono)
    for groups in ([[f] for f in allf], [[0], list(range(1, nf))]):
        for I, gI in enumerate(groups):
            y = {}
            for J, gJ in enumerate(groups):
                blk = go.assemble_multifield(pb, fe, stiff, mass, src, gI, gJ)
                for g, v in global_mul(blk, np.ones(len(gJ) * n)).items():
                    y[g] = y.get(g, 0.0) + v
                b_blk = rhs_map(blk)
            for ii, f in enumerate(gI):
                for g in range(n):
                    gm = group_gid(fe, nf, f, g)
                    gb = group_gid(fe, len(gI), ii, g)
                    assert abs(y[gb] - y_mono[gm]) < 1e-10
                    assert abs(b_blk[gb] - b_mono[gm]) < 1e-10


@pytest.mark.parametrize("parts", [(2, 2), (1, 1)])
def test_single_field_block_is_single_field_assembly(parts):
    pb = reference_problem(parts)
    fe = go.build_fespace(pb)
    stiff, mass, src = FORMS[3]
    for i in range(3):
        for j in range(3):
            if stiff[i][j] == 0 and mass[i][j] == 0:
                continue
            blk = go.assemble_multifield(pb, fe, stiff, mass, src, [i], [j])
            pb1 = reference_problem(parts)
            pb1.stiff, pb1.mass, pb1.f_const = float(stiff[i][j]), float(mass[i][j]), 0.0
            ref = go.assemble(pb1, fe, "full")
            for A, B in zip(blk, ref):
                assert np.array_equal(A.rowptr, B.rowptr) and np.array_equal(A.colidx, B.colidx)
                assert np.array_equal(A.col_ghost_gids, B.col_ghost_gids)
                assert np.array_equal(A.vals, B.vals)
        # the field's right-hand side: src_i (int v) minus the lifting with the row's tables
        blk = go.assemble_multifield(pb, fe, stiff, mass, src, [i], [i])
        pb1 = reference_problem(parts)
        pb1.stiff, pb1.mass, pb1.f_const = float(sum(stiff[i])), float(sum(mass[i])), src[i]
        ref = go.assemble(pb1, fe, "full")
        for A, B in zip(blk, ref):
            assert np.allclose(A.b, B.b, rtol=0, atol=1e-13)


@pytest.mark.parametrize("parts", [(2, 2), (3, 1)])
def test_multifield_gids(parts):
    pb = reference_problem(parts)
    fe = go.build_fespace(pb)
    for nf in (1, 2, 3):
        g = go.multifield_gids(fe, nf)
        n = fe.dofs[0].ngdofs
        assert g[0].ngdofs == nf * n
        own = np.concatenate([d.own_to_global for d in g])
        assert np.array_equal(own, np.arange(nf * n))          # part-contiguous, field by field
        for p, d in enumerate(g):
            nfree = len(fe.dofs[p].ldof_to_gdof)
            for f in range(nf):
                for l in range(nfree):
                    sg = int(fe.dofs[p].ldof_to_gdof[l])
                    assert d.ldof_to_gdof[f * nfree + l] == group_gid(fe, nf, f, sg)
        if nf == 1:
            for p in range(len(g)):
                assert np.array_equal(g[p].ldof_to_gdof, fe.dofs[p].ldof_to_gdof)


@pytest.mark.parametrize("parts", [(2, 2), (2, 1), (1, 2)])
@pytest.mark.parametrize("nf", [2, 3])
def test_sub_assembled_rows_multifield(parts, nf):
    """SubAssembledRows (the reference's default for multi-field assemblers): the owned rows
    give the FullyAssembledRows operator, ghost rows are explicit zeros over the row fields'
    copies of the scalar ghost rows, and each field's ghost columns keep the scalar
    SubAssembledRows first-appearance order."""
    pb = reference_problem(parts)
    fe = go.build_fespace(pb)
    stiff, mass, src = FORMS[nf]
    allf = list(range(nf))
    fa = go.assemble_multifield(pb, fe, stiff, mass, src, allf, allf, strategy="full")
    sa = go.assemble_multifield(pb, fe, stiff, mass, src, allf, allf, strategy="sub")
    x = np.random.default_rng(5).normal(size=nf * fe.dofs[0].ngdofs)
    y_fa, y_sa = global_mul(fa, x), global_mul_owned(sa, x)
    assert all(abs(y_fa[k] - y_sa[k]) <= 1e-12 * max(1.0, abs(y_fa[k])) for k in y_fa)
    assert rhs_map(fa) == pytest.approx(rhs_map_owned(sa), rel=1e-13, abs=1e-13)
    scalar = go.assemble(pb, fe, "sub")
    for p, (M, Sc) in enumerate(zip(sa, scalar)):
        nown = len(M.row_own_gids)
        assert np.all(M.vals[M.rowptr[nown]:] == 0.0) and np.all(M.b[nown:] == 0.0)
        want_rows = np.concatenate([[group_gid(fe, nf, jj, g) for g in Sc.row_ghost_gids] for jj in range(nf)])
        assert np.array_equal(M.row_ghost_gids, want_rows.astype(np.int64))
        for jj in range(nf):
            mine = [g for g in M.col_ghost_gids if any(group_gid(fe, nf, jj, s) == g for s in Sc.col_ghost_gids)]
            want = [group_gid(fe, nf, jj, s) for s in Sc.col_ghost_gids]
            assert mine == want


def global_mul_owned(mats, x):
    y = {}
    for M in mats:
        cols = np.concatenate([M.col_own_gids, M.col_ghost_gids])
        for r in range(len(M.row_own_gids)):
            y[int(M.row_own_gids[r])] = sum(M.vals[e] * x[cols[M.colidx[e]]] for e in range(M.rowptr[r], M.rowptr[r + 1]))
    return y


def rhs_map_owned(mats):
    return {int(g): float(b) for M in mats for g, b in zip(M.row_own_gids, M.b[:len(M.row_own_gids)])}
