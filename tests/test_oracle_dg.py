"""Discontinuous Galerkin in the oracle (CPU): the DG part of the reference's Poisson
known-answer test (test/PoissonTests.jl:47-77) -- Q2 with conformity L2 on (0,4)^2, 4x4
cells, symmetric interior penalty gamma = 10, h = 2, Nitsche Dirichlet on the bottom/left
sides, g = n.grad(u) on the top/right sides -- reproduces u = (x+y)^2 (L2 error < 1e-9)."""
import numpy as np
import pytest
import scipy.sparse as sps
import scipy.sparse.linalg as spla

import gridap_oracle as go


def kat_system(parts, k=2):
    u = lambda x, y: (x + y) ** 2
    g = lambda x, y, nx, ny: 2.0 * (x + y) * (nx + ny)
    return go.dg_system(parts, (4, 4), (0, 4, 0, 4), k, 2 * k, 10.0, 2.0, -4.0, (1, 0, 1, 0), (0, 1, 0, 1), u, g), u


def gathered(mats, ndofs):
    rows, cols, vals, b = [], [], [], np.zeros(ndofs)
    for M in mats:
        gcols = np.concatenate([M.col_own_gids, M.col_ghost_gids])
        for r in range(M.nrows):
            for e in range(M.rowptr[r], M.rowptr[r + 1]):
                rows.append(M.row_own_gids[r]); cols.append(gcols[M.colidx[e]]); vals.append(M.vals[e])
        b[M.row_own_gids] = M.b
    return sps.csr_matrix((vals, (rows, cols)), shape=(ndofs, ndofs)), b


@pytest.mark.parametrize("parts", [(1, 1), (2, 2), (2, 1), (1, 2)])
def test_dg_poisson_kat_oracle(parts):
    (mats, gid0, ndofs), u = kat_system(parts)
    A, b = gathered(mats, ndofs)
    assert abs(A - A.T).max() < 1e-12          # SIPG is symmetric
    x = spla.spsolve(A.tocsc(), b)
    assert go.dg_l2_error(parts, (4, 4), (0, 4, 0, 4), 2, 4, x, gid0, u) < 1e-9


def test_dg_numbering_is_partition_invariant():
    """The gathered operator is the same for every partition, up to the dof renumbering."""
    (m1, g1, n1), _ = kat_system((1, 1))
    (m4, g4, n4), _ = kat_system((2, 2))
    A1, b1 = gathered(m1, n1)
    A4, b4 = gathered(m4, n4)
    nn = 9
    perm = np.concatenate([np.arange(g4[c], g4[c] + nn) for c in range(16)])   # cell-major -> (2,2) gids
    base = np.concatenate([np.arange(g1[c], g1[c] + nn) for c in range(16)])
    P = sps.csr_matrix((np.ones(len(perm)), (perm, base)), shape=(n4, n1))
    assert abs(P @ A1 @ P.T - A4).max() < 1e-12
    assert np.abs(P @ b1 - b4).max() < 1e-12
