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


SA_CASES = [((2, 2), (4, 4), 1), ((3, 1), (5, 3), 2), ((2, 1, 2), (3, 2, 3), 1), ((1, 2, 2), (2, 3, 2), 1)]


@pytest.mark.parametrize("parts,n,k", SA_CASES)
def test_dg_sub_assembled_rows_parts(parts, n, k):
    """SubAssembledRows local parts of the SIPG system: the owned rows give the same
    operator as FullyAssembledRows, ghost rows hold explicit zeros only and are the dofs of
    the ghost cells just below the owned box (the faces a part owns are those whose cell
    with the larger global id it owns), and the ghost columns come in first-appearance
    order: those ghost cells by local id, then the ghost cells just above the owned box,
    owner by owner in ascending order, lexicographic within an owner."""
    dim = len(n)
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.5 * d))
    u = (lambda x, y: x * y + 1.0) if dim == 2 else (lambda x, y, z: x * y + z)
    g = (lambda x, y, nx, ny: x - ny) if dim == 2 else (lambda x, y, z, nx, ny, nz: x - ny + nz)
    ds = (1, 0) * dim
    ns = (0, 1) * dim
    args = (parts, n, domain, k, 2 * k, 6.0, 0.7, 1.5, ds, ns, u, g)
    fa, gid0, ndofs = go.dg_system(*args, strategy="full")
    sa, gid0b, _ = go.dg_system(*args, strategy="sub")
    assert np.array_equal(gid0, gid0b)
    A_fa, b_fa = go.gather_global(fa, ndofs)
    A_sa, b_sa = go.gather_global(sa, ndofs)
    assert abs(A_fa - A_sa).max() <= 1e-12 * abs(A_fa).max()
    assert np.abs(b_fa - b_sa).max() <= 1e-12 * np.abs(b_fa).max()
    P = go.make_partition(parts, n)
    nn = (k + 1) ** dim
    for p, M in enumerate(sa):
        nown = len(M.row_own_gids)
        ghost_vals = M.vals[M.rowptr[nown]:]
        assert np.all(ghost_vals == 0.0) and np.all(M.b[nown:] == 0.0)
        lcells = [int(c) for c in P.local_cells(p)]
        own = [c for c in lcells if P.cell_owner(P.cell_coords(c)) == p]
        own_set = set(own)

        def neighbour(c, d, s):
            ci = list(P.cell_coords(c)); ci[d] += s
            return P.cell_gid(tuple(ci)) if 0 <= ci[d] < n[d] else None
        lower = [c for c in lcells if c not in own_set and any(neighbour(c, d, +1) in own_set for d in range(dim))]
        upper = [c for c in lcells if c not in own_set and any(neighbour(c, d, -1) in own_set for d in range(dim))]
        upper.sort(key=lambda c: (P.cell_owner(P.cell_coords(c)), c))
        dofs = lambda cells: np.concatenate([np.arange(gid0[c], gid0[c] + nn) for c in cells]) if cells else \
            np.zeros(0, dtype=np.int64)
        assert np.array_equal(M.row_ghost_gids, dofs(lower)), f"ghost rows part {p}"
        assert np.array_equal(M.col_ghost_gids, dofs(lower + upper)), f"ghost cols part {p}"
