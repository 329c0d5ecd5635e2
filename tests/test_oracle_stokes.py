"""The oracle's restatement of the multi-field test with fields on different spaces
(test/MultiFieldTests.jl:14-57: vector Q2 velocity, discontinuous P1 pressure with the
zero-mean constraint, a Stokes form), checked on the CPU against that test's known
answers: the L2 errors of the solved velocity and pressure below 1e-9.  Also: the
corrected pressure has zero mean, and the result does not depend on which pressure DOF
the zero-mean space fixes (the mean correction removes the constant)."""
import numpy as np
import pytest

import stokes_oracle as so


def _case(domain):
    x0, x1, y0, y1 = domain
    mean = 0.5 * (x0 + x1) + 0.5 * (y0 + y1)   # mean of x + y over the rectangle
    u = lambda x, y: ((x + y) ** 2, (x - y) ** 2)
    p = lambda x, y: x + y - mean
    f = lambda x, y: (-4.0 + 1.0, -4.0 + 1.0)   # -lap u + grad p
    g = lambda x, y: 4.0 * y                     # div u
    return u, p, f, g


@pytest.mark.parametrize("n,domain", [((4, 4), (0.0, 4.0, 0.0, 4.0)),        # the reference test's mesh
                                      ((6, 5), (0.0, 1.5, -1.0, 0.25))],
                         ids=["reference_4x4", "rect_6x5"])
def test_stokes_known_answer(n, domain):
    u, p, f, g = _case(domain)
    S = so.stokes_system(n, domain, 2, u, p, f, g)
    uv, pv = so.stokes_solve(S)
    eu, ep = so.stokes_l2_errors(S, uv, pv, u, p)
    assert eu < 1e-9 and ep < 1e-9
    assert abs(float(pv @ S.dvol)) <= 1e-12 * S.vol   # zero mean after the correction


def test_stokes_mean_correction_is_independent_of_the_fixed_dof():
    """Fixing another pressure DOF (the first, or one in the middle) gives the same velocity
    and, after the mean correction, the same pressure."""
    domain = (0.0, 4.0, 0.0, 4.0)
    u, p, f, g = _case(domain)
    S = so.stokes_system((4, 4), domain, 2, u, p, f, g)
    uv, pv = so.stokes_solve(S)
    for other in (0, 23):
        T = so.stokes_system((4, 4), domain, 2, u, p, f, g, p_fixed=other)
        uv2, pv2 = so.stokes_solve(T)
        assert np.abs(uv2 - uv).max() <= 1e-11 * np.abs(uv).max()
        assert np.abs(pv2 - pv).max() <= 1e-11 * np.abs(pv).max()


def _gather(mats, ng):
    import scipy.sparse as sp
    I, J, V = [], [], []
    b = np.zeros(ng)
    for M in mats:
        cols = np.concatenate([M.col_own_gids, M.col_ghost_gids])
        nown = len(M.row_own_gids)
        for r in range(nown):
            for e in range(M.rowptr[r], M.rowptr[r + 1]):
                I.append(int(M.row_own_gids[r]))
                J.append(int(cols[M.colidx[e]]))
                V.append(M.vals[e])
        b[M.row_own_gids] = M.b[:nown]
    return sp.csr_matrix((V, (I, J)), shape=(ng, ng)), b


@pytest.mark.parametrize("parts,n,domain", [((1, 1), (4, 4), (0.0, 4.0, 0.0, 4.0)),
                                            ((2, 1), (4, 4), (0.0, 4.0, 0.0, 4.0)),
                                            ((2, 2), (4, 4), (0.0, 4.0, 0.0, 4.0)),
                                            ((3, 2), (6, 5), (0.0, 1.5, -1.0, 0.25))],
                         ids=["p1x1", "p2x1", "p2x2", "p3x2_rect"])
def test_stokes_distributed_matches_serial(parts, n, domain):
    """The distributed restatement (vector Q2 and zero-mean discontinuous P1 spaces on the
    Cartesian partition, their multi-field numbering, SubAssembledRows local parts) gathers
    to the serial system that the known answers pin: same fixed pressure DOF, owned rows
    equal entry by entry under the gid -> serial map (1e-12 of the largest entry), the same
    right-hand side, ghost rows holding explicit zeros only, part-contiguous gids, and the
    gathered solve reproduces the known answers."""
    import scipy.sparse.linalg as spla
    u, p, f, g = _case(domain)
    S = so.stokes_system(n, domain, 2, u, p, f, g)
    D = so.stokes_parts(parts, n, 2)
    assert (D.pfix_cell, D.pfix_m) == (n[0] * n[1] - 1, 2)
    ng = D.mf[0].ngdofs
    assert ng == S.A.shape[0]
    first = 0
    for d in D.mf:   # owned gids are consecutive per part, parts in order
        own = np.sort(d.own_to_global)
        assert np.array_equal(own, np.arange(first, first + len(own)))
        first += len(own)
    mats = so.stokes_sub_assembled(D, domain, 2, u, f, g)
    for M in mats:
        nown = len(M.row_own_gids)
        assert np.all(M.vals[M.rowptr[nown]:] == 0.0)
    Ad, bd = _gather(mats, ng)
    s = so.stokes_gid_to_serial(D, 2)
    assert len(np.unique(s)) == ng
    As = S.A.tocsr()[s][:, s]
    scale = np.abs(As).max()
    assert abs(Ad - As).max() <= 1e-12 * scale
    assert np.abs(bd - S.b[s]).max() <= 1e-12 * max(np.abs(S.b).max(), 1.0)
    x = spla.splu(Ad.tocsc()).solve(bd)
    xs = np.zeros(ng)
    xs[s] = x
    uv = S.u_dir.copy()
    free = S.vel_free >= 0
    uv[free] = xs[S.vel_free[free]]
    ndof_p = len(S.dvol)
    pv = np.zeros(ndof_p)
    pv[np.delete(np.arange(ndof_p), S.p_fixed)] = xs[S.nu_free:]
    pv += -float(pv @ S.dvol) / S.vol
    eu, ep = so.stokes_l2_errors(S, uv, pv, u, p)
    assert eu < 1e-9 and ep < 1e-9
