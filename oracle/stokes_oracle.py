"""CPU oracle for the reference's multi-field test with fields on different spaces.

TEST INFRASTRUCTURE ONLY: nothing in the shipped library imports this module.

``test/MultiFieldTests.jl:14-81`` assembles and solves a Stokes problem on a 2D
``CartesianDiscreteModel`` (domain (0,4)^2, 4x4 cells):

* velocity: vector-valued Lagrangian Q_k (k = 2), Dirichlet on the whole boundary with
  u = ((x+y)^2, (x-y)^2) (``:25, :28, :35``);
* pressure: scalar Lagrangian of order k-1 on the P space (``space=:P``), discontinuous,
  with the zero-mean constraint (``constraint=:zeromean``, ``:26, :36``), exact
  p = x + y - mean(x + y);
* a((u,p),(v,q)) = int(grad v : grad u - q div u - div v p), l((v,q)) = int(v.f - q g) with
  f = -lap u + grad p and g = div u (``:32-33, :49-50``), quadrature degree 2k (``:24``);
* its known answers: the L2 errors of the solved u and p below 1e-9 (``:54-57``).

The zero-mean space is ``FESpaceWithConstantFixed`` on the last free DOF of the
pressure space (``src/FESpaces.jl:872-910``) plus the mean correction of
``FEFunction`` (``src/FESpaces.jl:912-941, 958-975``): the fixed DOF takes the value 0,
the system is solved for the others, and then every pressure DOF (the fixed one too) is
shifted by c = -(sum_i p_i int(psi_i)) / |Omega| (``_compute_new_fixedval``).

Restated here on the gathered (serial) system, which is what the known answers pin:
velocity DOFs 2 per node of the k-refined node lattice (x fastest), pressure DOFs 3 per
cell (cells x fastest).  The discontinuous P1 element of Gridap's ``space=:P`` on a
square (Gridap.jl 0.20, third party): the monomials 1, x, y with nodal DOFs at the
exponent points (0,0), (1,0), (0,1) of the reference square, in that order; the
fixed DOF (the last free one) is then the third DOF of the last cell.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gridap_oracle import gauss_legendre, lagrange_1d, quad_points_per_dir


@dataclass
class StokesSystem:
    A: sp.csr_matrix          # free velocity DOFs, then the free pressure DOFs
    b: np.ndarray
    nu_free: int              # free velocity DOFs
    vel_free: np.ndarray      # global velocity DOF -> free index (-1: Dirichlet)
    u_dir: np.ndarray         # value of every velocity DOF (Dirichlet values, 0 elsewhere)
    p_fixed: int              # the pressure DOF fixed by the zero-mean space
    dvol: np.ndarray          # int(psi_i) over the domain, per pressure DOF
    vol: float
    n: tuple
    domain: tuple
    k: int


def _p1_square(xi, eta):
    """Nodal P1 basis on the reference square for the nodes (0,0), (1,0), (0,1) and its
    reference gradients."""
    val = np.array([1.0 - xi - eta, xi, eta])
    grd = np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])
    return val, grd


def _cell_tables(k, h, degree):
    """Tensor Gauss points of one cell: weights (with |J|), reference coordinates, the
    velocity shape values / physical gradients (cell-local nodes lexicographic, x fastest)
    and the pressure basis values."""
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    V, D = lagrange_1d(k, xq)
    pts = [(a, b) for b in range(nq) for a in range(nq)]   # x fastest
    nn = (k + 1) ** 2
    W = np.zeros(len(pts))
    xi = np.zeros((len(pts), 2))
    phi = np.zeros((len(pts), nn))
    gphi = np.zeros((len(pts), nn, 2))
    psi = np.zeros((len(pts), 3))
    for q, (a, b) in enumerate(pts):
        W[q] = wq[a] * wq[b] * h[0] * h[1]
        xi[q] = (xq[a], xq[b])
        for j in range(k + 1):
            for i in range(k + 1):
                n_ = i + (k + 1) * j
                phi[q, n_] = V[a, i] * V[b, j]
                gphi[q, n_, 0] = D[a, i] * V[b, j] / h[0]
                gphi[q, n_, 1] = V[a, i] * D[b, j] / h[1]
        psi[q], _ = _p1_square(xq[a], xq[b])
    return W, xi, phi, gphi, psi


def stokes_system(n=(4, 4), domain=(0.0, 4.0, 0.0, 4.0), k=2, u=None, p=None, f=None, g=None,
                  p_fixed=None) -> StokesSystem:
    """The gathered Stokes system of test/MultiFieldTests.jl on a Cartesian mesh (free
    unknowns only: the velocity's Dirichlet values lifted to the right-hand side, the
    zero-mean space's fixed pressure DOF removed).  p_fixed: the pressure DOF to fix
    (default the last one, as the reference's zero-mean space does)."""
    x0, x1, y0, y1 = domain
    h = ((x1 - x0) / n[0], (y1 - y0) / n[1])
    degree = 2 * k
    W, xi, phi, gphi, psi = _cell_tables(k, h, degree)
    N0, N1 = k * n[0] + 1, k * n[1] + 1
    nnode = N0 * N1
    ndof_u = 2 * nnode
    ncell = n[0] * n[1]
    ndof_p = 3 * ncell
    # Dirichlet velocity DOFs: every boundary node, both components
    boundary = np.zeros(nnode, dtype=bool)
    for Y in range(N1):
        for X in range(N0):
            if X in (0, N0 - 1) or Y in (0, N1 - 1):
                boundary[X + N0 * Y] = True
    u_dir = np.zeros(ndof_u)
    for Y in range(N1):
        for X in range(N0):
            if boundary[X + N0 * Y]:
                xy = (x0 + X * h[0] / k, y0 + Y * h[1] / k)
                uv = u(*xy)
                u_dir[2 * (X + N0 * Y)] = uv[0]
                u_dir[2 * (X + N0 * Y) + 1] = uv[1]
    vel_free = -np.ones(ndof_u, dtype=np.int64)
    nu_free = 0
    for node in range(nnode):
        if not boundary[node]:
            vel_free[2 * node] = nu_free
            vel_free[2 * node + 1] = nu_free + 1
            nu_free += 2
    if p_fixed is None:
        p_fixed = ndof_p - 1   # the last free DOF of the pressure space
    pres_free = np.arange(ndof_p, dtype=np.int64)
    pres_free[p_fixed] = -1
    pres_free[p_fixed + 1:] -= 1
    nfree = nu_free + ndof_p - 1
    I, J, Vv = [], [], []
    b = np.zeros(nfree)
    dvol = np.zeros(ndof_p)
    nn = (k + 1) ** 2
    for cy in range(n[1]):
        for cx in range(n[0]):
            c = cx + n[0] * cy
            nodes = [(k * cx + i) + N0 * (k * cy + j) for j in range(k + 1) for i in range(k + 1)]
            udofs = [2 * nd + a for a in range(2) for nd in nodes]   # component-major in the cell
            pdofs = [3 * c + m for m in range(3)]
            # element matrix over (u component-major, p)
            Ke = np.zeros((2 * nn + 3, 2 * nn + 3))
            fe = np.zeros(2 * nn + 3)
            for q in range(len(W)):
                xq = (x0 + (cx + xi[q, 0]) * h[0], y0 + (cy + xi[q, 1]) * h[1])
                G = gphi[q]
                lap = G @ G.T
                for a in range(2):
                    Ke[a * nn:(a + 1) * nn, a * nn:(a + 1) * nn] += W[q] * lap
                    # -q div u and -div v p
                    Ke[2 * nn:, a * nn:(a + 1) * nn] -= W[q] * np.outer(psi[q], G[:, a])
                    Ke[a * nn:(a + 1) * nn, 2 * nn:] -= W[q] * np.outer(G[:, a], psi[q])
                fv = f(*xq)
                for a in range(2):
                    fe[a * nn:(a + 1) * nn] += W[q] * fv[a] * phi[q]
                fe[2 * nn:] -= W[q] * g(*xq) * psi[q]
                dvol[pdofs] += W[q] * psi[q]
            # global free indices of the element's DOFs (-1: Dirichlet velocity or fixed pressure)
            gidx = [vel_free[d] for d in udofs] + [nu_free + pres_free[d] if pres_free[d] >= 0 else -1 for d in pdofs]
            dval = np.array([u_dir[d] if vel_free[d] < 0 else 0.0 for d in udofs] + [0.0, 0.0, 0.0])
            fe = fe - Ke @ dval   # lifting of the Dirichlet velocity values (the fixed pressure is 0)
            for i_, gi in enumerate(gidx):
                if gi < 0:
                    continue
                b[gi] += fe[i_]
                for j_, gj in enumerate(gidx):
                    if gj >= 0 and Ke[i_, j_] != 0.0:
                        I.append(gi)
                        J.append(gj)
                        Vv.append(Ke[i_, j_])
    A = sp.csr_matrix((Vv, (I, J)), shape=(nfree, nfree))
    return StokesSystem(A=A, b=b, nu_free=nu_free, vel_free=vel_free, u_dir=u_dir, p_fixed=p_fixed,
                        dvol=dvol, vol=(x1 - x0) * (y1 - y0), n=tuple(n), domain=tuple(domain), k=k)


def stokes_solve(S: StokesSystem):
    """Solve the gathered system (sparse LU, as the reference's BackslashSolver on the
    gathered matrix) and return (velocity DOF values, pressure DOF values) with the
    zero-mean correction applied."""
    x = spla.splu(S.A.tocsc()).solve(S.b)
    uvals = S.u_dir.copy()
    free = S.vel_free >= 0
    uvals[free] = x[S.vel_free[free]]
    ndof_p = len(S.dvol)
    pvals = np.zeros(ndof_p)
    pfree = np.delete(np.arange(ndof_p), S.p_fixed)
    pvals[pfree] = x[S.nu_free:]
    c = -float(pvals @ S.dvol) / S.vol   # the fixed DOF holds 0
    return uvals, pvals + c


def stokes_l2_errors(S: StokesSystem, uvals, pvals, u, p, degree=None):
    """sqrt(sum(int((u-uh).(u-uh)))) and the same for p, with the test's quadrature."""
    k = S.k
    x0, x1, y0, y1 = S.domain
    n = S.n
    h = ((x1 - x0) / n[0], (y1 - y0) / n[1])
    W, xi, phi, gphi, psi = _cell_tables(k, h, 2 * k if degree is None else degree)
    N0 = k * n[0] + 1
    eu = ep = 0.0
    for cy in range(n[1]):
        for cx in range(n[0]):
            c = cx + n[0] * cy
            nodes = [(k * cx + i) + N0 * (k * cy + j) for j in range(k + 1) for i in range(k + 1)]
            u0 = uvals[[2 * nd for nd in nodes]]
            u1 = uvals[[2 * nd + 1 for nd in nodes]]
            pc = pvals[3 * c:3 * c + 3]
            for q in range(len(W)):
                xq = (x0 + (cx + xi[q, 0]) * h[0], y0 + (cy + xi[q, 1]) * h[1])
                ue = u(*xq)
                d0 = ue[0] - phi[q] @ u0
                d1 = ue[1] - phi[q] @ u1
                eu += W[q] * (d0 * d0 + d1 * d1)
                dp = p(*xq) - psi[q] @ pc
                ep += W[q] * dp * dp
    return float(np.sqrt(eu)), float(np.sqrt(ep))


# --------------------------------------------------------------------------------------
# Distributed: the multi-field space of two different spaces on the Cartesian partition
# --------------------------------------------------------------------------------------
import gridap_oracle as _go   # noqa: E402  (helpers of the single-space restatement)


@dataclass
class StokesParts:
    P: object                 # gridap_oracle.Partition
    vspaces: list             # velocity LocalSpace per part (vector Q_k)
    pspaces: list             # pressure LocalSpace per part (after the zero-mean fix)
    vdofs: list               # velocity DofIndices per part
    pdofs: list               # pressure DofIndices per part
    mf: list                  # multi-field DofIndices per part (velocity lids, then pressure lids)
    pfix_gid: int             # the pressure gid the zero-mean space fixed (before renumbering)
    pfix_cell: int            # ... its global cell and its P1 DOF there
    pfix_m: int


def _pressure_local_space(P, p, fixed_lid=None):
    """The discontinuous P1 space on part p's local cells: 3 DOFs per cell, cells in local
    order, each cell's DOFs in basis order; every DOF is the cell's own (L2 conformity).
    fixed_lid: the local DOF the zero-mean space fixes here (FESpaceWithConstantFixed:
    it becomes the Dirichlet DOF -1 and the free DOFs after it move down by one)."""
    cells = P.local_cells(p)
    n = 3 * len(cells)
    lid = np.arange(n, dtype=np.int64)
    if fixed_lid is not None:
        lid = np.where(lid > fixed_lid, lid - 1, lid)
        lid[fixed_lid] = -1
    return _go.LocalSpace(part=p, box_lo=tuple(P.loc_lo[p]), box_hi=tuple(P.loc_hi[p]), cells=cells,
                          cell_dofs=lid.reshape(-1, 3), dof_node=np.zeros((n, P.dim), dtype=np.int64),
                          dof_comp=np.zeros(n, dtype=np.int64), dir_node=np.zeros((0, P.dim), dtype=np.int64),
                          dir_comp=np.zeros(0, dtype=np.int64), nfree=n - (fixed_lid is not None),
                          ndir=int(fixed_lid is not None))


def _multifield_gids_of(field_dofs):
    """generate_multi_field_gids (src/MultiField.jl:356-420) for fields on different spaces
    (ConsecutiveMultiFieldStyle): a part's local ids are its fields' free local ids one
    field after the other; each part numbers its owned DOFs field by field from the
    exclusive scan of the parts' owned counts; ghosts get the owner's number through each
    field's own ghost exchange (propagate_to_ghost_multifield!, :422-451)."""
    nparts = len(field_dofs[0])
    noids = [sum(fd[p].n_own for fd in field_dofs) for p in range(nparts)]
    firstgid = np.concatenate([[0], np.cumsum(noids)[:-1]]).astype(np.int64)
    offs = [[0] * len(field_dofs) for _ in range(nparts)]
    for p in range(nparts):
        o = 0
        for f, fd in enumerate(field_dofs):
            offs[p][f] = o
            o += len(fd[p].ldof_to_gdof)
    lid_gid, lid_part = [], []
    for p in range(nparts):
        nl = sum(len(fd[p].ldof_to_gdof) for fd in field_dofs)
        g = np.full(nl, -1, dtype=np.int64)
        o = np.zeros(nl, dtype=np.int32)
        gid = firstgid[p]
        for f, fd in enumerate(field_dofs):
            d = fd[p]
            for flid in np.nonzero(d.own_mask)[0]:
                g[offs[p][f] + flid] = gid
                gid += 1
            o[offs[p][f]:offs[p][f] + len(d.ldof_to_gdof)] = d.ldof_to_owner
        lid_gid.append(g)
        lid_part.append(o)
    for f, fd in enumerate(field_dofs):
        g2l = [{int(x): i for i, x in enumerate(d.ldof_to_gdof)} for d in fd]
        for p in range(nparts):
            d = fd[p]
            for flid in d.ghost_lids:
                q = int(d.ldof_to_owner[flid])
                qlid = g2l[q][int(d.ldof_to_gdof[flid])]
                lid_gid[p][offs[p][f] + flid] = lid_gid[q][offs[q][f] + qlid]
    ng = int(sum(noids))
    out = [_go.DofIndices(p, ng, lid_gid[p], lid_part[p]) for p in range(nparts)]
    for d in out:
        assert (d.ldof_to_gdof >= 0).all()
    return out


def stokes_parts(np_, n, k=2) -> StokesParts:
    """The distributed spaces of test/MultiFieldTests.jl: V (vector Q_k, Dirichlet on the
    whole boundary), Q (discontinuous P1 with the zero-mean constraint: the last free gid
    fixed on every part that holds it, FESpaces.jl:872-892, then generate_gids again on
    the fixed local spaces) and the multi-field numbering of [V, Q]."""
    P = _go.make_partition(np_, n)
    sides = (1,) * (2 * P.dim)
    vspaces = [_go.build_local_space(P, p, k, P.dim, sides) for p in range(P.nparts)]
    vdofs, _ = _go.generate_gids(P, vspaces)
    q0 = [_pressure_local_space(P, p) for p in range(P.nparts)]
    qd0, _ = _go.generate_gids(P, q0)
    fix = qd0[0].ngdofs - 1
    pspaces = []
    fcell = fm = -1
    for p in range(P.nparts):
        hit = np.nonzero(qd0[p].ldof_to_gdof == fix)[0]
        lid = int(hit[0]) if len(hit) else None
        if lid is not None:
            fcell, fm = int(q0[p].cells[lid // 3]), lid % 3
        pspaces.append(_pressure_local_space(P, p, lid))
    pdofs, _ = _go.generate_gids(P, pspaces)
    mf = _multifield_gids_of([vdofs, pdofs])
    return StokesParts(P, vspaces, pspaces, vdofs, pdofs, mf, fix, fcell, fm)


def _stokes_cell_tables(k, h, degree):
    """Reference blocks of one cell in Gridap's local orders: velocity DOFs component-major
    over the cell's nodes in Gridap's node order (cell_local_nodes), pressure DOFs in basis
    order.  Returns the point tables too, for the load vectors."""
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    V, D = lagrange_1d(k, xq)
    lnodes = _go.cell_local_nodes(2, k)
    nn = len(lnodes)
    pts = [(a, b) for b in range(nq) for a in range(nq)]
    W = np.array([wq[a] * wq[b] * h[0] * h[1] for (a, b) in pts])
    xi = np.array([(xq[a], xq[b]) for (a, b) in pts])
    phi = np.array([[V[a, o[0]] * V[b, o[1]] for o in lnodes] for (a, b) in pts])
    gx = np.array([[D[a, o[0]] * V[b, o[1]] / h[0] for o in lnodes] for (a, b) in pts])
    gy = np.array([[V[a, o[0]] * D[b, o[1]] / h[1] for o in lnodes] for (a, b) in pts])
    psi = np.array([_p1_square(xq[a], xq[b])[0] for (a, b) in pts])
    Kuu = np.zeros((2 * nn, 2 * nn))
    Kpu = np.zeros((3, 2 * nn))
    for q in range(len(pts)):
        lap = np.outer(gx[q], gx[q]) + np.outer(gy[q], gy[q])
        for c, gc in enumerate((gx[q], gy[q])):
            Kuu[c * nn:(c + 1) * nn, c * nn:(c + 1) * nn] += W[q] * lap
            Kpu[:, c * nn:(c + 1) * nn] -= W[q] * np.outer(psi[q], gc)
    return Kuu, Kpu, Kpu.T.copy(), W, xi, phi, psi, lnodes


def stokes_sub_assembled(S: StokesParts, domain, k, u, f, g):
    """SubAssembledRows local parts of the Stokes system (Algebra.jl:593-646 over the
    multi-field index sets), as gridap_oracle._multifield_sub_assembled does for fields on
    one space: owned cells only, the cell's block matrix walked block column outer and block
    row inner over the touched blocks (uu, pu, up; the pp block has no term), each block
    column-major, Dirichlet and fixed DOFs skipped; ghost-row triplets zeroed, sent to the
    owner and appended there; rows owned then touched ghosts, columns owned then ghosts in
    first appearance; b complete on owned rows."""
    P = S.P
    n = P.n
    x0, x1, y0, y1 = domain
    h = ((x1 - x0) / n[0], (y1 - y0) / n[1])
    Kuu, Kpu, Kup, W, xi, phi, psi, lnodes = _stokes_cell_tables(k, h, 2 * k)
    nn = len(lnodes)
    blocks = {(0, 0): Kuu, (1, 0): Kpu, (0, 1): Kup}
    N0 = k * n[0] + 1
    nrg = S.mf[0].ngdofs
    bglob = np.zeros(nrg)
    coo = []
    for p in range(P.nparts):
        vs, ps = S.vspaces[p], S.pspaces[p]
        nv = vs.nfree
        lg = S.mf[p].ldof_to_gdof
        I, J, V = [], [], []
        for ic, gcell in enumerate(vs.cells):
            ci = P.cell_coords(int(gcell))
            if P.cell_owner(ci) != p:
                continue
            vd = vs.cell_dofs[ic]                      # velocity cell DOFs (component-major)
            pd = ps.cell_dofs[ic]
            ids = [np.where(vd >= 0, vd, -1), np.where(pd >= 0, nv + pd, -1)]
            for jb in (0, 1):                          # block columns outer
                for ib in (0, 1):                      # block rows inner
                    Ke = blocks.get((ib, jb))
                    if Ke is None:
                        continue
                    ri, cj = ids[ib], ids[jb]
                    for c in range(len(cj)):
                        if cj[c] < 0:
                            continue
                        for a in range(len(ri)):
                            if ri[a] < 0:
                                continue
                            I.append(int(ri[a])); J.append(int(cj[c])); V.append(Ke[a, c])
            # load vector and the lifting of the Dirichlet velocity values
            fu = np.zeros(2 * nn)
            fp = np.zeros(3)
            for q in range(len(W)):
                xq = (x0 + (ci[0] + xi[q, 0]) * h[0], y0 + (ci[1] + xi[q, 1]) * h[1])
                fv = f(*xq)
                for c in range(2):
                    fu[c * nn:(c + 1) * nn] += W[q] * fv[c] * phi[q]
                fp -= W[q] * g(*xq) * psi[q]
            ud = np.zeros(2 * nn)
            for c in range(2):
                for a, off in enumerate(lnodes):
                    if vd[c * nn + a] < 0:
                        X = (k * ci[0] + off[0], k * ci[1] + off[1])
                        ud[c * nn + a] = u(x0 + X[0] * h[0] / k, y0 + X[1] * h[1] / k)[c]
            fu = fu - Kuu @ ud
            fp = fp - Kpu @ ud
            for a in range(2 * nn):
                if vd[a] >= 0:
                    bglob[lg[vd[a]]] += fu[a]
            for m in range(3):
                if pd[m] >= 0:
                    bglob[lg[nv + pd[m]]] += fp[m]
        I = np.array(I, dtype=np.int64); J = np.array(J, dtype=np.int64)
        coo.append((lg[I], lg[J], np.array(V, dtype=np.float64)))
    owner = {}
    for p in range(P.nparts):
        for gg, o in zip(S.mf[p].ldof_to_gdof, S.mf[p].ldof_to_owner):
            owner[int(gg)] = int(o)
    sent, kept = {}, []
    for p in range(P.nparts):
        Ig, Jg, Vv = coo[p]
        Vk = Vv.copy()
        for t in range(len(Ig)):
            q = owner[int(Ig[t])]
            if q != p:
                sent.setdefault((p, q), []).append((int(Ig[t]), int(Jg[t]), float(Vv[t])))
                Vk[t] = 0.0
        kept.append((Ig, Jg, Vk))
    out = []
    for p in range(P.nparts):
        Ig, Jg, Vv = kept[p]
        trip = list(zip(Ig.tolist(), Jg.tolist(), Vv.tolist()))
        for q in range(P.nparts):
            trip += sent.get((q, p), [])
        di = S.mf[p]
        own_g = di.own_to_global
        rlid = {int(gg): l for l, gg in enumerate(di.ldof_to_gdof)}
        ghost_rows = sorted({rlid[r] for (r, c, v) in trip if owner[r] != p})
        grow_g = np.array([int(di.ldof_to_gdof[l]) for l in ghost_rows], dtype=np.int64)
        gcol_g, seen = [], set()
        for (r, c, v) in trip:
            if owner[c] != p and c not in seen:
                seen.add(c)
                gcol_g.append(c)
        gcol_g = np.array(gcol_g, dtype=np.int64)
        rmap = {int(x): i for i, x in enumerate(own_g)}
        rmap.update({int(x): len(own_g) + i for i, x in enumerate(grow_g)})
        cmap = {int(x): i for i, x in enumerate(own_g)}
        cmap.update({int(x): len(own_g) + i for i, x in enumerate(gcol_g)})
        Il = np.array([rmap[r] for (r, c, v) in trip], dtype=np.int64)
        Jl = np.array([cmap[c] for (r, c, v) in trip], dtype=np.int64)
        Vl = np.array([v for (r, c, v) in trip], dtype=np.float64)
        nrows, ncols = len(own_g) + len(grow_g), len(own_g) + len(gcol_g)
        rowptr, colidx, vals = _go._compress(nrows, Il, Jl, Vl, ncols)
        og = lambda gs: np.array([owner[int(x)] for x in gs], dtype=np.int32)
        out.append(_go.LocalMatrix(p, nrows, ncols, rowptr, colidx, vals, own_g, grow_g, og(grow_g),
                                   own_g, gcol_g, og(gcol_g),
                                   np.concatenate([bglob[own_g], np.zeros(len(grow_g))])))
    return out


def stokes_gid_to_serial(S: StokesParts, k=2):
    """Map of every multi-field gid to the serial system's free unknown (velocity free DOFs
    in lattice order, then the pressure DOFs without the serial fixed one), so that the
    distributed and serial systems can be compared: velocity DOF (node, component), pressure
    DOF (global cell, basis index)."""
    P = S.P
    n = P.n
    N0, N1 = k * n[0] + 1, k * n[1] + 1
    vfree = {}
    c_ = 0
    for node in range(N0 * N1):
        X, Y = node % N0, node // N0
        if X in (0, N0 - 1) or Y in (0, N1 - 1):
            continue
        vfree[2 * node] = c_
        vfree[2 * node + 1] = c_ + 1
        c_ += 2
    nu = c_
    ncell = n[0] * n[1]
    out = np.full(S.mf[0].ngdofs, -1, dtype=np.int64)
    for p in range(P.nparts):
        vs, ps = S.vspaces[p], S.pspaces[p]
        nv = vs.nfree
        lg = S.mf[p].ldof_to_gdof
        for lid in range(nv):
            X = vs.dof_node[lid]
            node = int(X[0] + N0 * X[1])
            out[lg[lid]] = vfree[2 * node + int(vs.dof_comp[lid])]
        for ic, gcell in enumerate(ps.cells):
            for m in range(3):
                lid = ps.cell_dofs[ic, m]
                if lid < 0:
                    continue
                sdof = 3 * int(gcell) + m
                last = 3 * ncell - 1
                out[lg[nv + lid]] = nu + (sdof if sdof < last else sdof - 1)
    assert (out >= 0).all()
    return out
