"""CPU oracle for the GridapDistributed assembly-and-solve path.

TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library imports this module:
it is the checker that the CUDA path is compared against, and (through
``oracle_core.c``) the timed CPU baseline.  Only ``tests/``, ``__graft_entry__.smoke``
and ``bench.py``'s CPU-baseline leg may use it.

It restates, in plain numpy/Python, what the reference computes on its
``with_debug`` path for a non-periodic ``CartesianDiscreteModel``:

* cell partition with a one-cell ghost layer
  (``src/PArraysExtras.jl:5-84``, ``src/Geometry.jl:378-411``);
* per-part Lagrangian Q_k DOF numbering on the owned+ghost box.  This part is
  Gridap.jl 0.20 (third party, not in the reference tree): vertices, then edges,
  then faces, then cells, each face numbered at its first appearance when the
  cells are visited in order, free DOFs positive and Dirichlet DOFs negative.
  It is restated from that published algorithm; the reference's own tests pin
  only its consequences (DOF counts, exact solutions), not the order;
* ``generate_gids`` (``src/FESpaces.jl:139-261``): owner = max owner rank of the
  cells around a DOF, owned DOFs numbered part-contiguously in local order,
  ghost ids fetched from the owners through cell-wise exchanges;
* element matrices/vectors by tensor Gauss quadrature (Gridap ``integrate``,
  called from ``src/CellData.jl:234-259``) with Dirichlet lifting;
* the COO builders and ``create_from_nz`` for both strategies
  (``src/Algebra.jl:537-646, 720-793, 919-962, 1048-1257``):
  SubAssembledRows (ghost-row triplets zeroed but kept, sent to the row owner and
  appended there; ghost columns in first-appearance order) and FullyAssembledRows
  (no ghost rows, ghost columns sorted by local DOF id);
* the gathered sparse LU behind ``\\`` (PartitionedArrays 0.3, third party) via
  scipy's SuperLU, a Jacobi-PCG in FP64, and ``consistent!`` for ``FEFunction``
  (``src/FESpaces.jl:354-371``, ``src/Algebra.jl:270-293``).

Conventions: every index here is 0-based (the reference is 1-based).  Parts are
numbered x-fastest (``CartesianIndices(np)``), cells and lattice nodes
lexicographically x-fastest.  The "node lattice" of an order-k space is the
k-refined vertex grid: global node coordinates ``X_d`` in ``[0, k*n_d]``.
"""
from __future__ import annotations

import itertools
import math
from dataclasses import dataclass, field

import numpy as np

# --------------------------------------------------------------------------------------
# A1. Cartesian cell partition (src/PArraysExtras.jl:21-84)
# --------------------------------------------------------------------------------------


def local_range(p1: int, np_: int, n: int, ghost: bool = False):
    """0-based half-open cell range of 1-based part ``p1`` along one direction.

    Restates ``_local_range`` (src/PArraysExtras.jl:72-84): ``divrem(n,np)``, the
    last ``rem`` parts get one extra cell, the ghost layer extends one cell each
    way, clamped to the mesh (non-periodic)."""
    l, rem = divmod(n, np_)
    offset = l * (p1 - 1)
    if rem >= (np_ - p1 + 1):
        l += 1
        offset += p1 - (np_ - rem) - 1
    g = 1 if ghost else 0
    start = 1 + offset - g
    stop = l + offset + g
    start = max(1, start)
    stop = min(n, stop)
    return start - 1, stop  # 0-based [lo, hi)


@dataclass
class Partition:
    """Cell partition of ``n`` cells into ``np`` parts (src/PArraysExtras.jl:21-70)."""

    np: tuple
    n: tuple
    own_lo: list = field(default_factory=list)   # per part, per dim
    own_hi: list = field(default_factory=list)
    loc_lo: list = field(default_factory=list)
    loc_hi: list = field(default_factory=list)

    @property
    def dim(self):
        return len(self.n)

    @property
    def nparts(self):
        return int(np.prod(self.np))

    def part_coords(self, p):
        c = []
        for d in range(self.dim):
            c.append(p % self.np[d])
            p //= self.np[d]
        return tuple(c)

    def part_id(self, coords):
        p = 0
        for d in reversed(range(self.dim)):
            p = p * self.np[d] + coords[d]
        return p

    def cell_part_coord(self, d, cidx):
        """Part coordinate along ``d`` owning cell index ``cidx`` (src/PArraysExtras.jl:26-36)."""
        for pc in range(self.np[d]):
            lo, hi = local_range(pc + 1, self.np[d], self.n[d])
            if lo <= cidx < hi:
                return pc
        raise ValueError("cell index out of range")

    def local_cells(self, p):
        """Global lexicographic ids of the local (owned+ghost) cells of part ``p``,
        in the local model's cell order (box lexicographic, x fastest)."""
        ranges = [range(self.loc_lo[p][d], self.loc_hi[p][d]) for d in range(self.dim)]
        out = []
        for ci in itertools.product(*reversed(ranges)):
            ci = tuple(reversed(ci))
            out.append(self.cell_gid(ci))
        return np.array(out, dtype=np.int64)

    def cell_gid(self, ci):
        g = 0
        for d in reversed(range(self.dim)):
            g = g * self.n[d] + ci[d]
        return g

    def cell_coords(self, gid):
        c = []
        for d in range(self.dim):
            c.append(gid % self.n[d])
            gid //= self.n[d]
        return tuple(c)

    def cell_owner(self, ci):
        return self.part_id(tuple(self.cell_part_coord(d, ci[d]) for d in range(self.dim)))

    def ghost_maps(self, p):
        """``ghost_to_global``, ``ghost_to_owner`` and ``perm`` of part ``p`` in the
        order produced by ``_block_with_constant_size`` (src/PArraysExtras.jl:40-69)."""
        lcells = self.local_cells(p)
        n_own = int(np.prod([self.own_hi[p][d] - self.own_lo[p][d] for d in range(self.dim)]))
        g2g, g2o, perm = [], [], np.zeros(len(lcells), dtype=np.int64)
        i_own = 0
        i_gh = 0
        for i, g in enumerate(lcells):
            ci = self.cell_coords(int(g))
            owned = all(self.own_lo[p][d] <= ci[d] < self.own_hi[p][d] for d in range(self.dim))
            if owned:
                perm[i] = i_own
                i_own += 1
            else:
                g2g.append(int(g))
                g2o.append(self.cell_owner(ci))
                perm[i] = n_own + i_gh
                i_gh += 1
        return np.array(g2g, dtype=np.int64), np.array(g2o, dtype=np.int32), perm


def make_partition(np_, n):
    """``_uniform_partition(ranks, np, n, ghost=true)`` (src/PArraysExtras.jl:5-19)."""
    P = Partition(tuple(np_), tuple(n))
    for p in range(P.nparts):
        pc = P.part_coords(p)
        ol, oh, ll, lh = [], [], [], []
        for d in range(P.dim):
            a, b = local_range(pc[d] + 1, P.np[d], P.n[d])
            c, e = local_range(pc[d] + 1, P.np[d], P.n[d], ghost=True)
            ol.append(a); oh.append(b); ll.append(c); lh.append(e)
        P.own_lo.append(ol); P.own_hi.append(oh); P.loc_lo.append(ll); P.loc_hi.append(lh)
    return P


# --------------------------------------------------------------------------------------
# A3. Reference element, local Q_k numbering (Gridap 0.20 conforming FE space)
# --------------------------------------------------------------------------------------

# Gridap polytope orderings (vertex ids lexicographic, x fastest).
QUAD_EDGES = [(0, 1), (2, 3), (0, 2), (1, 3)]
HEX_EDGES = [(0, 1), (2, 3), (4, 5), (6, 7), (0, 2), (1, 3), (4, 6), (5, 7),
             (0, 4), (1, 5), (2, 6), (3, 7)]
HEX_FACES = [(0, 1, 2, 3), (4, 5, 6, 7), (0, 1, 4, 5), (2, 3, 6, 7), (0, 2, 4, 6), (1, 3, 5, 7)]


def vertex_offsets(dim):
    return [tuple((v >> d) & 1 for d in range(dim)) for v in range(1 << dim)]


def cell_local_nodes(dim, k):
    """Cell-local node offsets (in k-refined lattice units, each in [0,k]) in Gridap's
    Lagrangian node order: vertices, then own nodes of each edge (in edge order,
    increasing along the edge), then own nodes of each face (lexicographic in the
    face's first/second axes), then the interior nodes (lexicographic)."""
    verts = vertex_offsets(dim)
    nodes = [tuple(k * c for c in v) for v in verts]
    edges = QUAD_EDGES if dim == 2 else HEX_EDGES
    for (a, b) in edges:
        va, vb = np.array(verts[a]), np.array(verts[b])
        for t in range(1, k):
            nodes.append(tuple(int(x) for x in k * va + t * (vb - va)))
    if dim == 3:
        for (a, b, c, _) in HEX_FACES:
            va, vb, vc = np.array(verts[a]), np.array(verts[b]), np.array(verts[c])
            for t in range(1, k):
                for s in range(1, k):
                    nodes.append(tuple(int(x) for x in k * va + s * (vb - va) + t * (vc - va)))
    rng = [range(1, k)] * dim
    for ci in itertools.product(*rng):
        nodes.append(tuple(reversed(ci)))
    assert len(nodes) == (k + 1) ** dim
    return nodes


@dataclass
class LocalSpace:
    """One part's local FE space on its owned+ghost box."""

    part: int
    box_lo: tuple            # cell range of the local box
    box_hi: tuple
    cells: np.ndarray        # global cell ids in local order
    cell_dofs: np.ndarray    # (ncells, ndofs_cell): free lid >= 0, Dirichlet -(d+1)
    dof_node: np.ndarray     # (nfree, dim) global lattice coords of each free dof
    dof_comp: np.ndarray     # (nfree,)
    dir_node: np.ndarray     # (ndir, dim)
    dir_comp: np.ndarray
    nfree: int
    ndir: int


def dirichlet_node(X, N, dirichlet_sides):
    """A lattice node is Dirichlet iff it lies on a flagged boundary plane.
    ``dirichlet_sides[2d]`` flags the plane x_d = 0, ``[2d+1]`` x_d = max."""
    for d in range(len(N)):
        if dirichlet_sides[2 * d] and X[d] == 0:
            return True
        if dirichlet_sides[2 * d + 1] and X[d] == N[d] - 1:
            return True
    return False


def build_local_space(P: Partition, p: int, k: int, ncomp: int, dirichlet_sides):
    """Gridap-order conforming numbering on the local box of part ``p``.

    Faces are numbered by dimension (vertices, edges, faces, cells); vertices in
    lexicographic order, higher faces at first appearance while visiting the
    cells in local order and their local faces in polytope order.  DOFs are
    numbered face by face (own nodes component-major), then split into free
    (0,1,2,...) and Dirichlet (-1,-2,...) in that same order."""
    dim = P.dim
    lo = tuple(P.loc_lo[p]); hi = tuple(P.loc_hi[p])
    m = tuple(hi[d] - lo[d] for d in range(dim))
    N = tuple(k * P.n[d] + 1 for d in range(dim))
    verts = vertex_offsets(dim)
    edges = QUAD_EDGES if dim == 2 else HEX_EDGES
    faces2 = [] if dim == 2 else HEX_FACES
    lnodes = cell_local_nodes(dim, k)

    cell_list = []
    for ci in itertools.product(*[range(m[d]) for d in reversed(range(dim))]):
        cell_list.append(tuple(reversed(ci)))

    def vid(vc):
        g = 0
        for d in reversed(range(dim)):
            g = g * (m[d] + 1) + vc[d]
        return g

    nverts = int(np.prod([mm + 1 for mm in m]))
    # face own nodes (global lattice coordinates), by face id within each dimension
    face_nodes = []   # list over faces (all dims, in dimension order) of list of lattice coords
    # vertices
    vert_nodes = [None] * nverts
    for vc in itertools.product(*[range(mm + 1) for mm in reversed(m)]):
        vc = tuple(reversed(vc))
        vert_nodes[vid(vc)] = [tuple(k * (lo[d] + vc[d]) for d in range(dim))]
    face_nodes.extend(vert_nodes)

    def first_appearance(local_faces, nown_fn):
        seen = {}
        out = []
        for ci in cell_list:
            for lf in local_faces:
                key = tuple(sorted(vid(tuple(ci[d] + verts[v][d] for d in range(dim))) for v in lf))
                if key in seen:
                    continue
                seen[key] = len(out)
                out.append(nown_fn(ci, lf))
        return out

    def edge_own(ci, e):
        a, b = e
        va, vb = np.array(verts[a]), np.array(verts[b])
        base = np.array([k * (lo[d] + ci[d]) for d in range(dim)])
        return [tuple(int(x) for x in base + k * va + t * (vb - va)) for t in range(1, k)]

    def face_own(ci, f):
        a, b, c, _ = f
        va, vb, vc = np.array(verts[a]), np.array(verts[b]), np.array(verts[c])
        base = np.array([k * (lo[d] + ci[d]) for d in range(dim)])
        return [tuple(int(x) for x in base + k * va + s * (vb - va) + t * (vc - va))
                for t in range(1, k) for s in range(1, k)]

    if k > 1:
        face_nodes.extend(first_appearance(edges, edge_own))
        if dim == 3:
            face_nodes.extend(first_appearance(faces2, face_own))
        for ci in cell_list:
            base = [k * (lo[d] + ci[d]) for d in range(dim)]
            own = []
            for off in itertools.product(*[range(1, k)] * dim):
                off = tuple(reversed(off))
                own.append(tuple(base[d] + off[d] for d in range(dim)))
            face_nodes.append(own)

    # DOFs face by face, component-major within a face, then the free/Dirichlet split
    node_comp_to_lid = {}
    dof_node, dof_comp, dir_node, dir_comp = [], [], [], []
    for fn in face_nodes:
        for c in range(ncomp):
            for X in fn:
                if dirichlet_node(X, N, dirichlet_sides):
                    dir_node.append(X); dir_comp.append(c)
                    node_comp_to_lid[(X, c)] = -len(dir_node)
                else:
                    dof_node.append(X); dof_comp.append(c)
                    node_comp_to_lid[(X, c)] = len(dof_node) - 1

    nnode = len(lnodes)
    cell_dofs = np.zeros((len(cell_list), nnode * ncomp), dtype=np.int64)
    cells = np.zeros(len(cell_list), dtype=np.int64)
    for ic, ci in enumerate(cell_list):
        gci = tuple(lo[d] + ci[d] for d in range(dim))
        cells[ic] = P.cell_gid(gci)
        for c in range(ncomp):
            for a, off in enumerate(lnodes):
                X = tuple(k * gci[d] + off[d] for d in range(dim))
                cell_dofs[ic, c * nnode + a] = node_comp_to_lid[(X, c)]
    return LocalSpace(part=p, box_lo=lo, box_hi=hi, cells=cells, cell_dofs=cell_dofs,
                      dof_node=np.array(dof_node, dtype=np.int64).reshape(-1, dim),
                      dof_comp=np.array(dof_comp, dtype=np.int64),
                      dir_node=np.array(dir_node, dtype=np.int64).reshape(-1, dim),
                      dir_comp=np.array(dir_comp, dtype=np.int64),
                      nfree=len(dof_node), ndir=len(dir_node))


# --------------------------------------------------------------------------------------
# A4. generate_gids (src/FESpaces.jl:139-261)
# --------------------------------------------------------------------------------------


@dataclass
class DofIndices:
    """``LocalIndices(ngdofs, me, ldof_to_gdof, ldof_to_owner)`` of one part (0-based)."""

    part: int
    ngdofs: int
    ldof_to_gdof: np.ndarray
    ldof_to_owner: np.ndarray

    @property
    def own_mask(self):
        return self.ldof_to_owner == self.part

    @property
    def n_own(self):
        return int(self.own_mask.sum())

    @property
    def own_to_global(self):
        return self.ldof_to_gdof[self.own_mask]

    @property
    def ghost_lids(self):
        return np.nonzero(~self.own_mask)[0]


def generate_gids(P: Partition, spaces):
    """Restates ``generate_gids`` step by step, including the three cell-wise
    owner->ghost exchanges (src/FESpaces.jl:139-261)."""
    nparts = P.nparts
    cell_owner = []
    cell_is_own = []
    gid_to_lcell = []
    for p in range(nparts):
        owners = np.array([P.cell_owner(P.cell_coords(int(g))) for g in spaces[p].cells], dtype=np.int32)
        cell_owner.append(owners)
        cell_is_own.append(owners == p)
        gid_to_lcell.append({int(g): i for i, g in enumerate(spaces[p].cells)})

    # FESpaces.jl:145-163 local max owner
    ldof_to_owner = []
    for p in range(nparts):
        s = spaces[p]
        o = np.full(s.nfree, -1, dtype=np.int32)
        for c in range(len(s.cells)):
            for ld in s.cell_dofs[c]:
                if ld >= 0:
                    o[ld] = max(o[ld], cell_owner[p][c])
        ldof_to_owner.append(o)

    def dof_to_cell(vals):
        # dof_wise_to_cell_wise! over owned cells (FESpaces.jl:70-90); -1 elsewhere
        out = []
        for p in range(nparts):
            s = spaces[p]
            cw = np.full(s.cell_dofs.shape, -1, dtype=np.int64)
            for c in np.nonzero(cell_is_own[p])[0]:
                for i, ld in enumerate(s.cell_dofs[c]):
                    if ld >= 0:
                        cw[c, i] = vals[p][ld]
            out.append(cw)
        return out

    def fetch_ghost(cw):
        # owner -> ghost copy of cell-wise data (FESpaces.jl:130-137)
        new = [a.copy() for a in cw]
        for p in range(nparts):
            for c in np.nonzero(~cell_is_own[p])[0]:
                q = int(cell_owner[p][c])
                cq = gid_to_lcell[q][int(spaces[p].cells[c])]
                new[p][c] = cw[q][cq]
        return new

    def cell_to_dof(vals, cw):
        # cell_wise_to_dof_wise! over ghost cells (FESpaces.jl:92-109)
        for p in range(nparts):
            s = spaces[p]
            for c in np.nonzero(~cell_is_own[p])[0]:
                for i, ld in enumerate(s.cell_dofs[c]):
                    if ld >= 0:
                        vals[p][ld] = cw[p][c, i]

    cw = fetch_ghost(dof_to_cell(ldof_to_owner))
    cell_to_dof(ldof_to_owner, cw)
    nodofs = [int((ldof_to_owner[p] == p).sum()) for p in range(nparts)]
    first_gdof = np.concatenate([[0], np.cumsum(nodofs)[:-1]]).astype(np.int64)
    ldof_to_gdof = []
    for p in range(nparts):
        g = np.full(spaces[p].nfree, -1, dtype=np.int64)
        own = ldof_to_owner[p] == p
        g[own] = first_gdof[p] + np.arange(int(own.sum()))
        ldof_to_gdof.append(g)
    cw = fetch_ghost(dof_to_cell(ldof_to_gdof))
    for p in range(nparts):   # FESpaces.jl:215-233
        s = spaces[p]
        for c in np.nonzero(~cell_is_own[p])[0]:
            for i, ld in enumerate(s.cell_dofs[c]):
                if ld >= 0 and ldof_to_owner[p][ld] == cell_owner[p][c]:
                    ldof_to_gdof[p][ld] = cw[p][c, i]
    cw = fetch_ghost(dof_to_cell(ldof_to_gdof))
    cell_to_dof(ldof_to_gdof, cw)
    ngdofs = int(sum(nodofs))
    out = [DofIndices(p, ngdofs, ldof_to_gdof[p], ldof_to_owner[p]) for p in range(nparts)]
    for d in out:
        assert (d.ldof_to_gdof >= 0).all()
    return out, first_gdof


# --------------------------------------------------------------------------------------
# A7. Reference element integrals (Gridap integrate with tensor Gauss quadrature)
# --------------------------------------------------------------------------------------


def gauss_legendre(npts):
    x, w = np.polynomial.legendre.leggauss(npts)
    return 0.5 * (x + 1.0), 0.5 * w


def lagrange_1d(k, x):
    """Values and derivatives of the k+1 equispaced Lagrange polynomials on [0,1]."""
    nodes = np.linspace(0.0, 1.0, k + 1)
    x = np.atleast_1d(x)
    V = np.ones((len(x), k + 1))
    D = np.zeros((len(x), k + 1))
    for a in range(k + 1):
        others = [b for b in range(k + 1) if b != a]
        den = np.prod([nodes[a] - nodes[b] for b in others])
        val = np.ones(len(x))
        for b in others:
            val = val * (x - nodes[b])
        V[:, a] = val / den
        der = np.zeros(len(x))
        for b in others:
            t = np.ones(len(x))
            for c in others:
                if c != b:
                    t = t * (x - nodes[c])
            der += t
        D[:, a] = der / den
    return V, D


def quad_points_per_dir(degree):
    """Tensor Gauss rule with ceil((degree+1)/2) points per direction."""
    return (degree + 2) // 2


def reference_point_tables(dim, k, h, degree):
    """Weights ``W[q] = w_q |J|``, values ``phi[q, i]`` and gradients ``grad[q, i, d]`` of
    the cell's shape functions at the tensor Gauss points (points x fastest), in Gridap's
    cell-local node order -- what Gridap's integrate evaluates per point
    (CellData integrate, src/CellData.jl:234-259)."""
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    V, D = lagrange_1d(k, xq)
    lnodes = cell_local_nodes(dim, k)
    nn = len(lnodes)
    detJ = float(np.prod(h))
    qidx = list(itertools.product(*[range(nq)] * dim))
    nqt = len(qidx)
    phi = np.zeros((nqt, nn))
    grad = np.zeros((nqt, nn, dim))
    W = np.zeros(nqt)
    for iq, qi in enumerate(qidx):
        qi = tuple(reversed(qi))
        W[iq] = np.prod([wq[qi[d]] for d in range(dim)]) * detJ
        for a, off in enumerate(lnodes):
            vals = [V[qi[d], off[d]] for d in range(dim)]
            phi[iq, a] = np.prod(vals)
            for d in range(dim):
                g = D[qi[d], off[d]] / h[d]
                for e in range(dim):
                    if e != d:
                        g *= vals[e]
                grad[iq, a, d] = g
    return W, phi, grad


def quadrature_points(pb, cells=None):
    """Physical coordinates of the tensor Gauss points of the given global cells (all by
    default): array (cells, nq^dim, dim), points x fastest."""
    nq = quad_points_per_dir(pb.degree)
    xq, _ = gauss_legendre(nq)
    dim = pb.dim
    cells = np.arange(int(np.prod(pb.n))) if cells is None else np.asarray(cells)
    cc = np.stack(np.unravel_index(cells, tuple(reversed(pb.n)))[::-1], axis=1)   # (cells, dim), x first
    qi = np.indices((nq,) * dim).reshape(dim, -1)[::-1].T                          # (nqt, dim), x fastest
    out = np.empty((len(cells), len(qi), dim))
    for d in range(dim):
        out[:, :, d] = pb.domain[2 * d] + (cc[:, d][:, None] + xq[qi[:, d]][None, :]) * pb.h[d]
    return out


def stiffness_from_points(W, grad, c):
    """``K[i,j] = sum_q c_q W_q grad(phi_i).grad(phi_j)`` for coefficient values c at the points."""
    return np.einsum("q,qid,qjd->ij", W * c, grad, grad)


def elasticity_from_points(W, grad, c, nu):
    """Element matrix of ``int E C1 eps(u):eps(v)`` with E at the points (``c``), in the
    component-major vector DOF order of reference_elasticity."""
    nn, dim = grad.shape[1], grad.shape[2]
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    G = np.einsum("q,qic,qjd->icjd", W * c, grad, grad)
    K = np.zeros((dim * nn, dim * nn))
    lap = np.einsum("icjc->ij", G)
    for a in range(dim):
        for b in range(dim):
            blk = lam * G[:, a, :, b] + mu * G[:, b, :, a]
            if a == b:
                blk = blk + mu * lap
            K[a * nn:(a + 1) * nn, b * nn:(b + 1) * nn] = blk
    return K


def reference_matrices(dim, k, h, degree):
    """Element stiffness ``Kh[i,j] = sum_q w_q |J| grad(phi_i).grad(phi_j)``, mass
    ``Mh`` and load ``Fh[i] = sum_q w_q |J| phi_i`` for an axis-aligned cell of
    sizes ``h``, in Gridap's cell-local node order."""
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    V, D = lagrange_1d(k, xq)
    lnodes = cell_local_nodes(dim, k)
    nn = len(lnodes)
    detJ = float(np.prod(h))
    qidx = list(itertools.product(*[range(nq)] * dim))
    nqt = len(qidx)
    phi = np.zeros((nqt, nn))
    grad = np.zeros((nqt, nn, dim))
    W = np.zeros(nqt)
    for iq, qi in enumerate(qidx):
        qi = tuple(reversed(qi))
        W[iq] = np.prod([wq[qi[d]] for d in range(dim)]) * detJ
        for a, off in enumerate(lnodes):
            vals = [V[qi[d], off[d]] for d in range(dim)]
            phi[iq, a] = np.prod(vals)
            for d in range(dim):
                g = D[qi[d], off[d]] / h[d]
                for e in range(dim):
                    if e != d:
                        g *= vals[e]
                grad[iq, a, d] = g
    K = np.einsum("q,qid,qjd->ij", W, grad, grad)
    M = np.einsum("q,qi,qj->ij", W, phi, phi)
    F = np.einsum("q,qi->i", W, phi)
    return K, M, F


def reference_elasticity(dim, k, h, degree, nu):
    """Element matrix of ``int C eps(u):eps(v)`` for E = 1 on an axis-aligned cell of
    sizes ``h``, in Gridap's vector cell-DOF order (component-major: entry ``c*nn + a``
    is component c of node a).  With u = phi_j e_d and v = phi_i e_c:
    C eps(u):eps(v) = lam d_c(phi_i) d_d(phi_j) + mu (delta_cd grad(phi_i).grad(phi_j)
    + d_d(phi_i) d_c(phi_j)), lam = nu/((1+nu)(1-2nu)), mu = 1/(2(1+nu))."""
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    V, D = lagrange_1d(k, xq)
    lnodes = cell_local_nodes(dim, k)
    nn = len(lnodes)
    detJ = float(np.prod(h))
    qidx = list(itertools.product(*[range(nq)] * dim))
    grad = np.zeros((len(qidx), nn, dim))
    W = np.zeros(len(qidx))
    for iq, qi in enumerate(qidx):
        qi = tuple(reversed(qi))
        W[iq] = np.prod([wq[qi[d]] for d in range(dim)]) * detJ
        for a, off in enumerate(lnodes):
            vals = [V[qi[d], off[d]] for d in range(dim)]
            for d in range(dim):
                g = D[qi[d], off[d]] / h[d]
                for e in range(dim):
                    if e != d:
                        g *= vals[e]
                grad[iq, a, d] = g
    lam = nu / ((1 + nu) * (1 - 2 * nu))
    mu = 1.0 / (2 * (1 + nu))
    G = np.einsum("q,qic,qjd->icjd", W, grad, grad)   # int d_c phi_i d_d phi_j
    K = np.zeros((dim * nn, dim * nn))
    lap = np.einsum("icjc->ij", G)
    for c in range(dim):
        for d in range(dim):
            blk = lam * G[:, c, :, d] + mu * G[:, d, :, c]
            if c == d:
                blk = blk + mu * lap
            K[c * nn:(c + 1) * nn, d * nn:(d + 1) * nn] = blk
    return K


# --------------------------------------------------------------------------------------
# Problem description
# --------------------------------------------------------------------------------------


@dataclass
class Problem:
    """A scalar diffusion problem ``-div(kappa grad u) = f`` on a Cartesian box, or
    (``physics="elasticity"``) linear elasticity ``a(u,v) = int C(E) eps(u):eps(v)``,
    ``l(v) = int v.force`` with a vector space of ``ncomp = dim`` components, E per cell
    in ``kappa`` and Poisson ratio ``nu``."""

    np: tuple
    n: tuple
    domain: tuple
    order: int = 1
    degree: int = 2
    dirichlet_sides: tuple = None   # 2*dim flags; default: whole boundary
    kappa: np.ndarray = None        # per global cell (lexicographic); default 1
    kappa_qp: np.ndarray = None     # or per global cell and Gauss point (cells, nq^dim), points x
                                    # fastest: a coefficient that varies inside the cells (E for elasticity)
    f_const: float = 0.0            # constant source
    f_nodal: np.ndarray = None      # or nodal source values on the global lattice (b = M f)
    u_dir: np.ndarray = None        # Dirichlet values on the global lattice (dense), default 0;
                                    # elasticity: (lattice nodes, dim), components of a node together
    neumann: dict = None            # {side: g(*xyz, *normal)}, side 2d (x_d = min) / 2d+1 (max): l += int(v g)dGamma
    physics: str = "poisson"        # or "elasticity"
    nu: float = 0.3                 # Poisson ratio (elasticity)
    force: tuple = None             # body force (elasticity), default 0
    stiff: float = 1.0              # a(u,v) = int kappa (stiff grad(u).grad(v) + mass u v)
    mass: float = 0.0

    @property
    def ncomp(self):
        return self.dim if self.physics == "elasticity" else 1

    def __post_init__(self):
        dim = len(self.n)
        if self.dirichlet_sides is None:
            self.dirichlet_sides = (1,) * (2 * dim)
        if self.kappa is None:
            self.kappa = np.ones(int(np.prod(self.n)))
        self.kappa = np.asarray(self.kappa, dtype=np.float64)

    @property
    def dim(self):
        return len(self.n)

    @property
    def h(self):
        return tuple((self.domain[2 * d + 1] - self.domain[2 * d]) / self.n[d] for d in range(self.dim))

    @property
    def lattice(self):
        return tuple(self.order * self.n[d] + 1 for d in range(self.dim))

    def node_lin(self, X):
        N = self.lattice
        X = np.asarray(X)
        g = np.zeros(X.shape[:-1], dtype=np.int64)
        for d in reversed(range(self.dim)):
            g = g * N[d] + X[..., d]
        return g

    def node_xyz(self, X):
        X = np.asarray(X, dtype=np.float64)
        out = np.empty_like(X)
        for d in range(self.dim):
            out[..., d] = self.domain[2 * d] + X[..., d] * self.h[d] / self.order
        return out


@dataclass
class FESpaceData:
    P: Partition
    spaces: list
    dofs: list
    first_gdof: np.ndarray


def build_fespace(pb: Problem) -> FESpaceData:
    P = make_partition(pb.np, pb.n)
    spaces = [build_local_space(P, p, pb.order, pb.ncomp, pb.dirichlet_sides) for p in range(P.nparts)]
    dofs, first = generate_gids(P, spaces)
    return FESpaceData(P, spaces, dofs, first)


# --------------------------------------------------------------------------------------
# A8/A10. Cell matrices/vectors and the COO numeric loop
# --------------------------------------------------------------------------------------


def cell_contributions(pb: Problem, sp: LocalSpace, Kh, Mh, Fh):
    """Per local cell: element matrix ``kappa_c*Kh`` and element vector
    ``f-term - K_e[:,D] u_D`` (Dirichlet lifting with the trial space's values)."""
    dim = pb.dim
    lnodes = np.array(cell_local_nodes(dim, pb.order))
    mats, vecs = [], []
    if pb.physics == "elasticity":
        # element DOFs component-major (c * nnode + a), as Kel; u_dir: (lattice nodes, dim)
        assert pb.f_nodal is None, "elasticity: constant body force"
        Kel = reference_elasticity(dim, pb.order, pb.h, pb.degree, pb.nu)
        if pb.kappa_qp is not None:
            Wq, _, Gq = reference_point_tables(dim, pb.order, pb.h, pb.degree)
        force = pb.force if pb.force is not None else (0.0,) * dim
        be = np.concatenate([force[c] * Fh for c in range(dim)])
        ud_all = None if pb.u_dir is None else np.asarray(pb.u_dir, dtype=np.float64).reshape(-1, dim)
        for ic, g in enumerate(sp.cells):
            if pb.kappa_qp is not None:
                Ke = elasticity_from_points(Wq, Gq, pb.kappa_qp[g], pb.nu)
            else:
                Ke = pb.kappa[g] * Kel
            bv = be.copy()
            if ud_all is not None:
                ci = np.array(P_cell_coords(pb.n, int(g)))
                nl = pb.node_lin(pb.order * ci[None, :] + lnodes)
                ud = np.where(sp.cell_dofs[ic] < 0, np.concatenate([ud_all[nl, c] for c in range(dim)]), 0.0)
                bv = bv - Ke @ ud
            mats.append(Ke)
            vecs.append(bv)
        return mats, vecs
    nbt = neumann_tables(pb) if pb.neumann else None
    if pb.kappa_qp is not None:
        assert pb.stiff == 1.0 and pb.mass == 0.0, "point coefficients: stiffness form"
        Wq, _, Gq = reference_point_tables(dim, pb.order, pb.h, pb.degree)
    for ic, g in enumerate(sp.cells):
        if pb.kappa_qp is not None:
            Ke = stiffness_from_points(Wq, Gq, pb.kappa_qp[g])
        else:
            kap = pb.kappa[g]
            Ke = kap * Kh if (pb.stiff == 1.0 and pb.mass == 0.0) else kap * (pb.stiff * Kh + pb.mass * Mh)
        ci = np.array(P_cell_coords(pb.n, int(g)))
        X = pb.order * ci[None, :] + lnodes
        if pb.f_nodal is not None:
            be = Mh @ pb.f_nodal[pb.node_lin(X)]
        else:
            be = pb.f_const * Fh
        dofs = sp.cell_dofs[ic]
        if pb.u_dir is not None:
            ud = np.where(dofs < 0, pb.u_dir[pb.node_lin(X)], 0.0)
            be = be - Ke @ ud
        if nbt is not None:
            be = be + neumann_cell_load(pb, ci, lnodes, nbt)
        mats.append(Ke)
        vecs.append(be)
    return mats, vecs


def neumann_tables(pb: Problem):
    nq = quad_points_per_dir(pb.degree)
    xq, wq = gauss_legendre(nq)
    V, _ = lagrange_1d(pb.order, xq)
    return nq, xq, wq, V


def neumann_cell_load(pb: Problem, ci, lnodes, tabs):
    """``int(v g)dGamma`` over the cell's faces on the Neumann sides (Gridap boundary
    triangulation restricted to the cell; g evaluated at the face Gauss points)."""
    nq, xq, wq, V = tabs
    dim, k, h = pb.dim, pb.order, pb.h
    be = np.zeros(len(lnodes))
    for side, gfun in pb.neumann.items():
        d, hi = side // 2, side % 2
        if ci[d] != (pb.n[d] - 1 if hi else 0):
            continue
        tang = [t for t in range(dim) if t != d]
        normal = [0.0] * dim
        normal[d] = 1.0 if hi else -1.0
        for qi in itertools.product(*[range(nq)] * len(tang)):
            qi = tuple(reversed(qi))
            w = 1.0
            xyz = [0.0] * dim
            xyz[d] = pb.domain[2 * d + hi]
            for j, t in enumerate(tang):
                w *= wq[qi[j]] * h[t]
                xyz[t] = pb.domain[2 * t] + (ci[t] + xq[qi[j]]) * h[t]
            gv = gfun(*xyz, *normal)
            for a, off in enumerate(lnodes):
                if off[d] != (k if hi else 0):
                    continue   # the node's basis function vanishes on this face
                phi = np.prod([V[qi[j], off[t]] for j, t in enumerate(tang)])
                be[a] += w * phi * gv
    return be


def P_cell_coords(n, gid):
    c = []
    for d in range(len(n)):
        c.append(gid % n[d])
        gid //= n[d]
    return c


@dataclass
class LocalMatrix:
    """One part of a ``PSparseMatrix``: local CSR (sorted columns, duplicates summed,
    explicit zeros kept) and its row/col ``OwnAndGhostIndices``."""

    part: int
    nrows: int
    ncols: int
    rowptr: np.ndarray
    colidx: np.ndarray
    vals: np.ndarray
    row_own_gids: np.ndarray
    row_ghost_gids: np.ndarray
    row_ghost_owner: np.ndarray
    col_own_gids: np.ndarray
    col_ghost_gids: np.ndarray
    col_ghost_owner: np.ndarray
    b: np.ndarray      # RHS over the rows (ghost entries zero after assemble!)


def _compress(nrows, I, J, V, ncols):
    """Local ``sparse(I,J,V,m,n)``: duplicates summed in COO order, columns sorted
    within each row (CSR view of the same matrix)."""
    order = np.lexsort((np.arange(len(I)), J, I))
    I, J, V = I[order], J[order], V[order]
    if len(I):
        new = np.ones(len(I), dtype=bool)
        new[1:] = (I[1:] != I[:-1]) | (J[1:] != J[:-1])
        starts = np.nonzero(new)[0]
        vals = np.add.reduceat(V, starts)
        rows, cols = I[starts], J[starts]
    else:
        vals = np.zeros(0); rows = np.zeros(0, dtype=np.int64); cols = np.zeros(0, dtype=np.int64)
    rowptr = np.zeros(nrows + 1, dtype=np.int64)
    np.add.at(rowptr, rows + 1, 1)
    rowptr = np.cumsum(rowptr)
    return rowptr, cols.astype(np.int64), vals


def assemble(pb: Problem, fe: FESpaceData, strategy: str = "sub"):
    """``assemble_matrix_and_vector`` with a DistributedSparseMatrixAssembler.

    ``strategy`` is ``"sub"`` (SubAssembledRows, the default, Algebra.jl:593-646) or
    ``"full"`` (FullyAssembledRows, Algebra.jl:549-579)."""
    P, spaces, dofs = fe.P, fe.spaces, fe.dofs
    nparts = P.nparts
    Kh, Mh, Fh = reference_matrices(pb.dim, pb.order, pb.h, pb.degree)
    coo = []
    bloc = []
    for p in range(nparts):
        sp, di = spaces[p], dofs[p]
        owners = np.array([P.cell_owner(P.cell_coords(int(g))) for g in sp.cells])
        mats, vecs = cell_contributions(pb, sp, Kh, Mh, Fh)
        own_dof = di.ldof_to_owner == p
        I, J, V = [], [], []
        b = np.zeros(sp.nfree)
        touched = np.zeros(sp.nfree, dtype=bool)
        for ic in range(len(sp.cells)):
            if strategy == "sub" and owners[ic] != p:
                continue   # Triangulation(no_ghost) (Geometry.jl:802-847)
            cd = sp.cell_dofs[ic]
            Ke, be = mats[ic], vecs[ic]
            nd = len(cd)
            for j in range(nd):          # Gridap add_entries!: column-major loop
                gj = cd[j]
                if gj < 0:
                    continue
                for i in range(nd):
                    gi = cd[i]
                    if gi < 0:
                        continue
                    if strategy == "full" and not own_dof[gi]:
                        continue   # FESpaces.jl:808-816
                    I.append(gi); J.append(gj); V.append(Ke[i, j])
            for i in range(nd):
                gi = cd[i]
                if gi < 0:
                    continue
                if strategy == "full" and not own_dof[gi]:
                    continue
                b[gi] += be[i]
                touched[gi] = True
        coo.append([np.array(I, dtype=np.int64), np.array(J, dtype=np.int64), np.array(V, dtype=np.float64)])
        bloc.append((b, touched))

    # to_global_indices! (Algebra.jl:600-601)
    gI, gJ, gV = [], [], []
    for p in range(nparts):
        I, J, V = coo[p]
        gI.append(dofs[p].ldof_to_gdof[I]); gJ.append(dofs[p].ldof_to_gdof[J]); gV.append(V.copy())

    gid_owner = np.zeros(dofs[0].ngdofs, dtype=np.int32)
    for p in range(nparts):
        gid_owner[dofs[p].ldof_to_gdof] = dofs[p].ldof_to_owner

    mats_out = []
    if strategy == "sub":
        # rows: owned + ghost rows touched by I, sorted by FE-space lid (Algebra.jl:931-962, 919-928)
        row_ghost = []
        for p in range(nparts):
            di = dofs[p]
            lids = coo[p][0]
            gmask = ~di.own_mask[lids]
            gl = np.unique(lids[gmask])        # sorted by local dof id
            row_ghost.append(gl)
        # Jo and triplet routing (Algebra.jl:1048-1131)
        gJo = [gid_owner[gJ[p]] for p in range(nparts)]
        send = {}
        for p in range(nparts):
            rown = gid_owner[gI[p]]
            for q in sorted(set(rown.tolist()) - {p}):
                sel = np.nonzero(rown == q)[0]    # COO order preserved
                send[(p, q)] = (gI[p][sel].copy(), gJ[p][sel].copy(), gJo[p][sel].copy(), gV[p][sel].copy())
                gV[p][sel] = 0.0                  # zeroed, not removed (Algebra.jl:1084)
        for q in range(nparts):
            for p in range(nparts):               # received data appended in ascending sender order
                if (p, q) in send:
                    a, b_, c, v = send[(p, q)]
                    gI[q] = np.concatenate([gI[q], a]); gJ[q] = np.concatenate([gJ[q], b_])
                    gJo[q] = np.concatenate([gJo[q], c]); gV[q] = np.concatenate([gV[q], v])
        for p in range(nparts):
            di = dofs[p]
            own_g = di.own_to_global
            n_own = len(own_g)
            rg_l = row_ghost[p]
            rg_g = di.ldof_to_gdof[rg_l]
            rg_o = di.ldof_to_owner[rg_l]
            # cols: ghost cols in first-appearance order among non-owned J (Algebra.jl:1210-1238)
            seen = {}
            cg_g, cg_o = [], []
            for j, jo in zip(gJ[p].tolist(), gJo[p].tolist()):
                if jo != p and j not in seen:
                    seen[j] = len(cg_g); cg_g.append(j); cg_o.append(jo)
            cg_g = np.array(cg_g, dtype=np.int64); cg_o = np.array(cg_o, dtype=np.int32)
            row_map = {int(g): i for i, g in enumerate(own_g)}
            for i, g in enumerate(rg_g):
                row_map[int(g)] = n_own + i
            col_map = {int(g): i for i, g in enumerate(own_g)}
            for i, g in enumerate(cg_g):
                col_map[int(g)] = n_own + i
            I = np.array([row_map[int(g)] for g in gI[p]], dtype=np.int64)
            J = np.array([col_map[int(g)] for g in gJ[p]], dtype=np.int64)
            nrows = n_own + len(rg_g); ncols = n_own + len(cg_g)
            rowptr, colidx, vals = _compress(nrows, I, J, gV[p], ncols)
            mats_out.append(LocalMatrix(p, nrows, ncols, rowptr, colidx, vals, own_g, rg_g, rg_o,
                                        own_g, cg_g, cg_o, None))
        # RHS: _rhs_callback + assemble! (Algebra.jl:720-753, 786-789)
        bfull = np.zeros(dofs[0].ngdofs)
        for p in range(nparts):
            b, touched = bloc[p]
            np.add.at(bfull, dofs[p].ldof_to_gdof, np.where(touched, b, 0.0))
        for p in range(nparts):
            M = mats_out[p]
            M.b = np.concatenate([bfull[M.row_own_gids], np.zeros(len(M.row_ghost_gids))])
    else:
        for p in range(nparts):
            di = dofs[p]
            own_g = di.own_to_global
            n_own = len(own_g)
            J_l = coo[p][1]
            # cols: touched ghost lids sorted by FE-space lid (Algebra.jl:1245-1257, 919-928)
            gl = np.unique(J_l[~di.own_mask[J_l]])
            cg_g = di.ldof_to_gdof[gl]; cg_o = di.ldof_to_owner[gl]
            row_map = {int(g): i for i, g in enumerate(own_g)}
            col_map = dict(row_map)
            for i, g in enumerate(cg_g):
                col_map[int(g)] = n_own + i
            I = np.array([row_map[int(g)] for g in gI[p]], dtype=np.int64)
            J = np.array([col_map[int(g)] for g in gJ[p]], dtype=np.int64)
            rowptr, colidx, vals = _compress(n_own, I, J, gV[p], n_own + len(cg_g))
            b, _ = bloc[p]
            M = LocalMatrix(p, n_own, n_own + len(cg_g), rowptr, colidx, vals, own_g,
                            np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int32),
                            own_g, cg_g, cg_o.astype(np.int32), b[di.own_mask])
            mats_out.append(M)
    return mats_out


# --------------------------------------------------------------------------------------
# A14-A16. Gathered operator, solve, consistent!
# --------------------------------------------------------------------------------------


def gather_global(mats, ngdofs):
    """Owned rows of every part in part order = the global matrix in gid order."""
    import scipy.sparse as sps
    rows, cols, vals = [], [], []
    b = np.zeros(ngdofs)
    for M in mats:
        n_own = len(M.row_own_gids)
        colg = np.concatenate([M.col_own_gids, M.col_ghost_gids])
        for r in range(n_own):
            s, e = M.rowptr[r], M.rowptr[r + 1]
            rows.append(np.full(e - s, M.row_own_gids[r]))
            cols.append(colg[M.colidx[s:e]])
            vals.append(M.vals[s:e])
        b[M.row_own_gids] = M.b[:n_own]
    A = sps.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                       shape=(ngdofs, ngdofs))
    return A, b


def solve_lu(mats, ngdofs):
    """``A \\ b`` on a PSparseMatrix: gather to one part, sparse LU, scatter."""
    import scipy.sparse.linalg as spla
    A, b = gather_global(mats, ngdofs)
    return spla.splu(A.tocsc()).solve(b)


def pcg_jacobi(A, b, rtol=1e-8, maxit=100000, x0=None):
    """Jacobi-preconditioned CG in FP64; stops at ||b-Ax|| <= rtol*||b||."""
    x = np.zeros_like(b) if x0 is None else x0.copy()
    dinv = 1.0 / A.diagonal()
    r = b - A @ x
    z = dinv * r
    p = z.copy()
    rz = r @ z
    nb = np.linalg.norm(b)
    it = 0
    while np.linalg.norm(r) > rtol * nb and it < maxit:
        Ap = A @ p
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        z = dinv * r
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        it += 1
    return x, it


def consistent_local(x_global, dofs):
    """``change_ghost(..., make_consistent=true)`` onto the FE-space gids: every
    local DOF (owned and ghost) gets the owner's value."""
    return [x_global[d.ldof_to_gdof] for d in dofs]


def nodal_solution(pb: Problem, fe: FESpaceData, x_global):
    """Dense lattice array of the FE solution's nodal values (free from x, Dirichlet
    from u_dir)."""
    N = pb.lattice
    u = np.zeros(int(np.prod(N))) if pb.u_dir is None else pb.u_dir.copy()
    for sp, d in zip(fe.spaces, fe.dofs):
        u[pb.node_lin(sp.dof_node)] = x_global[d.ldof_to_gdof]
    return u


def l2_error(pb: Problem, u_nodal, u_exact):
    """``sqrt(sum(integrate(abs2(u - uh))))`` with the problem's quadrature degree."""
    dim, k = pb.dim, pb.order
    nq = quad_points_per_dir(pb.degree)
    xq, wq = gauss_legendre(nq)
    V, _ = lagrange_1d(k, xq)
    h = pb.h
    err = 0.0
    lnodes = np.array(cell_local_nodes(dim, k))
    qidx = [tuple(reversed(q)) for q in itertools.product(*[range(nq)] * dim)]
    for g in range(int(np.prod(pb.n))):
        ci = np.array(P_cell_coords(pb.n, g))
        X = k * ci[None, :] + lnodes
        ue = u_nodal[pb.node_lin(X)]
        for qi in qidx:
            phi = np.array([np.prod([V[qi[d], off[d]] for d in range(dim)]) for off in lnodes])
            xyz = [pb.domain[2 * d] + (ci[d] + xq[qi[d]]) * h[d] for d in range(dim)]
            w = np.prod([wq[qi[d]] for d in range(dim)]) * np.prod(h)
            err += w * (u_exact(*xyz) - phi @ ue) ** 2
    return math.sqrt(err)


# --------------------------------------------------------------------------------------
# Multi-field systems over one scalar space (src/MultiField.jl)
# --------------------------------------------------------------------------------------


def multifield_gids(fe: FESpaceData, nfields: int):
    """``generate_multi_field_gids`` (src/MultiField.jl:356-420) for ``nfields`` copies of
    the space: local ids are field-major (f * nfree + lid, Gridap's MultiFieldFESpace);
    each part numbers its owned dofs field by field (each field's owned dofs in its own
    owned order) from the exclusive scan of the parts' owned counts; ghosts receive the
    owner's number through each field's own ghost exchange (propagate_to_ghost_multifield!,
    :422-451)."""
    dofs = fe.dofs
    nparts = len(dofs)
    noids = [nfields * d.n_own for d in dofs]
    firstgid = np.concatenate([[0], np.cumsum(noids)[:-1]]).astype(np.int64)
    lid_gid, lid_part = [], []
    for p, d in enumerate(dofs):
        nfree = len(d.ldof_to_gdof)
        g = np.full(nfields * nfree, -1, dtype=np.int64)
        o = np.zeros(nfields * nfree, dtype=np.int32)
        gid = firstgid[p]
        own = np.nonzero(d.own_mask)[0]          # own_to_local: owned lids in order
        for f in range(nfields):
            for flid in own:
                g[f * nfree + flid] = gid
                gid += 1
            o[f * nfree:(f + 1) * nfree] = d.ldof_to_owner
        lid_gid.append(g)
        lid_part.append(o)
    # ghost values from the owners, field by field (the single-field exchange)
    gid_to_lid = [{int(x): i for i, x in enumerate(d.ldof_to_gdof)} for d in dofs]
    for p, d in enumerate(dofs):
        nfree = len(d.ldof_to_gdof)
        for f in range(nfields):
            for flid in d.ghost_lids:
                q = int(d.ldof_to_owner[flid])
                qlid = gid_to_lid[q][int(d.ldof_to_gdof[flid])]
                qn = len(dofs[q].ldof_to_gdof)
                lid_gid[p][f * nfree + flid] = lid_gid[q][f * qn + qlid]
    ngids = int(sum(noids))
    out = [DofIndices(p, ngids, lid_gid[p], lid_part[p]) for p in range(nparts)]
    for d in out:
        assert (d.ldof_to_gdof >= 0).all()
    return out


def assemble_multifield(pb: Problem, fe: FESpaceData, stiff, mass, src, rf, cf, strategy="full"):
    """The matrix and right-hand side of the multi-field form
    ``sum_ij int kappa (stiff[i][j] grad(u_j).grad(v_i) + mass[i][j] u_j v_i)``,
    ``sum_i int src[i] v_i`` (minus the Dirichlet lifting of every field) restricted to
    the row fields ``rf`` and column fields ``cf`` (a block of BlockMultiFieldStyle, or
    the ConsecutiveMultiFieldStyle matrix for rf = cf = all fields): one LocalMatrix per
    part, the local compression of FESpaces.jl:808-816 / Algebra.jl:549-579, 1245-1257 over
    the multi-field index sets.  Blocks with stiff = mass = 0 add no entries.
    ``strategy="sub"``: SubAssembledRows (the default of the reference's multi-field
    assemblers, MultiField.jl:473-479), _multifield_sub_assembled."""
    if strategy == "sub":
        return _multifield_sub_assembled(pb, fe, stiff, mass, src, rf, cf)
    P, spaces, dofs = fe.P, fe.spaces, fe.dofs
    stiff = np.asarray(stiff, dtype=np.float64)
    mass = np.asarray(mass, dtype=np.float64)
    nf = stiff.shape[0]
    Kh, Mh, Fh = reference_matrices(pb.dim, pb.order, pb.h, pb.degree)
    T = [[stiff[i, j] * Kh + mass[i, j] * Mh for j in range(nf)] for i in range(nf)]
    touched = (stiff != 0.0) | (mass != 0.0)
    S = [sum(T[i][j] for j in range(nf)) for i in range(nf)]
    rg = multifield_gids(fe, len(rf))
    cg = multifield_gids(fe, len(cf))
    lnodes = np.array(cell_local_nodes(pb.dim, pb.order))
    out = []
    for p in range(P.nparts):
        sp, di = spaces[p], dofs[p]
        nfree = sp.nfree
        own_dof = di.ldof_to_owner == p
        I, J, V = [], [], []
        b = np.zeros(len(rf) * nfree)
        for ic, g in enumerate(sp.cells):
            kap = pb.kappa[g]
            cd = sp.cell_dofs[ic]
            nd = len(cd)
            ci = np.array(P_cell_coords(pb.n, int(g)))
            X = pb.order * ci[None, :] + lnodes
            for ii, i in enumerate(rf):
                for jj, j in enumerate(cf):
                    if not touched[i, j]:
                        continue
                    Ke = kap * T[i][j]
                    for c in range(nd):          # add_entries!: column-major
                        gj = cd[c]
                        if gj < 0:
                            continue
                        for a in range(nd):
                            gi = cd[a]
                            if gi < 0 or not own_dof[gi]:
                                continue
                            I.append(ii * nfree + gi); J.append(jj * nfree + gj); V.append(Ke[a, c])
                be = src[i] * Fh
                if pb.u_dir is not None:
                    ud = np.where(cd < 0, pb.u_dir[pb.node_lin(X)], 0.0)
                    be = be - kap * (S[i] @ ud)
                for a in range(nd):
                    gi = cd[a]
                    if gi >= 0 and own_dof[gi]:
                        b[ii * nfree + gi] += be[a]
        I = np.array(I, dtype=np.int64); J = np.array(J, dtype=np.int64); V = np.array(V, dtype=np.float64)
        rdi, cdi = rg[p], cg[p]
        rown = rdi.own_to_global
        cown = cdi.own_to_global
        gl = np.unique(J[~cdi.own_mask[J]]) if len(J) else np.zeros(0, dtype=np.int64)
        cg_g = cdi.ldof_to_gdof[gl]; cg_o = cdi.ldof_to_owner[gl]
        row_map = {int(x): k for k, x in enumerate(rown)}
        col_map = {int(x): k for k, x in enumerate(cown)}
        for k, x in enumerate(cg_g):
            col_map[int(x)] = len(cown) + k
        Ig = rdi.ldof_to_gdof[I]; Jg = cdi.ldof_to_gdof[J]
        Il = np.array([row_map[int(x)] for x in Ig], dtype=np.int64)
        Jl = np.array([col_map[int(x)] for x in Jg], dtype=np.int64)
        rowptr, colidx, vals = _compress(len(rown), Il, Jl, V, len(cown) + len(cg_g))
        out.append(LocalMatrix(p, len(rown), len(cown) + len(cg_g), rowptr, colidx, vals, rown,
                               np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int32),
                               cown, cg_g, cg_o.astype(np.int32), b[rdi.own_mask]))
    return out


def _multifield_sub_assembled(pb: Problem, fe: FESpaceData, stiff, mass, src, rf, cf):
    """SubAssembledRows local parts of a multi-field system (Algebra.jl:593-646 over
    the multi-field index sets):

    * each part integrates its owned cells only (Triangulation(no_ghost));
    * the COO follows Gridap's loops: cells in local order, and for a cell the block matrix
      (rows: the row fields' cell dofs, columns: the column fields') walked column-major,
      block columns outer and block rows inner over the touched blocks, each block
      column-major (add_entries!); Dirichlet dofs skipped;
    * triplets of rows owned by another part are copied to it and zeroed (not removed),
      the owner appends them, senders in ascending order (Algebra.jl:1048-1131);
    * rows: owned multi-field dofs, then the touched ghost dofs by local id (field-major:
      group position * free dofs + scalar local id); columns: owned, then the ghost dofs in
      order of first appearance (Algebra.jl:1210-1238); duplicates summed;
    * b: owned rows complete (the vector assemble!), ghost rows zero."""
    P, spaces, dofs = fe.P, fe.spaces, fe.dofs
    stiff = np.asarray(stiff, dtype=np.float64)
    mass = np.asarray(mass, dtype=np.float64)
    nf = stiff.shape[0]
    Kh, Mh, Fh = reference_matrices(pb.dim, pb.order, pb.h, pb.degree)
    T = [[stiff[i, j] * Kh + mass[i, j] * Mh for j in range(nf)] for i in range(nf)]
    touched = (stiff != 0.0) | (mass != 0.0)
    S = [sum(T[i][j] for j in range(nf)) for i in range(nf)]
    rg = multifield_gids(fe, len(rf))
    cg = multifield_gids(fe, len(cf))
    lnodes = np.array(cell_local_nodes(pb.dim, pb.order))
    # global right-hand side per row-group gid (owned rows complete)
    nrg = sum(len(d.own_to_global) for d in rg)
    bglob = np.zeros(nrg)
    coo = []
    for p in range(P.nparts):
        sp, di = spaces[p], dofs[p]
        nfree = sp.nfree
        owners = [P.cell_owner(P.cell_coords(int(g))) for g in sp.cells]
        I, J, V = [], [], []
        for ic, g in enumerate(sp.cells):
            if owners[ic] != p:
                continue
            kap = pb.kappa[g]
            cd = sp.cell_dofs[ic]
            nd = len(cd)
            ci = np.array(P_cell_coords(pb.n, int(g)))
            X = pb.order * ci[None, :] + lnodes
            for jj, j in enumerate(cf):              # block columns outer
                for ii, i in enumerate(rf):          # block rows inner
                    if not touched[i, j]:
                        continue
                    Ke = kap * T[i][j]
                    for c in range(nd):              # column-major inside the block
                        gj = cd[c]
                        if gj < 0:
                            continue
                        for a in range(nd):
                            gi = cd[a]
                            if gi < 0:
                                continue
                            I.append(ii * nfree + gi); J.append(jj * nfree + gj); V.append(Ke[a, c])
            for ii, i in enumerate(rf):
                be = src[i] * Fh
                if pb.u_dir is not None:
                    ud = np.where(cd < 0, pb.u_dir[pb.node_lin(X)], 0.0)
                    be = be - kap * (S[i] @ ud)
                for a in range(nd):
                    gi = cd[a]
                    if gi >= 0:
                        bglob[rg[p].ldof_to_gdof[ii * nfree + gi]] += be[a]
        I = np.array(I, dtype=np.int64); J = np.array(J, dtype=np.int64)
        coo.append((rg[p].ldof_to_gdof[I] if len(I) else I, cg[p].ldof_to_gdof[J] if len(J) else J,
                    np.array(V, dtype=np.float64)))
    row_owner = {}
    for p in range(P.nparts):
        for gg, o in zip(rg[p].ldof_to_gdof, rg[p].ldof_to_owner):
            row_owner[int(gg)] = int(o)
    col_owner = {}
    for p in range(P.nparts):
        for gg, o in zip(cg[p].ldof_to_gdof, cg[p].ldof_to_owner):
            col_owner[int(gg)] = int(o)
    sent, kept = {}, []
    for p in range(P.nparts):
        Ig, Jg, V = coo[p]
        Vk = V.copy()
        for t in range(len(Ig)):
            q = row_owner[int(Ig[t])]
            if q != p:
                sent.setdefault((p, q), []).append((int(Ig[t]), int(Jg[t]), float(V[t])))
                Vk[t] = 0.0
        kept.append((Ig, Jg, Vk))
    out = []
    for p in range(P.nparts):
        Ig, Jg, V = kept[p]
        trip = list(zip(Ig.tolist(), Jg.tolist(), V.tolist()))
        for q in range(P.nparts):
            trip += sent.get((q, p), [])
        rdi, cdi = rg[p], cg[p]
        rown, cown = rdi.own_to_global, cdi.own_to_global
        rlid = {int(gg): l for l, gg in enumerate(rdi.ldof_to_gdof)}
        ghost_rows = sorted({rlid[r] for (r, c, v) in trip if row_owner[r] != p})
        grow_g = np.array([int(rdi.ldof_to_gdof[l]) for l in ghost_rows], dtype=np.int64)
        gcol_g, seen = [], set()
        for (r, c, v) in trip:
            if col_owner[c] != p and c not in seen:
                seen.add(c); gcol_g.append(c)
        gcol_g = np.array(gcol_g, dtype=np.int64)
        rmap = {int(x): k for k, x in enumerate(rown)}
        rmap.update({int(x): len(rown) + k for k, x in enumerate(grow_g)})
        cmap = {int(x): k for k, x in enumerate(cown)}
        cmap.update({int(x): len(cown) + k for k, x in enumerate(gcol_g)})
        Il = np.array([rmap[r] for (r, c, v) in trip], dtype=np.int64)
        Jl = np.array([cmap[c] for (r, c, v) in trip], dtype=np.int64)
        Vl = np.array([v for (r, c, v) in trip], dtype=np.float64)
        nrows, ncols = len(rown) + len(grow_g), len(cown) + len(gcol_g)
        rowptr, colidx, vals = _compress(nrows, Il, Jl, Vl, ncols)
        own = lambda gs, m: np.array([m[int(x)] for x in gs], dtype=np.int32)
        out.append(LocalMatrix(p, nrows, ncols, rowptr, colidx, vals, rown, grow_g, own(grow_g, row_owner),
                               cown, gcol_g, own(gcol_g, col_owner),
                               np.concatenate([bglob[rown], np.zeros(len(grow_g))])))
    return out


# --------------------------------------------------------------------------------------
# Discontinuous Galerkin (test/PoissonTests.jl:47-77)
# --------------------------------------------------------------------------------------


def _shape_ref(dim, k, lnodes, xi):
    """Values (NN,) and reference gradients (NN, dim) of the Q_k basis (nodes lnodes,
    Gridap order) at the reference point xi in [0,1]^dim."""
    vals, ders = [], []
    for d in range(dim):
        v, dv = lagrange_1d(k, np.array([xi[d]]))
        vals.append(v[0]); ders.append(dv[0])
    nn = len(lnodes)
    phi = np.ones(nn)
    grad = np.ones((nn, dim))
    for a, node in enumerate(lnodes):
        for d in range(dim):
            phi[a] *= vals[d][node[d]]
            for e in range(dim):
                grad[a, e] *= ders[d][node[d]] if e == d else vals[d][node[d]]
    return phi, grad


def dg_system(np_, n, domain, k, degree, gamma, hpen, f, dirichlet_sides, neumann_sides, u_dir, g_neu,
              strategy="full"):
    """Symmetric interior penalty system of test/PoissonTests.jl:47-77 on a Cartesian
    model, assembled the way a finite-element code does it: cell loops for the volume
    terms, one loop over the interior faces (each face once, its 2x2-block matrix with
    [[w n]] = w+ n+ + w- n- and {q} = (q+ + q-)/2 at the physical face points) and the
    boundary faces (Nitsche terms on the Dirichlet sides, g on the Neumann sides).

    Numbering (Gridap's L2 spaces): a cell's dofs in reference node order; a part's owned
    cells lexicographic, parts in order; local dofs of every local cell in local-box
    order.  Returns one LocalMatrix per part with FullyAssembledRows columns (owned dofs,
    then the touched ghost dofs sorted by local id) and b over the owned rows.

    f: constant; u_dir(x), g_neu(x, normal): callables on the physical face points."""
    P = make_partition(np_, n)
    dim = len(n)
    nn = (k + 1) ** dim
    lnodes = cell_local_nodes(dim, k)
    h = [(domain[2 * d + 1] - domain[2 * d]) / n[d] for d in range(dim)]
    det = float(np.prod(h))
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    ncells = int(np.prod(n))
    # gids
    owner = np.array([P.cell_owner(P.cell_coords(c)) for c in range(ncells)], dtype=np.int32)
    ncell_own = np.bincount(owner, minlength=P.nparts)
    first = np.concatenate([[0], np.cumsum(nn * ncell_own)[:-1]]).astype(np.int64)
    rank = np.zeros(ncells, dtype=np.int64)
    seen = np.zeros(P.nparts, dtype=np.int64)
    for c in range(ncells):            # lexicographic = each owner's box order
        rank[c] = seen[owner[c]]
        seen[owner[c]] += 1
    gid0 = first[owner] + nn * rank
    ndofs = int(nn * ncells)

    def cell_x0(ci):
        return np.array([domain[2 * d] + ci[d] * h[d] for d in range(dim)])

    def phys_shape(ci, x):
        xi = (x - cell_x0(ci)) / np.array(h)
        phi, g = _shape_ref(dim, k, lnodes, xi)
        return phi, g / np.array(h)[None, :]

    rows, cols, vals = [], [], []
    b = np.zeros(ndofs)
    terms = {"cell": {}, "bnd": {}, "facet": {}}   # per owned-cell / boundary-face / interior-face matrices

    def add(c1, c2, M):
        for a in range(nn):
            for bb in range(nn):
                rows.append(gid0[c1] + a); cols.append(gid0[c2] + bb); vals.append(M[a, bb])

    qpts = list(itertools.product(range(nq), repeat=dim))
    for c in range(ncells):
        ci = P.cell_coords(c)
        Ke = np.zeros((nn, nn)); be = np.zeros(nn)
        for q in qpts:
            x = cell_x0(ci) + np.array([xq[q[d]] * h[d] for d in range(dim)])
            w = det * np.prod([wq[q[d]] for d in range(dim)])
            phi, gr = phys_shape(ci, x)
            Ke += w * gr @ gr.T
            be += w * f * phi
        add(c, c, Ke)
        terms["cell"][c] = Ke
        b[gid0[c]:gid0[c] + nn] += be
    pen = gamma / hpen
    for c in range(ncells):
        ci = P.cell_coords(c)
        for d in range(dim):
            tang = [t for t in range(dim) if t != d]
            fm = float(np.prod([h[t] for t in tang]))
            fq = list(itertools.product(range(nq), repeat=dim - 1))
            # the upper face of c along d: interior (with the next cell) or the x_d = max side
            for side in (0, 1):
                on_lower = side == 0 and ci[d] == 0
                if side == 0 and not on_lower:
                    continue   # interior lower faces are the upper faces of the previous cell
                nb = list(ci); nb[d] += 1
                interior = side == 1 and nb[d] < n[d]
                if side == 1 and not interior and ci[d] != n[d] - 1:
                    continue
                normal = np.zeros(dim); normal[d] = 1.0 if side == 1 else -1.0
                xd = domain[2 * d] + (ci[d] + side) * h[d]
                if interior:
                    cn = P.cell_gid(tuple(nb))
                    A = np.zeros((2 * nn, 2 * nn))
                    for qf in fq:
                        x = np.zeros(dim); x[d] = xd
                        for j, t in enumerate(tang):
                            x[t] = domain[2 * t] + (ci[t] + xq[qf[j]]) * h[t]
                        w = fm * np.prod([wq[qf[j]] for j in range(dim - 1)])
                        pp, gp = phys_shape(ci, x)        # + side (this cell), n+ = normal
                        pm, gm = phys_shape(nb, x)        # - side, n- = -normal
                        jv = np.concatenate([pp, -pm])    # [[w n]] . n+ for the 2nn basis
                        mg = 0.5 * np.concatenate([gp @ normal, gm @ normal])   # {grad w} . n+
                        A += w * (pen * np.outer(jv, jv) - np.outer(jv, mg) - np.outer(mg, jv))
                    add(c, c, A[:nn, :nn]); add(c, cn, A[:nn, nn:])
                    add(cn, c, A[nn:, :nn]); add(cn, cn, A[nn:, nn:])
                    terms["facet"][(c, cn)] = A     # rows/cols [lower cell dofs, upper cell dofs]
                    continue
                s = 2 * d + side
                if not (dirichlet_sides[s] or neumann_sides[s]):
                    continue
                A = np.zeros((nn, nn)); be = np.zeros(nn)
                for qf in fq:
                    x = np.zeros(dim); x[d] = xd
                    for j, t in enumerate(tang):
                        x[t] = domain[2 * t] + (ci[t] + xq[qf[j]]) * h[t]
                    w = fm * np.prod([wq[qf[j]] for j in range(dim - 1)])
                    phi, gr = phys_shape(ci, x)
                    dn = gr @ normal
                    if dirichlet_sides[s]:
                        A += w * (pen * np.outer(phi, phi) - np.outer(phi, dn) - np.outer(dn, phi))
                        be += w * (pen * phi - dn) * u_dir(*x)
                    else:
                        be += w * phi * g_neu(*x, *normal)
                if dirichlet_sides[s]:
                    add(c, c, A)
                    terms["bnd"][(c, s)] = A
                b[gid0[c]:gid0[c] + nn] += be
    if strategy == "sub":
        return _dg_sub_assembled(P, n, nn, first, ncell_own, gid0, terms, b), gid0, ndofs
    I = np.array(rows, dtype=np.int64); J = np.array(cols, dtype=np.int64); V = np.array(vals)
    # FullyAssembledRows local parts
    out = []
    for p in range(P.nparts):
        lcells = P.local_cells(p)
        lid_of = {}
        for i, cg in enumerate(lcells):
            for a in range(nn):
                lid_of[int(gid0[cg]) + a] = i * nn + a
        own0, own1 = int(first[p]), int(first[p] + nn * ncell_own[p])
        sel = (I >= own0) & (I < own1)
        Ip, Jp, Vp = I[sel] - own0, J[sel], V[sel]
        ghost = sorted({lid_of[int(j)] for j in Jp if not (own0 <= j < own1)})
        gmap = {l: i for i, l in enumerate(ghost)}
        lid_gid = {l: g for g, l in lid_of.items()}
        Jl = np.array([j - own0 if own0 <= j < own1 else (own1 - own0) + gmap[lid_of[int(j)]] for j in Jp],
                      dtype=np.int64)
        rowptr, colidx, vv = _compress(own1 - own0, Ip, Jl, Vp, (own1 - own0) + len(ghost))
        gg = np.array([lid_gid[l] for l in ghost], dtype=np.int64)
        gown = np.array([int(np.searchsorted(first, g, side="right") - 1) for g in gg], dtype=np.int32)
        own_g = np.arange(own0, own1, dtype=np.int64)
        out.append(LocalMatrix(p, own1 - own0, (own1 - own0) + len(ghost), rowptr, colidx, vv, own_g,
                               np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.int32),
                               own_g, gg, gown, b[own0:own1].copy()))
    return out, gid0, ndofs


def _dg_facet_order(P, p, n):
    """Interior faces of part p's local model in Gridap's face numbering: faces are
    numbered as the local cells (local-box order) meet them, each cell's faces in the
    n-cube's order (2D: y-, y+, x-, x+; 3D: z-, z+, y-, y+, x-, x+), so an interior face
    gets its number at its lower cell, as that cell's upper face in direction d.
    Returns [(lower cell, upper cell)] global ids, in that order."""
    dim = len(n)
    lcells = P.local_cells(p)
    in_local = set(int(c) for c in lcells)
    out = []
    for c in lcells:
        ci = P.cell_coords(int(c))
        for d in reversed(range(dim)):           # upper faces in the order z+, y+, x+
            nb = list(ci); nb[d] += 1
            if nb[d] < n[d]:
                cn = P.cell_gid(tuple(nb))
                if cn in in_local:
                    out.append((int(c), int(cn)))
    return out


def _dg_sub_assembled(P, n, nn, first, ncell_own, gid0, terms, b):
    """SubAssembledRows local parts of the SIPG system (Algebra.jl:593-646 over the local
    loops of Gridap's numeric assembly):

    * part p integrates its owned cells, the boundary faces of its owned cells and the
      interior faces it owns: a face belongs to the part owning the adjacent cell with the
      larger global id (Geometry.jl:864-882, _find_owned_skeleton_facets);
    * the local COO follows Gridap's loops: terms in the order of the form (cells,
      Dirichlet faces, skeleton), faces in the local face numbering (_dg_facet_order); an
      interior face's 2x2 block matrix has plus = the cell with the lower local id, and
      add_entries! walks blocks and entries column-major;
    * triplets of rows owned by another part are copied to it and zeroed (not removed)
      locally (Algebra.jl:1048-1131); the owner appends them, senders in ascending order;
    * rows: owned dofs, then the touched ghost dofs sorted by local id; columns: owned
      dofs, then the ghost dofs in order of first appearance in the (local + received)
      COO (Algebra.jl:1210-1238); duplicates summed (sparse()).
    b: owned rows complete, ghost rows zero (assemble!)."""
    cell_owner = {}
    for c in range(len(gid0)):
        cell_owner[c] = P.cell_owner(P.cell_coords(c))

    def blocks_colmajor(rows_cells, cols_cells, M):
        """(row gid, col gid, value) of a block matrix over the cells' dofs, column-major."""
        R = np.concatenate([np.arange(gid0[c], gid0[c] + nn) for c in rows_cells])
        Cc = np.concatenate([np.arange(gid0[c], gid0[c] + nn) for c in cols_cells])
        out = []
        nb = len(cols_cells)
        for jb in range(nb):                    # block columns
            for ib in range(len(rows_cells)):   # block rows
                for j in range(nn):
                    for i in range(nn):
                        out.append((int(R[ib * nn + i]), int(Cc[jb * nn + j]),
                                    float(M[ib * nn + i, jb * nn + j])))
        return out

    local_coo = []
    for p in range(P.nparts):
        coo = []
        lcells = [int(c) for c in P.local_cells(p)]
        for c in lcells:                                           # Omega (no_ghost)
            if cell_owner[c] == p and c in terms["cell"]:
                coo += blocks_colmajor([c], [c], terms["cell"][c])
        lpos = {c: i for i, c in enumerate(lcells)}
        mine = [(key, A) for key, A in terms["bnd"].items() if cell_owner[key[0]] == p]
        for (c, sd), A in sorted(mine, key=lambda t: (lpos[t[0][0]], t[0][1])):   # Gamma_d (no_ghost)
            coo += blocks_colmajor([c], [c], A)
        for (cl, cu) in _dg_facet_order(P, p, n):                  # Lambda (owned faces)
            if cell_owner[max(cl, cu)] != p:
                continue
            A = terms["facet"][(cl, cu)]                           # plus = lower local id = cl
            coo += blocks_colmajor([cl, cu], [cl, cu], A)
        local_coo.append(coo)
    row_owner = lambda g: int(np.searchsorted(first, g, side="right") - 1)
    sent = {}
    kept = []
    for p in range(P.nparts):
        k_ = []
        for (r, c, v) in local_coo[p]:
            q = row_owner(r)
            if q != p:
                sent.setdefault((p, q), []).append((r, c, v))
                k_.append((r, c, 0.0))
            else:
                k_.append((r, c, v))
        kept.append(k_)
    out = []
    for p in range(P.nparts):
        coo = list(kept[p])
        for q in range(P.nparts):
            coo += sent.get((q, p), [])
        own0, own1 = int(first[p]), int(first[p] + nn * ncell_own[p])
        lcells = [int(c) for c in P.local_cells(p)]
        lid_of = {}
        for i, cg in enumerate(lcells):
            for a in range(nn):
                lid_of[int(gid0[cg]) + a] = i * nn + a
        ghost_rows = sorted({lid_of[r] for (r, c, v) in coo if not (own0 <= r < own1)})
        lid_gid = {l: g for g, l in lid_of.items()}
        grow_g = np.array([lid_gid[l] for l in ghost_rows], dtype=np.int64)
        gcol_g = []
        seen = set()
        for (r, c, v) in coo:
            if not (own0 <= c < own1) and c not in seen:
                seen.add(c); gcol_g.append(c)
        gcol_g = np.array(gcol_g, dtype=np.int64)
        nown = own1 - own0
        rmap = {g: i for i, g in enumerate(range(own0, own1))}
        rmap.update({int(g): nown + i for i, g in enumerate(grow_g)})
        cmap = {g: i for i, g in enumerate(range(own0, own1))}
        cmap.update({int(g): nown + i for i, g in enumerate(gcol_g)})
        I = np.array([rmap[r] for (r, c, v) in coo], dtype=np.int64)
        J = np.array([cmap[c] for (r, c, v) in coo], dtype=np.int64)
        V = np.array([v for (r, c, v) in coo])
        nrows, ncols = nown + len(grow_g), nown + len(gcol_g)
        rowptr, colidx, vv = _compress(nrows, I, J, V, ncols)
        own_g = np.arange(own0, own1, dtype=np.int64)
        gown = lambda gs: np.array([row_owner(int(g)) for g in gs], dtype=np.int32)
        out.append(LocalMatrix(p, nrows, ncols, rowptr, colidx, vv, own_g, grow_g, gown(grow_g),
                               own_g, gcol_g, gown(gcol_g),
                               np.concatenate([b[own0:own1], np.zeros(len(grow_g))])))
    return out


def dg_l2_error(np_, n, domain, k, degree, x, gid0, u):
    """sqrt(sum(int (u - uh)^2 dOmega)) for DG dof values x (dg_system's numbering)."""
    dim = len(n)
    lnodes = cell_local_nodes(dim, k)
    h = [(domain[2 * d + 1] - domain[2 * d]) / n[d] for d in range(dim)]
    det = float(np.prod(h))
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    P = make_partition(np_, n)
    tot = 0.0
    for c in range(int(np.prod(n))):
        ci = P.cell_coords(c)
        xv = x[gid0[c]:gid0[c] + len(lnodes)]
        for q in itertools.product(range(nq), repeat=dim):
            xi = np.array([xq[q[d]] for d in range(dim)])
            phi, _ = _shape_ref(dim, k, lnodes, xi)
            pt = [domain[2 * d] + (ci[d] + xi[d]) * h[d] for d in range(dim)]
            w = det * np.prod([wq[q[d]] for d in range(dim)])
            tot += w * (u(*pt) - phi @ xv) ** 2
    return math.sqrt(tot)
