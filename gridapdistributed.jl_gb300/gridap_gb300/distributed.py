"""Python mirror of GridapDistributed's assembly-and-solve API over libgdgpu.so.

The names, argument meanings and return types follow the Julia API so that a
script reads like the reference's tests (``test/FESpacesTests.jl``,
``test/PoissonTests.jl``)::

    with_gb300(lambda distribute: ...)                  # with_debug(f)
    ranks = distribute(range(4))                         # distribute(LinearIndices((4,)))
    model = CartesianDiscreteModel(ranks, (2, 2), (0, 1, 0, 1), (16, 16))
    V = TestFESpace(model, ReferenceFE(lagrangian, float, 2), dirichlet_tags="boundary")
    U = TrialFESpace(lambda x, y: (x + y) ** 2, V)
    dΩ = Measure(Triangulation(model), 4)
    a = integral_grad_grad(kappa=None, measure=dΩ)      # a(u,v) = ∫(κ ∇v⋅∇u)dΩ
    l = integral_source(f=-4.0, measure=dΩ)             # l(v)   = ∫(v f)dΩ
    op = AffineFEOperator(a, l, U, V)                    # A = op.matrix, b = op.vector
    uh = solve(op)

Weak forms are limited to what the device kernels implement: cell-constant
diffusion ``∫(κ ∇v⋅∇u)`` and sources ``∫(v f)`` with constant or nodal f (the
latter assembled as M f).  Every compute call goes to the C ABI; nothing here
falls back to the CPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L

lagrangian = "lagrangian"


class SubAssembledRows:
    code = L.GD_SUB_ASSEMBLED_ROWS


class FullyAssembledRows:
    code = L.GD_FULLY_ASSEMBLED_ROWS


# --------------------------------------------------------------------------------------
# backend / ranks (with_debug + distribute)
# --------------------------------------------------------------------------------------
class GB300Backend:
    """One CUDA context; every part of a partition lives on this device."""

    def __init__(self, device: int = 0):
        L.load()
        h = C.c_void_p()
        L.call("gd_ctx_create", device, C.byref(h))
        self.handle = h
        self.device = device

    def distribute(self, ids):
        return Ranks(list(ids), self)

    def set_stream(self, stream_handle: int | None):
        L.call("gd_ctx_set_stream", self.handle, C.c_void_p(stream_handle or 0))

    def close(self):
        if self.handle:
            L.load().gd_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def with_gb300(f, device: int = 0):
    """``with_debug(f)`` counterpart: runs ``f(distribute)`` with all parts on one GPU."""
    be = GB300Backend(device)
    try:
        return f(be.distribute)
    finally:
        be.close()


@dataclass
class Ranks:
    ids: list
    backend: GB300Backend

    def __len__(self):
        return len(self.ids)


# --------------------------------------------------------------------------------------
# model (Geometry.jl:378-411)
# --------------------------------------------------------------------------------------
class DistributedDiscreteModel:
    def __init__(self, ranks: Ranks, parts, domain, cells):
        if int(np.prod(parts)) != len(ranks):
            raise ValueError("prod(parts) must equal the number of ranks")
        if len(domain) != 2 * len(cells) or len(parts) != len(cells):
            raise ValueError("domain/cells/parts dimensions disagree")
        self.ranks = ranks
        self.backend = ranks.backend
        self.dim = len(cells)
        self.parts = tuple(int(p) for p in parts)
        self.cells = tuple(int(c) for c in cells)
        self.domain = tuple(float(x) for x in domain)
        h = C.c_void_p()
        cells_a = np.array(self.cells, dtype=np.int64)
        parts_a = np.array(self.parts, dtype=np.int32)
        dom_a = np.array(self.domain, dtype=np.float64)
        L.call("gd_model_cartesian", self.backend.handle, self.dim, L.ptr(cells_a, C.c_int64),
               L.ptr(parts_a, C.c_int32), L.ptr(dom_a, C.c_double), C.byref(h))
        self.handle = h

    @property
    def num_parts(self):
        return int(np.prod(self.parts))

    def part_boxes(self, p):
        a = [np.zeros(self.dim, dtype=np.int64) for _ in range(4)]
        L.call("gd_model_part_boxes", self.handle, p, *[L.ptr(x, C.c_int64) for x in a])
        return tuple(tuple(int(v) for v in x) for x in a)   # own_lo, own_hi, loc_lo, loc_hi

    def __del__(self):
        try:
            if self.handle:
                L.load().gd_model_destroy(self.handle)
        except Exception:
            pass


def CartesianDiscreteModel(ranks, parts, domain, cells):
    return DistributedDiscreteModel(ranks, parts, domain, cells)


@dataclass
class Triangulation:
    model: DistributedDiscreteModel
    portion: object = None


@dataclass
class BoundaryTriangulation:
    """``Boundary(model, tags=...)``: the boundary faces on the tagged sides of the box
    ("left"/"right" = x min/max, "bottom"/"top" = y, "back"/"front" = z, or "boundary")."""

    model: DistributedDiscreteModel
    sides: np.ndarray


def Boundary(model, tags="boundary"):
    return BoundaryTriangulation(model, _sides_from_tags(model.dim, tags))


@dataclass
class Measure:
    trian: Triangulation
    degree: int


class VectorValue:
    """Tag for ``ReferenceFE(lagrangian, VectorValue, k)``: a vector Lagrangian space
    with as many components as the model's dimension (VectorValue{D,Float64})."""


def ReferenceFE(name, T, order, space=None):
    """``ReferenceFE(lagrangian, T, order; space)``: Lagrangian Q_k elements (``space`` the
    default Q space).  The P space of a cube (``space=:P``, the discontinuous pressure of the
    reference's Stokes test) is not built on the device and is refused, not replaced."""
    if name != lagrangian or T not in (float, np.float64, VectorValue):
        raise NotImplementedError("only Lagrangian Float64 and VectorValue reference FEs")
    if space not in (None, "Q", ":Q"):
        raise NotImplementedError(f"ReferenceFE(..., space={space}): only the Q space is built on the device")
    return ("lagrangian", VectorValue if T is VectorValue else float, int(order))


# --------------------------------------------------------------------------------------
# FE spaces and gids (FESpaces.jl:139-261, 570-614)
# --------------------------------------------------------------------------------------
@dataclass
class LocalIndices:
    """``LocalIndices(ngdofs, me, ldof_to_gdof, ldof_to_owner)`` (0-based)."""

    n_global: int
    part: int
    local_to_global: np.ndarray
    local_to_owner: np.ndarray

    @property
    def own_mask(self):
        return self.local_to_owner == self.part

    def own_length(self):
        return int(self.own_mask.sum())

    def local_length(self):
        return len(self.local_to_global)


@dataclass
class OwnAndGhostIndices:
    n_global: int
    part: int
    own_to_global: np.ndarray
    ghost_to_global: np.ndarray
    ghost_to_owner: np.ndarray

    def local_length(self):
        return len(self.own_to_global) + len(self.ghost_to_global)

    def own_length(self):
        return len(self.own_to_global)

    @property
    def local_to_global(self):
        return np.concatenate([self.own_to_global, self.ghost_to_global])


class PRange:
    def __init__(self, partition):
        self._partition = partition

    def partition(self):
        return self._partition

    def __len__(self):
        return self._partition[0].n_global if self._partition else 0


def _sides_from_tags(dim, dirichlet_tags):
    if dirichlet_tags is None or dirichlet_tags == [] or dirichlet_tags == ():
        return np.zeros(2 * dim, dtype=np.int32)
    if isinstance(dirichlet_tags, str):
        dirichlet_tags = [dirichlet_tags]
    names = ["left", "right", "bottom", "top", "back", "front"]   # x0 x1 y0 y1 z0 z1
    s = np.zeros(2 * dim, dtype=np.int32)
    for t in dirichlet_tags:
        if t == "boundary":
            s[:] = 1
        elif t in names[: 2 * dim]:
            s[names.index(t)] = 1
        else:
            raise NotImplementedError(f"dirichlet tag {t!r}: use 'boundary' or one of {names[:2*dim]}")
    return s


class DistributedSingleFieldFESpace:
    def __init__(self, model: DistributedDiscreteModel, reffe, dirichlet_tags="boundary"):
        self.model = model
        self.order = reffe[2]
        self.ncomp = model.dim if reffe[1] is VectorValue else 1
        self.sides = _sides_from_tags(model.dim, dirichlet_tags)
        h = C.c_void_p()
        L.call("gd_space_create", model.handle, self.order, self.ncomp, L.ptr(self.sides, C.c_int32), C.byref(h))
        self.handle = h
        self._gids = None
        self.dirichlet_values = None

    def num_free_dofs(self):
        n = C.c_int64()
        L.call("gd_space_num_free_dofs", self.handle, C.byref(n))
        return n.value

    def local_sizes(self, p):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        L.call("gd_space_local_sizes", self.handle, p, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    @property
    def gids(self) -> PRange:
        """``get_free_dof_ids(V)``: the DOF PRange built by generate_gids."""
        if self._gids is None:
            n = self.num_free_dofs()
            parts = []
            for p in range(self.model.num_parts):
                nl, _, _ = self.local_sizes(p)
                g = np.zeros(nl, dtype=np.int64)
                o = np.zeros(nl, dtype=np.int32)
                L.call("gd_space_get_gids", self.handle, p, L.ptr(g, C.c_int64), L.ptr(o, C.c_int32))
                parts.append(LocalIndices(n, p, g, o))
            self._gids = PRange(parts)
        return self._gids

    def dof_nodes(self, p):
        nl, _, _ = self.local_sizes(p)
        out = np.zeros(nl, dtype=np.int64)
        L.call("gd_space_dof_nodes", self.handle, p, L.ptr(out, C.c_int64))
        return out

    # lattice helpers ------------------------------------------------------------------
    @property
    def lattice(self):
        return tuple(self.order * c + 1 for c in self.model.cells)

    def lattice_xyz(self):
        """Coordinates of every global lattice node, (N, dim), x fastest."""
        N = self.lattice
        idx = np.indices(tuple(reversed(N))).reshape(self.model.dim, -1)[::-1]
        h = [(self.model.domain[2 * d + 1] - self.model.domain[2 * d]) / (self.order * self.model.cells[d])
             for d in range(self.model.dim)]
        return np.stack([self.model.domain[2 * d] + idx[d] * h[d] for d in range(self.model.dim)], axis=1)

    def __del__(self):
        try:
            if self.handle:
                L.load().gd_space_destroy(self.handle)
        except Exception:
            pass


def TestFESpace(model, reffe, dirichlet_tags="boundary", conformity=None, constraint=None):
    if constraint is not None:
        # ZeroMeanFESpace (FESpaces.jl:663-668, 872-910) is not built on the device
        raise NotImplementedError(f"TestFESpace(..., constraint={constraint}): not built on the device")
    if conformity in ("L2", ":L2"):
        from .dg import DistributedDGFESpace
        if reffe[1] is not float:
            raise NotImplementedError("discontinuous spaces: scalar fields")
        return DistributedDGFESpace(model, reffe[2])
    if conformity not in (None, "H1", ":H1"):
        raise NotImplementedError("conforming (H1) and discontinuous (L2) spaces")
    return DistributedSingleFieldFESpace(model, reffe, dirichlet_tags)


FESpace = TestFESpace


def TrialFESpace(u, V: DistributedSingleFieldFESpace):
    """``TrialFESpace(u, V)``: nodal interpolation of ``u`` on the Dirichlet nodes.

    ``u`` is a number, a vectorised callable of the coordinates, or a dense
    array over the global node lattice.  On a vector space: a constant vector (tuple), a
    callable returning one array (or number) per component, or a dense array of shape
    (lattice nodes, ncomp)."""
    if u is None or (np.isscalar(u) and u == 0):
        L.call("gd_space_set_dirichlet", V.handle, None, L.GD_HOST)
        V.dirichlet_values = None
        return V
    vals = _lattice_values(V, u)
    L.call("gd_space_set_dirichlet", V.handle, L.ptr(vals, C.c_double), L.GD_HOST)
    V.dirichlet_values = vals
    return V


def _lattice_values(V, u):
    """Nodal interpolation of u over the global node lattice, in the layout of the Dirichlet
    values: (lattice nodes,) or, on a vector space, (lattice nodes, ncomp).  u: a number, a
    vectorised callable of the coordinates (a tuple of components on a vector space), a
    constant vector, a dense array, or an FEFunction (its nodal values)."""
    nn = int(np.prod(V.lattice))
    if isinstance(u, FEFunction):
        return u.nodal_values()
    if V.ncomp > 1:
        if callable(u):
            xyz = V.lattice_xyz()
            comps = u(*[xyz[:, d] for d in range(V.model.dim)])
            if len(comps) != V.ncomp:
                raise ValueError(f"u returns {len(comps)} components, the space has {V.ncomp}")
            vals = np.stack([np.broadcast_to(np.asarray(c, dtype=np.float64), (nn,)) for c in comps], axis=1)
        else:
            vals = np.asarray(u, dtype=np.float64)
            if vals.ndim == 1 and vals.shape[0] == V.ncomp:
                vals = np.broadcast_to(vals, (nn, V.ncomp))
            vals = vals.reshape(nn, V.ncomp)
        return np.ascontiguousarray(vals)
    if callable(u):
        xyz = V.lattice_xyz()
        vals = np.asarray(u(*[xyz[:, d] for d in range(V.model.dim)]), dtype=np.float64)
        return np.broadcast_to(vals, (xyz.shape[0],)).copy()
    if np.isscalar(u):
        return np.full(nn, float(u))
    return np.ascontiguousarray(np.asarray(u, dtype=np.float64).reshape(nn))


# --------------------------------------------------------------------------------------
# weak forms (restricted vocabulary) and assembly (FESpaces.jl:746-862, Algebra.jl)
# --------------------------------------------------------------------------------------
@dataclass
class GradGradForm:
    """a(u,v) = ∫( κ ∇(v)⋅∇(u) )dΩ with κ per global cell (None = 1), or -- a CellField
    that varies inside the cells -- κ at the Gauss points of every cell (``kappa_qp``,
    shape (cells, nq^dim), points x fastest), its element matrices formed in ``precision``
    ("fp64", "bf16", "bf16x3", "bf16x6")."""

    kappa: np.ndarray | None
    measure: Measure
    kappa_qp: np.ndarray | None = None
    precision: str = "fp64"


@dataclass
class ElasticityForm:
    """a(u,v) = ∫( ε(v) ⊙ (σ∘ε(u)) )dΩ, σ(ε) = λ tr(ε) I + 2μ ε with Young's modulus E per
    global cell (None = 1) and Poisson ratio nu (λ, μ from E and nu)."""

    E: np.ndarray | None
    nu: float
    measure: Measure
    E_qp: np.ndarray | None = None
    precision: str = "fp64"


@dataclass
class SourceForm:
    """l(v) = ∫( v f )dΩ with f constant or nodal (dense over the lattice); for a vector
    space f is a constant vector (body force)."""

    f: object
    measure: Measure


@dataclass
class BoundarySourceForm:
    """l(v) = ∫( v g )dΓ on a BoundaryTriangulation; g is a vectorised callable of the
    coordinates and the outward unit normal, g(x, y[, z], nx, ny[, nz])."""

    g: object
    measure: Measure


class LinearFormSum(list):
    """A sum of linear forms, e.g. ∫( v f )dΩ + ∫( v g )dΓn."""

    def __add__(self, other):
        return LinearFormSum(list(self) + [other])


def _form_add(self, other):
    return LinearFormSum([self, other])


SourceForm.__add__ = _form_add
BoundarySourceForm.__add__ = _form_add


def integral_boundary_source(g, measure: Measure):
    return BoundarySourceForm(g, measure)


def boundary_quadrature_points(trian: BoundaryTriangulation, degree: int):
    """Face Gauss points of the flagged sides, in the layout gd_add_boundary_source
    expects: list of (side, coordinates (nfaces * nq^(dim-1), dim))."""
    model = trian.model
    dim = model.dim
    nq = (int(degree) + 2) // 2
    xq, _ = _gauss01(nq)
    h = [(model.domain[2 * d + 1] - model.domain[2 * d]) / model.cells[d] for d in range(dim)]
    out = []
    for side in range(2 * dim):
        if not trian.sides[side]:
            continue
        d = side // 2
        tang = [t for t in range(dim) if t != d]
        fc = np.indices(tuple(model.cells[t] for t in reversed(tang))).reshape(len(tang), -1)[::-1]
        qq = np.indices((nq,) * len(tang)).reshape(len(tang), -1)[::-1]
        pts = np.empty((fc.shape[1], qq.shape[1], dim))
        pts[:, :, d] = model.domain[2 * d + (side & 1)]
        for j, t in enumerate(tang):
            pts[:, :, t] = model.domain[2 * t] + (fc[j][:, None] + xq[qq[j]][None, :]) * h[t]
        out.append((side, pts.reshape(-1, dim)))
    return out


def _point_values(coef, measure):
    """A coefficient given as a function of the coordinates (evaluated at the Gauss points
    on the host, like the Dirichlet values of TrialFESpace) or as per-point values."""
    if callable(coef):
        model = measure.trian.model
        ncells = int(np.prod(model.cells))
        xq = quadrature_points(model, measure.degree).reshape(ncells, -1, model.dim)
        v = coef(*[xq[:, :, d] for d in range(model.dim)])
        return np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), xq.shape[:2]))
    return np.ascontiguousarray(coef, dtype=np.float64)


def integral_grad_grad(kappa=None, measure: Measure = None, precision: str = "fp64"):
    """∫( κ ∇(v)⋅∇(u) )dΩ: κ per cell (1-D array), at the Gauss points (2-D array
    (cells, nq^dim)) or a function of the coordinates (sampled at the Gauss points)."""
    if callable(kappa) or (kappa is not None and np.ndim(kappa) == 2):
        if precision not in L.QP_PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(L.QP_PRECISIONS)}")
        return GradGradForm(None, measure, _point_values(kappa, measure), precision)
    return GradGradForm(None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64), measure)


def integral_elasticity(E=None, nu=0.3, measure: Measure = None, precision: str = "fp64"):
    """∫( ε(v) ⊙ (σ∘ε(u)) )dΩ with E per cell, at the Gauss points, or a function of x."""
    if callable(E) or (E is not None and np.ndim(E) == 2):
        if precision not in L.QP_PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(L.QP_PRECISIONS)}")
        return ElasticityForm(None, float(nu), measure, _point_values(E, measure), precision)
    return ElasticityForm(None if E is None else np.ascontiguousarray(E, dtype=np.float64), float(nu), measure)


def integral_source(f=0.0, measure: Measure = None):
    return SourceForm(f, measure)


class DGAssembler:
    """``SparseMatrixAssembler(V, V, strategy)`` on a DG space: the strategy of its system."""

    def __init__(self, V, strategy):
        self.V, self.strategy = V, strategy


def SparseMatrixAssembler(U, V, strategy=None):
    from .dg import DistributedDGFESpace
    from .multifield import DistributedMultiFieldFESpace, MultiFieldAssembler
    if isinstance(V, DistributedDGFESpace):
        return DGAssembler(V, strategy or SubAssembledRows())
    if isinstance(U, DistributedMultiFieldFESpace) or isinstance(V, DistributedMultiFieldFESpace):
        return MultiFieldAssembler(U, V, strategy)
    return DistributedSparseMatrixAssembler(U, V, strategy or SubAssembledRows())


class DistributedSparseMatrixAssembler:
    def __init__(self, U, V, strategy):
        self.U, self.V, self.strategy = U, V, strategy
        h = C.c_void_p()
        L.call("gd_assembler_create", U.handle, V.handle, strategy.code, C.byref(h))
        self.handle = h
        self._symbolic = False

    def symbolic(self):
        if not self._symbolic:
            L.call("gd_assemble_symbolic", self.handle)
            self._symbolic = True

    def numeric(self, a, l):
        self.symbolic()
        bnd = []
        if isinstance(l, (list, tuple)):
            vol = [f for f in l if isinstance(f, SourceForm)]
            bnd = [f for f in l if isinstance(f, BoundarySourceForm)]
            if len(vol) > 1:
                raise NotImplementedError("one volume source term")
            l = vol[0] if vol else None
        elif isinstance(l, BoundarySourceForm):
            bnd, l = [l], None
        self._numeric(a, l)
        for bf in bnd:
            self._boundary(bf)

    def _boundary(self, bf):
        trian = bf.measure.trian
        dim = trian.model.dim
        vals = []
        for side, pts in boundary_quadrature_points(trian, bf.measure.degree):
            normal = [0.0] * dim
            normal[side // 2] = 1.0 if side & 1 else -1.0
            v = bf.g(*[pts[:, d] for d in range(dim)], *[np.full(len(pts), c) for c in normal])
            vals.append(np.broadcast_to(np.asarray(v, dtype=np.float64), (len(pts),)))
        g = np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1))
        sides = np.ascontiguousarray(trian.sides, dtype=np.int32)
        L.call("gd_add_boundary_source", self.handle, L.ptr(sides, C.c_int32), L.vptr(g), int(bf.measure.degree),
               L.GD_HOST)

    def _numeric(self, a, l):
        if isinstance(a, ElasticityForm) and a.E_qp is not None:
            c = L.gd_elasticity_qp()
            c.E_qp = a.E_qp.ctypes.data
            c.nu = a.nu
            f = l.f if l is not None else (0.0,) * self.V.model.dim
            f = tuple(float(x) for x in (f if not np.isscalar(f) else (0.0,) * self.V.model.dim))
            for i in range(3):
                c.force[i] = f[i] if i < len(f) else 0.0
            c.degree = int(a.measure.degree if a.measure is not None else 2 * self.V.order)
            c.precision = L.QP_PRECISIONS[a.precision]
            c.where = L.GD_HOST
            L.call("gd_assemble_elasticity_qp", self.handle, C.byref(c))
            return
        if isinstance(a, GradGradForm) and a.kappa_qp is not None:
            c = L.gd_qp_coeffs()
            c.kappa_qp = a.kappa_qp.ctypes.data
            f = l.f if l is not None else 0.0
            keep = None
            if np.isscalar(f):
                c.f_nodal = None
                c.f_const = float(f)
            else:
                keep = np.ascontiguousarray(f, dtype=np.float64)
                c.f_nodal = keep.ctypes.data
                c.f_const = 0.0
            c.degree = int(a.measure.degree if a.measure is not None else 2 * self.V.order)
            c.precision = L.QP_PRECISIONS[a.precision]
            c.where = L.GD_HOST
            L.call("gd_assemble_qp", self.handle, C.byref(c))
            return
        if isinstance(a, ElasticityForm):
            c = L.gd_elasticity()
            c.E = None if a.E is None else a.E.ctypes.data
            c.nu = a.nu
            f = l.f if l is not None else (0.0,) * self.V.model.dim
            f = tuple(float(x) for x in (f if not np.isscalar(f) else (0.0,) * self.V.model.dim))
            for i in range(3):
                c.force[i] = f[i] if i < len(f) else 0.0
            c.degree = int(a.measure.degree if a.measure is not None else 2 * self.V.order)
            c.where = L.GD_HOST
            L.call("gd_assemble_elasticity", self.handle, C.byref(c))
            return
        keep = []
        c = L.gd_coeffs()
        c.kappa = None if a.kappa is None else a.kappa.ctypes.data
        if a.kappa is not None:
            keep.append(a.kappa)
        f = l.f if l is not None else 0.0
        if np.isscalar(f):
            c.f_nodal = None
            c.f_const = float(f)
        else:
            fa = np.ascontiguousarray(f, dtype=np.float64)
            keep.append(fa)
            c.f_nodal = fa.ctypes.data
            c.f_const = 0.0
        c.degree = int(a.measure.degree if a.measure is not None else 2 * self.V.order)
        c.where = L.GD_HOST
        L.call("gd_assemble_numeric", self.handle, C.byref(c))

    def __del__(self):
        try:
            if self.handle:
                L.load().gd_assembler_destroy(self.handle)
        except Exception:
            pass


class PSparseMatrix:
    """A PSparseMatrix whose parts live on the device; host copies on request."""

    def __init__(self, assem: DistributedSparseMatrixAssembler):
        self.assem = assem
        self._parts = None

    @property
    def n_global(self):
        return self.assem.V.num_free_dofs()

    def _export(self):
        if self._parts is not None:
            return self._parts
        import scipy.sparse as sps
        V = self.assem.V
        out = []
        for p in range(V.model.num_parts):
            nr, nc, nnz, ngr, ngc = (C.c_int64() for _ in range(5))
            L.call("gd_matrix_sizes", self.assem.handle, p, *[C.byref(x) for x in (nr, nc, nnz, ngr, ngc)])
            rp = np.zeros(nr.value + 1, dtype=np.int64)
            ci = np.zeros(nnz.value, dtype=np.int32)
            vv = np.zeros(nnz.value, dtype=np.float64)
            grg = np.zeros(ngr.value, dtype=np.int64)
            gro = np.zeros(ngr.value, dtype=np.int32)
            gcg = np.zeros(ngc.value, dtype=np.int64)
            gco = np.zeros(ngc.value, dtype=np.int32)
            L.call("gd_matrix_export", self.assem.handle, p, L.ptr(rp, C.c_int64), L.ptr(ci, C.c_int32),
                   L.ptr(vv, C.c_double), L.ptr(grg, C.c_int64), L.ptr(gro, C.c_int32), L.ptr(gcg, C.c_int64),
                   L.ptr(gco, C.c_int32))
            _, nown, first = V.local_sizes(p)
            own = np.arange(first, first + nown, dtype=np.int64)
            rows = OwnAndGhostIndices(self.n_global, p, own, grg, gro)
            cols = OwnAndGhostIndices(self.n_global, p, own, gcg, gco)
            mat = sps.csr_matrix((vv, ci, rp), shape=(nr.value, nc.value))
            out.append((mat, rows, cols, (rp, ci, vv)))
        self._parts = out
        return out

    @property
    def matrix_partition(self):
        return [m for m, _, _, _ in self._export()]

    @property
    def row_partition(self):
        return [r for _, r, _, _ in self._export()]

    @property
    def col_partition(self):
        return [c for _, _, c, _ in self._export()]

    def csr_parts(self):
        return [raw for _, _, _, raw in self._export()]

    def __matmul__(self, x):
        return self.mul(x)

    def mul(self, x: np.ndarray) -> np.ndarray:
        """``A*x`` for a global vector (PVector over the owned rows)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n_global)
        L.call("gd_spmv", self.assem.handle, L.vptr(x), L.vptr(y), L.GD_HOST)
        return y

    def solve(self, rtol=1e-12, maxit=100000, method="jacobi_pcg", b=None):
        """``A \\ b``: for the assembled right-hand side, or for ``b`` (a PVector, an
        AssembledPVector or a global array in gid order) when given.

        ``method``: "jacobi_pcg" (FP64 Jacobi-PCG) or "mixed_ir" (FP64 iterative
        refinement around FP32 Jacobi-PCG with FP64 inner products)."""
        codes = {"jacobi_pcg": L.GD_SOLVE_JACOBI_PCG, "mixed_ir": L.GD_SOLVE_MIXED_IR}
        x = np.zeros(self.n_global)
        st = L.gd_solve_stats()
        if b is None:
            L.call("gd_solve", self.assem.handle, codes[method], float(rtol), int(maxit), L.vptr(x), L.GD_HOST,
                   C.byref(st))
        else:
            bv = b.global_values() if hasattr(b, "global_values") else b
            bv = np.ascontiguousarray(bv, dtype=np.float64)
            if bv.shape != (self.n_global,):
                raise ValueError(f"solve: b has {bv.shape[0]} entries, the matrix {self.n_global} rows")
            L.call("gd_solve_rhs", self.assem.handle, codes[method], float(rtol), int(maxit), L.vptr(bv), L.vptr(x),
                   L.GD_HOST, C.byref(st))
        self.last_stats = st
        return x


class PVector:
    def __init__(self, assem: DistributedSparseMatrixAssembler, matrix: PSparseMatrix):
        self.assem = assem
        self.matrix = matrix

    @property
    def partition(self):
        out = []
        for p, (mat, rows, _, _) in enumerate(self.matrix._export()):
            b = np.zeros(mat.shape[0])
            L.call("gd_vector_export", self.assem.handle, p, L.ptr(b, C.c_double))
            out.append(b)
        return out

    def global_values(self):
        b = np.zeros(self.matrix.n_global)
        L.call("gd_system_download", self.assem.handle, L.ptr(b, C.c_double), None)
        return b


def collect_cell_matrix_and_vector(U, V, a, l, uhd=None):
    return (a, l)


def collect_cell_matrix(U, V, a):
    """``collect_cell_matrix(U, V, a(du, dv))``: the bilinear form alone."""
    return _MatrixData(a)


def collect_cell_vector(V, l):
    """``collect_cell_vector(V, l(dv))``: the linear form alone (no Dirichlet lifting)."""
    return _VectorData(l)


@dataclass
class _MatrixData:
    a: object


@dataclass
class _VectorData:
    l: object


def _matrix_form(data):
    return data.a if isinstance(data, _MatrixData) else data


def _check_owner(obj, assem, what):
    if obj.assem is not assem:
        raise ValueError(f"{what} was allocated by another assembler")


def assemble_matrix_and_vector(assem: DistributedSparseMatrixAssembler, data):
    a, l = data
    assem.numeric(a, l)
    A = PSparseMatrix(assem)
    return A, PVector(assem, A)


def allocate_matrix_and_vector(assem: DistributedSparseMatrixAssembler, data):
    """The symbolic phase: a PSparseMatrix with the pattern and zero values and its PVector,
    to be filled by ``assemble_matrix_and_vector_`` (Julia's ``assemble_matrix_and_vector!``)."""
    assem.symbolic()
    A = PSparseMatrix(assem)
    return A, PVector(assem, A)


def assemble_matrix_and_vector_(A: "PSparseMatrix", b: "PVector", assem: DistributedSparseMatrixAssembler, data):
    """``assemble_matrix_and_vector!(A, b, assem, data)``: new values into the pattern of A."""
    _check_owner(A, assem, "the matrix")
    _check_owner(b, assem, "the vector")
    a, l = data
    assem.numeric(a, l)
    A._parts = None
    return A, b


def assemble_matrix(assem: DistributedSparseMatrixAssembler, data):
    """``assemble_matrix(assem, collect_cell_matrix(U, V, a))``.  The device assembles the
    right-hand side alongside (with f = 0); a PVector made from this assembler later shows it."""
    assem.numeric(_matrix_form(data), None)
    return PSparseMatrix(assem)


def allocate_matrix(assem: DistributedSparseMatrixAssembler, data):
    assem.symbolic()
    return PSparseMatrix(assem)


def assemble_matrix_(A: "PSparseMatrix", assem: DistributedSparseMatrixAssembler, data):
    """``assemble_matrix!(A, assem, data)``."""
    _check_owner(A, assem, "the matrix")
    assem.numeric(_matrix_form(data), None)
    A._parts = None
    return A


def _vector_coeffs(V, l):
    if isinstance(l, _VectorData):
        l = l.l
    if not isinstance(l, SourceForm):
        raise NotImplementedError("assemble_vector: one volume source term int(v f)")
    c = L.gd_coeffs()
    c.kappa = None
    keep = None
    if np.isscalar(l.f):
        c.f_nodal = None
        c.f_const = float(l.f)
    else:
        keep = np.ascontiguousarray(l.f, dtype=np.float64)
        c.f_nodal = keep.ctypes.data
        c.f_const = 0.0
    c.degree = int(l.measure.degree if l.measure is not None else 2 * V.order)
    c.where = L.GD_HOST
    return c, keep


def assemble_vector(assem: DistributedSparseMatrixAssembler, data):
    """``assemble_vector(assem, collect_cell_vector(V, l))``: the load vector alone, a new
    vector (the assembler's matrix and right-hand side are not touched)."""
    b = allocate_vector(assem, data)
    return assemble_vector_(b, assem, data)


def allocate_vector(assem: DistributedSparseMatrixAssembler, data):
    assem.symbolic()
    return AssembledPVector(assem, np.zeros(assem.V.num_free_dofs()))


def assemble_vector_(b: "AssembledPVector", assem: DistributedSparseMatrixAssembler, data):
    """``assemble_vector!(b, assem, data)``."""
    _check_owner(b, assem, "the vector")
    assem.symbolic()
    c, keep = _vector_coeffs(assem.V, data)
    L.call("gd_assemble_vector", assem.handle, C.byref(c), L.ptr(b.values, C.c_double), L.GD_HOST)
    return b


class AssembledPVector:
    """A PVector from ``assemble_vector``: global values over the owned rows (gid order); the
    per-part layout is the assembler's row partition (owned rows, then its ghost rows, which
    hold zeros)."""

    def __init__(self, assem: DistributedSparseMatrixAssembler, values: np.ndarray):
        self.assem = assem
        self.values = np.ascontiguousarray(values, dtype=np.float64)

    def __len__(self):
        return len(self.values)

    def global_values(self):
        return self.values.copy()

    @property
    def partition(self):
        out = []
        V = self.assem.V
        for p in range(V.model.num_parts):
            nr, nc, nnz, ngr, ngc = (C.c_int64() for _ in range(5))
            L.call("gd_matrix_sizes", self.assem.handle, p, *[C.byref(x) for x in (nr, nc, nnz, ngr, ngc)])
            _, nown, first = V.local_sizes(p)
            out.append(np.concatenate([self.values[first:first + nown], np.zeros(ngr.value)]))
        return out


class AffineFEOperator:
    def __init__(self, a, l, U, V, assem=None):
        from .dg import DistributedDGFESpace, assemble_dg
        from .multifield import MultiFieldAssembler, assemble_multifield
        self.U, self.V = U, V
        self.a, self.l = a, l
        if isinstance(V, DistributedDGFESpace):
            if U is not V:
                raise NotImplementedError("DG: trial space = test space")
            strategy = getattr(assem, "strategy", None)
            self.assem = assem
            self.matrix, self.vector = assemble_dg(V, a, l, strategy)
            return
        self.assem = assem if assem is not None else SparseMatrixAssembler(U, V)
        if isinstance(self.assem, MultiFieldAssembler):
            self.matrix, self.vector = assemble_multifield(self.assem, a, l)
        else:
            self.matrix, self.vector = assemble_matrix_and_vector(self.assem, (a, l))


class FEFunction:
    """``FEFunction(U, x)`` / ``FEFunction(U, x, dirichlet_values)``: free values made
    consistent on every part; the Dirichlet values are the trial space's unless given (in
    the trial space's layout: one value per lattice node, (nodes, ncomp) on vector spaces)."""

    def __init__(self, U: DistributedSingleFieldFESpace, x: np.ndarray, dirichlet_values=None):
        self.U = U
        self.free_values = np.ascontiguousarray(x, dtype=np.float64)
        self.dirichlet_values = (None if dirichlet_values is None
                                 else np.ascontiguousarray(dirichlet_values, dtype=np.float64))

    def _dirichlet(self):
        return self.dirichlet_values if self.dirichlet_values is not None else self.U.dirichlet_values

    def local_values(self, p):
        nl, _, _ = self.U.local_sizes(p)
        out = np.zeros(nl)
        L.call("gd_fe_function_local", self.U.handle, p, L.vptr(self.free_values), L.GD_HOST,
               L.ptr(out, C.c_double))
        return out

    def nodal_values(self):
        """Dense lattice array of nodal values, (nodes,) or (nodes, ncomp): free values from
        x, Dirichlet values from this function (else from the trial space)."""
        N, nc = int(np.prod(self.U.lattice)), self.U.ncomp
        shape = (N,) if nc == 1 else (N, nc)
        d = self._dirichlet()
        u = np.zeros(shape) if d is None else np.asarray(d, dtype=np.float64).reshape(shape).copy()
        for p in range(self.U.model.num_parts):
            nodes, vals = self.U.dof_nodes(p), self.local_values(p)
            if nc == 1:
                u[nodes] = vals
            else:
                u[nodes, np.arange(len(nodes)) % nc] = vals
        return u


# interpolation (FESpaces.jl interpolate* on the distributed spaces; the function is
# evaluated at the lattice nodes on the host, like the Dirichlet values of TrialFESpace)
def zero_free_values(U: DistributedSingleFieldFESpace) -> np.ndarray:
    return np.zeros(U.num_free_dofs())


def zero_dirichlet_values(U: DistributedSingleFieldFESpace) -> np.ndarray:
    N = int(np.prod(U.lattice))
    return np.zeros(N if U.ncomp == 1 else (N, U.ncomp))


def get_dirichlet_dof_values(U: DistributedSingleFieldFESpace) -> np.ndarray:
    """The trial space's Dirichlet values (lattice layout; only Dirichlet nodes are read)."""
    return zero_dirichlet_values(U) if U.dirichlet_values is None else U.dirichlet_values.copy()


def _free_values_of(U, u) -> np.ndarray:
    """u at every free DOF of U, global order."""
    if isinstance(u, FEFunction) and u.U is U:
        return u.free_values.copy()
    lat = _lattice_values(U, u)
    out = np.zeros(U.num_free_dofs())
    for p in range(U.model.num_parts):
        li = U.gids.partition()[p]
        own = li.local_to_owner == p
        nodes = U.dof_nodes(p)[own]
        if U.ncomp == 1:
            out[li.local_to_global[own]] = lat[nodes]
        else:
            comp = np.arange(len(li.local_to_global))[own] % U.ncomp
            out[li.local_to_global[own]] = lat[nodes, comp]
    return out


def interpolate(u, U: DistributedSingleFieldFESpace) -> FEFunction:
    """``interpolate(u, U)``: u at the free DOFs; the Dirichlet values stay the space's."""
    return FEFunction(U, _free_values_of(U, u))


def interpolate_everywhere(u, U: DistributedSingleFieldFESpace) -> FEFunction:
    """``interpolate_everywhere(u, U)``: u at the free and at the Dirichlet DOFs."""
    return FEFunction(U, _free_values_of(U, u), _lattice_values(U, u))


def interpolate_dirichlet(u, U: DistributedSingleFieldFESpace) -> FEFunction:
    """``interpolate_dirichlet(u, U)``: zero free values, u at the Dirichlet DOFs."""
    return FEFunction(U, zero_free_values(U), _lattice_values(U, u))


def interpolate_everywhere_(u, free_values, dirichlet_values, U: DistributedSingleFieldFESpace) -> FEFunction:
    """``interpolate_everywhere!(u, free_values, dirichlet_values, U)``."""
    free_values[...] = _free_values_of(U, u)
    dirichlet_values[...] = np.asarray(_lattice_values(U, u)).reshape(np.shape(dirichlet_values))
    return FEFunction(U, free_values, dirichlet_values)


def interpolate_dirichlet_(u, free_values, dirichlet_values, U: DistributedSingleFieldFESpace) -> FEFunction:
    """``interpolate_dirichlet!(u, free_values, dirichlet_values, U)``."""
    free_values[...] = 0.0
    dirichlet_values[...] = np.asarray(_lattice_values(U, u)).reshape(np.shape(dirichlet_values))
    return FEFunction(U, free_values, dirichlet_values)


def _gauss01(nq):
    x, w = np.polynomial.legendre.leggauss(nq)
    return 0.5 * (x + 1.0), 0.5 * w


def quadrature_points(model: DistributedDiscreteModel, degree: int):
    """Physical coordinates (ncells * nq^dim, dim) of the tensor Gauss points of every
    global cell (cells lexicographic, points x fastest), nq = (degree + 2) // 2."""
    dim = model.dim
    nq = (int(degree) + 2) // 2
    xq, _ = _gauss01(nq)
    h = [(model.domain[2 * d + 1] - model.domain[2 * d]) / model.cells[d] for d in range(dim)]
    cells = np.indices(tuple(reversed(model.cells))).reshape(dim, -1)[::-1]        # (dim, ncells), x fastest
    q = np.indices((nq,) * dim).reshape(dim, -1)[::-1]                              # (dim, nqt), x fastest
    out = np.empty((cells.shape[1], q.shape[1], dim))
    for d in range(dim):
        out[:, :, d] = model.domain[2 * d] + (cells[d][:, None] + xq[q[d]][None, :]) * h[d]
    return out.reshape(-1, dim)


def l2_error(uh: "FEFunction", u_exact, measure: Measure) -> float:
    """``sqrt(sum(∫( abs2(u - uh) )dΩ))`` on the device; ``u_exact`` is a vectorised callable
    of the coordinates (a tuple of components on vector spaces)."""
    from .dg import DGFEFunction, dg_l2_error
    if isinstance(uh, DGFEFunction):
        return dg_l2_error(uh, u_exact, measure)
    U = uh.U
    xyz = quadrature_points(U.model, measure.degree)
    vals = u_exact(*[xyz[:, d] for d in range(U.model.dim)])
    if U.ncomp > 1:
        vals = np.stack([np.broadcast_to(np.asarray(v, dtype=np.float64), (xyz.shape[0],)) for v in vals], axis=1)
    else:
        vals = np.broadcast_to(np.asarray(vals, dtype=np.float64), (xyz.shape[0],))
    vals = np.ascontiguousarray(vals, dtype=np.float64).reshape(-1)
    err = C.c_double()
    # a function with its own Dirichlet values: the space carries them for this call
    own = uh.dirichlet_values
    swap = own is not None and own is not U.dirichlet_values
    if swap:
        L.call("gd_space_set_dirichlet", U.handle, L.ptr(own, C.c_double), L.GD_HOST)
    try:
        L.call("gd_l2_error", U.handle, L.vptr(uh.free_values), L.vptr(vals), int(measure.degree), L.GD_HOST,
               C.byref(err))
    finally:
        if swap:
            L.call("gd_space_set_dirichlet", U.handle,
                   None if U.dirichlet_values is None else L.ptr(U.dirichlet_values, C.c_double), L.GD_HOST)
    return err.value


def solve(op: AffineFEOperator, rtol=1e-12, maxit=100000):
    from .dg import DGFEFunction, DistributedDGFESpace
    x = op.matrix.solve(rtol=rtol, maxit=maxit)
    if isinstance(op.U, DistributedDGFESpace):
        return DGFEFunction(op.U, x)
    return FEFunction(op.U, x)
