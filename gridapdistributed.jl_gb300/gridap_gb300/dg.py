"""Discontinuous Galerkin over the C ABI (``gd_dg_*``), mirroring the DG part of the
reference's Poisson test (test/PoissonTests.jl:47-77)::

    V_dg = FESpace(model, ReferenceFE(lagrangian, float, k), conformity="L2")
    Λ = Skeleton(model); Γd = Boundary(model, tags=...); Γn = Boundary(model, tags=...)
    dΩ, dΛ, dΓd, dΓn = Measure(Ω, 2k), Measure(Λ, 2k), Measure(Γd, 2k), Measure(Γn, 2k)
    a_dg = integral_sipg(gamma, h, dΩ, dΓd, dΛ)                      # a_dg(u, v)
    l_dg = integral_sipg_source(f, u, g, gamma, h, dΩ, dΓn, dΓd)     # l_dg(v)
    op = AffineFEOperator(a_dg, l_dg, V_dg, V_dg)
    uh = solve(op); l2_error(uh, u, dΩ)

The bilinear form is the symmetric interior penalty form of that test; f is a number or
a vectorised callable of the coordinates, u (the Dirichlet data) and g (the Neumann
data, called with the coordinates and the outward normal's components) are callables.
Assembly follows FullyAssembledRows (each owned row summed by its part): the global
operator equals the reference's; its SubAssembledRows local parts are not reproduced.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .distributed import (BoundaryTriangulation, LocalIndices, Measure, OwnAndGhostIndices, PRange,
                          boundary_quadrature_points, quadrature_points)


class DistributedDGFESpace:
    """``FESpace(model, reffe, conformity=:L2)``: discontinuous scalar Q_k, k <= 3."""

    def __init__(self, model, order):
        self.model = model
        self.order = order
        self.ncomp = 1
        h = C.c_void_p()
        L.call("gd_dg_space_create", model.handle, int(order), C.byref(h))
        self.handle = h
        self._gids = None

    def num_free_dofs(self):
        n = C.c_int64()
        L.call("gd_dg_num_free_dofs", self.handle, C.byref(n))
        return n.value

    def local_sizes(self, p):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        L.call("gd_dg_local_sizes", self.handle, p, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    @property
    def gids(self) -> PRange:
        if self._gids is None:
            n = self.num_free_dofs()
            parts = []
            for p in range(self.model.num_parts):
                nl, _, _ = self.local_sizes(p)
                g = np.zeros(nl, dtype=np.int64)
                o = np.zeros(nl, dtype=np.int32)
                L.call("gd_dg_get_gids", self.handle, p, L.ptr(g, C.c_int64), L.ptr(o, C.c_int32))
                parts.append(LocalIndices(n, p, g, o))
            self._gids = PRange(parts)
        return self._gids

    def __del__(self):
        try:
            if self.handle:
                L.load().gd_dg_space_destroy(self.handle)
        except Exception:
            pass


@dataclass
class SkeletonTriangulation:
    """``Skeleton(model)``: the interior faces."""

    model: object


def Skeleton(model):
    return SkeletonTriangulation(model)


@dataclass
class SIPGForm:
    """∫(∇v⋅∇u)dΩ + ∫((γ/h) v u − v (n⋅∇u) − (n⋅∇v) u)dΓd
    + ∫((γ/h) jump(v n)⋅jump(u n) − jump(v n)⋅mean(∇u) − mean(∇v)⋅jump(u n))dΛ."""

    gamma: float
    h: float
    measure: Measure
    dirichlet: Measure | None
    skeleton: Measure


@dataclass
class SIPGSource:
    """∫(v f)dΩ + ∫(v g)dΓn + ∫((γ/h) v u − (n⋅∇v) u)dΓd."""

    f: object
    u: object
    g: object
    gamma: float
    h: float
    measure: Measure
    neumann: Measure | None
    dirichlet: Measure | None


def integral_sipg(gamma, h, measure: Measure, dirichlet: Measure | None, skeleton: Measure):
    return SIPGForm(float(gamma), float(h), measure, dirichlet, skeleton)


def integral_sipg_source(f, u, g, gamma, h, measure: Measure, neumann: Measure | None = None,
                         dirichlet: Measure | None = None):
    return SIPGSource(f, u, g, float(gamma), float(h), measure, neumann, dirichlet)


def _face_values(fn, trian: BoundaryTriangulation, degree, with_normal):
    dim = trian.model.dim
    vals = []
    for side, pts in boundary_quadrature_points(trian, degree):
        args = [pts[:, d] for d in range(dim)]
        if with_normal:
            normal = [0.0] * dim
            normal[side // 2] = 1.0 if side & 1 else -1.0
            args += [np.full(len(pts), c) for c in normal]
        v = fn(*args)
        vals.append(np.broadcast_to(np.asarray(v, dtype=np.float64), (len(pts),)))
    return np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(1))


class DGMatrix:
    """The assembled SIPG operator: a PSparseMatrix over the DG dofs (per part the owned
    rows, and the touched ghost rows under SubAssembledRows) with its right-hand side;
    parts live on the device."""

    def __init__(self, V: DistributedDGFESpace):
        self.V = V
        self._parts = None

    @property
    def n_global(self):
        return self.V.num_free_dofs()

    def _export(self):
        if self._parts is not None:
            return self._parts
        import scipy.sparse as sps
        out = []
        for p in range(self.V.model.num_parts):
            a, b, n, gr, g = (C.c_int64() for _ in range(5))
            L.call("gd_dg_matrix_sizes", self.V.handle, p, C.byref(a), C.byref(b), C.byref(n), C.byref(gr),
                   C.byref(g))
            rp = np.zeros(a.value + 1, dtype=np.int64)
            ci = np.zeros(n.value, dtype=np.int32)
            vv = np.zeros(n.value, dtype=np.float64)
            rg = np.zeros(gr.value, dtype=np.int64)
            ro = np.zeros(gr.value, dtype=np.int32)
            gg = np.zeros(g.value, dtype=np.int64)
            go = np.zeros(g.value, dtype=np.int32)
            bb = np.zeros(a.value, dtype=np.float64)
            L.call("gd_dg_matrix_export", self.V.handle, p, L.ptr(rp, C.c_int64), L.ptr(ci, C.c_int32),
                   L.ptr(vv, C.c_double), L.ptr(rg, C.c_int64), L.ptr(ro, C.c_int32), L.ptr(gg, C.c_int64),
                   L.ptr(go, C.c_int32), L.ptr(bb, C.c_double))
            _, nown, first = self.V.local_sizes(p)
            own = np.arange(first, first + nown, dtype=np.int64)
            rows = OwnAndGhostIndices(self.n_global, p, own, rg, ro)
            cols = OwnAndGhostIndices(self.n_global, p, own, gg, go)
            out.append((sps.csr_matrix((vv, ci, rp), shape=(a.value, b.value)), rows, cols, (rp, ci, vv), bb))
        self._parts = out
        return out

    def csr_parts(self):
        return [raw for _, _, _, raw, _ in self._export()]

    @property
    def row_partition(self):
        return [r for _, r, _, _, _ in self._export()]

    @property
    def col_partition(self):
        return [c for _, _, c, _, _ in self._export()]

    def rhs_parts(self):
        return [b for _, _, _, _, b in self._export()]

    def mul(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n_global)
        L.call("gd_dg_spmv", self.V.handle, L.vptr(x), L.vptr(y), L.GD_HOST)
        return y

    def __matmul__(self, x):
        return self.mul(x)

    def solve(self, rtol=1e-12, maxit=100000, method="jacobi_pcg"):
        if method != "jacobi_pcg":
            raise NotImplementedError("DG systems: FP64 Jacobi-PCG")
        x = np.zeros(self.n_global)
        st = L.gd_solve_stats()
        L.call("gd_dg_solve", self.V.handle, float(rtol), int(maxit), L.vptr(x), L.GD_HOST, C.byref(st))
        self.last_stats = st
        return x


class DGVector:
    def __init__(self, matrix: DGMatrix):
        self.matrix = matrix

    @property
    def partition(self):
        return self.matrix.rhs_parts()

    def global_values(self):
        """The owned entries of every part in gid order (ghost rows left out)."""
        rows = self.matrix.row_partition
        return np.concatenate([b[:len(r.own_to_global)] for b, r in zip(self.matrix.rhs_parts(), rows)])


def assemble_dg(V: DistributedDGFESpace, a: SIPGForm, l: SIPGSource, strategy=None):
    """``assemble_matrix_and_vector`` for the SIPG forms on a DG space; ``strategy`` is
    SubAssembledRows() (the reference's default) or FullyAssembledRows()."""
    from .distributed import SubAssembledRows
    strategy = strategy if strategy is not None else SubAssembledRows()
    L.call("gd_dg_set_strategy", V.handle, strategy.code)
    model = V.model
    dim = model.dim
    deg = int(a.measure.degree)
    for m in (a.dirichlet, a.skeleton, l.neumann, l.dirichlet, l.measure):
        if m is not None and int(m.degree) != deg:
            raise NotImplementedError("one quadrature degree for the cells and the faces")
    if l is not None and (l.gamma != a.gamma or l.h != a.h):
        raise ValueError("the linear form's penalty must match the bilinear form's")
    dsides = np.zeros(2 * dim, dtype=np.int32) if a.dirichlet is None else \
        np.ascontiguousarray(a.dirichlet.trian.sides, dtype=np.int32)
    nsides = np.zeros(2 * dim, dtype=np.int32) if l is None or l.neumann is None else \
        np.ascontiguousarray(l.neumann.trian.sides, dtype=np.int32)
    keep = [dsides, nsides]
    F = L.gd_dg_form()
    F.gamma, F.h, F.degree, F.where = a.gamma, a.h, deg, L.GD_HOST
    F.dirichlet_sides = dsides.ctypes.data
    F.neumann_sides = nsides.ctypes.data
    F.f_const, F.f_qp = 0.0, None
    F.ud_qp = F.g_qp = None
    if l is not None:
        if callable(l.f):
            xyz = quadrature_points(model, deg)
            fq = np.ascontiguousarray(np.broadcast_to(np.asarray(l.f(*[xyz[:, d] for d in range(dim)]),
                                                                 dtype=np.float64), (xyz.shape[0],)))
            keep.append(fq)
            F.f_qp = fq.ctypes.data
        else:
            F.f_const = float(l.f if l.f is not None else 0.0)
        if dsides.any():
            ud = _face_values(l.u, a.dirichlet.trian, deg, False)
            keep.append(ud)
            F.ud_qp = ud.ctypes.data
        if nsides.any():
            g = _face_values(l.g, l.neumann.trian, deg, True)
            keep.append(g)
            F.g_qp = g.ctypes.data
    L.call("gd_dg_assemble", V.handle, C.byref(F))
    A = DGMatrix(V)
    return A, DGVector(A)


class DGFEFunction:
    def __init__(self, V: DistributedDGFESpace, x: np.ndarray):
        self.U = V
        self.free_values = np.ascontiguousarray(x, dtype=np.float64)


def dg_l2_error(uh: DGFEFunction, u_exact, measure: Measure) -> float:
    V = uh.U
    xyz = quadrature_points(V.model, measure.degree)
    vals = np.ascontiguousarray(np.broadcast_to(np.asarray(u_exact(*[xyz[:, d] for d in range(V.model.dim)]),
                                                           dtype=np.float64), (xyz.shape[0],)))
    err = C.c_double()
    L.call("gd_dg_l2_error", V.handle, L.vptr(uh.free_values), L.vptr(vals), int(measure.degree), L.GD_HOST,
           C.byref(err))
    return err.value
