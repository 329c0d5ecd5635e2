"""Multi-field spaces, forms and block assembly over the C ABI (``gd_mfield_*``,
``gd_mfmat_*``), mirroring GridapDistributed's MultiField API (src/MultiField.jl)::

    Y = MultiFieldFESpace([V, V])                                   # ConsecutiveMultiFieldStyle
    Yb = MultiFieldFESpace([V, V], style=BlockMultiFieldStyle())    # one block per field
    X, Xb = MultiFieldFESpace([U, U]), MultiFieldFESpace([U, U], style=BlockMultiFieldStyle())
    a = integral_multifield(stiffness=[[1, 0], [0, 0]], mass=[[0, 0], [1, 1]], measure=dΩ)
    l = integral_multifield_source([1.0, 1.0], dΩ)
    op = AffineFEOperator(a, l, X, Y, SparseMatrixAssembler(X, Y, FullyAssembledRows()))
    op.matrix       # PSparseMatrix over the multi-field gids, or a BlockPMatrix

The fields share one scalar test space (and one trial space); the bilinear form is
``sum_ij ∫(κ (stiffness[i][j] ∇(u_j)⋅∇(v_i) + mass[i][j] u_j v_i))dΩ``, the linear form
``sum_i ∫(src[i] v_i)dΩ`` — the vocabulary of the reference's block-assembler test
(test/BlockSparseMatrixAssemblersTests.jl:111-114).  Assembly strategy: SubAssembledRows
(the default of the reference's multi-field assemblers) or FullyAssembledRows (the strategy
that test passes to its assemblers).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from .distributed import (DistributedSingleFieldFESpace, LocalIndices, Measure, OwnAndGhostIndices, PRange,
                          SubAssembledRows)


class ConsecutiveMultiFieldStyle:
    """All fields in one numbering (the default style)."""


class BlockMultiFieldStyle:
    """``BlockMultiFieldStyle(NB, SB)``: NB blocks of SB[k] consecutive fields (default:
    one block per field).  Field permutations are not supported."""

    def __init__(self, nblocks=None, sizes=None, permutation=None):
        if permutation is not None:
            raise NotImplementedError("field permutations")
        self.nblocks, self.sizes = nblocks, sizes

    def groups(self, nfields):
        if self.nblocks is None:
            return [[f] for f in range(nfields)]
        sizes = self.sizes if self.sizes is not None else (1,) * self.nblocks
        if len(sizes) != self.nblocks or sum(sizes) != nfields:
            raise ValueError("BlockMultiFieldStyle: block sizes must add up to the number of fields")
        out, f = [], 0
        for s in sizes:
            out.append(list(range(f, f + s)))
            f += s
        return out


class DistributedMultiFieldFESpace:
    def __init__(self, spaces, style=None):
        spaces = list(spaces)
        if not spaces or any(not isinstance(s, DistributedSingleFieldFESpace) for s in spaces):
            raise TypeError("MultiFieldFESpace: a list of single-field spaces")
        if any(s is not spaces[0] for s in spaces):
            raise NotImplementedError("multi-field spaces whose fields share one scalar space")
        if spaces[0].ncomp != 1:
            raise NotImplementedError("scalar fields")
        self.fields = spaces
        self.space = spaces[0]
        self.style = style if style is not None else ConsecutiveMultiFieldStyle()
        self._gids = {}

    def num_fields(self):
        return len(self.fields)

    def __len__(self):
        return len(self.fields)

    def __getitem__(self, i):
        return self.fields[i]

    @property
    def model(self):
        return self.space.model

    def groups(self):
        if isinstance(self.style, BlockMultiFieldStyle):
            return self.style.groups(len(self.fields))
        return [list(range(len(self.fields)))]

    def num_free_dofs(self):
        return len(self.fields) * self.space.num_free_dofs()


def MultiFieldFESpace(spaces, style=None):
    return DistributedMultiFieldFESpace(spaces, style)


@dataclass
class MultiFieldForm:
    """a((u_j), (v_i)) = Σ_ij ∫(κ (stiffness[i][j] ∇(u_j)⋅∇(v_i) + mass[i][j] u_j v_i))dΩ."""

    stiffness: np.ndarray
    mass: np.ndarray
    measure: Measure
    kappa: np.ndarray | None = None


@dataclass
class MultiFieldSource:
    """l((v_i)) = Σ_i ∫(src[i] v_i)dΩ."""

    src: np.ndarray
    measure: Measure


def integral_multifield(stiffness=None, mass=None, measure: Measure = None, kappa=None):
    n = len(stiffness if stiffness is not None else mass)
    st = np.zeros((n, n)) if stiffness is None else np.asarray(stiffness, dtype=np.float64)
    ms = np.zeros((n, n)) if mass is None else np.asarray(mass, dtype=np.float64)
    if st.shape != (n, n) or ms.shape != (n, n):
        raise ValueError("stiffness and mass are n x n")
    k = None if kappa is None else np.ascontiguousarray(kappa, dtype=np.float64)
    return MultiFieldForm(st, ms, measure, k)


def integral_multifield_source(src, measure: Measure = None):
    return MultiFieldSource(np.asarray(src, dtype=np.float64), measure)


class MultiFieldAssembler:
    """``SparseMatrixAssembler(X, Y, strategy)`` for multi-field spaces (SubAssembledRows by
    default, as the reference's): the scalar assembler of the shared space plus the field
    set (gd_mfield)."""

    def __init__(self, X: DistributedMultiFieldFESpace, Y: DistributedMultiFieldFESpace, strategy=None):
        strategy = strategy or SubAssembledRows()
        if X.num_fields() != Y.num_fields() or X.space is not Y.space:
            raise NotImplementedError("trial and test fields on one shared scalar space")
        if type(X.style) is not type(Y.style) or X.groups() != Y.groups():
            raise ValueError("trial and test spaces must have the same multi-field style")
        self.X, self.Y, self.strategy = X, Y, strategy
        V = Y.space
        h = C.c_void_p()
        L.call("gd_assembler_create", V.handle, V.handle, strategy.code, C.byref(h))
        self.handle = h
        L.call("gd_assemble_symbolic", self.handle)
        m = C.c_void_p()
        L.call("gd_mfield_create", self.handle, Y.num_fields(), C.byref(m))
        self.mfield = m
        self._mats = []

    def numeric(self, a: MultiFieldForm, l: MultiFieldSource | None):
        n = self.Y.num_fields()
        st = np.ascontiguousarray(a.stiffness, dtype=np.float64)
        ms = np.ascontiguousarray(a.mass, dtype=np.float64)
        src = np.zeros(n) if l is None else np.ascontiguousarray(l.src, dtype=np.float64)
        if st.shape != (n, n) or src.shape != (n,):
            raise ValueError("form sizes do not match the number of fields")
        c = L.gd_coeffs()
        c.kappa = None if a.kappa is None else a.kappa.ctypes.data
        c.f_nodal = None
        c.f_const = 0.0
        c.degree = int(a.measure.degree if a.measure is not None else 2 * self.Y.space.order)
        c.where = L.GD_HOST
        L.call("gd_mfield_assemble", self.mfield, L.ptr(st, C.c_double), L.ptr(ms, C.c_double),
               L.ptr(src, C.c_double), C.byref(c))
        for mat in self._mats:
            mat._refresh()

    def matrix(self, rf, cf):
        mat = MultiFieldMatrix(self, rf, cf)
        self._mats.append(mat)
        return mat

    def gids(self, fields):
        """PRange of the multi-field space of `fields` (generate_multi_field_gids)."""
        V = self.Y.space
        nf = len(fields)
        f = np.ascontiguousarray(fields, dtype=np.int32)
        parts = []
        for p in range(V.model.num_parts):
            nl, _, _ = V.local_sizes(p)
            g = np.zeros(nf * nl, dtype=np.int64)
            o = np.zeros(nf * nl, dtype=np.int32)
            L.call("gd_mfield_gids", self.mfield, nf, L.ptr(f, C.c_int32), p, L.ptr(g, C.c_int64),
                   L.ptr(o, C.c_int32))
            parts.append(LocalIndices(nf * V.num_free_dofs(), p, g, o))
        return PRange(parts)

    def __del__(self):
        try:
            lib = L.load()
            for mat in self._mats:
                mat._destroy()
            if self.mfield:
                lib.gd_mfield_destroy(self.mfield)
            if self.handle:
                lib.gd_assembler_destroy(self.handle)
        except Exception:
            pass


class MultiFieldMatrix:
    """A PSparseMatrix over the multi-field numbering of row fields `rf` and column
    fields `cf` (a block of a BlockPMatrix, or the whole ConsecutiveMultiFieldStyle
    matrix), with its right-hand side; parts live on the device."""

    def __init__(self, assem: MultiFieldAssembler, rf, cf):
        self.assem, self.rf, self.cf = assem, list(rf), list(cf)
        r = np.ascontiguousarray(rf, dtype=np.int32)
        c = np.ascontiguousarray(cf, dtype=np.int32)
        h = C.c_void_p()
        L.call("gd_mfmat_create", assem.mfield, len(r), L.ptr(r, C.c_int32), len(c), L.ptr(c, C.c_int32),
               C.byref(h))
        self.handle = h
        self._parts = None

    def _refresh(self):
        L.call("gd_mfmat_refresh", self.handle)
        self._parts = None

    def _destroy(self):
        if self.handle:
            L.load().gd_mfmat_destroy(self.handle)
            self.handle = None

    @property
    def n_rows(self):
        return len(self.rf) * self.assem.Y.space.num_free_dofs()

    @property
    def n_cols(self):
        return len(self.cf) * self.assem.Y.space.num_free_dofs()

    def _export(self):
        if self._parts is not None:
            return self._parts
        import scipy.sparse as sps
        V = self.assem.Y.space
        nr, nc = len(self.rf), len(self.cf)
        out = []
        for p in range(V.model.num_parts):
            a, b, n, gr, g = (C.c_int64() for _ in range(5))
            L.call("gd_mfmat_sizes", self.handle, p, C.byref(a), C.byref(b), C.byref(n), C.byref(gr), C.byref(g))
            rp = np.zeros(a.value + 1, dtype=np.int64)
            ci = np.zeros(n.value, dtype=np.int32)
            vv = np.zeros(n.value, dtype=np.float64)
            rg = np.zeros(gr.value, dtype=np.int64)
            ro = np.zeros(gr.value, dtype=np.int32)
            gg = np.zeros(g.value, dtype=np.int64)
            go = np.zeros(g.value, dtype=np.int32)
            bb = np.zeros(a.value, dtype=np.float64)
            L.call("gd_mfmat_export", self.handle, p, L.ptr(rp, C.c_int64), L.ptr(ci, C.c_int32),
                   L.ptr(vv, C.c_double), L.ptr(rg, C.c_int64), L.ptr(ro, C.c_int32), L.ptr(gg, C.c_int64),
                   L.ptr(go, C.c_int32), L.ptr(bb, C.c_double))
            _, nown, first = V.local_sizes(p)
            rows = OwnAndGhostIndices(self.n_rows, p, np.arange(nr * first, nr * (first + nown), dtype=np.int64),
                                      rg, ro)
            cols = OwnAndGhostIndices(self.n_cols, p, np.arange(nc * first, nc * (first + nown), dtype=np.int64),
                                      gg, go)
            mat = sps.csr_matrix((vv, ci, rp), shape=(a.value, b.value))
            out.append((mat, rows, cols, (rp, ci, vv), bb))
        self._parts = out
        return out

    @property
    def matrix_partition(self):
        return [m for m, _, _, _, _ in self._export()]

    @property
    def row_partition(self):
        return [r for _, r, _, _, _ in self._export()]

    @property
    def col_partition(self):
        return [c for _, _, c, _, _ in self._export()]

    def csr_parts(self):
        return [raw for _, _, _, raw, _ in self._export()]

    def rhs_parts(self):
        return [b for _, _, _, _, b in self._export()]

    def mul(self, x: np.ndarray) -> np.ndarray:
        """``A*x``: x over the column fields' numbering, the result over the rows'."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.shape != (self.n_cols,):
            raise ValueError("x has the column numbering's length")
        y = np.zeros(self.n_rows)
        L.call("gd_mfmat_spmv", self.handle, L.vptr(x), L.vptr(y), L.GD_HOST)
        return y

    def __matmul__(self, x):
        return self.mul(x)


class MultiFieldVector:
    """A PVector over a row numbering: the right-hand side rows of `matrix`."""

    def __init__(self, matrix: MultiFieldMatrix):
        self.matrix = matrix

    @property
    def partition(self):
        return self.matrix.rhs_parts()

    def global_values(self):
        """The owned entries of every part in gid order (ghost rows left out)."""
        rows = self.matrix.row_partition
        return np.concatenate([b[:len(r.own_to_global)] for b, r in zip(self.matrix.rhs_parts(), rows)])


class BlockPMatrix:
    """``BlockPMatrix``: blocks[I][J] over row group I and column group J
    (src/BlockPartitionedArrays.jl)."""

    def __init__(self, blocks):
        self.blocks = blocks

    def mul(self, xs):
        """``mul!(y, A, x)`` block by block (BlockPartitionedArrays.jl:330-350)."""
        out = []
        for row in self.blocks:
            y = None
            for A, x in zip(row, xs):
                v = A.mul(x)
                y = v if y is None else y + v
            out.append(y)
        return out


class BlockPVector:
    def __init__(self, blocks):
        self.blocks = blocks

    def global_values(self):
        return [b.global_values() for b in self.blocks]


def assemble_multifield(assem: MultiFieldAssembler, a: MultiFieldForm, l: MultiFieldSource | None):
    """``assemble_matrix_and_vector`` for multi-field spaces: a PSparseMatrix/PVector
    pair (consecutive style) or a BlockPMatrix/BlockPVector pair (block style)."""
    assem.numeric(a, l)
    groups = assem.Y.groups()
    if isinstance(assem.Y.style, BlockMultiFieldStyle):
        blocks = [[assem.matrix(gI, gJ) for gJ in groups] for gI in groups]
        return BlockPMatrix(blocks), BlockPVector([MultiFieldVector(row[0]) for row in blocks])
    A = assem.matrix(groups[0], groups[0])
    return A, MultiFieldVector(A)


def restrict_to_field(space: DistributedMultiFieldFESpace, x: np.ndarray, field: int) -> np.ndarray:
    """``restrict_to_field`` for a global vector in the multi-field numbering of
    `space` (consecutive style) or of the block holding `field` (block style): the
    field's values in the single-field numbering."""
    V = space.space
    groups = space.groups()
    g = next(gr for gr in groups if field in gr)
    jj = g.index(field)
    out = np.zeros(V.num_free_dofs())
    for p in range(V.model.num_parts):
        _, nown, first = V.local_sizes(p)
        out[first:first + nown] = x[len(g) * first + jj * nown: len(g) * first + (jj + 1) * nown]
    return out
