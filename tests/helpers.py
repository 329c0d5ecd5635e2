"""Shared helpers: build the same problem for the oracle and for the GPU library."""
import numpy as np

import gridap_oracle as go


def lattice_xyz(pb):
    N = pb.lattice
    idx = np.indices(tuple(reversed(N))).reshape(pb.dim, -1)[::-1]
    return np.stack([pb.domain[2 * d] + idx[d] * pb.h[d] / pb.order for d in range(pb.dim)], axis=1)


def make_problem(dim, n, parts, order, sides=None, seed=None, f=1.0, u=None, domain=None, f_nodal=False):
    domain = domain or tuple(v for _ in range(dim) for v in (0.0, 1.0))
    ncells = int(np.prod(n))
    kappa = None
    if seed is not None:
        kappa = np.exp(np.random.default_rng(seed).normal(size=ncells))
    pb = go.Problem(np=parts, n=n, domain=domain, order=order, degree=2 * order, dirichlet_sides=sides,
                    kappa=kappa, f_const=f)
    if u is not None:
        xyz = lattice_xyz(pb)
        pb.u_dir = np.asarray(u(*[xyz[:, d] for d in range(dim)]), dtype=np.float64)
    if f_nodal:
        pb.f_nodal = np.random.default_rng(1000 + (seed or 0)).normal(size=int(np.prod(pb.lattice)))
    return pb


def row_scaled_error(vals_a, vals_b, rowptr):
    """max over entries of |a-b| / max|b| in the entry's row (0 for empty rows)."""
    err = 0.0
    for r in range(len(rowptr) - 1):
        s, e = rowptr[r], rowptr[r + 1]
        if e == s:
            continue
        scale = max(np.abs(vals_b[s:e]).max(), 1e-300)
        err = max(err, float(np.abs(vals_a[s:e] - vals_b[s:e]).max() / scale))
    return err


def row_scaled_error_fast(vals_a, vals_b, rowptr):
    """row_scaled_error, vectorised for millions of rows."""
    rowptr = np.asarray(rowptr)
    nonempty = np.diff(rowptr) > 0
    if not nonempty.any():
        return 0.0
    starts = rowptr[:-1][nonempty]
    scale = np.maximum.reduceat(np.abs(vals_b), starts)
    diff = np.maximum.reduceat(np.abs(np.asarray(vals_a) - vals_b), starts)
    return float((diff / np.maximum(scale, 1e-300)).max())


def gpu_system(backend, pb, strategy):
    """The problem's operator through the Python mirror of the reference API (on the GPU)."""
    import gridap_gb300 as G
    ranks = backend.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    tags = ["left", "right", "bottom", "top", "back", "front"]
    sides = [t for t, s in zip(tags, pb.dirichlet_sides) if s]
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, pb.order), dirichlet_tags=sides)
    U = G.TrialFESpace(pb.u_dir, V) if pb.u_dir is not None else G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    a = G.integral_grad_grad(pb.kappa, dO)
    l = G.integral_source(pb.f_nodal if pb.f_nodal is not None else pb.f_const, dO)
    strat = G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows()
    assem = G.SparseMatrixAssembler(U, V, strat)
    op = G.AffineFEOperator(a, l, U, V, assem)
    return model, V, U, op


def export_part(handle, p):
    """One part of the assembled PSparseMatrix and PVector straight from the C ABI:
    rowptr, colidx, vals, ghost-row gids, ghost-column gids, rhs."""
    import ctypes as C
    import gridap_gb300 as G
    L = G._lib
    nr, nc, nnz, ngr, ngc = (C.c_int64() for _ in range(5))
    L.call("gd_matrix_sizes", handle, p, *[C.byref(x) for x in (nr, nc, nnz, ngr, ngc)])
    rp = np.zeros(nr.value + 1, dtype=np.int64)
    ci = np.zeros(nnz.value, dtype=np.int32)
    vv = np.zeros(nnz.value, dtype=np.float64)
    grg = np.zeros(ngr.value, dtype=np.int64)
    gro = np.zeros(ngr.value, dtype=np.int32)
    gcg = np.zeros(ngc.value, dtype=np.int64)
    gco = np.zeros(ngc.value, dtype=np.int32)
    b = np.zeros(nr.value, dtype=np.float64)
    L.call("gd_matrix_export", handle, p, L.ptr(rp, C.c_int64), L.ptr(ci, C.c_int32), L.ptr(vv, C.c_double),
           L.ptr(grg, C.c_int64), L.ptr(gro, C.c_int32), L.ptr(gcg, C.c_int64), L.ptr(gco, C.c_int32))
    L.call("gd_vector_export", handle, p, L.ptr(b, C.c_double))
    return dict(rowptr=rp, colidx=ci, vals=vv, row_ghost_gids=grg, col_ghost_gids=gcg, b=b)
