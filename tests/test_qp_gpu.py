"""Quadrature-point coefficients on the GPU (gd_assemble_qp / gd_assemble_elasticity_qp).

A coefficient known at the Gauss points of every cell (a CellField that varies inside the
cells, CellData integrate, src/CellData.jl:234-259) gives K_e = sum_q c_q H_q.  Checked
against the oracle's FP64 restatement:

* GD_QP_FP64 (element matrices in FP64 on the CUDA cores): patterns bit-exact, values
  within 1e-12 x max|row|, rhs within 1e-12 x max|b| -- the same bar as the cell-wise path;
* the tensor-core modes (tcgen05, BF16 operands split into 1, 2 or 3 terms, FP32
  accumulation, FP32 element matrices): values within the stated bound of each mode,
  relative to the row's largest entry: bf16 3e-2, bf16x3 3e-4, bf16x6 3e-6;
* the manufactured solutions of tests/test_oracle_qp.py through the device solve
  (kappa = 1 + x + 2y with a linear u; E = 2 + x + y with an affine displacement):
  FP64 mode 1e-9, bf16x6 1e-5;
* at sizes with many work items per CTA (the operand ring and both TMEM accumulators
  cycle): the tensor-core element matrices against the FP64 mode on the GPU itself.
"""
import ctypes as C

import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem, row_scaled_error, row_scaled_error_fast, export_part

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "bf16": 3e-2, "bf16x3": 3e-4, "bf16x6": 3e-6}
TAGS = ["left", "right", "bottom", "top", "back", "front"]


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def qp_system(backend, pb, strategy, precision):
    import gridap_gb300 as G
    ranks = backend.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    sides = [t for t, s in zip(TAGS, pb.dirichlet_sides) if s]
    ref = G.ReferenceFE(G.lagrangian, G.VectorValue if pb.physics == "elasticity" else float, pb.order)
    V = G.TestFESpace(model, ref, dirichlet_tags=sides)
    U = G.TrialFESpace(pb.u_dir, V) if pb.u_dir is not None else G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    if pb.physics == "elasticity":
        a = G.integral_elasticity(pb.kappa_qp, pb.nu, dO, precision=precision)
        l = G.integral_source(tuple(pb.force) if pb.force is not None else (0.0,) * pb.dim, dO)
    else:
        a = G.integral_grad_grad(pb.kappa_qp, dO, precision=precision)
        l = G.integral_source(pb.f_nodal if pb.f_nodal is not None else pb.f_const, dO)
    strat = G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows()
    assem = G.SparseMatrixAssembler(U, V, strat)
    op = G.AffineFEOperator(a, l, U, V, assem)
    return model, V, U, op


def random_qp(pb, seed):
    """A smooth positive coefficient with cell-to-cell and in-cell variation."""
    xq = go.quadrature_points(pb)
    rng = np.random.default_rng(seed)
    a = rng.normal(size=3)
    g = sum(a[d] * np.sin((d + 2) * np.pi * xq[:, :, d]) for d in range(pb.dim))
    return np.exp(0.5 * g) * (1.0 + 0.5 * rng.random(size=(xq.shape[0], 1)))


def compare(op, ref, tol, label):
    A = op.matrix
    b_parts = op.vector.partition
    for p, M in enumerate(ref):
        rp, ci, vv = A.csr_parts()[p]
        assert np.array_equal(rp, M.rowptr), f"{label} rowptr part {p}"
        assert np.array_equal(ci, M.colidx), f"{label} colidx part {p}"
        assert np.array_equal(A.row_partition[p].ghost_to_global, M.row_ghost_gids)
        assert np.array_equal(A.col_partition[p].ghost_to_global, M.col_ghost_gids)
        err = row_scaled_error(vv, M.vals, M.rowptr)
        assert err <= tol, f"{label} values part {p}: {err}"
        scale = max(np.abs(M.b).max(initial=0.0), 1e-300)
        berr = np.abs(b_parts[p] - M.b).max(initial=0.0) / scale
        assert berr <= tol, f"{label} rhs part {p}: {berr}"


SCALAR = [
    dict(dim=2, n=(5, 4), parts=(2, 2), order=1, seed=1),
    dict(dim=2, n=(4, 3), parts=(2, 1), order=2, seed=2, u=lambda x, y: 1.0 + x * y),
    dict(dim=2, n=(3, 3), parts=(1, 2), order=3, seed=3, sides=(1, 0, 1, 1)),
    dict(dim=3, n=(4, 3, 3), parts=(2, 2, 1), order=1, seed=4, f_nodal=True),
    dict(dim=3, n=(3, 3, 2), parts=(2, 1, 2), order=2, seed=5, u=lambda x, y, z: x - y + 2 * z),
    dict(dim=3, n=(2, 3, 2), parts=(1, 2, 2), order=3, seed=6, sides=(1, 1, 0, 1, 1, 0)),
]


def case_id(c):
    return f"{c['dim']}d_q{c['order']}_n{'x'.join(map(str, c['n']))}"


@pytest.mark.parametrize("precision", ["fp64", "bf16x6", "bf16x3", "bf16"])
@pytest.mark.parametrize("case", SCALAR, ids=case_id)
def test_scalar_point_coefficients_against_oracle(backend, case, precision):
    pb = make_problem(**case)
    pb.kappa_qp = random_qp(pb, case["seed"])
    fe = go.build_fespace(pb)
    for strategy in ("sub", "full"):
        ref = go.assemble(pb, fe, strategy)
        _, V, U, op = qp_system(backend, pb, strategy, precision)
        compare(op, ref, TOL[precision], f"{precision}/{strategy}")


def elasticity_problem(dim, n, parts, order, seed, u=False):
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.25 * d))
    sides = (1, 0) + (0, 0) * (dim - 1)   # clamped at x = 0
    pb = go.Problem(np=parts, n=n, domain=domain, order=order, degree=2 * order, physics="elasticity", nu=0.3,
                    dirichlet_sides=sides, force=(0.0, -1.0, 0.5)[:dim])
    pb.kappa_qp = random_qp(pb, seed)
    if u:
        N = pb.lattice
        X = np.stack(np.meshgrid(*[np.arange(N[d]) for d in range(dim)], indexing="ij"), axis=-1).reshape(-1, dim)
        uD = np.zeros((int(np.prod(N)), dim))
        uD[pb.node_lin(X)] = 0.1 * pb.node_xyz(X)[:, ::-1]
        pb.u_dir = uD
    return pb


ELASTIC = [((2, (4, 3), (2, 1), 1), True), ((2, (3, 3), (2, 2), 2), False),
           ((3, (3, 2, 2), (2, 1, 2), 1), True), ((3, (2, 3, 2), (1, 2, 1), 2), False)]


@pytest.mark.parametrize("precision", ["fp64", "bf16x6", "bf16x3"])
@pytest.mark.parametrize("case", ELASTIC, ids=[f"{c[0][0]}d_vq{c[0][3]}" for c in ELASTIC])
def test_elasticity_point_modulus_against_oracle(backend, case, precision):
    (dim, n, parts, order), with_u = case
    pb = elasticity_problem(dim, n, parts, order, seed=10 * dim + order, u=with_u)
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, "sub")
    _, V, U, op = qp_system(backend, pb, "sub", precision)
    compare(op, ref, TOL[precision], precision)


@pytest.mark.parametrize("precision,bound", [("fp64", 1e-9), ("bf16x6", 1e-5)])
@pytest.mark.parametrize("dim,n,parts,order", [(2, (6, 5), (2, 2), 2), (3, (4, 4, 3), (2, 2, 1), 1),
                                               (3, (3, 3, 3), (2, 1, 2), 2)])
def test_variable_kappa_known_answer(backend, dim, n, parts, order, precision, bound):
    """kappa = 1 + x + 2y at the Gauss points, u = x + y (+ z), f = -3: reproduced."""
    import gridap_gb300 as G
    from test_oracle_qp import diffusion_kat_problem
    pb, u = diffusion_kat_problem(dim, n, parts, order)
    _, V, U, op = qp_system(backend, pb, "sub", precision)
    x = op.matrix.solve(rtol=1e-13)
    uh = G.FEFunction(U, x)
    dO = G.Measure(G.Triangulation(V.model), pb.degree)
    err = G.l2_error(uh, u, dO)
    assert err < bound, err


@pytest.mark.parametrize("precision,bound", [("fp64", 1e-9), ("bf16x6", 1e-5)])
@pytest.mark.parametrize("dim,order,parts,n", [(2, 2, (2, 2), (3, 3)), (3, 1, (2, 1, 2), (3, 2, 2)),
                                                (3, 2, (1, 2, 1), (2, 3, 2))])
def test_variable_modulus_known_answer(backend, dim, order, parts, n, precision, bound):
    """E = 2 + x + y at the Gauss points, affine displacement with its body force."""
    from test_oracle_qp import elasticity_kat_problem
    pb, B, t = elasticity_kat_problem(dim, n, parts, order, seed=90 + 10 * dim + order)
    fe = go.build_fespace(pb)
    _, V, U, op = qp_system(backend, pb, "sub", precision)
    x = op.matrix.solve(rtol=1e-13)
    for sp, d in zip(fe.spaces, fe.dofs):
        want = (pb.node_xyz(sp.dof_node) @ B.T + t)[np.arange(len(sp.dof_comp)), sp.dof_comp]
        assert np.abs(x[d.ldof_to_gdof] - want).max() <= bound * max(1.0, np.abs(want).max())


LARGE = [
    # scalar Q2 3D: 27 points (K padded to 32), 6 entry tiles
    dict(dim=3, n=(26, 24, 22), parts=(2, 2, 2), order=2, physics="poisson"),
    # scalar Q3 3D: 64 points (K = 64, 128-cell tiles), 32 entry tiles
    dict(dim=3, n=(13, 12, 11), parts=(2, 1, 2), order=3, physics="poisson"),
    # scalar Q1 3D: 8 points (K padded to 16)
    dict(dim=3, n=(60, 50, 40), parts=(2, 2, 2), order=1, physics="poisson"),
    # vector Q2 3D elasticity: 6561 entries, 52 entry tiles
    dict(dim=3, n=(18, 16, 14), parts=(2, 2, 2), order=2, physics="elasticity"),
]


@pytest.mark.parametrize("case", LARGE, ids=["q2", "q3", "q1", "vq2"])
def test_tensor_core_modes_against_fp64_mode_at_size(backend, case):
    dim, n, parts, order = case["dim"], case["n"], case["parts"], case["order"]
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.1 * d))
    if case["physics"] == "elasticity":
        pb = go.Problem(np=parts, n=n, domain=domain, order=order, degree=2 * order, physics="elasticity", nu=0.3,
                        dirichlet_sides=(1, 0, 0, 0, 0, 0), force=(0.0, 0.0, -1.0))
    else:
        pb = go.Problem(np=parts, n=n, domain=domain, order=order, degree=2 * order, f_const=1.0)
    pb.kappa_qp = random_qp(pb, 77)
    _, V, U, op = qp_system(backend, pb, "sub", "fp64")
    h = op.matrix.assem.handle
    ref = [export_part(h, p) for p in range(int(np.prod(parts)))]
    for precision in ("bf16x6", "bf16x3", "bf16"):
        a = op.a.__class__(**{**op.a.__dict__, "precision": precision})
        op.matrix.assem.numeric(a, op.l)
        for p, M in enumerate(ref):
            got = export_part(h, p)
            assert np.array_equal(got["colidx"], M["colidx"])
            err = row_scaled_error_fast(got["vals"], M["vals"], M["rowptr"])
            assert err <= TOL[precision], f"{precision} part {p}: {err}"
            berr = np.abs(got["b"] - M["b"]).max(initial=0.0) / max(np.abs(M["b"]).max(initial=0.0), 1e-300)
            assert berr <= TOL[precision], f"{precision} rhs part {p}: {berr}"


def test_qp_info_and_bad_coefficients(backend):
    import gridap_gb300 as G
    L = G._lib
    pb = make_problem(3, (3, 3, 3), (1, 1, 1), 2, seed=8)
    pb.kappa_qp = random_qp(pb, 8)
    _, V, U, op = qp_system(backend, pb, "sub", "bf16x6")
    h = op.matrix.assem.handle
    pts, ent, kp, et = (C.c_int32() for _ in range(4))
    L.call("gd_qp_info", h, C.byref(pts), C.byref(ent), C.byref(kp), C.byref(et), None, None)
    assert (pts.value, ent.value, kp.value, et.value) == (27, 729, 32, 6)
    bad = pb.kappa_qp.copy()
    bad[3, 5] = -1.0
    c = L.gd_qp_coeffs()
    c.kappa_qp = bad.ctypes.data
    c.f_nodal = None
    c.f_const = 1.0
    c.degree = pb.degree
    c.precision = L.GD_QP_BF16X6
    c.where = L.GD_HOST
    rc = L.load().gd_assemble_qp(h, C.byref(c))
    assert rc == 8   # GD_ERR_NUMERIC
