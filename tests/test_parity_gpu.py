"""GPU parity: the CUDA path against the CPU oracle, through the C ABI.

Bit-exact: DOF numbering, gids and owners, row/column index sets, local CSR
patterns.  FP64 values: |gpu - oracle| <= 1e-12 * (max |oracle| in the row).
Solutions: relative difference to the oracle's gathered sparse LU <= 1e-8.
"""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import export_part, gpu_system, make_problem, row_scaled_error

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12     # FP64 matrix/vector entries, relative to the row scale
SOL_TOL = 1e-8      # solution vs gathered sparse LU


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


CASES = [
    dict(dim=2, n=(4, 4), parts=(2, 2), order=1),
    dict(dim=2, n=(5, 4), parts=(2, 2), order=2, seed=1),
    dict(dim=2, n=(6, 5), parts=(2, 1), order=3, sides=(1, 0, 1, 0), seed=2),
    dict(dim=2, n=(7, 3), parts=(3, 1), order=2, seed=3),
    dict(dim=2, n=(4, 4), parts=(1, 1), order=1),
    dict(dim=3, n=(5, 4, 3), parts=(2, 2, 1), order=1, seed=4),
    dict(dim=3, n=(6, 6, 6), parts=(2, 2, 2), order=1, seed=5),
    dict(dim=3, n=(4, 3, 5), parts=(2, 1, 2), order=2, seed=6),
    dict(dim=3, n=(3, 4, 3), parts=(1, 2, 2), order=3, sides=(1, 0, 1, 0, 1, 0), seed=7),
    dict(dim=3, n=(4, 4, 4), parts=(2, 2, 2), order=1, sides=(0, 0, 0, 0, 0, 0), seed=8),
    dict(dim=3, n=(5, 5, 5), parts=(2, 2, 2), order=2, sides=(1, 0, 0, 0, 0, 0), seed=9, f_nodal=True),
    # Q1 with free boundary nodes, a nodal source and non-zero Dirichlet values (lifting)
    dict(dim=3, n=(6, 5, 4), parts=(2, 1, 2), order=1, sides=(1, 1, 0, 1, 1, 0), seed=10, f_nodal=True,
         u=lambda x, y, z: x + 2 * y + z * z),
    dict(dim=2, n=(6, 4), parts=(2, 2), order=1, sides=(0, 1, 1, 0), seed=11, f_nodal=True,
         u=lambda x, y: 1.0 + x * y),
    dict(dim=3, n=(7, 6, 5), parts=(3, 2, 1), order=1, seed=12, u=lambda x, y, z: 2.0 - x),
    # cube cells, an odd number of them (the coefficient scaling's last single cell)
    dict(dim=3, n=(5, 3, 7), parts=(1, 1, 2), order=1, seed=13, domain=(0, 1.25, 0, 0.75, 0, 1.75)),
]


def case_id(c):
    cube = "_cube" if "domain" in c else ""
    return f"{c['dim']}d_n{'x'.join(map(str, c['n']))}_p{''.join(map(str, c['parts']))}_q{c['order']}{cube}"


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_parity_against_oracle(backend, case, strategy):
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, strategy)
    model, V, U, op = gpu_system(backend, pb, strategy)
    # A4: gids and owners, bit-exact; local DOF order via the lattice node of each DOF
    assert V.num_free_dofs() == fe.dofs[0].ngdofs
    for p, (d, sp) in enumerate(zip(fe.dofs, fe.spaces)):
        li = V.gids.partition()[p]
        assert np.array_equal(li.local_to_global, d.ldof_to_gdof), f"gids part {p}"
        assert np.array_equal(li.local_to_owner, d.ldof_to_owner), f"owners part {p}"
        assert np.array_equal(V.dof_nodes(p), pb.node_lin(sp.dof_node)), f"local numbering part {p}"
    # A11: local matrices, index sets bit-exact, values to VAL_TOL
    A = op.matrix
    b_parts = op.vector.partition
    for p, M in enumerate(ref):
        rp, ci, vv = A.csr_parts()[p]
        rows, cols = A.row_partition[p], A.col_partition[p]
        assert np.array_equal(rows.own_to_global, M.row_own_gids)
        assert np.array_equal(rows.ghost_to_global, M.row_ghost_gids), f"ghost rows part {p}"
        assert np.array_equal(rows.ghost_to_owner, M.row_ghost_owner)
        assert np.array_equal(cols.ghost_to_global, M.col_ghost_gids), f"ghost cols part {p}"
        assert np.array_equal(cols.ghost_to_owner, M.col_ghost_owner)
        assert np.array_equal(rp, M.rowptr), f"rowptr part {p}"
        assert np.array_equal(ci, M.colidx), f"colidx part {p}"
        assert row_scaled_error(vv, M.vals, M.rowptr) <= VAL_TOL
        scale = max(np.abs(M.b).max(), 1e-300)
        assert np.abs(b_parts[p] - M.b).max() <= VAL_TOL * scale


@pytest.mark.parametrize("case", [CASES[6], CASES[14], CASES[7], CASES[8], CASES[2]], ids=case_id)
def test_mul_matches_gathered_oracle(backend, case):
    """A14 `mul!`: Q1 rows (the sliced-ELL copy, exact zeros of cube cells dropped) and Q2/Q3
    rows (lane groups on the CSR) against the oracle's gathered matrix; twice, so the second
    product reuses the cached copy.  |y - y_ref| <= 1e-12 * max |y_ref|."""
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    A_ref, _ = go.gather_global(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    _, V, U, op = gpu_system(backend, pb, "sub")
    rng = np.random.default_rng(17)
    for _ in range(2):
        x = rng.normal(size=fe.dofs[0].ngdofs)
        y_ref = A_ref @ x
        y = op.matrix.mul(x)
        assert np.abs(y - y_ref).max() <= 1e-12 * np.abs(y_ref).max()


def test_c1_poisson2d_q2_128(backend):
    """The C1 configuration at full size: 2D Q2 on 128 x 128 cells, parts (2,2), quadrature
    degree 4, u = (x+y)^2 on the boundary, f = -4 (test/PoissonTests.jl:14-45 on a 128^2
    mesh).  Local parts against the oracle (pattern bit-exact, values 1e-12), the device FP64
    solve against the oracle's gathered sparse LU (1e-8), and the known answer: Q2 reproduces
    (x+y)^2, L2 error < 1e-9 (the discretisation error is zero; the solver's at rtol 1e-13 is
    ~1e-12)."""
    import gridap_gb300 as G
    u = lambda x, y: (x + y) ** 2
    pb = make_problem(2, (128, 128), (2, 2), 2, f=-4.0, u=u)
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, "sub")
    model, V, U, op = gpu_system(backend, pb, "sub")
    A = op.matrix
    for p, M in enumerate(ref):
        rp, ci, vv = A.csr_parts()[p]
        assert np.array_equal(rp, M.rowptr), f"rowptr part {p}"
        assert np.array_equal(ci, M.colidx), f"colidx part {p}"
        assert row_scaled_error(vv, M.vals, M.rowptr) <= VAL_TOL
        assert np.abs(op.vector.partition[p] - M.b).max() <= VAL_TOL * np.abs(M.b).max()
    x_ref = go.solve_lu(ref, fe.dofs[0].ngdofs)
    uh = G.solve(op, rtol=1e-13)
    assert op.matrix.last_stats.converged
    assert np.abs(uh.free_values - x_ref).max() / np.abs(x_ref).max() <= SOL_TOL
    dO = G.Measure(G.Triangulation(model), pb.degree)
    assert G.l2_error(uh, u, dO) < 1e-9


@pytest.mark.parametrize("case", [CASES[1], CASES[6], CASES[7]], ids=case_id)
def test_solve_matches_gathered_lu(backend, case):
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    x_ref = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    _, V, U, op = gpu_system(backend, pb, "sub")
    x = op.matrix.solve(rtol=1e-13)
    assert op.matrix.last_stats.converged
    assert np.abs(x - x_ref).max() / np.abs(x_ref).max() <= SOL_TOL


@pytest.mark.parametrize("case", [CASES[6], CASES[7], CASES[13],
                                  dict(dim=3, n=(12, 10, 8), parts=(2, 2, 2), order=1, seed=30),
                                  dict(dim=3, n=(9, 8, 7), parts=(2, 2, 1), order=1, seed=31,
                                       sides=(1, 0, 1, 1, 0, 1)),
                                  # cube cells (the lattice inner iteration): rows of 12 nodes (no
                                  # padding), of 10 (warps start mid-row), of 141 (rows across warps)
                                  dict(dim=3, n=(11, 7, 6), parts=(1, 2, 1), order=1, seed=32,
                                       sides=(0, 1, 1, 0, 1, 1), domain=(0, 1.375, 0, 0.875, 0, 0.75)),
                                  dict(dim=3, n=(9, 8, 7), parts=(2, 2, 1), order=1, seed=34,
                                       sides=(1, 0, 1, 1, 0, 1), domain=(0, 1.125, 0, 1.0, 0, 0.875)),
                                  dict(dim=3, n=(140, 4, 3), parts=(2, 1, 1), order=1, seed=33,
                                       domain=(0, 17.5, 0, 0.5, 0, 0.375)),
                                  # 11 blocks of the persistent kernel whose chunks start and end
                                  # mid-row, Dirichlet and natural sides mixed
                                  dict(dim=3, n=(35, 30, 28), parts=(2, 2, 1), order=1, seed=35,
                                       sides=(1, 1, 0, 1, 1, 0), domain=(0, 4.375, 0, 3.75, 0, 3.5)),
                                  # rows of 141 nodes over 8 blocks of the persistent kernel
                                  dict(dim=3, n=(140, 30, 4), parts=(2, 1, 1), order=1, seed=37,
                                       sides=(1, 0, 1, 1, 0, 1), domain=(0, 17.5, 0, 3.75, 0, 0.5))],
                         ids=case_id)
def test_mixed_solver_matches_gathered_lu(backend, case):
    """FP64 refinement around FP32 CG (matrix-free on cube Q1, FP32 CSR otherwise)."""
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    x_ref = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    _, V, U, op = gpu_system(backend, pb, "sub")
    x = op.matrix.solve(rtol=1e-12, method="mixed_ir")
    assert op.matrix.last_stats.converged
    assert op.matrix.last_stats.rel_residual <= 1e-12
    assert np.abs(x - x_ref).max() / np.abs(x_ref).max() <= SOL_TOL


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("parts", [(2, 2), (1, 1), (2, 1), (1, 2)])
def test_fespaces_kat_on_gpu(backend, parts, strategy):
    """test/FESpacesTests.jl:10-59 on the GPU path: Q1, u = x+y, L2 error < 1e-9."""
    import gridap_gb300 as G
    pb = make_problem(2, (4, 4), parts, 1, f=0.0, u=lambda x, y: x + y, domain=(0, 4, 0, 4))
    pb.degree = 3
    _, V, U, op = gpu_system(backend, pb, strategy)
    uh = G.solve(op, rtol=1e-14)
    assert go.l2_error(pb, uh.nodal_values(), lambda x, y: x + y) < 1e-9
    r = op.matrix.mul(uh.free_values) - op.vector.global_values()
    assert np.abs(r).max() < 1e-10


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("parts", [(2, 2), (1, 1), (2, 1), (1, 2)])
def test_fespaces_assemble_tests_sequence(backend, parts, strategy):
    """test/FESpacesTests.jl:12-70 (`assemble_tests`) call by call on the GPU path: Q1 on
    (0,4)^2 with 4 x 4 cells, u = x+y on the boundary, a = int(grad v . grad u), l = int(0 v),
    degree 3.  assemble_matrix_and_vector (and the local matrix sizes), allocate_matrix_and_vector
    + assemble_matrix_and_vector!, AffineFEOperator, assemble_matrix and allocate_matrix +
    assemble_matrix! solved against the operator's vector: L2 error < 1e-9 each; then
    assemble_vector and allocate_vector + assemble_vector! of int(1 v) on a fresh assembler:
    sum(b) == length(b) to 1e-12 (no Dirichlet lifting in a vector-only assembly)."""
    import gridap_gb300 as G
    u = lambda x, y: x + y
    ranks = backend.distribute(range(int(np.prod(parts))))
    model = G.CartesianDiscreteModel(ranks, parts, (0, 4, 0, 4), (4, 4))
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, 1), dirichlet_tags="boundary")
    U = G.TrialFESpace(u, V)
    das = G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows()
    dO = G.Measure(G.Triangulation(model), 3)
    a = G.integral_grad_grad(None, dO)
    l = G.integral_source(0.0, dO)
    assem = G.SparseMatrixAssembler(U, V, das)
    err = lambda x: G.l2_error(G.FEFunction(U, x), u, dO)

    data = G.collect_cell_matrix_and_vector(U, V, a, l)
    A1, b1 = G.assemble_matrix_and_vector(assem, data)
    assert err(A1.solve(rtol=1e-14)) < 1e-9
    for mat, rows, cols in zip(A1.matrix_partition, A1.row_partition, A1.col_partition):
        assert mat.shape == (rows.local_length(), cols.local_length())
    A2, b2 = G.allocate_matrix_and_vector(assem, data)
    G.assemble_matrix_and_vector_(A2, b2, assem, data)
    assert err(A2.solve(rtol=1e-14)) < 1e-9
    op = G.AffineFEOperator(a, l, U, V, G.SparseMatrixAssembler(U, V, das))
    assert err(G.solve(op, rtol=1e-14).free_values) < 1e-9
    mdata = G.collect_cell_matrix(U, V, a)
    A3 = G.assemble_matrix(assem, mdata)
    assert err(A3.solve(rtol=1e-14, b=op.vector)) < 1e-9
    A4 = G.allocate_matrix(assem, mdata)
    G.assemble_matrix_(A4, assem, mdata)
    assert err(A4.solve(rtol=1e-14, b=op.vector)) < 1e-9

    vecdata = G.collect_cell_vector(V, G.integral_source(1.0, dO))
    assem = G.SparseMatrixAssembler(U, V, das)
    bv1 = G.assemble_vector(assem, vecdata)
    assert abs(bv1.global_values().sum() - len(bv1)) < 1e-12
    bv2 = G.allocate_vector(assem, vecdata)
    G.assemble_vector_(bv2, assem, vecdata)
    assert abs(bv2.global_values().sum() - len(bv2)) < 1e-12
    assert all(len(bp) == rows.local_length() for bp, rows in zip(bv2.partition, A1.row_partition))


def test_poisson_q2_kat_on_gpu(backend):
    """test/PoissonTests.jl:14-45 (all-Dirichlet): Q2 reproduces (x+y)^2."""
    import gridap_gb300 as G
    pb = make_problem(2, (4, 4), (2, 2), 2, f=-4.0, u=lambda x, y: (x + y) ** 2, domain=(0, 4, 0, 4))
    _, V, U, op = gpu_system(backend, pb, "sub")
    uh = G.solve(op, rtol=1e-14)
    assert go.l2_error(pb, uh.nodal_values(), lambda x, y: (x + y) ** 2) < 1e-9


def test_vector_kat_on_gpu(backend):
    """test/FESpacesTests.jl:61-70: sum(b) == length(b) for ∫(1*v)."""
    pb = go.Problem(np=(2, 2), n=(4, 4), domain=(0, 4, 0, 4), order=1, degree=3, f_const=1.0)
    _, V, U, op = gpu_system(backend, pb, "sub")
    b = op.vector.global_values()
    assert abs(b.sum() - len(b)) < 1e-12


@pytest.mark.parametrize("fixture_case", ["fespaces_q1_2x2", "poisson_q2_2x2", "diffusion_q1_3d"])
@pytest.mark.parametrize("strategy", ["sub", "full"])
def test_gpu_against_golden_fixtures(backend, fixture_case, strategy):
    from pathlib import Path
    import make_golden as mg
    g = np.load(Path(__file__).resolve().parent / "golden" / f"{fixture_case}_{strategy}.npz")
    pb = make_problem(**mg.CASES[fixture_case])
    _, V, U, op = gpu_system(backend, pb, strategy)
    for p in range(int(np.prod(pb.np))):
        rp, ci, vv = op.matrix.csr_parts()[p]
        assert np.array_equal(V.gids.partition()[p].local_to_global, g[f"p{p}_gid"])
        assert np.array_equal(rp, g[f"p{p}_rowptr"]) and np.array_equal(ci, g[f"p{p}_colidx"])
        assert row_scaled_error(vv, g[f"p{p}_vals"], g[f"p{p}_rowptr"]) <= VAL_TOL
    x = op.matrix.solve(rtol=1e-14)
    assert np.abs(x - g["x"]).max() / max(np.abs(g["x"]).max(), 1e-300) <= SOL_TOL


def test_nonpositive_kappa_is_rejected(backend):
    import gridap_gb300 as G
    pb = make_problem(2, (4, 4), (2, 2), 1, seed=1)
    pb.kappa[3] = -1.0
    with pytest.raises(G._lib.GdError) as e:
        gpu_system(backend, pb, "sub")
    assert e.value.status == 8


CLASS_SUM_CASES = [
    dict(dim=2, n=(37, 29), parts=(2, 2), order=2, seed=61),
    dict(dim=2, n=(23, 31), parts=(2, 1), order=3, sides=(1, 0, 1, 1), seed=62, domain=(0, 1.0, 0, 0.6)),
    dict(dim=2, n=(30, 26), parts=(2, 2), order=2, seed=63, f_nodal=True, u=lambda x, y: 1.0 + x * x - y),
    dict(dim=2, n=(40, 40), parts=(2, 2), order=2, u=lambda x, y: (x + y) ** 2),
]


@pytest.mark.parametrize("case", CLASS_SUM_CASES, ids=["q2", "q3_rect_sides", "q2_fn_ud", "q2_c1_like"])
def test_2d_class_sum_rows_match_per_cell_rows(backend, case):
    """2D Q2/Q3 rows: one reference value times the sum of the shared cells' coefficients
    (the default) against the per-cell sum, on square and rectangular cells, with partial
    Dirichlet sides, nodal sources and Dirichlet lifting: values within 1e-14 x max|row|,
    rhs within 1e-14 x max|b|; both against the oracle at the parity tolerance."""
    import gridap_gb300 as G
    pb = make_problem(**case)
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, "sub")
    _, V, U, op = gpu_system(backend, pb, "sub")
    assem = op.matrix.assem
    got = {}
    for cs in (1, 0):
        G._lib.call("gd_assembler_set_class_sums", assem.handle, cs)
        assem.numeric(op.a, op.l)
        got[cs] = [export_part(assem.handle, p) for p in range(int(np.prod(pb.np)))]
    G._lib.call("gd_assembler_set_class_sums", assem.handle, 1)
    for p, M in enumerate(ref):
        a, b = got[1][p], got[0][p]
        assert np.array_equal(a["rowptr"], b["rowptr"]) and np.array_equal(a["colidx"], b["colidx"])
        assert row_scaled_error(a["vals"], b["vals"], a["rowptr"]) <= 1e-14
        bscale = max(np.abs(b["b"]).max(initial=0.0), 1e-300)
        assert np.abs(a["b"] - b["b"]).max(initial=0.0) <= 1e-14 * bscale
        for g in (a, b):
            assert row_scaled_error(g["vals"], M.vals, M.rowptr) <= VAL_TOL
            assert np.abs(g["b"] - M.b).max(initial=0.0) <= VAL_TOL * max(np.abs(M.b).max(initial=0.0), 1e-300)
