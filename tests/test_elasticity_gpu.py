"""Vector-valued spaces and linear elasticity on the GPU path against the oracle:
DOF numbering (gids, owners), the PSparseMatrix parts (pattern bit-exact, values
1e-12 row-relative, ghost row/column index sets) and the solution against the
gathered sparse LU."""
import numpy as np
import pytest

import gridap_oracle as go

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
SOL_TOL = 1e-8

CASES = [
    dict(n=(3, 4, 2), parts=(2, 2, 1), order=1, sides=(1, 0, 0, 0, 0, 0), seed=60),
    dict(n=(4, 3, 3), parts=(2, 1, 2), order=2, sides=(1, 0, 0, 0, 0, 0), seed=61),
    dict(n=(3, 3, 4), parts=(2, 2, 2), order=2, sides=None, seed=62),
    dict(n=(5, 2, 3), parts=(3, 1, 1), order=1, sides=(1, 1, 1, 0, 0, 1), seed=63),
    dict(n=(4, 4), parts=(2, 2), order=2, sides=(1, 0, 0, 0), seed=64),
    dict(n=(5, 3), parts=(2, 1), order=1, sides=None, seed=65),
]


def case_id(c):
    return f"{len(c['n'])}d_q{c['order']}_{'x'.join(map(str, c['n']))}_p{''.join(map(str, c['parts']))}"


def problem(c):
    dim = len(c["n"])
    E = np.exp(0.5 * np.random.default_rng(c["seed"]).normal(size=int(np.prod(c["n"]))))
    force = (0.0, 0.0, -1.0) if dim == 3 else (0.3, -1.0)
    return go.Problem(np=c["parts"], n=c["n"], domain=tuple(v for _ in range(dim) for v in (0.0, 1.0)),
                      order=c["order"], degree=2 * c["order"], dirichlet_sides=c["sides"], kappa=E,
                      physics="elasticity", nu=0.3, force=force)


def gpu_system(be, pb, strategy):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    tags = ["left", "right", "bottom", "top", "back", "front"]
    sides = [t for t, s in zip(tags, pb.dirichlet_sides) if s]
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, G.VectorValue, pb.order), dirichlet_tags=sides)
    U = G.TrialFESpace(pb.u_dir if pb.u_dir is not None else 0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    a = G.integral_elasticity(pb.kappa, pb.nu, dO)
    l = G.integral_source(pb.force, dO)
    strat = G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows()
    op = G.AffineFEOperator(a, l, U, V, G.SparseMatrixAssembler(U, V, strat))
    return V, op


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_elasticity_matches_oracle(backend, case, strategy):
    pb = problem(case)
    fe = go.build_fespace(pb)
    parts = go.assemble(pb, fe, strategy)
    V, op = gpu_system(backend, pb, strategy)
    assert V.num_free_dofs() == fe.dofs[0].ngdofs
    for p in range(len(parts)):
        li = V.gids.partition()[p]
        assert np.array_equal(li.local_to_global, fe.dofs[p].ldof_to_gdof)
        assert np.array_equal(li.local_to_owner, fe.dofs[p].ldof_to_owner)
    A = op.matrix
    b_parts = op.vector.partition
    for p, (rp, ci, vv) in enumerate(A.csr_parts()):
        O = parts[p]
        rows, cols = A.row_partition[p], A.col_partition[p]
        assert np.array_equal(rows.ghost_to_global, O.row_ghost_gids)
        assert np.array_equal(rows.ghost_to_owner, O.row_ghost_owner)
        assert np.array_equal(cols.ghost_to_global, O.col_ghost_gids)
        assert np.array_equal(cols.ghost_to_owner, O.col_ghost_owner)
        assert np.array_equal(rp, O.rowptr), f"rowptr part {p}"
        assert np.array_equal(ci, O.colidx), f"colidx part {p}"
        for r in range(len(rp) - 1):
            s, e = rp[r], rp[r + 1]
            if e > s:
                rs = max(np.abs(O.vals[s:e]).max(), 1e-300)
                assert np.abs(vv[s:e] - O.vals[s:e]).max() <= VAL_TOL * rs
        if len(O.b):
            bs = max(np.abs(O.b).max(), 1e-300)
            assert np.abs(b_parts[p] - O.b).max() <= VAL_TOL * bs


@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[4]], ids=case_id)
def test_elasticity_solution_matches_gathered_lu(backend, case):
    pb = problem(case)
    fe = go.build_fespace(pb)
    x_ref = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    V, op = gpu_system(backend, pb, "sub")
    for method in ("jacobi_pcg", "mixed_ir"):
        x = op.matrix.solve(rtol=1e-12, method=method)
        assert op.matrix.last_stats.converged
        assert np.abs(x - x_ref).max() / np.abs(x_ref).max() <= SOL_TOL


def test_vector_space_rejects_order_3(backend):
    import gridap_gb300 as G
    from gridap_gb300._lib import GdError
    ranks = backend.distribute(range(2))
    model = G.CartesianDiscreteModel(ranks, (2, 1, 1), (0, 1, 0, 1, 0, 1), (2, 2, 2))
    with pytest.raises(GdError):
        G.TestFESpace(model, G.ReferenceFE(G.lagrangian, G.VectorValue, 3))


def lattice_field(pb, fn):
    """Dense (lattice nodes, dim) array of fn(xyz) in lattice order (x fastest)."""
    dim, N = pb.dim, pb.lattice
    X = np.stack(np.meshgrid(*[np.arange(N[d]) for d in range(dim)], indexing="ij"), axis=-1).reshape(-1, dim)
    u = np.empty((int(np.prod(N)), dim))
    u[pb.node_lin(X)] = fn(pb.node_xyz(X))
    return u


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[4], CASES[5]], ids=case_id)
def test_elasticity_dirichlet_values_match_oracle(backend, case, strategy):
    """TrialFESpace(u, V) on a vector space: the lifted right-hand side (b -= K[:,D] u_D,
    E per cell) against the oracle's, 1e-12 relative; the matrix does not change."""
    pb = problem(case)
    pb.u_dir = lattice_field(pb, lambda x: np.stack([np.sin(1.0 + x[:, d]) * (d + 1.0) + x[:, 0] * x[:, -1]
                                                     for d in range(pb.dim)], axis=1))
    fe = go.build_fespace(pb)
    parts = go.assemble(pb, fe, strategy)
    V, op = gpu_system(backend, pb, strategy)
    for p, (rp, ci, vv) in enumerate(op.matrix.csr_parts()):
        O = parts[p]
        assert np.array_equal(ci, O.colidx)
        if len(O.vals):
            assert np.abs(vv - O.vals).max() <= VAL_TOL * np.abs(O.vals).max()
        if len(O.b):
            assert np.abs(op.vector.partition[p] - O.b).max() <= VAL_TOL * max(np.abs(O.b).max(), 1e-300)


@pytest.mark.parametrize("dim,order,parts,n", [(2, 1, (2, 1), (4, 3)), (2, 2, (2, 2), (3, 3)),
                                                (3, 1, (2, 1, 2), (4, 3, 3)), (3, 2, (1, 2, 1), (2, 3, 2))])
def test_affine_displacement_kat_on_gpu(backend, dim, order, parts, n):
    """Known answer: u = B x + t on the whole boundary, E constant, no body force; the
    affine field has constant stress and lies in the space, so the device solve
    reproduces it: L2 error < 1e-9 (and the oracle's LU, tests/test_oracle_elasticity.py)."""
    import gridap_gb300 as G
    rng = np.random.default_rng(90 + 10 * dim + order)
    B, t = rng.normal(size=(dim, dim)), rng.normal(size=dim)
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.5 * d))
    ranks = backend.distribute(range(int(np.prod(parts))))
    model = G.CartesianDiscreteModel(ranks, parts, domain, n)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, G.VectorValue, order), dirichlet_tags="boundary")
    u = lambda *x: tuple(sum(B[c, d] * x[d] for d in range(dim)) + t[c] for c in range(dim))
    U = G.TrialFESpace(u, V)
    dO = G.Measure(G.Triangulation(model), 2 * order)
    op = G.AffineFEOperator(G.integral_elasticity(np.full(int(np.prod(n)), 2.5), 0.3, dO),
                            G.integral_source((0.0,) * dim, dO), U, V)
    uh = G.solve(op, rtol=1e-14)
    assert op.matrix.last_stats.converged
    assert G.l2_error(uh, u, dO) < 1e-9
