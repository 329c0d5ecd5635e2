"""Discontinuous Galerkin on the GPU.

- The DG part of the reference's Poisson known-answer test (test/PoissonTests.jl:47-77):
  Q2 with conformity L2 on (0,4)^2, 4x4 cells, symmetric interior penalty gamma = 10,
  h = 2, Nitsche Dirichlet data on the bottom/left sides and g = n.grad(u) on the
  top/right sides reproduces u = (x+y)^2: L2 error < 1e-9, through the Python mirror.
- The assembled local parts against the oracle's restatement (tests/test_oracle_dg.py
  pins it to the same known answer), for both strategies: pattern, ghost row and ghost
  column gids and owners bit-exact (SubAssembledRows: the faces a part owns, the zeroed
  ghost rows and the first-appearance column order of the oracle's loop restatement);
  values |gpu - oracle| <= 1e-12 * max |oracle| in the row; right-hand side <= 1e-12.
- The DG dof numbering (gids and owners of every part's local dofs) bit-exact.
"""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import row_scaled_error

pytestmark = pytest.mark.gpu

TAGS = ["left", "right", "bottom", "top", "back", "front"]
VAL_TOL = 1e-12


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def gpu_dg(be, parts, n, domain, k, gamma, hpen, f, dsides, nsides, u, g, strategy=None):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(parts))))
    model = G.CartesianDiscreteModel(ranks, parts, domain, n)
    V = G.FESpace(model, G.ReferenceFE(G.lagrangian, float, k), conformity="L2")
    deg = 2 * k
    dO = G.Measure(G.Triangulation(model), deg)
    dL = G.Measure(G.Skeleton(model), deg)
    dGd = G.Measure(G.Boundary(model, tags=[TAGS[s] for s in range(len(dsides)) if dsides[s]]), deg) \
        if any(dsides) else None
    dGn = G.Measure(G.Boundary(model, tags=[TAGS[s] for s in range(len(nsides)) if nsides[s]]), deg) \
        if any(nsides) else None
    a = G.integral_sipg(gamma, hpen, dO, dGd, dL)
    l = G.integral_sipg_source(f, u, g, gamma, hpen, dO, dGn, dGd)
    assem = None
    if strategy is not None:
        assem = G.SparseMatrixAssembler(V, V, G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows())
    return model, V, G.AffineFEOperator(a, l, V, V, assem), dO


@pytest.mark.parametrize("parts", [(1, 1), (2, 2), (2, 1), (1, 2)])
def test_dg_poisson_kat_on_gpu(backend, parts):
    """test/PoissonTests.jl:47-77 on the GPU path."""
    import gridap_gb300 as G
    u = lambda x, y: (x + y) ** 2
    g = lambda x, y, nx, ny: 2.0 * (x + y) * (nx + ny)
    _, V, op, dO = gpu_dg(backend, parts, (4, 4), (0, 4, 0, 4), 2, 10.0, 2.0, -4.0, (1, 0, 1, 0), (0, 1, 0, 1), u, g)
    uh = G.solve(op, rtol=1e-14)
    assert op.matrix.last_stats.converged
    assert G.l2_error(uh, u, dO) < 1e-9


CASES = [
    dict(parts=(2, 2), n=(4, 4), domain=(0, 4, 0, 4), k=2, dsides=(1, 0, 1, 0), nsides=(0, 1, 0, 1)),
    dict(parts=(3, 1), n=(5, 3), domain=(0, 1, 0, 0.6), k=1, dsides=(1, 1, 0, 0), nsides=(0, 0, 1, 0)),
    dict(parts=(1, 2), n=(3, 4), domain=(-1, 2, 0, 1), k=3, dsides=(0, 0, 0, 1), nsides=(1, 0, 0, 0)),
    dict(parts=(2, 1, 2), n=(3, 2, 3), domain=(0, 1, 0, 1, 0, 1), k=1, dsides=(1, 0, 0, 0, 1, 1),
         nsides=(0, 1, 1, 0, 0, 0)),
    dict(parts=(1, 2, 2), n=(2, 3, 2), domain=(0, 2, 0, 3, 0, 1), k=2, dsides=(0, 1, 1, 0, 0, 0),
         nsides=(1, 0, 0, 0, 0, 1)),
]


def case_id(c):
    return f"{len(c['n'])}d_q{c['k']}_{'x'.join(map(str, c['n']))}_p{''.join(map(str, c['parts']))}"


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("case", CASES, ids=case_id)
def test_dg_parts_match_oracle(backend, case, strategy):
    dim = len(case["n"])
    if dim == 2:
        u = lambda x, y: np.sin(x) + x * y
        g = lambda x, y, nx, ny: 0.5 + x - y * nx
    else:
        u = lambda x, y, z: np.cos(x) + y * z
        g = lambda x, y, z, nx, ny, nz: 1.0 + x * ny - z * nz
    gamma, hpen, f = 7.5, 0.8, 1.25
    model, V, op, _ = gpu_dg(backend, case["parts"], case["n"], case["domain"], case["k"], gamma, hpen, f,
                             case["dsides"], case["nsides"], u, g, strategy)
    ref, gid0, ndofs = go.dg_system(case["parts"], case["n"], case["domain"], case["k"], 2 * case["k"], gamma, hpen,
                                    f, case["dsides"], case["nsides"], u, g, strategy=strategy)
    assert V.num_free_dofs() == ndofs
    A = op.matrix
    for p, (M, (rp, ci, vv), rows, cols, b) in enumerate(zip(ref, A.csr_parts(), A.row_partition, A.col_partition,
                                                              A.rhs_parts())):
        assert np.array_equal(rp, M.rowptr), f"rowptr part {p}"
        assert np.array_equal(ci, M.colidx), f"colidx part {p}"
        assert np.array_equal(rows.ghost_to_global, M.row_ghost_gids), f"ghost rows part {p}"
        assert np.array_equal(rows.ghost_to_owner, M.row_ghost_owner)
        assert np.array_equal(cols.ghost_to_global, M.col_ghost_gids), f"ghost cols part {p}"
        assert np.array_equal(cols.ghost_to_owner, M.col_ghost_owner)
        assert row_scaled_error(vv, M.vals, M.rowptr) <= VAL_TOL
        assert np.abs(b - M.b).max() <= VAL_TOL * max(np.abs(M.b).max(), 1e-300)
    # dof numbering of every part's local cells
    P = go.make_partition(case["parts"], case["n"])
    nn = (case["k"] + 1) ** dim
    for p, li in enumerate(V.gids.partition()):
        lc = P.local_cells(p)
        expect = np.concatenate([np.arange(gid0[c], gid0[c] + nn) for c in lc])
        assert np.array_equal(li.local_to_global, expect), f"gids part {p}"
    # mul! against the gathered oracle operator
    x = np.random.default_rng(3).normal(size=ndofs)
    y = A.mul(x)
    for M in ref:
        gcols = np.concatenate([M.col_own_gids, M.col_ghost_gids])
        for r in range(len(M.row_own_gids)):
            s = sum(M.vals[e] * x[gcols[M.colidx[e]]] for e in range(M.rowptr[r], M.rowptr[r + 1]))
            assert abs(y[M.row_own_gids[r]] - s) <= 1e-12 * max(1.0, abs(s))
