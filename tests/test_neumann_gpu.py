"""Neumann boundary terms, l(v) = int(v f)dOmega + int(v g)dGamma_n: the reference's
Poisson known-answer test (test/PoissonTests.jl:14-45: Q2 reproduces (x+y)^2 with
Dirichlet on left/bottom and g = n.grad(u) on top/right) through the GPU path, and the
assembled right-hand side against the oracle for general g."""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem

pytestmark = pytest.mark.gpu

VAL_TOL = 1e-12
TAGS = ["left", "right", "bottom", "top", "back", "front"]


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def gpu_op(be, pb, neumann_sides, g, strategy="sub"):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, float, pb.order),
                      dirichlet_tags=[t for t, s in zip(TAGS, pb.dirichlet_sides) if s])
    U = G.TrialFESpace(pb.u_dir, V) if pb.u_dir is not None else G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    dG = G.Measure(G.Boundary(model, tags=[TAGS[s] for s in neumann_sides]), pb.degree)
    a = G.integral_grad_grad(pb.kappa, dO)
    l = G.integral_source(pb.f_nodal if pb.f_nodal is not None else pb.f_const, dO) + \
        G.integral_boundary_source(g, dG)
    strat = G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows()
    op = G.AffineFEOperator(a, l, U, V, G.SparseMatrixAssembler(U, V, strat))
    return op, dO


@pytest.mark.parametrize("strategy", ["sub", "full"])
@pytest.mark.parametrize("parts", [(1, 1), (2, 2), (2, 1), (1, 2)])
def test_poisson_neumann_kat_on_gpu(backend, parts, strategy):
    import gridap_gb300 as G
    u = lambda x, y: (x + y) ** 2
    g = lambda x, y, nx, ny: 2.0 * (x + y) * (nx + ny)   # n . grad(u)
    pb = make_problem(2, (4, 4), parts, 2, f=-4.0, u=u, domain=(0, 4, 0, 4), sides=(1, 0, 1, 0))
    op, dO = gpu_op(backend, pb, [1, 3], g, strategy)
    uh = G.solve(op, rtol=1e-14)
    assert G.l2_error(uh, u, dO) < 1e-9


CASES = [
    dict(dim=3, n=(4, 3, 5), parts=(2, 1, 2), order=1, sides=(1, 0, 0, 1, 1, 0), seed=80),
    dict(dim=3, n=(3, 3, 2), parts=(1, 2, 2), order=3, sides=(0, 1, 1, 0, 0, 0), seed=81),
    dict(dim=2, n=(5, 4), parts=(2, 2), order=2, sides=(1, 0, 0, 0), seed=82),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c['dim']}d_q{c['order']}")
def test_neumann_rhs_matches_oracle(backend, case):
    pb = make_problem(**case)
    dim = pb.dim
    neu = [s for s in range(2 * dim) if not pb.dirichlet_sides[s]]
    if dim == 3:
        g = lambda x, y, z, nx, ny, nz: np.sin(2 * x) * np.cos(y) + z + 0.5 * nx - ny
    else:
        g = lambda x, y, nx, ny: np.sin(2 * x) * np.cos(y) + 0.5 * nx - ny
    pb.neumann = {s: g for s in neu}
    fe = go.build_fespace(pb)
    parts = go.assemble(pb, fe, "sub")
    op, _ = gpu_op(backend, pb, neu, g)
    for p, bp in enumerate(op.vector.partition):
        O = parts[p]
        if len(O.b):
            assert np.abs(bp - O.b).max() <= VAL_TOL * max(np.abs(O.b).max(), 1e-300)
