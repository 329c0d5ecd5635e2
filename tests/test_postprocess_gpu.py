"""Device post-processing: the L2 error of a solution, as the reference's tests form it
(sqrt(sum(int(abs2(u - uh))dOmega))), against the oracle's host restatement and on the
reference's known-answer problems."""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def backend():
    import gridap_gb300 as G
    be = G.GB300Backend(0)
    yield be
    be.close()


def system(be, pb, strategy="sub", vector=False, nu=0.3, force=None):
    import gridap_gb300 as G
    ranks = be.distribute(range(int(np.prod(pb.np))))
    model = G.CartesianDiscreteModel(ranks, pb.np, pb.domain, pb.n)
    tags = ["left", "right", "bottom", "top", "back", "front"]
    sides = [t for t, s in zip(tags, pb.dirichlet_sides) if s]
    T = G.VectorValue if vector else float
    V = G.TestFESpace(model, G.ReferenceFE(G.lagrangian, T, pb.order), dirichlet_tags=sides)
    U = G.TrialFESpace(pb.u_dir, V) if pb.u_dir is not None else G.TrialFESpace(0.0, V)
    dO = G.Measure(G.Triangulation(model), pb.degree)
    if vector:
        a = G.integral_elasticity(pb.kappa, nu, dO)
        l = G.integral_source(force, dO)
    else:
        a = G.integral_grad_grad(pb.kappa, dO)
        l = G.integral_source(pb.f_nodal if pb.f_nodal is not None else pb.f_const, dO)
    strat = G.SubAssembledRows() if strategy == "sub" else G.FullyAssembledRows()
    op = G.AffineFEOperator(a, l, U, V, G.SparseMatrixAssembler(U, V, strat))
    return model, V, U, op, dO


@pytest.mark.parametrize("strategy", ["sub", "full"])
def test_fespaces_kat_l2_error_on_device(backend, strategy):
    """test/FESpacesTests.jl:10-59: Q1 reproduces u = x + y."""
    import gridap_gb300 as G
    u = lambda x, y: x + y
    pb = make_problem(2, (4, 4), (2, 2), 1, f=0.0, u=u, domain=(0, 4, 0, 4))
    pb.degree = 3
    model, V, U, op, dO = system(backend, pb, strategy)
    uh = G.solve(op, rtol=1e-14)
    assert G.l2_error(uh, u, dO) < 1e-9


def test_poisson_q2_kat_l2_error_on_device(backend):
    """test/PoissonTests.jl:14-45: Q2 reproduces (x + y)^2."""
    import gridap_gb300 as G
    u = lambda x, y: (x + y) ** 2
    pb = make_problem(2, (4, 4), (2, 2), 2, f=-4.0, u=u, domain=(0, 4, 0, 4))
    model, V, U, op, dO = system(backend, pb)
    uh = G.solve(op, rtol=1e-14)
    assert G.l2_error(uh, u, dO) < 1e-9


@pytest.mark.parametrize("case", [dict(dim=3, n=(6, 5, 4), parts=(2, 2, 1), order=1, seed=70),
                                  dict(dim=3, n=(3, 4, 3), parts=(2, 1, 2), order=3, seed=71),
                                  dict(dim=2, n=(5, 6), parts=(2, 2), order=2, seed=72)])
def test_l2_error_matches_oracle(backend, case):
    import gridap_gb300 as G
    pb = make_problem(**case)
    model, V, U, op, dO = system(backend, pb)
    uh = G.solve(op, rtol=1e-13)
    if pb.dim == 3:
        ue = lambda x, y, z: np.sin(3 * x) * np.cos(2 * y) + z * z
    else:
        ue = lambda x, y: np.sin(3 * x) * np.cos(2 * y)
    dev = G.l2_error(uh, ue, dO)
    ref = go.l2_error(pb, uh.nodal_values(), ue)
    assert abs(dev - ref) <= 1e-10 * ref


def test_vector_l2_norm_matches_componentwise_oracle(backend):
    import gridap_gb300 as G
    pb = go.Problem(np=(2, 2, 1), n=(4, 3, 3), domain=(0, 1, 0, 1, 0, 1), order=2, degree=4,
                    dirichlet_sides=(1, 0, 0, 0, 0, 0),
                    kappa=np.exp(0.5 * np.random.default_rng(73).normal(size=36)))
    model, V, U, op, dO = system(backend, pb, vector=True, force=(0.0, 0.0, -1.0))
    x = op.matrix.solve(rtol=1e-13)
    uh = G.FEFunction(U, x)
    dev = G.l2_error(uh, lambda x_, y_, z_: (0.0 * x_, 0.0 * x_, 0.0 * x_), dO)
    # per-component lattice arrays from the gids of the vector dofs
    N = int(np.prod(V.lattice))
    comps = np.zeros((3, N))
    for p in range(model.num_parts):
        li = V.gids.partition()[p]
        nodes = V.dof_nodes(p)
        comp = np.arange(len(nodes)) % 3
        comps[comp, nodes] = x[li.local_to_global]
    ref = np.sqrt(sum(go.l2_error(pb, comps[c], lambda x_, y_, z_: 0.0) ** 2 for c in range(3)))
    assert abs(dev - ref) <= 1e-10 * ref


@pytest.mark.parametrize("parts", [(2, 2), (1, 1), (2, 1), (1, 2)])
def test_fespaces_interpolation_kat_on_gpu(backend, parts):
    """test/FESpacesTests.jl:88-139 (`_interpolation_tests` with a Julia function): Q1 on
    (0,4)^2, 4 x 4 cells, u = x+y, U = TrialFESpace(u, V).  interpolate, interpolate_everywhere
    (of u and of an FEFunction), interpolate_everywhere!, interpolate_dirichlet(!), and
    FEFunction(U, free, dirichlet): L2 error of u - uh < 1e-9 (degree 3), computed on the device.
    Then a space with zero Dirichlet values: a function carrying its own Dirichlet values is
    measured with them, and afterwards the space's own (zero) values are back in place."""
    import gridap_gb300 as G
    u = lambda x, y: x + y
    ranks = backend.distribute(range(int(np.prod(parts))))
    model = G.CartesianDiscreteModel(ranks, parts, (0, 4, 0, 4), (4, 4))
    reffe = G.ReferenceFE(G.lagrangian, float, 1)
    V = G.TestFESpace(model, reffe, dirichlet_tags="boundary")
    U = G.TrialFESpace(u, V)
    dO = G.Measure(G.Triangulation(model), 3)
    err = lambda uh: G.l2_error(uh, u, dO)
    assert G.zero_free_values(U).shape == (U.num_free_dofs(),)
    assert err(G.interpolate(u, U)) < 1e-9
    free_values = G.zero_free_values(U)
    dirichlet_values = G.get_dirichlet_dof_values(U)
    uh_dir = G.interpolate_dirichlet_(u, free_values, dirichlet_values, U)
    assert np.all(uh_dir.free_values == 0.0)
    uh_e = G.interpolate_everywhere(u, U)
    assert err(uh_e) < 1e-9
    uh_e_ = G.interpolate_everywhere_(u, free_values, G.zero_dirichlet_values(U), U)
    assert err(uh_e_) < 1e-9
    assert err(G.interpolate_everywhere(uh_e, U)) < 1e-9
    assert err(G.interpolate_everywhere_(uh_e, free_values, dirichlet_values, U)) < 1e-9
    assert err(G.FEFunction(U, free_values, dirichlet_values)) < 1e-9

    V0 = G.TestFESpace(model, reffe, dirichlet_tags="boundary")
    U0 = G.TrialFESpace(0.0, V0)
    assert err(G.interpolate_everywhere(u, U0)) < 1e-9     # its own Dirichlet values
    assert err(G.interpolate(u, U0)) > 1e-2                # the space's zero values again
    assert err(G.interpolate_dirichlet(u, U0)) > 1e-2      # zero free values
