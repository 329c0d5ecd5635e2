"""The oracle's elasticity element matrix and vector numbering, checked against
properties that hold for any correct restatement: the E = 1 element matrix is
symmetric, annihilates the rigid-body motions (dim translations and dim(dim-1)/2
linearised rotations) and is positive on their complement; the vector numbering of
orders 1 and 2 is the scalar node numbering with components interleaved."""
import itertools

import numpy as np
import pytest

import gridap_oracle as go


@pytest.mark.parametrize("dim,k", [(2, 1), (2, 2), (3, 1), (3, 2)])
def test_element_matrix_rigid_modes(dim, k):
    h = (0.5, 0.25, 0.125)[:dim]
    K = go.reference_elasticity(dim, k, h, 2 * k, 0.3)
    assert np.abs(K - K.T).max() <= 1e-13 * np.abs(K).max()
    nodes = np.array(go.cell_local_nodes(dim, k), dtype=float) / k * np.array(h)
    nn = len(nodes)
    modes = []
    for c in range(dim):                     # translations
        u = np.zeros((dim, nn))
        u[c] = 1.0
        modes.append(u.ravel())
    for a, b in itertools.combinations(range(dim), 2):   # rotations in the (a, b) plane
        u = np.zeros((dim, nn))
        u[a] = -nodes[:, b]
        u[b] = nodes[:, a]
        modes.append(u.ravel())
    for m in modes:
        assert np.abs(K @ m).max() <= 1e-12 * np.abs(K).max() * np.abs(m).max()
    ev = np.linalg.eigvalsh(K)
    nrig = len(modes)
    assert np.all(ev[nrig:] > 1e-8 * ev[-1])


@pytest.mark.parametrize("order", [1, 2])
def test_vector_numbering_interleaves_scalar(order):
    n, parts = (3, 2, 2), (2, 1, 2)
    pv = go.Problem(np=parts, n=n, domain=(0, 1, 0, 1, 0, 1), order=order, degree=2 * order,
                    dirichlet_sides=(1, 0, 0, 0, 0, 0), physics="elasticity")
    ps = go.Problem(np=parts, n=n, domain=(0, 1, 0, 1, 0, 1), order=order, degree=2 * order,
                    dirichlet_sides=(1, 0, 0, 0, 0, 0))
    fv, fs = go.build_fespace(pv), go.build_fespace(ps)
    for p in range(len(fv.spaces)):
        dv, ds = fv.dofs[p], fs.dofs[p]
        assert np.array_equal(dv.ldof_to_gdof, (3 * ds.ldof_to_gdof[:, None] + np.arange(3)).ravel())
        assert np.array_equal(dv.ldof_to_owner, np.repeat(ds.ldof_to_owner, 3))
        assert np.array_equal(fv.spaces[p].dof_comp, np.tile(np.arange(3), fs.spaces[p].nfree))


def test_small_elasticity_system_is_spd():
    pb = go.Problem(np=(2, 1, 1), n=(3, 2, 2), domain=(0, 1, 0, 1, 0, 1), order=2, degree=4,
                    dirichlet_sides=(1, 0, 0, 0, 0, 0), physics="elasticity", nu=0.3, force=(0, 0, -1.0))
    fe = go.build_fespace(pb)
    A, b = go.gather_global(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    Ad = A.toarray()
    assert np.abs(Ad - Ad.T).max() <= 1e-13 * np.abs(Ad).max()
    assert np.linalg.eigvalsh(Ad).min() > 0
    x = np.linalg.solve(Ad, b)
    assert x[2::3].mean() < 0     # the body force points down


def affine_problem(dim, order, parts, n, seed):
    """u_D = B x + t on the whole boundary, E constant, no body force: the stress of the
    affine field is constant, so it solves the problem and lies in the Q_k space."""
    rng = np.random.default_rng(seed)
    B, t = rng.normal(size=(dim, dim)), rng.normal(size=dim)
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.5 * d))
    pb = go.Problem(np=parts, n=n, domain=domain, order=order, degree=2 * order,
                    kappa=np.full(int(np.prod(n)), 2.5), physics="elasticity", nu=0.3)
    N = pb.lattice
    X = np.stack(np.meshgrid(*[np.arange(N[d]) for d in range(dim)], indexing="ij"), axis=-1).reshape(-1, dim)
    lin = pb.node_lin(X)
    u = np.empty((int(np.prod(N)), dim))
    u[lin] = pb.node_xyz(X) @ B.T + t
    pb.u_dir = u
    return pb, B, t


@pytest.mark.parametrize("dim,order,parts,n", [(2, 1, (2, 1), (3, 2)), (2, 2, (2, 2), (3, 3)),
                                                (3, 1, (2, 1, 2), (3, 2, 2)), (3, 2, (1, 2, 1), (2, 3, 2))])
def test_affine_displacement_is_reproduced(dim, order, parts, n):
    """Known answer for the Dirichlet lifting of vector spaces: the gathered LU solution
    equals the affine field at every free (node, component) to 1e-10."""
    pb, B, t = affine_problem(dim, order, parts, n, seed=70 + 10 * dim + order)
    fe = go.build_fespace(pb)
    x = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    for sp, d in zip(fe.spaces, fe.dofs):
        want = (pb.node_xyz(sp.dof_node) @ B.T + t)[np.arange(len(sp.dof_comp)), sp.dof_comp]
        assert np.abs(x[d.ldof_to_gdof] - want).max() <= 1e-10
