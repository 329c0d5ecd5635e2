"""The oracle's quadrature-point coefficients (CPU only).

A coefficient known at the Gauss points enters each element matrix as
K_e = sum_q c_q W_q grad(phi_i).grad(phi_j) (CellData integrate, src/CellData.jl:234-259).
Pinned by:
* consistency with the cell-constant path (pinned to the reference's known-answer tests):
  c_q = kappa_cell at every point gives the same matrices and vectors;
* manufactured solutions that the Galerkin method reproduces exactly because the exact
  solution lies in the space and the quadrature integrates both forms exactly:
  - diffusion, kappa = 1 + x + 2y sampled at the points, u = x + y (+ z), f = -3;
  - elasticity, E = 2 + x + y at the points, u = B x + t (constant strain), body force
    f = -sigma1 (1, 1, 0), sigma1 = the stress of E = 1.
"""
import numpy as np
import pytest

import gridap_oracle as go
from helpers import make_problem, row_scaled_error


def _kappa_qp_const(pb):
    nqt = go.quad_points_per_dir(pb.degree) ** pb.dim
    return np.repeat(pb.kappa[:, None], nqt, axis=1)


@pytest.mark.parametrize("dim,n,parts,order", [(2, (5, 4), (2, 2), 1), (2, (3, 3), (2, 1), 3),
                                               (3, (4, 3, 3), (2, 1, 2), 2), (3, (4, 4, 4), (2, 2, 2), 1)])
@pytest.mark.parametrize("strategy", ["sub", "full"])
def test_point_coefficients_constant_per_cell_match_cell_path(dim, n, parts, order, strategy):
    pb = make_problem(dim, n, parts, order, seed=5, u=(lambda *x: 1.0 + sum(x)))
    fe = go.build_fespace(pb)
    ref = go.assemble(pb, fe, strategy)
    pb.kappa_qp = _kappa_qp_const(pb)
    got = go.assemble(pb, fe, strategy)
    for M, Q in zip(ref, got):
        assert np.array_equal(M.rowptr, Q.rowptr) and np.array_equal(M.colidx, Q.colidx)
        assert row_scaled_error(Q.vals, M.vals, M.rowptr) <= 1e-13
        assert np.abs(Q.b - M.b).max(initial=0.0) <= 1e-13 * max(np.abs(M.b).max(initial=0.0), 1e-300)


def diffusion_kat_problem(dim, n, parts, order):
    """kappa = 1 + x + 2y at the Gauss points, u = x + y (+ z) on the boundary, f = -3."""
    u = (lambda x, y: x + y) if dim == 2 else (lambda x, y, z: x + y + z)
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.25 * d))
    pb = make_problem(dim, n, parts, order, f=-3.0, u=u, domain=domain)
    xq = go.quadrature_points(pb)
    pb.kappa_qp = 1.0 + xq[:, :, 0] + 2.0 * xq[:, :, 1]
    return pb, u


@pytest.mark.parametrize("dim,n,parts,order", [(2, (4, 3), (2, 2), 1), (2, (3, 3), (1, 2), 2),
                                               (3, (3, 3, 2), (2, 1, 2), 1), (3, (2, 2, 3), (1, 2, 2), 2)])
def test_variable_kappa_linear_solution_is_reproduced(dim, n, parts, order):
    pb, u = diffusion_kat_problem(dim, n, parts, order)
    fe = go.build_fespace(pb)
    x = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    assert go.l2_error(pb, go.nodal_solution(pb, fe, x), u) < 1e-10


def elasticity_kat_problem(dim, n, parts, order, seed):
    rng = np.random.default_rng(seed)
    B, t = rng.normal(size=(dim, dim)), rng.normal(size=dim)
    nu = 0.3
    domain = tuple(v for d in range(dim) for v in (0.0, 1.0 + 0.5 * d))
    pb = go.Problem(np=parts, n=n, domain=domain, order=order, degree=2 * order, physics="elasticity", nu=nu)
    xq = go.quadrature_points(pb)
    pb.kappa_qp = 2.0 + xq[:, :, 0] + xq[:, :, 1]
    eps = 0.5 * (B + B.T)
    lam, mu = nu / ((1 + nu) * (1 - 2 * nu)), 1.0 / (2 * (1 + nu))
    sigma1 = lam * np.trace(eps) * np.eye(dim) + 2 * mu * eps
    grad_e = np.zeros(dim)
    grad_e[0] = grad_e[1] = 1.0
    pb.force = tuple(-(sigma1 @ grad_e))
    N = pb.lattice
    X = np.stack(np.meshgrid(*[np.arange(N[d]) for d in range(dim)], indexing="ij"), axis=-1).reshape(-1, dim)
    uD = np.empty((int(np.prod(N)), dim))
    uD[pb.node_lin(X)] = pb.node_xyz(X) @ B.T + t
    pb.u_dir = uD
    return pb, B, t


@pytest.mark.parametrize("dim,order,parts,n", [(2, 1, (2, 1), (3, 2)), (2, 2, (2, 2), (3, 3)),
                                                (3, 1, (2, 1, 2), (3, 2, 2)), (3, 2, (1, 2, 1), (2, 3, 2))])
def test_variable_modulus_affine_displacement_is_reproduced(dim, order, parts, n):
    pb, B, t = elasticity_kat_problem(dim, n, parts, order, seed=90 + 10 * dim + order)
    fe = go.build_fespace(pb)
    x = go.solve_lu(go.assemble(pb, fe, "sub"), fe.dofs[0].ngdofs)
    for sp, d in zip(fe.spaces, fe.dofs):
        want = (pb.node_xyz(sp.dof_node) @ B.T + t)[np.arange(len(sp.dof_comp)), sp.dof_comp]
        assert np.abs(x[d.ldof_to_gdof] - want).max() <= 1e-10
