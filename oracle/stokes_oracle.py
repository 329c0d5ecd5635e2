"""CPU oracle for the reference's multi-field test with fields on different spaces.

TEST INFRASTRUCTURE ONLY: nothing in the shipped library imports this module.

``test/MultiFieldTests.jl:14-81`` assembles and solves a Stokes problem on a 2D
``CartesianDiscreteModel`` (domain (0,4)^2, 4x4 cells):

* velocity: vector-valued Lagrangian Q_k (k = 2), Dirichlet on the whole boundary with
  u = ((x+y)^2, (x-y)^2) (``:25, :28, :35``);
* pressure: scalar Lagrangian of order k-1 on the P space (``space=:P``), discontinuous,
  with the zero-mean constraint (``constraint=:zeromean``, ``:26, :36``), exact
  p = x + y - mean(x + y);
* a((u,p),(v,q)) = int(grad v : grad u - q div u - div v p), l((v,q)) = int(v.f - q g) with
  f = -lap u + grad p and g = div u (``:32-33, :49-50``), quadrature degree 2k (``:24``);
* its known answers: the L2 errors of the solved u and p below 1e-9 (``:54-57``).

The zero-mean space is ``FESpaceWithConstantFixed`` on the last free DOF of the
pressure space (``src/FESpaces.jl:872-910``) plus the mean correction of
``FEFunction`` (``src/FESpaces.jl:912-941, 958-975``): the fixed DOF takes the value 0,
the system is solved for the others, and then every pressure DOF (the fixed one too) is
shifted by c = -(sum_i p_i int(psi_i)) / |Omega| (``_compute_new_fixedval``).

Restated here on the gathered (serial) system, which is what the known answers pin:
velocity DOFs 2 per node of the k-refined node lattice (x fastest), pressure DOFs 3 per
cell (cells x fastest).  The discontinuous P1 element of Gridap's ``space=:P`` on a
square (Gridap.jl 0.20, third party): the monomials 1, x, y with nodal DOFs at the
exponent points (0,0), (1,0), (0,1) of the reference square, in that order; the
fixed DOF (the last free one) is then the third DOF of the last cell.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from gridap_oracle import gauss_legendre, lagrange_1d, quad_points_per_dir


@dataclass
class StokesSystem:
    A: sp.csr_matrix          # free velocity DOFs, then the free pressure DOFs
    b: np.ndarray
    nu_free: int              # free velocity DOFs
    vel_free: np.ndarray      # global velocity DOF -> free index (-1: Dirichlet)
    u_dir: np.ndarray         # value of every velocity DOF (Dirichlet values, 0 elsewhere)
    p_fixed: int              # the pressure DOF fixed by the zero-mean space
    dvol: np.ndarray          # int(psi_i) over the domain, per pressure DOF
    vol: float
    n: tuple
    domain: tuple
    k: int


def _p1_square(xi, eta):
    """Nodal P1 basis on the reference square for the nodes (0,0), (1,0), (0,1) and its
    reference gradients."""
    val = np.array([1.0 - xi - eta, xi, eta])
    grd = np.array([[-1.0, -1.0], [1.0, 0.0], [0.0, 1.0]])
    return val, grd


def _cell_tables(k, h, degree):
    """Tensor Gauss points of one cell: weights (with |J|), reference coordinates, the
    velocity shape values / physical gradients (cell-local nodes lexicographic, x fastest)
    and the pressure basis values."""
    nq = quad_points_per_dir(degree)
    xq, wq = gauss_legendre(nq)
    V, D = lagrange_1d(k, xq)
    pts = [(a, b) for b in range(nq) for a in range(nq)]   # x fastest
    nn = (k + 1) ** 2
    W = np.zeros(len(pts))
    xi = np.zeros((len(pts), 2))
    phi = np.zeros((len(pts), nn))
    gphi = np.zeros((len(pts), nn, 2))
    psi = np.zeros((len(pts), 3))
    for q, (a, b) in enumerate(pts):
        W[q] = wq[a] * wq[b] * h[0] * h[1]
        xi[q] = (xq[a], xq[b])
        for j in range(k + 1):
            for i in range(k + 1):
                n_ = i + (k + 1) * j
                phi[q, n_] = V[a, i] * V[b, j]
                gphi[q, n_, 0] = D[a, i] * V[b, j] / h[0]
                gphi[q, n_, 1] = V[a, i] * D[b, j] / h[1]
        psi[q], _ = _p1_square(xq[a], xq[b])
    return W, xi, phi, gphi, psi


def stokes_system(n=(4, 4), domain=(0.0, 4.0, 0.0, 4.0), k=2, u=None, p=None, f=None, g=None,
                  p_fixed=None) -> StokesSystem:
    """The gathered Stokes system of test/MultiFieldTests.jl on a Cartesian mesh (free
    unknowns only: the velocity's Dirichlet values lifted to the right-hand side, the
    zero-mean space's fixed pressure DOF removed).  p_fixed: the pressure DOF to fix
    (default the last one, as the reference's zero-mean space does)."""
    x0, x1, y0, y1 = domain
    h = ((x1 - x0) / n[0], (y1 - y0) / n[1])
    degree = 2 * k
    W, xi, phi, gphi, psi = _cell_tables(k, h, degree)
    N0, N1 = k * n[0] + 1, k * n[1] + 1
    nnode = N0 * N1
    ndof_u = 2 * nnode
    ncell = n[0] * n[1]
    ndof_p = 3 * ncell
    # Dirichlet velocity DOFs: every boundary node, both components
    boundary = np.zeros(nnode, dtype=bool)
    for Y in range(N1):
        for X in range(N0):
            if X in (0, N0 - 1) or Y in (0, N1 - 1):
                boundary[X + N0 * Y] = True
    u_dir = np.zeros(ndof_u)
    for Y in range(N1):
        for X in range(N0):
            if boundary[X + N0 * Y]:
                xy = (x0 + X * h[0] / k, y0 + Y * h[1] / k)
                uv = u(*xy)
                u_dir[2 * (X + N0 * Y)] = uv[0]
                u_dir[2 * (X + N0 * Y) + 1] = uv[1]
    vel_free = -np.ones(ndof_u, dtype=np.int64)
    nu_free = 0
    for node in range(nnode):
        if not boundary[node]:
            vel_free[2 * node] = nu_free
            vel_free[2 * node + 1] = nu_free + 1
            nu_free += 2
    if p_fixed is None:
        p_fixed = ndof_p - 1   # the last free DOF of the pressure space
    pres_free = np.arange(ndof_p, dtype=np.int64)
    pres_free[p_fixed] = -1
    pres_free[p_fixed + 1:] -= 1
    nfree = nu_free + ndof_p - 1
    I, J, Vv = [], [], []
    b = np.zeros(nfree)
    dvol = np.zeros(ndof_p)
    nn = (k + 1) ** 2
    for cy in range(n[1]):
        for cx in range(n[0]):
            c = cx + n[0] * cy
            nodes = [(k * cx + i) + N0 * (k * cy + j) for j in range(k + 1) for i in range(k + 1)]
            udofs = [2 * nd + a for a in range(2) for nd in nodes]   # component-major in the cell
            pdofs = [3 * c + m for m in range(3)]
            # element matrix over (u component-major, p)
            Ke = np.zeros((2 * nn + 3, 2 * nn + 3))
            fe = np.zeros(2 * nn + 3)
            for q in range(len(W)):
                xq = (x0 + (cx + xi[q, 0]) * h[0], y0 + (cy + xi[q, 1]) * h[1])
                G = gphi[q]
                lap = G @ G.T
                for a in range(2):
                    Ke[a * nn:(a + 1) * nn, a * nn:(a + 1) * nn] += W[q] * lap
                    # -q div u and -div v p
                    Ke[2 * nn:, a * nn:(a + 1) * nn] -= W[q] * np.outer(psi[q], G[:, a])
                    Ke[a * nn:(a + 1) * nn, 2 * nn:] -= W[q] * np.outer(G[:, a], psi[q])
                fv = f(*xq)
                for a in range(2):
                    fe[a * nn:(a + 1) * nn] += W[q] * fv[a] * phi[q]
                fe[2 * nn:] -= W[q] * g(*xq) * psi[q]
                dvol[pdofs] += W[q] * psi[q]
            # global free indices of the element's DOFs (-1: Dirichlet velocity or fixed pressure)
            gidx = [vel_free[d] for d in udofs] + [nu_free + pres_free[d] if pres_free[d] >= 0 else -1 for d in pdofs]
            dval = np.array([u_dir[d] if vel_free[d] < 0 else 0.0 for d in udofs] + [0.0, 0.0, 0.0])
            fe = fe - Ke @ dval   # lifting of the Dirichlet velocity values (the fixed pressure is 0)
            for i_, gi in enumerate(gidx):
                if gi < 0:
                    continue
                b[gi] += fe[i_]
                for j_, gj in enumerate(gidx):
                    if gj >= 0 and Ke[i_, j_] != 0.0:
                        I.append(gi)
                        J.append(gj)
                        Vv.append(Ke[i_, j_])
    A = sp.csr_matrix((Vv, (I, J)), shape=(nfree, nfree))
    return StokesSystem(A=A, b=b, nu_free=nu_free, vel_free=vel_free, u_dir=u_dir, p_fixed=p_fixed,
                        dvol=dvol, vol=(x1 - x0) * (y1 - y0), n=tuple(n), domain=tuple(domain), k=k)


def stokes_solve(S: StokesSystem):
    """Solve the gathered system (sparse LU, as the reference's BackslashSolver on the
    gathered matrix) and return (velocity DOF values, pressure DOF values) with the
    zero-mean correction applied."""
    x = spla.splu(S.A.tocsc()).solve(S.b)
    uvals = S.u_dir.copy()
    free = S.vel_free >= 0
    uvals[free] = x[S.vel_free[free]]
    ndof_p = len(S.dvol)
    pvals = np.zeros(ndof_p)
    pfree = np.delete(np.arange(ndof_p), S.p_fixed)
    pvals[pfree] = x[S.nu_free:]
    c = -float(pvals @ S.dvol) / S.vol   # the fixed DOF holds 0
    return uvals, pvals + c


def stokes_l2_errors(S: StokesSystem, uvals, pvals, u, p, degree=None):
    """sqrt(sum(int((u-uh).(u-uh)))) and the same for p, with the test's quadrature."""
    k = S.k
    x0, x1, y0, y1 = S.domain
    n = S.n
    h = ((x1 - x0) / n[0], (y1 - y0) / n[1])
    W, xi, phi, gphi, psi = _cell_tables(k, h, 2 * k if degree is None else degree)
    N0 = k * n[0] + 1
    eu = ep = 0.0
    for cy in range(n[1]):
        for cx in range(n[0]):
            c = cx + n[0] * cy
            nodes = [(k * cx + i) + N0 * (k * cy + j) for j in range(k + 1) for i in range(k + 1)]
            u0 = uvals[[2 * nd for nd in nodes]]
            u1 = uvals[[2 * nd + 1 for nd in nodes]]
            pc = pvals[3 * c:3 * c + 3]
            for q in range(len(W)):
                xq = (x0 + (cx + xi[q, 0]) * h[0], y0 + (cy + xi[q, 1]) * h[1])
                ue = u(*xq)
                d0 = ue[0] - phi[q] @ u0
                d1 = ue[1] - phi[q] @ u1
                eu += W[q] * (d0 * d0 + d1 * d1)
                dp = p(*xq) - psi[q] @ pc
                ep += W[q] * dp * dp
    return float(np.sqrt(eu)), float(np.sqrt(ep))
