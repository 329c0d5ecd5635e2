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
