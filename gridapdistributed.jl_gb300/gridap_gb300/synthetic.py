"""Seeded synthetic inputs for the benchmark configurations.

The coefficient fields are lognormal, kappa = exp(g), with g a Gaussian random
field of standard deviation sigma and squared-exponential correlation
exp(-r^2 / (2 l^2)).  g is drawn by spectral synthesis on a periodically embedded
grid twice the mesh size per direction (numpy PCG64, seed given by the caller),
evaluated at the cell centres and normalised to mean 0 and the target sigma.
"""
from __future__ import annotations

import numpy as np


def gaussian_random_field(cells, sigma=1.0, corr_len=0.1, seed=0, domain_len=1.0):
    """g at the cell centres of a uniform grid with ``cells`` cells per direction.

    Returns a flat float64 array in lexicographic cell order (x fastest)."""
    cells = tuple(int(c) for c in cells)
    dim = len(cells)
    rng = np.random.Generator(np.random.PCG64(seed))
    M = tuple(2 * c for c in cells)
    h = [domain_len / c for c in cells]
    # wavenumbers of the embedded periodic grid (axis order z,y,x for C-order arrays)
    ks = [2 * np.pi * np.fft.fftfreq(M[d], d=h[d]) for d in range(dim)]
    grids = np.meshgrid(*[ks[d] for d in reversed(range(dim))], indexing="ij", sparse=True)
    k2 = sum(g * g for g in grids)
    amp = np.exp(-k2 * corr_len * corr_len / 4.0)   # sqrt of the squared-exponential spectrum
    shape = tuple(reversed(M))
    noise = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    field = np.fft.ifftn(amp * noise).real
    field = field[tuple(slice(0, c) for c in reversed(cells))]
    field = field - field.mean()
    std = field.std()
    if std > 0:
        field = field * (sigma / std)
    return np.ascontiguousarray(field.reshape(-1), dtype=np.float64)


def lognormal_kappa(cells, sigma=1.0, corr_len=0.1, seed=0):
    return np.exp(gaussian_random_field(cells, sigma, corr_len, seed))


def gaussian_random_field_at_points(cells, points, sigma=1.0, corr_len=0.1, seed=0, domain_len=1.0):
    """g of gaussian_random_field (same seed, same cell-centre values) at arbitrary points
    of the unit box, by multilinear interpolation between the cell centres (constant
    beyond the outermost centres).  ``points``: array (..., dim).  The correlation length
    spans several cells, so the interpolation changes the field by O((h / l)^2)."""
    cells = tuple(int(c) for c in cells)
    dim = len(cells)
    g = gaussian_random_field(cells, sigma, corr_len, seed, domain_len).reshape(tuple(reversed(cells)))
    pts = np.asarray(points, dtype=np.float64)
    i0, t = [], []
    for d in range(dim):
        s = pts[..., d] / (domain_len / cells[d]) - 0.5
        lo = np.clip(np.floor(s).astype(np.int64), 0, max(cells[d] - 2, 0))
        i0.append(lo)
        t.append(np.clip(s - lo, 0.0, 1.0) if cells[d] > 1 else np.zeros_like(s))
    out = np.zeros(pts.shape[:-1])
    for corner in range(1 << dim):
        w = np.ones(pts.shape[:-1])
        idx = []
        for d in range(dim):
            b = (corner >> d) & 1
            w = w * (t[d] if b else 1.0 - t[d])
            idx.append(np.minimum(i0[d] + b, cells[d] - 1))
        out += w * g[tuple(reversed(idx))]
    return out


def lognormal_at_points(cells, points, sigma=1.0, corr_len=0.1, seed=0):
    return np.exp(gaussian_random_field_at_points(cells, points, sigma, corr_len, seed))


# The 3D variable-coefficient Poisson workload: 128^3 Q1 hex cells on the unit
# cube, parts (2,2,2), kappa = exp(g) (sigma 1, correlation length 0.1), f = 1,
# homogeneous Dirichlet on the whole boundary, quadrature degree 2.
POISSON3D_128 = dict(name="poisson3d_q1_128^3_parts2x2x2", dim=3, cells=(128, 128, 128), parts=(2, 2, 2),
                     domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), order=1, degree=2, sigma=1.0, corr_len=0.1,
                     f=1.0, seed=1000)


def gaussian_random_field_torch(cells, sigma=1.0, corr_len=0.1, seed=0, domain_len=1.0, device="cuda"):
    """Same spectral synthesis as gaussian_random_field, on the GPU with torch (for
    generating many training fields); a different random stream than the numpy one."""
    import torch
    cells = tuple(int(c) for c in cells)
    dim = len(cells)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    M = tuple(2 * c for c in cells)
    ks = [2 * torch.pi * torch.fft.fftfreq(M[d], d=domain_len / cells[d], device=device, dtype=torch.float64)
          for d in range(dim)]
    grids = torch.meshgrid(*[ks[d] for d in reversed(range(dim))], indexing="ij")
    k2 = sum(x * x for x in grids)
    amp = torch.exp(-k2 * corr_len * corr_len / 4.0)
    shape = tuple(reversed(M))
    noise = torch.complex(torch.randn(shape, generator=g, device=device, dtype=torch.float64),
                          torch.randn(shape, generator=g, device=device, dtype=torch.float64))
    field = torch.fft.ifftn(amp * noise).real[tuple(slice(0, c) for c in reversed(cells))]
    field = field - field.mean()
    field = field * (sigma / field.std())
    return field.reshape(-1).contiguous()


# Learned-preconditioner workloads: 96^3 and 192^3 Q1 cells on the unit cube, parts
# (2,2,2), kappa = exp(g) (sigma 1.5, correlation length 0.05), load M f with f ~ N(0,1)
# per node, homogeneous Dirichlet, solve to 1e-8 FP64 relative residual.
DIFFUSION3D_96 = dict(name="diffusion3d_q1_96^3_parts2x2x2_sigma1.5", dim=3, cells=(96, 96, 96), parts=(2, 2, 2),
                      domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), order=1, degree=2, sigma=1.5, corr_len=0.05,
                      seed=5000)
DIFFUSION3D_192 = dict(DIFFUSION3D_96, name="diffusion3d_q1_192^3_parts2x2x2_sigma1.5", cells=(192, 192, 192))


# Batched uneven workload: 64 independent 3D diffusion problems, cells per direction
# n ~ U{16..96}, order k ~ U{1,2,3}, kappa lognormal i.i.d. per cell (sigma 1), f = 1,
# homogeneous Dirichlet, parts (2,2,1) per problem.  Draw: numpy PCG64(seed); problem i's
# kappa uses PCG64(seed + 1 + i).
BATCHED3D_64 = dict(name="batched64_3d_q1-q3_16-96cells_parts2x2x1", nprobs=64, cells=(16, 96), orders=(1, 2, 3),
                    sigma=1.0, parts=(2, 2, 1), domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), f=1.0, seed=3000)


def batched_draw(w=BATCHED3D_64):
    """[(n, k, kappa_seed)] for the batch, in draw order."""
    rng = np.random.Generator(np.random.PCG64(w["seed"]))
    lo, hi = w["cells"]
    out = []
    for i in range(w["nprobs"]):
        n = int(rng.integers(lo, hi + 1))
        k = int(rng.integers(min(w["orders"]), max(w["orders"]) + 1))
        out.append((n, k, w["seed"] + 1 + i))
    return out


def batched_kappa(n, seed, sigma=1.0):
    rng = np.random.Generator(np.random.PCG64(seed))
    return np.exp(sigma * rng.standard_normal(n ** 3))


def batched_nnz_estimate(n, k):
    """Free DOFs and stored owned-row entries of one problem (all-Dirichlet): a Q_k node
    couples with 2k+1 nodes per direction at a cell vertex and k+1 inside a cell, so on
    average k+2 per direction."""
    dofs = (k * n - 1) ** 3
    return dofs, dofs * (k + 2) ** 3


# Linear elasticity workload: 64^3 hex cells on the unit cube, vector Q2, quadrature
# degree 4, parts (2,2,2), E = exp(g) (sigma 0.5, correlation length 0.1), nu = 0.3,
# body force (0,0,-1), clamped (all components) on x = 0.
ELASTICITY3D_64 = dict(name="elasticity3d_vq2_64^3_parts2x2x2", cells=(64, 64, 64), parts=(2, 2, 2),
                       domain=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), order=2, degree=4, sigma=0.5, corr_len=0.1,
                       nu=0.3, force=(0.0, 0.0, -1.0), seed=4000)
