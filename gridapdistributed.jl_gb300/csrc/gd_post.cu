// Boundary source terms and post-processing on the device.
//
// gd_add_boundary_source adds int(v g) dGamma over flagged boundary sides to the
// assembled right-hand side (the Neumann term of test/PoissonTests.jl:20-41, g given at
// the face Gauss points).  gd_l2_error is the L2 error sqrt(sum(int(abs2(u - u_h)) dOmega))
// of an FE function, as the reference's tests compute it (test/PoissonTests.jl:43-45,
// test/FESpacesTests.jl:36-40).  The exact solution comes sampled at the tensor Gauss
// points of every cell (the caller evaluates it; a device cannot call back into the
// host's function); u_h is evaluated from the cell's nodal values (free values by gid,
// Dirichlet values from the trial space) with the same 1D Lagrange tables as the
// assembly.  One thread per cell, FP64, block partials summed on the host in block order.
#include <cmath>
#include <string>
#include <vector>

#include "gd_internal.h"

namespace gd {

// lattice node -> gid (-1 for Dirichlet nodes) from each part's owned DOFs
__global__ void k_space_node_gid(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                                 const int32_t* __restrict__ lid_node, const int32_t* __restrict__ lid_owner,
                                 const int64_t* __restrict__ lid_gid, int32_t* __restrict__ node_gid) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int lo = 0, hi = g.nparts - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (parts[mid].lid_off <= t) lo = mid;
    else hi = mid - 1;
  }
  const DevPart& P = parts[lo];
  if (lid_owner[t] != lo) return;
  int64_t li = lid_node[t], X[3] = {0, 0, 0};
  for (int d = 0; d < g.dim; ++d) {
    X[d] = g.k * P.loc_lo[d] + li % P.nb[d];
    li /= P.nb[d];
  }
  node_gid[lattice_lin(g, X)] = (int32_t)lid_gid[t];
}

constexpr int kPostThreads = 128;
constexpr int kMaxQ = 8;   // quadrature points per direction

template <int DIM, int K>
__global__ void __launch_bounds__(kPostThreads)
k_l2_error(Geom g, int64_t ncells, int bs, const int32_t* __restrict__ node_gid, const double* __restrict__ x,
           const double* __restrict__ u_dir, const double* __restrict__ u_qp, int nq,
           const double* __restrict__ tab, double detJ, double* __restrict__ partial) {
  constexpr int KP1 = K + 1;
  constexpr int NN = DIM == 3 ? KP1 * KP1 * KP1 : KP1 * KP1;
  __shared__ double sV[kMaxQ * KP1];
  __shared__ double sW[kMaxQ];
  __shared__ double red[kPostThreads / 32];
  for (int i = threadIdx.x; i < nq * KP1; i += blockDim.x) sV[i] = tab[i];
  for (int i = threadIdx.x; i < nq; i += blockDim.x) sW[i] = tab[nq * KP1 + i];
  __syncthreads();
  int nqt = 1;
  for (int d = 0; d < DIM; ++d) nqt *= nq;
  double acc = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    int64_t cc[3] = {0, 0, 0}, r = c;
    for (int d = 0; d < DIM; ++d) {
      cc[d] = r % g.n[d];
      r /= g.n[d];
    }
    for (int comp = 0; comp < bs; ++comp) {
      double U[NN];
#pragma unroll
      for (int a = 0; a < NN; ++a) {
        int64_t X[3] = {0, 0, 0};
        for (int d = 0, rest = a; d < DIM; ++d) {
          X[d] = K * cc[d] + rest % KP1;
          rest /= KP1;
        }
        const int64_t lin = lattice_lin(g, X);
        const int32_t gid = node_gid[lin];
        U[a] = gid >= 0 ? x[(int64_t)bs * gid + comp] : (u_dir ? u_dir[(int64_t)bs * lin + comp] : 0.0);
      }
      for (int q = 0; q < nqt; ++q) {
        int qi[3] = {0, 0, 0};
        double w = detJ;
        for (int d = 0, rest = q; d < DIM; ++d) {
          qi[d] = rest % nq;
          rest /= nq;
          w *= sW[qi[d]];
        }
        double uh = 0.0;
#pragma unroll
        for (int a = 0; a < NN; ++a) {
          double phi = 1.0;
          for (int d = 0, rest = a; d < DIM; ++d) {
            phi *= sV[qi[d] * KP1 + rest % KP1];
            rest /= KP1;
          }
          uh = fma(phi, U[a], uh);
        }
        const double e = u_qp[(c * nqt + q) * bs + comp] - uh;
        acc = fma(w * e, e, acc);
      }
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    partial[blockIdx.x] = s;
  }
}

static int space_node_gid(gd_space* S, cudaStream_t st) {
  const Geom& g = S->geom;
  int64_t nnodes = 1;
  for (int d = 0; d < g.dim; ++d) nnodes *= g.N[d];
  if (S->lat_gid.p && S->lat_gid.n == (size_t)nnodes) return GD_OK;
  GD_TRY(dalloc(S->lat_gid, nnodes));
  GD_CUDA_TRY(cudaMemsetAsync(S->lat_gid.p, 0xFF, sizeof(int32_t) * nnodes, st));
  if (S->total_lids > 0)
    k_space_node_gid<<<(unsigned)((S->total_lids + 255) / 256), 256, 0, st>>>(g, S->d_parts.p, S->total_lids,
                                                                               S->lid_node.p, S->lid_owner.p,
                                                                               S->lid_gid.p, S->lat_gid.p);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// ---- boundary source l(v) += int(v g) dGamma on flagged sides ------------------------------
// One thread per owned row: the row's node X, on each flagged side it lies on, collects
// sum_q w_q |J_face| phi_X(x_q) g(x_q) over the boundary faces around it (up to 2^(dim-1)),
// phi_X restricted to the face being the product of the tangential 1D Lagrange factors.
// g_qp: faces side by side (flagged sides in order x-, x+, y-, y+, z-, z+), lexicographic
// over the face's cells in the remaining directions (lowest first), nq^(dim-1) points
// per face (lowest remaining direction fastest).
template <int DIM, int K>
__global__ void k_boundary_rhs(Geom g, int64_t nrows_own, const int32_t* __restrict__ row_node, int side_mask,
                               const int64_t* __restrict__ side_off, const double* __restrict__ g_qp, int nq,
                               const double* __restrict__ tab, double* __restrict__ rhs) {
  constexpr int KP1 = K + 1;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows_own) return;
  int64_t lin = row_node[r];
  int64_t X[3] = {0, 0, 0};
  for (int d = 0; d < DIM; ++d) {
    X[d] = lin % g.N[d];
    lin /= g.N[d];
  }
  const double* V = tab;          // [nq][KP1]
  const double* W = tab + nq * KP1;
  double b = 0.0;
  for (int s = 0; s < 2 * DIM; ++s) {
    if (!((side_mask >> s) & 1)) continue;
    const int d = s >> 1;
    if (X[d] != ((s & 1) ? g.N[d] - 1 : 0)) continue;
    int tang[2] = {0, 0}, nt = 0;
    for (int t = 0; t < DIM; ++t)
      if (t != d) tang[nt++] = t;
    int64_t clo[2] = {0, 0}, chi[2] = {0, 0};
    for (int j = 0; j < nt; ++j) {
      const int t = tang[j];
      const int64_t c = X[t] / K;
      if (X[t] % K == 0) {
        clo[j] = c - 1 < 0 ? 0 : c - 1;
        chi[j] = c > g.n[t] - 1 ? g.n[t] - 1 : c;
      } else {
        clo[j] = chi[j] = c;
      }
    }
    int nqf = 1;
    for (int j = 0; j < nt; ++j) nqf *= nq;
    for (int64_t c1 = clo[1]; c1 <= chi[1]; ++c1)
      for (int64_t c0 = clo[0]; c0 <= chi[0]; ++c0) {
        const int64_t cc[2] = {c0, c1};
        const int64_t f = nt == 1 ? c0 : c0 + g.n[tang[0]] * c1;
        int l[2] = {0, 0};
        for (int j = 0; j < nt; ++j) l[j] = (int)(X[tang[j]] - K * cc[j]);
        const double* gq = g_qp + (side_off[s] + f) * nqf;
        for (int q = 0; q < nqf; ++q) {
          double w = 1.0, phi = 1.0;
          for (int j = 0, rest = q; j < nt; ++j) {
            const int qj = rest % nq;
            rest /= nq;
            w *= W[qj] * g.h[tang[j]];
            phi *= V[qj * KP1 + l[j]];
          }
          b = fma(w * phi, gq[q], b);
        }
      }
  }
  rhs[r] += b;
}

}  // namespace gd

using namespace gd;

extern "C" int gd_add_boundary_source(gd_asm* A, const int32_t* sides, const double* g_qp, int degree, int where) {
  if (!A || !sides || !g_qp) return fail(GD_ERR_ARG, "gd_add_boundary_source: null argument");
  if (!A->numeric_done) return fail(GD_ERR_STATE, "gd_add_boundary_source: run the numeric assembly first");
  if (A->bs != 1) return fail(GD_ERR_UNSUPPORTED, "gd_add_boundary_source: scalar spaces only");
  const Geom& g = A->test->geom;
  const int nq = (degree + 2) / 2;
  if (nq < 1 || nq > kMaxQ) return fail(GD_ERR_ARG, "gd_add_boundary_source: quadrature degree out of range");
  cudaStream_t st = A->test->model->ctx->stream;
  int mask = 0;
  std::vector<int64_t> off(2 * kMaxDim + 1, 0);
  int64_t nfaces = 0;
  int nqf = 1;
  for (int d = 0; d + 1 < g.dim; ++d) nqf *= nq;
  for (int s = 0; s < 2 * g.dim; ++s) {
    off[s] = nfaces;
    if (!sides[s]) continue;
    mask |= 1 << s;
    int64_t nf = 1;
    for (int t = 0; t < g.dim; ++t)
      if (t != s / 2) nf *= g.n[t];
    nfaces += nf;
  }
  if (!mask) return GD_OK;
  const double* dg = g_qp;
  DBuf<double> hg, dtab;
  DBuf<int64_t> doff;
  if (where == GD_HOST) {
    GD_TRY(dalloc(hg, nfaces * nqf));
    GD_CUDA_TRY(cudaMemcpyAsync(hg.p, g_qp, sizeof(double) * nfaces * nqf, cudaMemcpyHostToDevice, st));
    dg = hg.p;
  }
  const int kp1 = g.k + 1;
  std::vector<double> xq, wq, tab(nq * kp1 + nq), dtmp(kp1);
  gauss_legendre01(nq, xq, wq);
  for (int q = 0; q < nq; ++q) {
    lagrange01(g.k, xq[q], &tab[q * kp1], dtmp.data());
    tab[nq * kp1 + q] = wq[q];
  }
  GD_TRY(dalloc(dtab, tab.size()));
  GD_TRY(dalloc(doff, off.size()));
  GD_CUDA_TRY(cudaMemcpyAsync(dtab.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaMemcpyAsync(doff.p, off.data(), sizeof(int64_t) * off.size(), cudaMemcpyHostToDevice, st));
  const int64_t R = A->ngdofs;
  if (R > 0) {
    const unsigned nb = (unsigned)((R + 127) / 128);
    const int sel = g.dim * 10 + g.k;
#define BND_LAUNCH(D, K) \
  k_boundary_rhs<D, K><<<nb, 128, 0, st>>>(g, R, A->row_node.p, mask, doff.p, dg, nq, dtab.p, A->rhs.p)
    switch (sel) {
      case 21: BND_LAUNCH(2, 1); break;
      case 22: BND_LAUNCH(2, 2); break;
      case 23: BND_LAUNCH(2, 3); break;
      case 31: BND_LAUNCH(3, 1); break;
      case 32: BND_LAUNCH(3, 2); break;
      case 33: BND_LAUNCH(3, 3); break;
      default: return fail(GD_ERR_UNSUPPORTED, "gd_add_boundary_source: unsupported dim/order");
    }
#undef BND_LAUNCH
    GD_CUDA_TRY(cudaGetLastError());
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

extern "C" int gd_l2_error(gd_space* S, const double* x, const double* u_qp, int degree, int where, double* err) {
  if (!S || !x || !u_qp || !err) return fail(GD_ERR_ARG, "gd_l2_error: null argument");
  const Geom& g = S->geom;
  const int nq = (degree + 2) / 2;
  if (nq < 1 || nq > kMaxQ) return fail(GD_ERR_ARG, "gd_l2_error: quadrature degree out of range");
  cudaStream_t st = S->model->ctx->stream;
  const int bs = S->ncomp;
  int64_t ncells = 1;
  for (int d = 0; d < g.dim; ++d) ncells *= g.n[d];
  int64_t nqt = 1;
  for (int d = 0; d < g.dim; ++d) nqt *= nq;
  GD_TRY(space_node_gid(S, st));
  const double* dx = x;
  const double* du = u_qp;
  DBuf<double> hx, hu;
  if (where == GD_HOST) {
    GD_TRY(dalloc(hx, std::max<int64_t>(S->ngdofs * bs, 1)));
    GD_TRY(dalloc(hu, std::max<int64_t>(ncells * nqt * bs, 1)));
    GD_CUDA_TRY(cudaMemcpyAsync(hx.p, x, sizeof(double) * S->ngdofs * bs, cudaMemcpyHostToDevice, st));
    GD_CUDA_TRY(cudaMemcpyAsync(hu.p, u_qp, sizeof(double) * ncells * nqt * bs, cudaMemcpyHostToDevice, st));
    dx = hx.p;
    du = hu.p;
  }
  // 1D tables: Lagrange values at the Gauss points, then the weights
  const int kp1 = g.k + 1;
  std::vector<double> xq, wq, tab(nq * kp1 + nq), dtmp(kp1);
  gauss_legendre01(nq, xq, wq);
  for (int q = 0; q < nq; ++q) {
    lagrange01(g.k, xq[q], &tab[q * kp1], dtmp.data());
    tab[nq * kp1 + q] = wq[q];
  }
  DBuf<double> dtab, part;
  GD_TRY(dalloc(dtab, tab.size()));
  GD_CUDA_TRY(cudaMemcpyAsync(dtab.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st));
  double detJ = 1.0;
  for (int d = 0; d < g.dim; ++d) detJ *= g.h[d];
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>((ncells + kPostThreads - 1) / kPostThreads, 4096));
  GD_TRY(dalloc(part, nb));
  const double* udir = S->has_dirichlet_values ? S->u_dir.p : nullptr;
  const int sel = g.dim * 10 + g.k;
#define L2_LAUNCH(D, K)                                                                                     \
  k_l2_error<D, K><<<nb, kPostThreads, 0, st>>>(g, ncells, bs, S->lat_gid.p, dx, udir, du, nq, dtab.p, detJ, \
                                                part.p)
  switch (sel) {
    case 21: L2_LAUNCH(2, 1); break;
    case 22: L2_LAUNCH(2, 2); break;
    case 23: L2_LAUNCH(2, 3); break;
    case 31: L2_LAUNCH(3, 1); break;
    case 32: L2_LAUNCH(3, 2); break;
    case 33: L2_LAUNCH(3, 3); break;
    default: return fail(GD_ERR_UNSUPPORTED, "gd_l2_error: unsupported dim/order");
  }
#undef L2_LAUNCH
  GD_CUDA_TRY(cudaGetLastError());
  std::vector<double> hp(nb);
  GD_CUDA_TRY(cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  double s = 0.0;
  for (int i = 0; i < nb; ++i) s += hp[i];
  *err = std::sqrt(s);
  return GD_OK;
}
