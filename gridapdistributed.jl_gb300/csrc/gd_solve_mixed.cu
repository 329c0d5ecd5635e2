// Mixed-precision solve behind `\`: FP64 iterative refinement around an FP32
// preconditioned CG whose operator is applied matrix-free.
//
// The reference's `\` gathers the system and factorises it (PartitionedArrays 0.3).
// On GB300 the FP64 pipe is ~60x slower than FP32 and a CSR SpMV moves 12 bytes per
// entry, so this solver keeps FP64 only where it sets the accuracy:
//   outer loop (FP64): r = b - A x with the assembled FP64 matrix, x += |r| d;
//   inner loop (FP32 vectors): CG on A d = r/|r| to a relative tolerance, with the
//   inner products, step lengths alpha/beta and the convergence test in FP64.
// For Q1 on cube cells the inner operator is rebuilt per row from the prescaled cell
// coefficients w = K2*kappa (FP32, one 4-byte value per cell) and a lattice-node ->
// gid map: an SpMV reads ~17 bytes per row instead of ~330 (27 entries x 12 bytes).
// Other spaces use an FP32 copy of the CSR values.  The preconditioner is Jacobi, or
// (gd_solve with GD_SOLVE_LEARNED_FCG) a trained network applied by gd_learned.cu,
// in which case the inner iteration is flexible CG.
#include <chrono>
#include <cmath>
#include <string>

#include "gd_internal.h"
#include "gd_solve_mixed.h"

namespace gd {

constexpr int kMxThreads = 256;
constexpr int kMxMaxBlocks = 1024;

__device__ inline double block_sum_d(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;
}

// node -> gid over the global lattice (-1: Dirichlet), from the owned DOFs of all parts
__global__ void k_node_gid(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                           const int32_t* __restrict__ lid_node, const int32_t* __restrict__ lid_owner,
                           const int64_t* __restrict__ lid_gid, int32_t* __restrict__ node_gid) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int lo = 0, hi = g.nparts - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (parts[mid].lid_off <= t) lo = mid; else hi = mid - 1;
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

__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = __double2float_rn(a[i]);
}

// Matrix-free FP32 Q1 operator on cube cells (3D): y = A x over the owned rows.
// v(center) = ratio * sum(w), face diagonals = sums of two w, corners = w, edges = 0.
__device__ __forceinline__ float mf_row(const Geom& g, uint32_t lin, const int32_t* __restrict__ node_gid,
                                        const float* __restrict__ wf, float ratio, const float* __restrict__ x) {
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
  const int64_t X0 = lin % N0, t = lin / N0, X1 = t % N1, X2 = t / N1;
  const int64_t n0 = g.n[0], n1 = g.n[1], n2 = g.n[2];
  float w[8];
#pragma unroll
  for (int a = 0; a < 8; ++a) {
    const int64_t cx = X0 - 1 + (a & 1), cy = X1 - 1 + ((a >> 1) & 1), cz = X2 - 1 + ((a >> 2) & 1);
    const bool cin = cx >= 0 && cx < n0 && cy >= 0 && cy < n1 && cz >= 0 && cz < n2;
    w[a] = cin ? __ldg(wf + cx + n0 * (cy + n1 * cz)) : 0.f;
  }
  float P[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) P[a] = w[a] + w[a + 4];
  float acc = 0.f;
#pragma unroll
  for (int s = 0; s < 27; ++s) {
    const int o0 = s % 3 - 1, o1 = (s / 3) % 3 - 1, o2 = s / 9 - 1;
    const int nz = (o0 != 0) + (o1 != 0) + (o2 != 0);
    if (nz == 1) continue;   // edge neighbours: exactly zero on cube cells
    const int a0 = (o0 + 1) >> 1, a1 = (o1 + 1) >> 1, a2 = (o2 + 1) >> 1;
    float v;
    if (nz == 0) v = ratio * ((P[0] + P[1]) + (P[2] + P[3]));
    else if (nz == 3) v = w[a0 + 2 * a1 + 4 * a2];
    else if (o2 == 0) v = P[a0 + 2 * a1];
    else if (o1 == 0) v = w[a0 + 4 * a2] + w[a0 + 2 + 4 * a2];
    else v = w[2 * a1 + 4 * a2] + w[1 + 2 * a1 + 4 * a2];
    const int64_t Y0 = X0 + o0, Y1 = X1 + o1, Y2 = X2 + o2;
    if (Y0 < 0 || Y0 >= g.N[0] || Y1 < 0 || Y1 >= g.N[1] || Y2 < 0 || Y2 >= g.N[2]) continue;
    const int32_t gid = __ldg(node_gid + Y0 + g.N[0] * (Y1 + g.N[1] * Y2));
    if (gid >= 0) acc = fmaf(v, __ldg(x + gid), acc);
  }
  return acc;
}

__global__ void __launch_bounds__(kMxThreads)
k_mf_apply(Geom g, int64_t n, const int32_t* __restrict__ row_node, const int32_t* __restrict__ node_gid,
           const float* __restrict__ wf, float ratio, const float* __restrict__ x, float* __restrict__ y,
           double* __restrict__ partial) {
  __shared__ double sh[kMxThreads / 32];
  float dot = 0.f;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const float v = mf_row(g, (uint32_t)row_node[r], node_gid, wf, ratio, x);
    y[r] = v;
    dot = fmaf(v, x[r], dot);
  }
  if (partial) {
    const double t = block_sum_d((double)dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// FP32 CSR operator (spaces without the cube structure)
__global__ void __launch_bounds__(kMxThreads)
k_csr32_apply(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
              const float* __restrict__ val, const float* __restrict__ x, float* __restrict__ y,
              double* __restrict__ partial) {
  __shared__ double sh[kMxThreads / 32];
  float dot = 0.f;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.f;
    for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) s = fmaf(val[e], __ldg(x + col[e]), s);
    y[r] = s;
    dot = fmaf(s, x[r], dot);
  }
  if (partial) {
    const double t = block_sum_d((double)dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// The same with G lanes per row (long rows: vector and high-order spaces), strided
// coalesced entries per lane and a shuffle tree; the group's first lane writes the row.
template <int G>
__global__ void __launch_bounds__(kMxThreads)
k_csr32_apply_g(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                const float* __restrict__ val, const float* __restrict__ x, float* __restrict__ y,
                double* __restrict__ partial) {
  __shared__ double sh[kMxThreads / 32];
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31, sub = lane / G, gl = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  float dot = 0.f;
  for (int64_t rb = warp * RPW; rb < n; rb += nw * RPW) {   // warp-uniform trip count
    const int64_t r = rb + sub;
    float s = 0.f;
    if (r < n) {
      const int64_t e1 = rowptr[r + 1];
      int64_t e = rowptr[r] + gl;
      for (; e + 3 * G < e1; e += 4 * G) {   // 4 independent entries in flight per lane
        int32_t c[4];
        float v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          c[u] = col[e + u * G];
          v[u] = val[e + u * G];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) s = fmaf(v[u], xv[u], s);
      }
      for (; e < e1; e += G) s = fmaf(val[e], __ldg(x + col[e]), s);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (r < n && gl == 0) {
      y[r] = s;
      dot = fmaf(s, x[r], dot);
    }
  }
  if (partial) {
    const double t = block_sum_d((double)dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// diagonal of the FP32 operator -> its inverse
__global__ void k_mx_dinv(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                          const double* __restrict__ val, float* __restrict__ dinv) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 0.0;
  for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e)
    if (col[e] == r) d = val[e];
  dinv[r] = d > 0.0 ? (float)(1.0 / d) : 0.f;
}

// r32 = r64 * inv, x32 = 0, z = dinv r, p = z; partials r.z, r.r
__global__ void k_mx_start(int64_t n, const double* __restrict__ r64, double inv, const float* __restrict__ dinv,
                           float* __restrict__ x, float* __restrict__ r, float* __restrict__ z, float* __restrict__ p,
                           int precond_external, double* __restrict__ prz, double* __restrict__ prr) {
  __shared__ double sh[kMxThreads / 32];
  float a = 0.f, b = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = (float)(r64[i] * inv);
    r[i] = ri;
    x[i] = 0.f;
    if (!precond_external) {
      const float zi = dinv[i] * ri;
      z[i] = zi;
      p[i] = zi;
      a = fmaf(ri, zi, a);
    }
    b = fmaf(ri, ri, b);
  }
  double t = block_sum_d((double)a, sh);
  if (threadIdx.x == 0) prz[blockIdx.x] = t;
  t = block_sum_d((double)b, sh);
  if (threadIdx.x == 0) prr[blockIdx.x] = t;
}

struct MxScalars {
  double rz, pq, alpha, beta, rr, rz_old, rzn_mixed;
  int32_t it;
};

// fixed-order sums of the block partials and the CG scalars (FP64)
// mode 0: rz, rr   1: alpha = rz/pq   2: beta = rz_new/rz, rz, rr   3: flexible beta
__global__ void k_mx_scalars(int mode, int nb, const double* __restrict__ pa, const double* __restrict__ pb,
                             const double* __restrict__ pc, MxScalars* __restrict__ sc) {
  __shared__ double sh[kMxThreads / 32];
  double a = 0.0, b = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += pa[i];
    if (pb) b += pb[i];
    if (pc) c += pc[i];
  }
  const double sa = block_sum_d(a, sh), sb = block_sum_d(b, sh), scc = block_sum_d(c, sh);
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    sc->rz = sa;
    sc->rr = sb;
  } else if (mode == 1) {
    sc->pq = sa;
    sc->alpha = sa != 0.0 ? sc->rz / sa : 0.0;
  } else if (mode == 2) {
    sc->beta = sc->rz != 0.0 ? sa / sc->rz : 0.0;
    sc->rz = sa;
    sc->rr = sb;
  } else {   // flexible CG: beta = (r_new . (z_new - z_old)) / (r_old . z_old), sa = r_new.z_new, scc = r_new.z_old
    sc->beta = sc->rz != 0.0 ? (sa - scc) / sc->rz : 0.0;
    sc->rz = sa;
    sc->rr = sb;
  }
}

// x += alpha p; r -= alpha q; partial r.r (and z = dinv r, partial r.z when Jacobi)
__global__ void k_mx_update(int64_t n, const MxScalars* __restrict__ sc, float* __restrict__ x, float* __restrict__ r,
                            float* __restrict__ z, const float* __restrict__ p, const float* __restrict__ q,
                            const float* __restrict__ dinv, int precond_external, double* __restrict__ prz,
                            double* __restrict__ prr) {
  __shared__ double sh[kMxThreads / 32];
  const float alpha = (float)sc->alpha;
  float a = 0.f, b = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] = fmaf(alpha, p[i], x[i]);
    const float ri = fmaf(-alpha, q[i], r[i]);
    r[i] = ri;
    if (!precond_external) {
      const float zi = dinv[i] * ri;
      z[i] = zi;
      a = fmaf(ri, zi, a);
    }
    b = fmaf(ri, ri, b);
  }
  double t = block_sum_d((double)a, sh);
  if (threadIdx.x == 0) prz[blockIdx.x] = t;
  t = block_sum_d((double)b, sh);
  if (threadIdx.x == 0) prr[blockIdx.x] = t;
}

// partials r.z_new and r.z_old for flexible CG (after an external preconditioner wrote z)
__global__ void k_mx_dots_flex(int64_t n, const float* __restrict__ r, const float* __restrict__ z,
                               const float* __restrict__ zold, double* __restrict__ pa, double* __restrict__ pc) {
  __shared__ double sh[kMxThreads / 32];
  float a = 0.f, c = 0.f;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    a = fmaf(r[i], z[i], a);
    if (zold) c = fmaf(r[i], zold[i], c);
  }
  double t = block_sum_d((double)a, sh);
  if (threadIdx.x == 0) pa[blockIdx.x] = t;
  if (zold) {
    t = block_sum_d((double)c, sh);
    if (threadIdx.x == 0) pc[blockIdx.x] = t;
  }
}

__global__ void k_mx_pupdate(int64_t n, const MxScalars* __restrict__ sc, const float* __restrict__ z,
                             float* __restrict__ p) {
  const float beta = (float)sc->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = fmaf(beta, p[i], z[i]);
}

__global__ void k_mx_copy(int64_t n, const float* __restrict__ a, float* __restrict__ b) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// x64 += s * x32
__global__ void k_mx_accumulate(int64_t n, double s, const float* __restrict__ x32, double* __restrict__ x64) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x64[i] += s * (double)x32[i];
}

static int grid_mx(int64_t n) {
  int64_t b = (n + kMxThreads - 1) / kMxThreads;
  if (b > kMxMaxBlocks) b = kMxMaxBlocks;
  return (int)(b < 1 ? 1 : b);
}

// ---- setup of the FP32 operator (after every numeric assembly) -------------------------
int mixed_setup(gd_asm* A) {
  gd_space* S = A->test;
  const Geom& g = S->geom;
  cudaStream_t st = S->model->ctx->stream;
  const int64_t n = A->ngdofs;
  MixedState& M = A->mx;
  if (M.numeric_epoch == A->numeric_epoch && M.ready) return GD_OK;
  M.matrix_free = A->fast_q1 && A->q1c_cube && g.dim == 3 && !A->qp_values;
  int64_t ncells = 1, nnodes = 1;
  for (int d = 0; d < g.dim; ++d) {
    ncells *= g.n[d];
    nnodes *= g.N[d];
  }
  if (M.f32.n < (size_t)(6 * n)) GD_TRY(dalloc(M.f32, 6 * std::max<int64_t>(n, 1)));
  if (M.f64.n < (size_t)(2 * n)) GD_TRY(dalloc(M.f64, 2 * std::max<int64_t>(n, 1)));
  if (!M.red.p) GD_TRY(dalloc(M.red, 4 * kMxMaxBlocks + 64));
  float* dinv = M.f32.p + 5 * n;
  if (M.matrix_free) {
    if (M.node_gid.n != (size_t)nnodes) {
      GD_TRY(dalloc(M.node_gid, nnodes));
      GD_CUDA_TRY(cudaMemsetAsync(M.node_gid.p, 0xFF, sizeof(int32_t) * nnodes, st));
      if (S->total_lids > 0)
        k_node_gid<<<(unsigned)((S->total_lids + 255) / 256), 256, 0, st>>>(g, S->d_parts.p, S->total_lids,
                                                                             S->lid_node.p, S->lid_owner.p,
                                                                             S->lid_gid.p, M.node_gid.p);
      GD_CUDA_TRY(cudaGetLastError());
    }
    if (M.wf.n != (size_t)ncells) GD_TRY(dalloc(M.wf, ncells));
    k_to_f32<<<grid_mx(ncells), kMxThreads, 0, st>>>(ncells, A->w_cells.p, M.wf.p);
    GD_CUDA_TRY(cudaGetLastError());
    M.ratio = (float)A->mf_ratio;
  } else {
    if (M.vals32.n != (size_t)std::max<int64_t>(A->nnz_own, 1)) GD_TRY(dalloc(M.vals32, std::max<int64_t>(A->nnz_own, 1)));
    if (A->nnz_own > 0) k_to_f32<<<grid_mx(A->nnz_own), kMxThreads, 0, st>>>(A->nnz_own, A->vals.p, M.vals32.p);
    GD_CUDA_TRY(cudaGetLastError());
  }
  if (n > 0) k_mx_dinv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, A->rowptr.p, A->colgid.p, A->vals.p, dinv);
  GD_CUDA_TRY(cudaGetLastError());
  {   // lanes per row of the FP32 CSR operator, from the average row length
    const int64_t avg = n > 0 ? A->nnz_own / n : 0;
    M.csr_lanes = avg >= 256 ? 32 : avg >= 96 ? 16 : avg >= 48 ? 8 : 1;
  }
  M.numeric_epoch = A->numeric_epoch;
  M.ready = true;
  return GD_OK;
}

int mixed_apply(gd_asm* A, const float* x, float* y, double* partial, cudaStream_t st) {
  const int64_t n = A->ngdofs;
  MixedState& M = A->mx;
  const int gb = grid_mx(n);
  if (M.matrix_free)
    k_mf_apply<<<gb, kMxThreads, 0, st>>>(A->test->geom, n, A->row_node.p, M.node_gid.p, M.wf.p, M.ratio, x, y,
                                          partial);
  else if (M.csr_lanes == 32)
    k_csr32_apply_g<32><<<gb, kMxThreads, 0, st>>>(n, A->rowptr.p, A->colgid.p, M.vals32.p, x, y, partial);
  else if (M.csr_lanes == 16)
    k_csr32_apply_g<16><<<gb, kMxThreads, 0, st>>>(n, A->rowptr.p, A->colgid.p, M.vals32.p, x, y, partial);
  else if (M.csr_lanes == 8)
    k_csr32_apply_g<8><<<gb, kMxThreads, 0, st>>>(n, A->rowptr.p, A->colgid.p, M.vals32.p, x, y, partial);
  else
    k_csr32_apply<<<gb, kMxThreads, 0, st>>>(n, A->rowptr.p, A->colgid.p, M.vals32.p, x, y, partial);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// Mixed-precision refinement; `precond` applies z = M(r) when non-null (flexible CG).
int mixed_solve(gd_asm* A, double rtol, int maxit, double* x_out, int where, gd_solve_stats* stats,
                const MixedPrecond* precond) {
  GD_TRY(mixed_setup(A));
  if (A->mx.matrix_free && (!precond || precond->apply_lattice))
    return mixed_solve_lattice(A, rtol, maxit, x_out, where, stats, precond);
  cudaStream_t st = A->test->model->ctx->stream;
  const int64_t n = A->ngdofs;
  MixedState& M = A->mx;
  auto t0 = std::chrono::steady_clock::now();
  float* x = M.f32.p;
  float* r = x + n;
  float* z = r + n;
  float* p = z + n;
  float* q = p + n;
  float* dinv = q + n;
  double* x64 = M.f64.p;
  double* r64 = x64 + n;
  double* pa = M.red.p;
  double* pb = pa + kMxMaxBlocks;
  double* pc = pb + kMxMaxBlocks;
  MxScalars* sc = reinterpret_cast<MxScalars*>(pc + kMxMaxBlocks);
  const int gb = grid_mx(n);
  const int ext = precond != nullptr;
  float* zold = nullptr;
  if (ext) {
    if (M.zold.n < (size_t)n) GD_TRY(dalloc(M.zold, std::max<int64_t>(n, 1)));
    zold = M.zold.p;
  }
  GD_CUDA_TRY(cudaMemsetAsync(x64, 0, sizeof(double) * n, st));
  int total_inner = 0, outer = 0;
  double bnorm = 0.0, rel = 1.0, prev_rel = 1e300;
  const double inner_tol = 1e-5;
  int status = GD_OK;
  while (true) {
    // FP64 residual of the current iterate
    int gr = 0;
    GD_TRY(residual_fp64_asm(A, x64, A->rhs_override ? A->rhs_override : A->rhs.p, r64, pa, pb, st, &gr));
    k_mx_scalars<<<1, kMxThreads, 0, st>>>(0, gr, pa, pb, nullptr, sc);
    GD_CUDA_TRY(cudaGetLastError());
    MxScalars h{};
    GD_CUDA_TRY(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    const double rnorm = std::sqrt(h.rz);
    if (outer == 0) bnorm = std::sqrt(h.rr);
    rel = bnorm > 0.0 ? rnorm / bnorm : 0.0;
    if (!std::isfinite(rel)) {
      status = fail(GD_ERR_NUMERIC, "mixed solve: residual is not finite");
      break;
    }
    if (rel <= rtol || bnorm == 0.0) break;
    if (total_inner >= maxit) {
      status = fail(GD_ERR_NOTCONVERGED, "mixed solve: tolerance not reached in " + std::to_string(total_inner) + " iterations");
      break;
    }
    if (outer > 0 && rel > 0.5 * prev_rel) {   // refinement stalled
      status = fail(GD_ERR_STALL, "mixed solve: refinement stalled at relative residual " + std::to_string(rel));
      break;
    }
    prev_rel = rel;
    ++outer;
    // inner CG on A d = r / |r|
    k_mx_start<<<gb, kMxThreads, 0, st>>>(n, r64, 1.0 / rnorm, dinv, x, r, z, p, ext, pa, pb);
    GD_CUDA_TRY(cudaGetLastError());
    if (ext) {
      GD_TRY(precond->apply(precond->ctx, A, r, z, st));
      k_mx_copy<<<gb, kMxThreads, 0, st>>>(n, z, p);
      k_mx_dots_flex<<<gb, kMxThreads, 0, st>>>(n, r, z, nullptr, pa, nullptr);
      k_mx_scalars<<<1, kMxThreads, 0, st>>>(0, gb, pa, pb, nullptr, sc);   // rz and rr (pb from start)
    } else {
      k_mx_scalars<<<1, kMxThreads, 0, st>>>(0, gb, pa, pb, nullptr, sc);
    }
    GD_CUDA_TRY(cudaGetLastError());
    // inner tolerance: reach inner_tol, or a bit below what the outer loop still needs
    const double tol_in = std::max(inner_tol, 0.5 * rtol / rel);
    int it = 0;
    const int batch = 16;
    const int inner_max = maxit - total_inner;
    // external preconditioner: give up when 64 iterations do not halve the inner
    // residual, so a weak preconditioner hands over to Jacobi early
    bool inner_stall = false;
    double check_res = 1.0;
    int check_it = 0;
    while (it < inner_max) {
      const int nstep = std::min(batch, inner_max - it);
      for (int s = 0; s < nstep; ++s) {
        GD_TRY(mixed_apply(A, p, q, pa, st));
        k_mx_scalars<<<1, kMxThreads, 0, st>>>(1, gb, pa, nullptr, nullptr, sc);
        k_mx_update<<<gb, kMxThreads, 0, st>>>(n, sc, x, r, z, p, q, dinv, ext, pa, pb);
        if (ext) {
          k_mx_copy<<<gb, kMxThreads, 0, st>>>(n, z, zold);
          GD_TRY(precond->apply(precond->ctx, A, r, z, st));
          k_mx_dots_flex<<<gb, kMxThreads, 0, st>>>(n, r, z, zold, pa, pc);
          k_mx_scalars<<<1, kMxThreads, 0, st>>>(3, gb, pa, pb, pc, sc);
        } else {
          k_mx_scalars<<<1, kMxThreads, 0, st>>>(2, gb, pa, pb, nullptr, sc);
        }
        k_mx_pupdate<<<gb, kMxThreads, 0, st>>>(n, sc, z, p);
      }
      GD_CUDA_TRY(cudaGetLastError());
      it += nstep;
      GD_CUDA_TRY(cudaMemcpyAsync(&h, sc, sizeof(h), cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
      if (!std::isfinite(h.rr)) {
        inner_stall = ext;
        break;
      }
      if (std::sqrt(h.rr) <= tol_in) break;
      if (ext && it - check_it >= 64) {
        if (std::sqrt(h.rr) > 0.5 * check_res) {
          inner_stall = true;
          break;
        }
        check_res = std::sqrt(h.rr);
        check_it = it;
      }
    }
    total_inner += it;
    if (inner_stall) {
      status = fail(GD_ERR_STALL, "mixed solve: preconditioned inner iteration stagnated");
      break;
    }
    k_mx_accumulate<<<gb, kMxThreads, 0, st>>>(n, rnorm, x, x64);
    GD_CUDA_TRY(cudaGetLastError());
  }
  GD_CUDA_TRY(cudaMemcpyAsync(x_out, x64, sizeof(double) * n,
                              where == GD_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (stats) {
    stats->iterations = total_inner;
    stats->converged = rel <= rtol;
    stats->rel_residual = rel;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  M.last_outer = outer;
  return status;
}

}  // namespace gd
