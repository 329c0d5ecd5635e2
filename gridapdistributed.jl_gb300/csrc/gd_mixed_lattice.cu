// Lattice-order inner iteration of the mixed-precision solve (3D Q1 on cube cells).
//
// The FP32 inner CG keeps its vectors on the structured node lattice (x fastest; a
// Dirichlet node holds 0 in every vector) instead of in gid order, so the operator is
// a pure 21-point stencil with no node -> gid indirection: a node reads the 8
// prescaled coefficients w = K2*kappa of its cells and the search direction at its 21
// non-edge neighbours (edge neighbours of a cube Q1 stiffness are exactly zero).
// One Jacobi-CG iteration is two kernels:
//   k_lat_apply : p <- z + beta p (fused, ping-pong buffers), q = A p, alpha = rz / p.q
//   k_lat_update: x += alpha p, r -= alpha q, z = D^-1 r, beta = r.z_new / r.z_old
// The FP64 scalars are formed by whichever block finishes last (fixed-order sum of the
// per-block partials, so the result does not depend on the block schedule), which
// removes the single-block reduction kernels.  The outer FP64 refinement (residual with
// the assembled matrix, x64 += |r| d) is the same as for the gid-order path; gid <-> lattice
// conversions happen once per outer step.
#include <chrono>
#include <cmath>
#include <algorithm>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_solve_mixed.h"

namespace gd {

constexpr int kLatThreads = 256;
constexpr int kLatMaxBlocks = 152 * 16;
constexpr int kLatUnroll = 4;   // independent elements per thread per step

struct LatScalars {
  double rz, rr, pq, alpha, beta;
};

// device scratch of the lattice solve
struct LatRed {
  double part[3][kLatMaxBlocks];
  unsigned counter;
  unsigned pad;
  LatScalars sc;
};

struct LatGeom {
  int N[3];    // nodes per direction
  int n[3];    // cells per direction
  int ds[6];   // Dirichlet sides (x-, x+, y-, y+, z-, z+)
};

static LatGeom lat_geom(const Geom& g) {
  LatGeom L{};
  for (int d = 0; d < 3; ++d) {
    L.N[d] = (int)g.N[d];
    L.n[d] = (int)g.n[d];
    L.ds[2 * d] = g.dsides[2 * d];
    L.ds[2 * d + 1] = g.dsides[2 * d + 1];
  }
  return L;
}

__device__ inline double lat_block_sum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;   // valid in thread 0
}

// Sum over the block of FP32 thread partials: FP32 within a warp (5 shuffles), FP64
// across the warps.  GB300 issues FP64 adds ~60x slower than FP32 ones, so a block-wide
// FP64 shuffle tree would cost more than the vector update it closes.
__device__ inline double lat_block_sum_f(float v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) sh[wid] = (double)v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;   // valid in thread 0
}

// Block partials of NV sums (FP32 thread partials); returns true in the block that
// finished last, whose thread 0 then holds the FP64 totals in v (summed over the block
// partials in block order).
template <int NV>
__device__ bool lat_reduce(double (&v)[NV], const float (&f)[NV], LatRed* R) {
  __shared__ double sh[kLatThreads / 32];
  __shared__ int last;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    const double t = lat_block_sum_f(f[k], sh);
    if (threadIdx.x == 0) R->part[k][blockIdx.x] = t;
  }
  if (threadIdx.x == 0) {
    __threadfence();
    last = atomicAdd(&R->counter, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    // independent loads in flight (the grid is at most a few blocks per SM)
    double t[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int i = threadIdx.x + u * blockDim.x;
      t[u] = i < (int)gridDim.x ? __ldcg(&R->part[k][i]) : 0.0;
    }
    double a = (t[0] + t[1]) + (t[2] + t[3]);
    for (int i = threadIdx.x + 4 * blockDim.x; i < (int)gridDim.x; i += blockDim.x) a += __ldcg(&R->part[k][i]);
    v[k] = lat_block_sum(a, sh);
  }
  if (threadIdx.x == 0) R->counter = 0;
  return true;
}

__device__ inline bool lat_dirichlet(const LatGeom& g, int x, int y, int z) {
  return (g.ds[0] && x == 0) || (g.ds[1] && x == g.N[0] - 1) || (g.ds[2] && y == 0) || (g.ds[3] && y == g.N[1] - 1) ||
         (g.ds[4] && z == 0) || (g.ds[5] && z == g.N[2] - 1);
}

// r = r64[gid] * inv, x = 0, p = 0 (z = D^-1 r for Jacobi); sums r.z, r.r; beta = 0
__global__ void __launch_bounds__(kLatThreads)
k_lat_start(int nlat, const int32_t* __restrict__ node_gid, const double* __restrict__ r64, double inv,
            const float* __restrict__ dinvl, float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
            float* __restrict__ p, int jacobi, LatRed* R) {
  float a = 0.f, b = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    const float ri = g >= 0 ? (float)(r64[g] * inv) : 0.f;
    r[i] = ri;
    x[i] = 0.f;
    p[i] = 0.f;
    if (jacobi) {
      const float zi = dinvl[i] * ri;
      z[i] = zi;
      a = fmaf(ri, zi, a);
    }
    b = fmaf(ri, ri, b);
  }
  double v[2];
  const float f[2] = {a, b};
  if (lat_reduce<2>(v, f, R) && threadIdx.x == 0) {
    if (jacobi) R->sc.rz = v[0];
    R->sc.rr = v[1];
    R->sc.beta = 0.0;
  }
}

// pn = z + beta p_old (written to p_new), q = A pn, alpha = rz / pn.q.
// A thread takes 4 consecutive nodes of one lattice row (groups never wrap a row).  Each
// of the 9 neighbour rows is read once (6 values shared by the 4 nodes and their three
// x-offsets) and the 5x2x2 cell coefficients around the group once.  Every thread runs
// the same code: loads outside the lattice are predicated off and read as 0, which is
// exact, since a neighbour outside the lattice shares only outside cells (w = 0) with the
// node.  Dirichlet nodes get q = 0.  (Measured against a per-node variant with bounds
// checks, which diverged in nearly every warp, and against 2.5D shared-memory blocking,
// whose plane staging cost more instructions than it saved.)
__global__ void __launch_bounds__(kLatThreads, 4)
k_lat_apply(LatGeom lg, int nlat, const float* __restrict__ wf, float ratio, const float* __restrict__ z,
            const float* __restrict__ p_old, float* __restrict__ p_new, float* __restrict__ q, LatRed* R) {
  const float beta = (float)R->sc.beta;
  const int N0 = lg.N[0], N1 = lg.N[1], N2 = lg.N[2];
  const int n0 = lg.n[0], n1 = lg.n[1], n2 = lg.n[2];
  const int G = (N0 + 3) >> 2;   // groups per row
  const int ngroups = G * N1 * N2;
  (void)nlat;
  float dot = 0.f;
  for (int gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngroups; gi += gridDim.x * blockDim.x) {
    const int row = gi / G;
    const int X0 = 4 * (gi - row * G), X1 = row % N1, X2 = row / N1;
    const int i0 = X0 + N0 * row;
    bool xin[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) xin[k] = (unsigned)(X0 - 1 + k) < (unsigned)N0;
    bool cxin[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) cxin[k] = (unsigned)(X0 - 1 + k) < (unsigned)n0;
    // w[cz][cy][k]: cell (X0 - 1 + k, X1 - 1 + cy, X2 - 1 + cz), 0 outside
    float w[2][2][5];
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
      for (int cy = 0; cy < 2; ++cy) {
        const int Cy = X1 - 1 + cy, Cz = X2 - 1 + cz;
        const bool rin = (unsigned)Cy < (unsigned)n1 && (unsigned)Cz < (unsigned)n2;
        const float* wr = wf + (X0 - 1) + (ptrdiff_t)n0 * (Cy + (ptrdiff_t)n1 * Cz);
#pragma unroll
        for (int k = 0; k < 5; ++k) w[cz][cy][k] = rin && cxin[k] ? __ldg(wr + k) : 0.f;
      }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    float own[4];
#pragma unroll
    for (int o2 = -1; o2 <= 1; ++o2)
#pragma unroll
      for (int o1 = -1; o1 <= 1; ++o1) {
        const int nyz = (o1 != 0) + (o2 != 0);
        const bool rin = (unsigned)(X1 + o1) < (unsigned)N1 && (unsigned)(X2 + o2) < (unsigned)N2;
        const ptrdiff_t base = (ptrdiff_t)i0 - 1 + (ptrdiff_t)N0 * (o1 + (ptrdiff_t)N1 * o2);   // x = X0 - 1
        float v[6];
#pragma unroll
        for (int k = 0; k < 6; ++k) {
          const bool need = nyz != 0 || (k >= 1 && k <= 4);   // the centre row needs the own nodes only
          v[k] = need && rin && xin[k] ? fmaf(beta, __ldg(p_old + base + k), __ldg(z + base + k)) : 0.f;
        }
        const int a1 = (o1 + 1) >> 1, a2 = (o2 + 1) >> 1;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          if (nyz == 0) {
            own[j] = v[j + 1];
            float sw = 0.f;
#pragma unroll
            for (int cz = 0; cz < 2; ++cz)
#pragma unroll
              for (int cy = 0; cy < 2; ++cy) sw += w[cz][cy][j] + w[cz][cy][j + 1];
            acc[j] = fmaf(ratio * sw, v[j + 1], acc[j]);
            continue;
          }
#pragma unroll
          for (int o0 = -1; o0 <= 1; ++o0) {
            const int nz = nyz + (o0 != 0);
            if (nz <= 1) continue;   // edge neighbours are zero on cube cells
            const int a0 = (o0 + 1) >> 1;
            float c;
            if (nz == 3) c = w[a2][a1][j + a0];
            else if (o2 == 0) c = w[0][a1][j + a0] + w[1][a1][j + a0];
            else if (o1 == 0) c = w[a2][0][j + a0] + w[a2][1][j + a0];
            else c = w[a2][a1][j] + w[a2][a1][j + 1];
            acc[j] = fmaf(c, v[j + 1 + o0], acc[j]);
          }
        }
      }
    const bool ydir = (lg.ds[2] && X1 == 0) || (lg.ds[3] && X1 == N1 - 1) || (lg.ds[4] && X2 == 0) ||
                      (lg.ds[5] && X2 == N2 - 1);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int X = X0 + j;
      if (X >= N0) break;
      const bool dir = ydir || (lg.ds[0] && X == 0) || (lg.ds[1] && X == N0 - 1);
      const float qv = dir ? 0.f : acc[j];
      p_new[i0 + j] = own[j];
      q[i0 + j] = qv;
      dot = fmaf(own[j], qv, dot);
    }
  }
  double v[1];
  const float f[1] = {dot};
  if (lat_reduce<1>(v, f, R) && threadIdx.x == 0) {
    R->sc.pq = v[0];
    R->sc.alpha = v[0] != 0.0 ? R->sc.rz / v[0] : 0.0;
  }
}

// x += alpha p, r -= alpha q; Jacobi: z = D^-1 r, beta = r.z / rz_old; sums r.z, r.r
__global__ void __launch_bounds__(kLatThreads)
k_lat_update(int nlat, float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
             const float* __restrict__ p, const float* __restrict__ q, const float* __restrict__ dinvl, int jacobi,
             LatRed* R) {
  const float alpha = (float)R->sc.alpha;
  float a = 0.f, b = 0.f;
  const int stride = gridDim.x * blockDim.x;
  for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < nlat; i0 += kLatUnroll * stride) {
    float xv[kLatUnroll], pv[kLatUnroll], qv[kLatUnroll], rv[kLatUnroll], dv[kLatUnroll];
#pragma unroll
    for (int u = 0; u < kLatUnroll; ++u) {
      const int i = i0 + u * stride;
      const bool ok = i < nlat;
      xv[u] = ok ? x[i] : 0.f;
      pv[u] = ok ? p[i] : 0.f;
      qv[u] = ok ? q[i] : 0.f;
      rv[u] = ok ? r[i] : 0.f;
      dv[u] = ok && jacobi ? dinvl[i] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kLatUnroll; ++u) {
      const int i = i0 + u * stride;
      if (i >= nlat) break;
      x[i] = fmaf(alpha, pv[u], xv[u]);
      const float ri = fmaf(-alpha, qv[u], rv[u]);
      r[i] = ri;
      if (jacobi) {
        const float zi = dv[u] * ri;
        z[i] = zi;
        a = fmaf(ri, zi, a);
      }
      b = fmaf(ri, ri, b);
    }
  }
  double v[2];
  const float f[2] = {a, b};
  if (lat_reduce<2>(v, f, R) && threadIdx.x == 0) {
    if (jacobi) {
      R->sc.beta = R->sc.rz != 0.0 ? v[0] / R->sc.rz : 0.0;
      R->sc.rz = v[0];
    }
    R->sc.rr = v[1];
  }
}

// flexible CG after the preconditioner wrote z: rz = r.z; beta = (r.z - r.z_old) / rz_old
__global__ void __launch_bounds__(kLatThreads)
k_lat_dots(int nlat, const float* __restrict__ r, const float* __restrict__ z, const float* __restrict__ zold,
           LatRed* R) {
  float a = 0.f, c = 0.f;
  const int stride = gridDim.x * blockDim.x;
  for (int i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < nlat; i0 += kLatUnroll * stride) {
    float rv[kLatUnroll], zv[kLatUnroll], ov[kLatUnroll];
#pragma unroll
    for (int u = 0; u < kLatUnroll; ++u) {
      const int i = i0 + u * stride;
      const bool ok = i < nlat;
      rv[u] = ok ? r[i] : 0.f;
      zv[u] = ok ? z[i] : 0.f;
      ov[u] = ok && zold ? zold[i] : 0.f;
    }
#pragma unroll
    for (int u = 0; u < kLatUnroll; ++u) {
      a = fmaf(rv[u], zv[u], a);
      c = fmaf(rv[u], ov[u], c);
    }
  }
  double v[2];
  const float f[2] = {a, c};
  if (lat_reduce<2>(v, f, R) && threadIdx.x == 0) {
    R->sc.beta = zold && R->sc.rz != 0.0 ? (v[0] - v[1]) / R->sc.rz : 0.0;
    R->sc.rz = v[0];
  }
}

// x64[gid] += s * x (free nodes)
__global__ void k_lat_accumulate(int nlat, const int32_t* __restrict__ node_gid, double s, const float* __restrict__ x,
                                 double* __restrict__ x64) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    if (g >= 0) x64[g] += s * (double)x[i];
  }
}

// lattice copy of a gid-order vector (0 on Dirichlet nodes)
__global__ void k_lat_from_gid(int nlat, const int32_t* __restrict__ node_gid, const float* __restrict__ v,
                               float* __restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    out[i] = g >= 0 ? v[g] : 0.f;
  }
}

// fixed-order host sums of two arrays of nb block partials
static int sum_partials_host(const double* pa, const double* pb, int nb, double out[2], cudaStream_t st) {
  std::vector<double> h(2 * (size_t)nb);
  GD_CUDA_TRY(cudaMemcpyAsync(h.data(), pa, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(h.data() + nb, pb, sizeof(double) * nb, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  out[0] = out[1] = 0.0;
  for (int i = 0; i < nb; ++i) {
    out[0] += h[i];
    out[1] += h[nb + i];
  }
  return GD_OK;
}

// a few resident blocks per SM: the partial count (and the last block's final sum)
// stays small, and each thread streams several elements
static int lat_grid(int64_t n) {
  static int cap[64] = {0};
  int dev = 0;
  int c = 152 * 4;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    if (!cap[dev]) {
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cap[dev] = sms > 0 ? std::min(4 * sms, kLatMaxBlocks) : 152 * 4;
    }
    c = cap[dev];
  }
  int64_t b = (n + kLatThreads - 1) / kLatThreads;
  if (b > c) b = c;
  return (int)(b < 1 ? 1 : b);
}

int lattice_setup(gd_asm* A) {
  MixedState& M = A->mx;
  const Geom& g = A->test->geom;
  const int64_t nlat = g.N[0] * g.N[1] * g.N[2];
  cudaStream_t st = A->test->model->ctx->stream;
  if (M.lat.n != (size_t)(kLatVectors * nlat)) GD_TRY(dalloc(M.lat, kLatVectors * nlat));
  if (!M.latred.p) {
    GD_TRY(dalloc(M.latred, (sizeof(LatRed) + sizeof(double) - 1) / sizeof(double)));
    GD_CUDA_TRY(cudaMemsetAsync(M.latred.p, 0, sizeof(LatRed), st));
  }
  const float* dinv = M.f32.p + 5 * A->ngdofs;
  float* dinvl = M.lat.p + 7 * nlat;
  k_lat_from_gid<<<lat_grid(nlat), kLatThreads, 0, st>>>((int)nlat, M.node_gid.p, dinv, dinvl);
  GD_CUDA_TRY(cudaGetLastError());
  M.lat_epoch = M.numeric_epoch;
  return GD_OK;
}

const float* lattice_dinv(const gd_asm* A) {
  const Geom& g = A->test->geom;
  return A->mx.lat.p + 7 * (g.N[0] * g.N[1] * g.N[2]);
}

// Mixed-precision refinement with the lattice-order inner CG (Jacobi, or flexible CG
// around `precond->apply_lattice`).
int mixed_solve_lattice(gd_asm* A, double rtol, int maxit, double* x_out, int where, gd_solve_stats* stats,
                        const MixedPrecond* precond) {
  GD_TRY(mixed_setup(A));
  MixedState& M = A->mx;
  if (M.lat_epoch != M.numeric_epoch || !M.lat.p) GD_TRY(lattice_setup(A));
  cudaStream_t st = A->test->model->ctx->stream;
  const int64_t n = A->ngdofs;
  const Geom& g = A->test->geom;
  const int64_t nl64 = g.N[0] * g.N[1] * g.N[2];
  if (nl64 >= (int64_t)1 << 31) return fail(GD_ERR_UNSUPPORTED, "mixed solve: node lattice exceeds 2^31 nodes");
  const int nlat = (int)nl64;
  const LatGeom lg = lat_geom(g);
  auto t0 = std::chrono::steady_clock::now();
  float* x = M.lat.p;
  float* r = x + nl64;
  float* zb[2] = {r + nl64, r + 2 * nl64};
  float* pb[2] = {r + 3 * nl64, r + 4 * nl64};
  float* q = r + 5 * nl64;
  float* dinvl = r + 6 * nl64;
  LatRed* R = reinterpret_cast<LatRed*>(M.latred.p);
  double* x64 = M.f64.p;
  double* r64 = x64 + n;
  double* pa = M.red.p;
  double* pbb = pa + 1024;
  const int gb = lat_grid(nl64);
  const int ext = precond != nullptr;
  GD_CUDA_TRY(cudaMemsetAsync(x64, 0, sizeof(double) * n, st));
  GD_CUDA_TRY(cudaMemsetAsync(&R->counter, 0, sizeof(unsigned), st));
  int total_inner = 0, outer = 0;
  double bnorm = 0.0, rel = 1.0, prev_rel = 1e300;
  const double inner_tol = 1e-5;
  int status = GD_OK;
  while (true) {
    int gr = 0;
    GD_TRY(residual_fp64(n, A->rowptr.p, A->colgid.p, A->vals.p, x64, A->rhs_override ? A->rhs_override : A->rhs.p,
                         r64, pa, pbb, st, &gr));
    double h2[2];
    GD_TRY(sum_partials_host(pa, pbb, gr, h2, st));
    const double rnorm = std::sqrt(h2[0]);
    if (outer == 0) bnorm = std::sqrt(h2[1]);
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
    if (outer > 0 && rel > 0.5 * prev_rel) {
      status = fail(GD_ERR_STALL, "mixed solve: refinement stalled at relative residual " + std::to_string(rel));
      break;
    }
    prev_rel = rel;
    ++outer;
    int zc = 0, pc = 0;   // current z and p buffers
    k_lat_start<<<gb, kLatThreads, 0, st>>>(nlat, M.node_gid.p, r64, 1.0 / rnorm, dinvl, x, r, zb[zc], pb[pc], !ext, R);
    GD_CUDA_TRY(cudaGetLastError());
    if (ext) {
      GD_TRY(precond->apply_lattice(precond->ctx, A, r, zb[zc], st));
      k_lat_dots<<<gb, kLatThreads, 0, st>>>(nlat, r, zb[zc], nullptr, R);
      GD_CUDA_TRY(cudaGetLastError());
    }
    const double tol_in = std::max(inner_tol, 0.5 * rtol / rel);
    int it = 0;
    const int batch = 16;
    const int inner_max = maxit - total_inner;
    bool inner_stall = false;
    double check_res = 1.0;
    int check_it = 0;
    LatScalars h{};
    while (it < inner_max) {
      const int nstep = std::min(batch, inner_max - it);
      for (int s = 0; s < nstep; ++s) {
        k_lat_apply<<<gb, kLatThreads, 0, st>>>(lg, nlat, M.wf.p, M.ratio, zb[zc], pb[pc], pb[pc ^ 1], q, R);
        pc ^= 1;
        if (ext) {
          k_lat_update<<<gb, kLatThreads, 0, st>>>(nlat, x, r, nullptr, pb[pc], q, dinvl, 0, R);
          GD_TRY(precond->apply_lattice(precond->ctx, A, r, zb[zc ^ 1], st));
          k_lat_dots<<<gb, kLatThreads, 0, st>>>(nlat, r, zb[zc ^ 1], zb[zc], R);
          zc ^= 1;
        } else {
          k_lat_update<<<gb, kLatThreads, 0, st>>>(nlat, x, r, zb[zc], pb[pc], q, dinvl, 1, R);
        }
      }
      GD_CUDA_TRY(cudaGetLastError());
      it += nstep;
      GD_CUDA_TRY(cudaMemcpyAsync(&h, &R->sc, sizeof(h), cudaMemcpyDeviceToHost, st));
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
    k_lat_accumulate<<<gb, kLatThreads, 0, st>>>(nlat, M.node_gid.p, rnorm, x, x64);
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
