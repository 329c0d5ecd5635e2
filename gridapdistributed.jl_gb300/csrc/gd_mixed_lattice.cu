// Lattice-order inner iteration of the mixed-precision solve (3D Q1 on cube cells).
//
// The FP32 inner CG keeps its vectors on the structured node lattice (x fastest; a
// Dirichlet node holds 0 in every vector) instead of in gid order, so the operator is
// a pure 21-point stencil with no node -> gid indirection: a node reads the 8
// prescaled coefficients w = K2*kappa of its cells and the search direction at its 21
// non-edge neighbours (edge neighbours of a cube Q1 stiffness are exactly zero).
// One Jacobi-CG iteration is two phases:
//   apply : p <- z + beta p (ping-pong buffers), q <- A z + beta q (= A p), alpha = rz / p.q
//   update: x += alpha p, r -= alpha q, z = D^-1 r, beta = r.z_new / r.z_old
// The Jacobi solve runs all iterations in one cooperative launch (k_pad_cg, grid
// barriers between the phases); the flexible CG around an external preconditioner runs
// them as kernels (k_lat_apply, k_lat_update, k_lat_dots), whose FP64 scalars are formed
// by whichever block finishes last (fixed-order sum of the per-block partials, so the
// result does not depend on the block schedule).  The outer FP64 refinement (residual with
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

// grid barrier state and results of the persistent inner CG (reset before every launch)
struct alignas(128) LatSync {
  unsigned count;                  // blocks arrived at the current barrier (own 128-byte line)
  unsigned pad[31];
  unsigned long long totw[3];      // published totals, tagged with the barrier number
  int err;                         // a barrier wait ran out
  int it;                          // CG steps taken
};

// device scratch of the lattice solve
struct LatRed {
  double part[3][kLatMaxBlocks];
  unsigned counter;
  unsigned pad;
  LatScalars sc;
  LatSync sync;
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

// r = r64[gid] * inv, x = p = q = 0 (z = D^-1 r for Jacobi); sums r.z, r.r; beta = 0
__global__ void __launch_bounds__(kLatThreads)
k_lat_start(int nlat, const int32_t* __restrict__ node_gid, const double* __restrict__ r64, double inv,
            const float* __restrict__ dinvl, float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
            float* __restrict__ p, float* __restrict__ q, int jacobi, LatRed* R) {
  float a = 0.f, b = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    const float ri = g >= 0 ? (float)(r64[g] * inv) : 0.f;
    r[i] = ri;
    x[i] = 0.f;
    p[i] = 0.f;
    q[i] = 0.f;
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

// pn = z + beta p_old (written to p_new), q <- A z + beta q (= A pn, since q held A p_old),
// alpha = rz / pn.q; only z is read at the neighbours, p and q at the node itself.
// A thread takes 4 consecutive nodes of one lattice row (groups never wrap a row).  Each
// of the 9 neighbour rows is read once (6 values shared by the 4 nodes and their three
// x-offsets) and the 5x2x2 cell coefficients around the group once.  Every thread runs
// the same code: loads outside the lattice are predicated off and read as 0, which is
// exact, since a neighbour outside the lattice shares only outside cells (w = 0) with the
// node.  Dirichlet nodes get A z = 0 (q stays 0 there).  (Measured against a per-node
// variant with bounds checks, which diverged in nearly every warp, and against 2.5D
// shared-memory blocking, whose plane staging cost more instructions than it saved.)
//
// Body of k_lat_apply over the groups gi = g0, g0 + gs, ...; returns the thread's p.q partial.
__device__ __forceinline__ float lat_apply_groups(const LatGeom& lg, const float* __restrict__ wf, float ratio,
                                                  float beta, const float* __restrict__ z,
                                                  const float* __restrict__ p_old, float* __restrict__ p_new,
                                                  float* __restrict__ q, int g0, int gs) {
  const int N0 = lg.N[0], N1 = lg.N[1], N2 = lg.N[2];
  const int n0 = lg.n[0], n1 = lg.n[1], n2 = lg.n[2];
  const int G = (N0 + 3) >> 2;   // groups per row
  const int ngroups = G * N1 * N2;
  float dot = 0.f;
  for (int gi = g0; gi < ngroups; gi += gs) {
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
          v[k] = need && rin && xin[k] ? __ldg(z + base + k) : 0.f;
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
      const float qv = fmaf(beta, q[i0 + j], dir ? 0.f : acc[j]);
      const float pv = fmaf(beta, p_old[i0 + j], own[j]);
      p_new[i0 + j] = pv;
      q[i0 + j] = qv;
      dot = fmaf(pv, qv, dot);
    }
  }
  return dot;
}

__global__ void __launch_bounds__(kLatThreads, 4)
k_lat_apply(LatGeom lg, int nlat, const float* __restrict__ wf, float ratio, const float* __restrict__ z,
            const float* __restrict__ p_old, float* __restrict__ p_new, float* __restrict__ q, LatRed* R) {
  (void)nlat;
  const float dot = lat_apply_groups(lg, wf, ratio, (float)R->sc.beta, z, p_old, p_new, q,
                                           blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
  double v[1];
  const float f[1] = {dot};
  if (lat_reduce<1>(v, f, R) && threadIdx.x == 0) {
    R->sc.pq = v[0];
    R->sc.alpha = v[0] != 0.0 ? R->sc.rz / v[0] : 0.0;
  }
}

// x += alpha p, r -= alpha q; Jacobi: z = D^-1 r, beta = r.z / rz_old; sums r.z, r.r
__device__ __forceinline__ void lat_update_elems(int nlat, float alpha, float* __restrict__ x, float* __restrict__ r,
                                                 float* __restrict__ z, const float* __restrict__ p,
                                                 const float* __restrict__ q, const float* __restrict__ dinvl,
                                                 int jacobi, int t0, int stride, float& a, float& b) {
  for (int i0 = t0; i0 < nlat; i0 += kLatUnroll * stride) {
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
}

__global__ void __launch_bounds__(kLatThreads)
k_lat_update(int nlat, float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
             const float* __restrict__ p, const float* __restrict__ q, const float* __restrict__ dinvl, int jacobi,
             LatRed* R) {
  float a = 0.f, b = 0.f;
  lat_update_elems(nlat, (float)R->sc.alpha, x, r, z, p, q, dinvl, jacobi, blockIdx.x * blockDim.x + threadIdx.x,
                   gridDim.x * blockDim.x, a, b);
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

// ---- persistent Jacobi-CG ------------------------------------------------------------
//
// The whole inner Jacobi-CG of one outer step in one cooperative launch: every CG step
// runs the apply body and the update body of the kernels above, separated by grid
// barriers, so a step costs two barriers instead of two launches with their tails.
// Every block re-sums the block partials in the same fixed order (FP64), so all blocks
// hold bit-identical alpha, beta and r.r and take the same convergence decision.
// The barrier's wait is bounded by wall time: a block that waits past the limit sets the
// error flag, every other block sees it in its own wait, and all blocks return; the host
// reports GD_ERR_TIMEOUT.  (A cooperative launch keeps every block resident, so the
// limit is only ever reached if the launch was not co-resident.)

constexpr unsigned long long kLatSyncTimeoutNs = 2000000000ull;   // 2 s per barrier
// k_pad_cg: one block of 768 threads per SM (80 registers per thread): 152 arrivals per
// grid barrier instead of 456 with 3 blocks of 256, the same 24 warps per SM
constexpr int kPadThreads = 768;
constexpr int kPadBlocksPerSM = 1;

__device__ __forceinline__ unsigned long long lat_globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Memory-order primitives at GPU scope (PTX ISA memory consistency model): an acq_rel
// arrival, release stores and acquire loads replace full fences around the grid barrier.
__device__ __forceinline__ unsigned atom_add_acq_rel_gpu(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}
__device__ __forceinline__ void st_release_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_acquire_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu(unsigned long long* p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// A published total: the FP32 value in the low word and the barrier number in the high
// word of one 64-bit store, so a waiter reads the total and learns that it is current in
// one single-copy-atomic load.
__device__ __forceinline__ unsigned long long lat_tag(float v, unsigned epoch) {
  return ((unsigned long long)epoch << 32) | (unsigned long long)__float_as_uint(v);
}
__device__ __forceinline__ float lat_untag(unsigned long long w) { return __uint_as_float((unsigned)(w & 0xffffffffull)); }
__device__ __forceinline__ bool lat_tag_is(unsigned long long w, unsigned epoch) { return (unsigned)(w >> 32) == epoch; }

// Grid barrier fused with an all-reduce of NV sums of FP32 thread partials f, published
// in the total words W .. W+NV-1.  FP32 throughout, in a fixed order: the warp tree, the
// block's warps in order (thread 0), then in the last block to arrive warp 0 over the
// block partials (lane l takes l, l + 32, ... in order; then the xor tree; lane 0's
// result).  So the totals do not depend on the arrival order, and no FP64 instruction
// (a slow pipe on this part) sits on the barrier's critical path; the thread partials
// are FP32 sums already.  Thread 0 stores the block partials and arrives on the count
// with an acq_rel add (releasing the block's writes, which the block barrier before it
// orders, and acquiring the earlier arrivals').  Lane 0 of the last block resets the
// count and publishes each total with the barrier number `epoch` (counted by every block;
// the words start at 0): relaxed stores, the last one a release.  The others poll their
// total words (the last with an acquire load) until all carry `epoch`; the block barrier
// after the wait orders the rest of the block behind it.  Every thread returns the
// totals.  The wait is bounded by wall time: past the limit a block sets the error flag,
// blocks still waiting see it (checked every 256 polls), and all return false.
template <int NV, int W>
__device__ bool lat_allreduce(LatRed* R, const float (&f)[NV], unsigned nb, unsigned epoch, float (&out)[NV],
                              unsigned long long timeout_ns = kLatSyncTimeoutNs) {
  __shared__ float wsum[NV][32];   // up to 32 warps per block
  __shared__ int last_s, ok_s;
  __shared__ unsigned long long w_s[NV];
  LatSync* S = &R->sync;
  float* part = reinterpret_cast<float*>(R->part[0]);   // NV arrays of kLatMaxBlocks floats
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  float v[NV];
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    v[j] = f[j];
    for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_down_sync(0xffffffffu, v[j], o);
  }
  if (lane == 0)
#pragma unroll
    for (int j = 0; j < NV; ++j) wsum[j][wid] = v[j];
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      float t = 0.f;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += wsum[j][w];
      part[j * kLatMaxBlocks + blockIdx.x] = t;
    }
    last_s = atom_add_acq_rel_gpu(&S->count, 1u) == nb - 1;
  }
  __syncthreads();
  if (last_s) {
    if (wid == 0) {
      float a[NV];
#pragma unroll
      for (int j = 0; j < NV; ++j) a[j] = 0.f;
      for (int i0 = lane; i0 < (int)nb; i0 += 32 * 8) {   // 8 independent loads per lane in flight
        float t[NV][8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int i = i0 + 32 * u;
#pragma unroll
          for (int j = 0; j < NV; ++j) t[j][u] = i < (int)nb ? __ldcg(part + j * kLatMaxBlocks + i) : 0.f;
        }
#pragma unroll
        for (int j = 0; j < NV; ++j)
#pragma unroll
          for (int u = 0; u < 8; ++u) a[j] += t[j][u];
      }
#pragma unroll
      for (int j = 0; j < NV; ++j)
        for (int o = 16; o > 0; o >>= 1) a[j] += __shfl_xor_sync(0xffffffffu, a[j], o);
      if (lane == 0) {
        S->count = 0u;
#pragma unroll
        for (int j = 0; j < NV; ++j) {
          const unsigned long long w = lat_tag(a[j], epoch);
          if (j < NV - 1) st_relaxed_gpu(&S->totw[W + j], w);
          else st_release_gpu(&S->totw[W + j], w);
          w_s[j] = w;
        }
      }
    }
  } else if (threadIdx.x == 0) {
    volatile int* verr = &S->err;
    int ok = 1;
    unsigned long long w[NV];
    auto current = [&]() {
#pragma unroll
      for (int j = 0; j < NV - 1; ++j) w[j] = ld_relaxed_gpu(&S->totw[W + j]);
      w[NV - 1] = ld_acquire_gpu(&S->totw[W + NV - 1]);
      bool c = true;
#pragma unroll
      for (int j = 0; j < NV; ++j) c = c && lat_tag_is(w[j], epoch);
      return c;
    };
    if (!current()) {
      const unsigned long long t0 = lat_globaltimer();
      unsigned ns = 32, polls = 0;
      while (!current()) {
        if ((++polls & 255u) == 0) {
          if (*verr) {
            ok = 0;
            break;
          }
          if (lat_globaltimer() - t0 > timeout_ns) {
            atomicExch(&S->err, 1);
            ok = 0;
            break;
          }
        }
        __nanosleep(ns);
        if (ns < 64) ns <<= 1;
      }
    }
#pragma unroll
    for (int j = 0; j < NV; ++j) w_s[j] = w[j];
    ok_s = ok;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) out[j] = lat_untag(w_s[j]);
  return last_s || ok_s != 0;
}

// Padded lattice of the persistent Jacobi-CG.  Node (X, Y, Z) sits at
// ((Z + 1) R1 + Y + 1) P0 + X: the row pitch P0 is N0 rounded up to a multiple of 4, so a
// thread's 4 nodes X0..X0+3 (X0 = 4k) are one aligned float4, and the rows y = -1, N1
// and planes z = -1, N2 are zero ghost rows, so no neighbour load needs a bounds test.
// Cell (c0, c1, c2) coefficients use the same layout (cell rows c1 = -1 and c1 >= n1 are
// zero, as are the columns c0 >= n0).  Entries outside the lattice are 0 in every vector.
struct PadGeom {
  int N[3];   // nodes per direction
  int P0;     // row pitch (floats), a multiple of 4
  int R1;     // storage rows per plane, N1 + 2
  int L;      // floats per padded vector, P0 R1 (N2 + 2)
  int ds[6];  // Dirichlet sides
};

static PadGeom pad_geom(const Geom& g) {
  PadGeom P{};
  for (int d = 0; d < 3; ++d) P.N[d] = (int)g.N[d];
  P.P0 = (P.N[0] + 3) & ~3;
  P.R1 = P.N[1] + 2;
  P.L = (int)((int64_t)P.P0 * P.R1 * (P.N[2] + 2));
  for (int k = 0; k < 6; ++k) P.ds[k] = g.dsides[k];
  return P;
}

static bool pad_fits(const Geom& g) {
  const int64_t L = (((g.N[0] + 3) / 4) * 4) * (g.N[1] + 2) * (g.N[2] + 2);
  return L < ((int64_t)1 << 31) - 64;
}

// padded copies of the lattice D^-1 (nodes) and the cell coefficients; 0 elsewhere
__global__ void k_pad_setup(PadGeom pg, const float* __restrict__ dinvl, const float* __restrict__ wf,
                            float* __restrict__ dpad, float* __restrict__ wpad) {
  const int N0 = pg.N[0], N1 = pg.N[1], N2 = pg.N[2];
  const int n0 = N0 - 1, n1 = N1 - 1, n2 = N2 - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pg.L; i += gridDim.x * blockDim.x) {
    const int X = i % pg.P0, t = i / pg.P0;
    const int Y = t % pg.R1 - 1, Z = t / pg.R1 - 1;
    float d = 0.f, w = 0.f;
    if (X < N0 && Y >= 0 && Y < N1 && Z >= 0 && Z < N2) d = dinvl[X + N0 * (Y + N1 * Z)];
    if (X < n0 && Y >= 0 && Y < n1 && Z >= 0 && Z < n2) w = wf[X + n0 * (Y + n1 * Z)];
    dpad[i] = d;
    wpad[i] = w;
  }
}

// r = r64[gid] * inv, x = p = q = 0, z = D^-1 r on the padded lattice; sums r.z, r.r; beta = 0
__global__ void __launch_bounds__(kLatThreads)
k_pad_start(PadGeom pg, const int32_t* __restrict__ node_gid, const double* __restrict__ r64, double inv,
            const float* __restrict__ dpad, float* __restrict__ x, float* __restrict__ r, float* __restrict__ z,
            float* __restrict__ p, float* __restrict__ q, LatRed* R) {
  const int N0 = pg.N[0], N1 = pg.N[1], N2 = pg.N[2];
  float a = 0.f, b = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < pg.L; i += gridDim.x * blockDim.x) {
    const int X = i % pg.P0, t = i / pg.P0;
    const int Y = t % pg.R1 - 1, Z = t / pg.R1 - 1;
    float ri = 0.f;
    if (X < N0 && Y >= 0 && Y < N1 && Z >= 0 && Z < N2) {
      const int32_t g = node_gid[X + N0 * (Y + N1 * Z)];
      if (g >= 0) ri = (float)(r64[g] * inv);
    }
    const float zi = dpad[i] * ri;
    r[i] = ri;
    z[i] = zi;
    x[i] = 0.f;
    p[i] = 0.f;
    q[i] = 0.f;
    a = fmaf(ri, zi, a);
    b = fmaf(ri, ri, b);
  }
  double v[2];
  const float f[2] = {a, b};
  if (lat_reduce<2>(v, f, R) && threadIdx.x == 0) {
    R->sc.rz = v[0];
    R->sc.rr = v[1];
    R->sc.beta = 0.0;
  }
}

// x64[gid] += s * x (free nodes), x on the padded lattice
__global__ void k_pad_accumulate(PadGeom pg, const int32_t* __restrict__ node_gid, double s,
                                 const float* __restrict__ x, double* __restrict__ x64) {
  const int N0 = pg.N[0], N1 = pg.N[1];
  const int nlat = N0 * N1 * pg.N[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlat; i += gridDim.x * blockDim.x) {
    const int32_t g = node_gid[i];
    if (g < 0) continue;
    const int X = i % N0, t = i / N0;
    const int Y = t % N1, Z = t / N1;
    x64[g] += s * (double)x[((Z + 1) * pg.R1 + Y + 1) * pg.P0 + X];
  }
}

// The apply phase on the padded lattice.  With p_new = z + beta p, A p_new = A z + beta q
// (q = A p from the previous step), so the stencil reads only z at the neighbours and p
// and q are updated in place from the thread's own values:
//   q <- A z + beta q,  p <- z + beta p,  returns the thread's p.q partial
// (the 21-point stencil of k_lat_apply).  The block owns the groups c0 .. c1-1 (group =
// 4 nodes of one row, rows in lattice order); lane l of a warp takes group wb + l, so a
// warp's groups are consecutive and the x-halo values X0 - 1 and X0 + 4 of a row come
// from the neighbouring lanes by shuffle (lanes 0 and 31 load their outer halo
// themselves), and are 0 at the ends of a row.  Per neighbour row that is one float4
// load instead of six scalar loads at a 16-byte lane stride.  Loads of z are plain
// (coherent after a grid barrier); the cell coefficients go through the read-only path.
__device__ __forceinline__ float pad_apply(const PadGeom& pg, const float* __restrict__ wpad, float ratio,
                                           float beta, const float* z, float* p, float* q, int c0, int c1) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int N0 = pg.N[0], N1 = pg.N[1], N2 = pg.N[2], P0 = pg.P0, R1 = pg.R1;
  const int Gp = P0 >> 2;
  float dot = 0.f;
  for (int wb = c0 + (threadIdx.x & ~31); wb < c1; wb += blockDim.x) {   // warp-uniform trip count
    // c0 and chunk ends are multiples of 32 (only the lattice's last chunk ends short), so
    // the lane after the last valid one is lane 31's successor or past the last group of
    // the last row (no right halo): shuffled halos never come from an invalid lane
    const bool valid = wb + lane < c1;
    const int gi = valid ? wb + lane : c1 - 1;
    const int row = gi / Gp;
    const int X0 = 4 * (gi - row * Gp), X1 = row % N1, X2 = row / N1;
    const bool hl = X0 > 0, hr = X0 + 4 < P0;   // the row continues left / right of the group
    const bool fetch = (lane == 0 && hl) || (lane == 31 && hr);
    const int eo = lane == 0 ? -1 : 4;
    const int ob = ((X2 + 1) * R1 + X1 + 1) * P0 + X0;
    const float4 pold = *reinterpret_cast<const float4*>(p + ob);
    const float4 qold = *reinterpret_cast<const float4*>(q + ob);
    // w[cz][cy][k]: cell (X0 - 1 + k, X1 - 1 + cy, X2 - 1 + cz)
    float w[2][2][5];
#pragma unroll
    for (int cz = 0; cz < 2; ++cz)
#pragma unroll
      for (int cy = 0; cy < 2; ++cy) {
        const int cb = ((X2 + cz) * R1 + X1 + cy) * P0 + X0;
        const float4 c4 = __ldg(reinterpret_cast<const float4*>(wpad + cb));
        const float e = lane == 0 && hl ? __ldg(wpad + cb - 1) : 0.f;
        float left = __shfl_up_sync(full, c4.w, 1);
        if (lane == 0) left = e;
        w[cz][cy][0] = hl ? left : 0.f;
        w[cz][cy][1] = c4.x;
        w[cz][cy][2] = c4.y;
        w[cz][cy][3] = c4.z;
        w[cz][cy][4] = c4.w;
      }
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    float own[4];
#pragma unroll
    for (int o2 = -1; o2 <= 1; ++o2)
#pragma unroll
      for (int o1 = -1; o1 <= 1; ++o1) {
        const int nyz = (o1 != 0) + (o2 != 0);
        const int nb = ((X2 + 1 + o2) * R1 + X1 + 1 + o1) * P0 + X0;
        const float4 z4 = *reinterpret_cast<const float4*>(z + nb);
        float v[6];
        v[1] = z4.x;
        v[2] = z4.y;
        v[3] = z4.z;
        v[4] = z4.w;
        v[0] = v[5] = 0.f;
        if (nyz != 0) {   // the centre row needs the own nodes only
          const float ev = fetch ? z[nb + eo] : 0.f;
          float l = __shfl_up_sync(full, v[4], 1);
          float rt = __shfl_down_sync(full, v[1], 1);
          if (lane == 0) l = ev;
          if (lane == 31) rt = ev;
          v[0] = hl ? l : 0.f;
          v[5] = hr ? rt : 0.f;
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
    if (valid) {
      const bool ydir = (pg.ds[2] && X1 == 0) || (pg.ds[3] && X1 == N1 - 1) || (pg.ds[4] && X2 == 0) ||
                        (pg.ds[5] && X2 == N2 - 1);
      const float po[4] = {pold.x, pold.y, pold.z, pold.w}, qo[4] = {qold.x, qold.y, qold.z, qold.w};
      float pv[4], qv[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int X = X0 + j;
        const bool dir = ydir || (pg.ds[0] && X == 0) || (pg.ds[1] && X == N0 - 1);
        // A z is 0 on Dirichlet nodes and past the row end (all coefficients there are 0)
        qv[j] = fmaf(beta, qo[j], dir ? 0.f : acc[j]);
        pv[j] = fmaf(beta, po[j], own[j]);
        dot = fmaf(pv[j], qv[j], dot);
      }
      *reinterpret_cast<float4*>(p + ob) = make_float4(pv[0], pv[1], pv[2], pv[3]);
      *reinterpret_cast<float4*>(q + ob) = make_float4(qv[0], qv[1], qv[2], qv[3]);
    }
  }
  return dot;
}

// The update phase over the block's groups (one float4 each), with the same group ->
// thread map as pad_apply, so a thread updates the p and q it wrote: x += alpha p,
// r -= alpha q, z = D^-1 r; accumulates r.z and r.r.  Ghost rows are never written.
__device__ __forceinline__ void pad_update(const PadGeom& pg, float alpha, float* x, float* r, float* z,
                                           const float* p, const float* q, const float* __restrict__ dpad, int c0,
                                           int c1, float& a, float& b) {
  const int Gp = pg.P0 >> 2, N1 = pg.N[1];
  for (int gi = c0 + threadIdx.x; gi < c1; gi += blockDim.x) {
    const int row = gi / Gp;
    const int X0 = 4 * (gi - row * Gp), X1 = row % N1, X2 = row / N1;
    const int o = ((X2 + 1) * pg.R1 + X1 + 1) * pg.P0 + X0;
    const float4 xv = *reinterpret_cast<const float4*>(x + o);
    const float4 rv = *reinterpret_cast<const float4*>(r + o);
    const float4 pv = *reinterpret_cast<const float4*>(p + o);
    const float4 qv = *reinterpret_cast<const float4*>(q + o);
    const float4 dv = __ldg(reinterpret_cast<const float4*>(dpad + o));
    float4 xo, ro, zo;
    xo.x = fmaf(alpha, pv.x, xv.x);
    xo.y = fmaf(alpha, pv.y, xv.y);
    xo.z = fmaf(alpha, pv.z, xv.z);
    xo.w = fmaf(alpha, pv.w, xv.w);
    ro.x = fmaf(-alpha, qv.x, rv.x);
    ro.y = fmaf(-alpha, qv.y, rv.y);
    ro.z = fmaf(-alpha, qv.z, rv.z);
    ro.w = fmaf(-alpha, qv.w, rv.w);
    zo.x = dv.x * ro.x;
    zo.y = dv.y * ro.y;
    zo.z = dv.z * ro.z;
    zo.w = dv.w * ro.w;
    *reinterpret_cast<float4*>(x + o) = xo;
    *reinterpret_cast<float4*>(r + o) = ro;
    *reinterpret_cast<float4*>(z + o) = zo;
    a = fmaf(ro.x, zo.x, fmaf(ro.y, zo.y, fmaf(ro.z, zo.z, fmaf(ro.w, zo.w, a))));
    b = fmaf(ro.x, ro.x, fmaf(ro.y, ro.y, fmaf(ro.z, ro.z, fmaf(ro.w, ro.w, b))));
  }
}

// Jacobi-CG on the padded lattice from the state k_pad_start left (R->sc: rz, rr,
// beta = 0; p = q = 0) until r.r <= tol2, r.r is not finite, or max_it steps.  Two fused
// barrier/all-reduces per step (p.q; r.z and r.r), so every block holds the same alpha,
// beta and r.r and takes the same exit.  Block 0 writes the step count and the final
// scalars.
__global__ void __launch_bounds__(kPadThreads, kPadBlocksPerSM)
k_pad_cg(PadGeom pg, const float* __restrict__ wpad, float ratio, float* x, float* r, float* z, float* p, float* q,
         const float* __restrict__ dpad, LatRed* R, int max_it, double tol2) {
  const unsigned nb = gridDim.x;
  // equal contiguous chunks of groups, a multiple of 32 each (whole warps)
  const int ngroups = (pg.P0 >> 2) * pg.N[1] * pg.N[2];
  const int chunk = ((ngroups + (int)nb - 1) / (int)nb + 31) & ~31;
  const int c0 = min((int)blockIdx.x * chunk, ngroups), c1 = min(c0 + chunk, ngroups);
  // CG scalars in FP32 (the vectors are FP32; the grid sums are FP32 in a fixed order)
  float rz = (float)R->sc.rz, rr = (float)R->sc.rr, beta = (float)R->sc.beta, alpha = 0.f;
  const float tol2f = (float)tol2;
  int it = 0;
  unsigned epoch = 0;   // grid barriers passed in this launch
  while (it < max_it && rr > tol2f && isfinite(rr)) {
    {
      const float f[1] = {pad_apply(pg, wpad, ratio, beta, z, p, q, c0, c1)};
      float pq[1];
      if (!lat_allreduce<1, 0>(R, f, nb, ++epoch, pq)) break;
      alpha = pq[0] != 0.f ? rz / pq[0] : 0.f;
    }
    float f[2] = {0.f, 0.f};
    pad_update(pg, alpha, x, r, z, p, q, dpad, c0, c1, f[0], f[1]);
    float s2[2];
    if (!lat_allreduce<2, 1>(R, f, nb, ++epoch, s2)) break;
    beta = rz != 0.f ? s2[0] / rz : 0.f;
    rz = s2[0];
    rr = s2[1];
    ++it;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    R->sc.rz = rz;
    R->sc.rr = rr;
    R->sc.alpha = alpha;
    R->sc.beta = beta;
    R->sync.it = it;
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

// Cooperative grid of k_pad_cg: the same number of blocks on every SM (kPadBlocksPerSM,
// resident by the register bound), so that equal chunks mean equal work per SM; fewer for
// small lattices.  0 when the device cannot launch cooperatively.
static int lat_coop_grid(int64_t ngroups) {
  static int cap[64] = {0};   // 0: not yet queried, -1: no cooperative launch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 0;
  if (!cap[dev]) {
    int coop = 0, sms = 0, per = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) coop = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pad_cg, kPadThreads, 0) != cudaSuccess) per = 0;
    cudaGetLastError();
    cap[dev] = coop && sms > 0 && per > 0 ? std::min(std::min(per, kPadBlocksPerSM) * sms, kLatMaxBlocks) : -1;
  }
  if (cap[dev] < 0) return 0;
  int64_t b = (ngroups + kPadThreads - 1) / kPadThreads;
  if (b > cap[dev]) b = cap[dev];
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
  // Jacobi: the persistent kernel on the padded lattice, where the device launches
  // cooperatively and the padded vectors index in 32 bits
  const PadGeom pg = pad_fits(g) ? pad_geom(g) : PadGeom{};
  const int64_t pls = ((int64_t)pg.L + 63) & ~(int64_t)63;   // padded vector stride (256-byte aligned)
  const int gc = ext || !pad_fits(g) ? 0 : lat_coop_grid((int64_t)(pg.P0 / 4) * pg.N[1] * pg.N[2]);
  if (gc > 0 && (M.plat.n != (size_t)(7 * pls) || M.plat_epoch != M.numeric_epoch)) {
    if (M.plat.n != (size_t)(7 * pls)) {
      GD_TRY(dalloc(M.plat, 7 * pls));
      GD_CUDA_TRY(cudaMemsetAsync(M.plat.p, 0, sizeof(float) * 7 * pls, st));
    }
    k_pad_setup<<<lat_grid(pg.L), kLatThreads, 0, st>>>(pg, dinvl, M.wf.p, M.plat.p + 5 * pls, M.plat.p + 6 * pls);
    GD_CUDA_TRY(cudaGetLastError());
    M.plat_epoch = M.numeric_epoch;
  }
  GD_CUDA_TRY(cudaMemsetAsync(x64, 0, sizeof(double) * n, st));
  GD_CUDA_TRY(cudaMemsetAsync(&R->counter, 0, sizeof(unsigned), st));
  int total_inner = 0, outer = 0;
  double bnorm = 0.0, rel = 1.0, prev_rel = 1e300;
  const double inner_tol = 1e-5;
  int status = GD_OK;
  while (true) {
    int gr = 0;
    GD_TRY(residual_fp64_asm(A, x64, A->rhs_override ? A->rhs_override : A->rhs.p, r64, pa, pbb, st, &gr));
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
    const double tol_in = std::max(inner_tol, 0.5 * rtol / rel);
    const int inner_max = maxit - total_inner;
    if (gc > 0) {
      // the whole Jacobi-CG of this outer step in one cooperative launch
      float* px = M.plat.p;
      float* pr = px + pls;
      float* pz = px + 2 * pls;
      float* pp = px + 3 * pls;
      float* pq = px + 4 * pls;
      const float* dpad = px + 5 * pls;
      const float* wpad = px + 6 * pls;
      k_pad_start<<<lat_grid(pg.L), kLatThreads, 0, st>>>(pg, M.node_gid.p, r64, 1.0 / rnorm, dpad, px, pr, pz, pp,
                                                           pq, R);
      GD_CUDA_TRY(cudaGetLastError());
      GD_CUDA_TRY(cudaMemsetAsync(&R->sync, 0, sizeof(LatSync), st));
      PadGeom pga = pg;
      float rat = M.ratio;
      int mi = inner_max;
      double t2 = tol_in * tol_in;
      void* args[] = {&pga, &wpad, &rat, &px, &pr, &pz, &pp, &pq, &dpad, &R, &mi, &t2};
      GD_CUDA_TRY(cudaLaunchCooperativeKernel((const void*)k_pad_cg, dim3(gc), dim3(kPadThreads), args, 0, st));
      LatSync hs{};
      GD_CUDA_TRY(cudaMemcpyAsync(&hs, &R->sync, sizeof(hs), cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
      if (hs.err) {
        status = fail(GD_ERR_TIMEOUT, "mixed solve: grid barrier of the inner iteration timed out");
        break;
      }
      total_inner += hs.it;
      k_pad_accumulate<<<gb, kLatThreads, 0, st>>>(pg, M.node_gid.p, rnorm, px, x64);
      GD_CUDA_TRY(cudaGetLastError());
      continue;
    }
    int zc = 0, pc = 0;   // current z and p buffers
    k_lat_start<<<gb, kLatThreads, 0, st>>>(nlat, M.node_gid.p, r64, 1.0 / rnorm, dinvl, x, r, zb[zc], pb[pc], q, !ext,
                                            R);
    GD_CUDA_TRY(cudaGetLastError());
    if (ext) {
      GD_TRY(precond->apply_lattice(precond->ctx, A, r, zb[zc], st));
      k_lat_dots<<<gb, kLatThreads, 0, st>>>(nlat, r, zb[zc], nullptr, R);
      GD_CUDA_TRY(cudaGetLastError());
    }
    int it = 0;
    bool inner_stall = false;
    double check_res = 1.0;
    int check_it = 0;
    LatScalars h{};
    auto enqueue = [&](int nstep) -> int {
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
      return GD_OK;
    };
    // Batches of 16, 8, 4 or 2 steps between convergence checks: after each batch the
    // observed per-step reduction of the residual estimates the steps still needed, and
    // the next batch is the largest size not above that estimate, so the last batch of a
    // refinement step does few steps past the tolerance (each costs a preconditioner
    // application).  Every size is even, so z and p return to the same buffers and one
    // captured graph per size replays every batch of that size of every outer step.  The
    // first batch of a solve runs uncaptured (the preconditioner's first-use setup).
    constexpr int kBatchSizes[4] = {16, 8, 4, 2};
    int bi = 0;
    double res_prev = 1.0;   // the inner residual is relative to the normalised start
    while (it < inner_max) {
      const int nstep = std::min(kBatchSizes[bi], inner_max - it);
      const uint64_t key[5] = {ext ? precond->graph_key : 0, (uint64_t)(uintptr_t)M.lat.p,
                               (uint64_t)(uintptr_t)R, (uint64_t)nlat, (uint64_t)gb};
      const bool graphable = ext && precond->graph_key != 0 && nstep == kBatchSizes[bi];
      if (!std::equal(key, key + 5, M.fcg_key)) {   // other buffers or preconditioner: drop all graphs
        for (auto& gx : M.fcg_graph) {
          if (gx) cudaGraphExecDestroy(gx);
          gx = nullptr;
        }
        if (graphable && (it > 0 || total_inner > 0)) std::copy(key, key + 5, M.fcg_key);
      }
      if (graphable && !M.fcg_graph[bi] && (it > 0 || total_inner > 0) && std::equal(key, key + 5, M.fcg_key)) {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
          const int rc = enqueue(nstep);
          const cudaError_t ce = cudaStreamEndCapture(st, &g);
          if (!(rc == GD_OK && ce == cudaSuccess && g && cudaGraphInstantiate(&M.fcg_graph[bi], g, 0) == cudaSuccess))
            M.fcg_graph[bi] = nullptr;
          if (g) cudaGraphDestroy(g);
        }
        cudaGetLastError();   // a failed capture leaves the uncaptured path below
      }
      if (graphable && M.fcg_graph[bi] && std::equal(key, key + 5, M.fcg_key)) {
        GD_CUDA_TRY(cudaGraphLaunch(M.fcg_graph[bi], st));
      } else {
        GD_TRY(enqueue(nstep));
      }
      it += nstep;
      GD_CUDA_TRY(cudaMemcpyAsync(&h, &R->sc, sizeof(h), cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
      if (!std::isfinite(h.rr)) {
        inner_stall = ext;
        break;
      }
      const double res = std::sqrt(h.rr);
      if (res <= tol_in) break;
      if (ext && it - check_it >= 64) {
        if (res > 0.5 * check_res) {
          inner_stall = true;
          break;
        }
        check_res = res;
        check_it = it;
      }
      // next batch size from the per-step reduction factor of this batch
      const double rho = res_prev > 0.0 && res < res_prev ? std::pow(res / res_prev, 1.0 / nstep) : 1.0;
      bi = 0;
      if (rho < 1.0) {
        const double need = std::log(tol_in / res) / std::log(rho);
        while (bi < 3 && kBatchSizes[bi] > need) ++bi;
      }
      res_prev = res;
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

namespace gd {

// One grid all-reduce across the launched blocks, waiting for `expected` arrivals: with
// expected > gridDim.x the last arrival never comes and every block's wait runs out
// after timeout_ns (a flag nothing sets), which is how the bounded wait is tested.
__global__ void k_barrier_probe(LatRed* R, unsigned expected, unsigned long long timeout_ns) {
  const float f[1] = {1.0f};
  float out[1];
  lat_allreduce<1, 0>(R, f, expected, 1u, out, timeout_ns);
}

}  // namespace gd

using namespace gd;

// Diagnostics: exercises the bounded wait of the persistent kernels' grid barrier.
extern "C" int gd_debug_barrier_probe(gd_ctx* ctx, int blocks, int expected, double timeout_s) {
  if (!ctx || blocks < 1 || blocks > 152 || expected < 1 || !(timeout_s > 0.0) || timeout_s > 5.0)
    return fail(GD_ERR_ARG, "gd_debug_barrier_probe: 1..152 blocks, expected >= 1, 0 < timeout <= 5 s");
  cudaStream_t st = ctx->stream;
  DBuf<double> buf;
  GD_TRY(dalloc(buf, (sizeof(LatRed) + sizeof(double) - 1) / sizeof(double)));
  LatRed* R = reinterpret_cast<LatRed*>(buf.p);
  unsigned ex = (unsigned)expected;
  unsigned long long tns = (unsigned long long)(timeout_s * 1e9);
  void* args[] = {&R, &ex, &tns};
  cudaError_t e = cudaMemsetAsync(buf.p, 0, sizeof(LatRed), st);
  if (e == cudaSuccess)
    e = cudaLaunchCooperativeKernel((const void*)k_barrier_probe, dim3(blocks), dim3(kLatThreads), args, 0, st);
  LatSync hs{};
  if (e == cudaSuccess) e = cudaMemcpyAsync(&hs, &R->sync, sizeof(hs), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dfreeb(buf);
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, std::string("gd_debug_barrier_probe: ") + cudaGetErrorString(e));
  if (hs.err) return fail(GD_ERR_TIMEOUT, "gd_debug_barrier_probe: the grid barrier wait ran out");
  return GD_OK;
}
