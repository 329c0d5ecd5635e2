// A14-A16: mul!, the solve behind `\`, and FEFunction's consistent!.
//
// The owned rows of all parts, stored first and in gid order, form the global
// matrix (global DOF ids are part-contiguous, FESpaces.jl:186-208), so SpMV runs over
// them with global column ids and needs no halo exchange: on one device the
// owner->ghost copy of consistent! is a gather from the global vector.
// The reference's `\` gathers A and b to one part and runs a sparse LU
// (PartitionedArrays 0.3); here the solve is Jacobi-preconditioned CG in FP64 with
// deterministic two-stage reductions.
#include <chrono>
#include <cmath>
#include <string>

#include "gd_internal.h"
#include "gd_solve_mixed.h"

namespace gd {

constexpr int kSpmvThreads = 128;                // one row per thread
constexpr int kRowsPerSpmvBlock = kSpmvThreads;
constexpr int kSpmvCap = 3584;                   // staged entries per chunk (43 KB)
constexpr int kStageBatch = 8;                   // staging loads per thread in flight
constexpr int kVecThreads = 256;
constexpr int kMaxPartials = 1024;             // blocks that write partial sums

// CG scalars on the device.  tol2 = (rtol |b|)^2: once r.r falls to it, `done` is set, the
// step count `iters` stops and later steps take alpha = 0 (x and r stay as they are), so
// the host, which checks every few steps, reads the exact iteration count.
struct Scalars {
  double rz, pq, alpha, beta, rr, bb, rz_new, tol2;
  int32_t done, iters;
};
static_assert(sizeof(Scalars) <= 16 * sizeof(double), "Scalars must fit its 16-double slot");

__device__ inline double block_sum(double v, double* sh) {
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

// Block sum of one FP64 value per thread with 127 adds (a shuffle tree would issue
// 5 adds per lane; GB300's FP64 pipe is the scarce unit in these kernels).
__device__ inline double block_sum_serial(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  if (threadIdx.x < kSpmvThreads / 32) {
    double s = 0.0;
    for (int i = 0; i < 32; ++i) s += sh[threadIdx.x * 32 + i];
    sh[kSpmvThreads + threadIdx.x] = s;
  }
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < kSpmvThreads / 32; ++i) s += sh[kSpmvThreads + i];
  __syncthreads();
  return s;   // valid in thread 0
}

// CSR rows on GB300: one thread per row, so a row costs one FP64 FMA per entry and no
// cross-lane adds; the block's contiguous entry range is staged through shared memory
// with coalesced loads (in chunks, so rows of any length work).  MODE 0: y = A x with an
// optional partial of y.w; MODE 1: r = b - A x with partials of r.r and b.b.
template <int MODE>
__device__ __forceinline__ void csr_rows(int64_t n, const int64_t* __restrict__ rowptr,
                                         const int32_t* __restrict__ col, const double* __restrict__ val,
                                         const double* __restrict__ x, const double* __restrict__ b,
                                         double* __restrict__ out, const double* __restrict__ w, double& s1,
                                         double& s2) {
  __shared__ double sval[kSpmvCap];
  __shared__ int32_t scol[kSpmvCap];
  for (int64_t r0 = (int64_t)blockIdx.x * kSpmvThreads; r0 < n; r0 += (int64_t)gridDim.x * kSpmvThreads) {
    const int64_t r = r0 + threadIdx.x;
    const int64_t rend = r0 + kSpmvThreads < n ? r0 + kSpmvThreads : n;
    const int64_t E0 = rowptr[r0], E1 = rowptr[rend];
    const bool valid = r < n;
    const int64_t rs = valid ? rowptr[r] : 0, re = valid ? rowptr[r + 1] : 0;
    double acc = 0.0;
    for (int64_t c0 = E0; c0 < E1; c0 += kSpmvCap) {
      const int cn = (int)(E1 - c0 < kSpmvCap ? E1 - c0 : kSpmvCap);
      __syncthreads();   // the previous chunk has been consumed
      // 8 values and 8 column ids per thread in flight at once (a chunk is at most 28 per
      // thread): the loads of one round, then the stores
      for (int i0 = threadIdx.x; i0 < cn; i0 += kStageBatch * kSpmvThreads) {
        double v[kStageBatch];
        int32_t c[kStageBatch];
#pragma unroll
        for (int u = 0; u < kStageBatch; ++u) {
          const int i = i0 + u * kSpmvThreads;
          if (i < cn) {
            v[u] = __ldcs(val + c0 + i);
            c[u] = __ldcs(col + c0 + i);
          }
        }
#pragma unroll
        for (int u = 0; u < kStageBatch; ++u) {
          const int i = i0 + u * kSpmvThreads;
          if (i < cn) {
            sval[i] = v[u];
            scol[i] = c[u];
          }
        }
      }
      __syncthreads();
      const int lo = (int)((rs > c0 ? rs : c0) - c0), hi = (int)((re < c0 + cn ? re : c0 + cn) - c0);
      // 8 gathers of x in flight before their FMAs (the row's FMA order is unchanged)
      int e = lo;
      for (; e + 8 <= hi; e += 8) {
        double xv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) xv[u] = __ldg(x + scol[e + u]);
#pragma unroll
        for (int u = 0; u < 8; ++u) acc = fma(sval[e + u], xv[u], acc);
      }
      for (; e < hi; ++e) acc = fma(sval[e], __ldg(x + scol[e]), acc);
    }
    if (valid) {
      if (MODE == 0) {
        out[r] = acc;
        if (w) s1 = fma(acc, w[r], s1);
      } else {
        const double bv = b[r];
        const double rv = bv - acc;
        if (out) out[r] = rv;
        s1 = fma(rv, rv, s1);
        s2 = fma(bv, bv, s2);
      }
    }
  }
}

// y = A x over owned rows; optional partial dot(y, w) per block.  Shared memory allows 5
// blocks per SM; the launch bound keeps the registers within that too.
__global__ void __launch_bounds__(kSpmvThreads, 5)
k_spmv(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
       const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y,
       const double* __restrict__ w, double* __restrict__ partial) {
  __shared__ double sh[kSpmvThreads + kSpmvThreads / 32];
  double dot = 0.0, unused = 0.0;
  csr_rows<0>(n, rowptr, col, val, x, nullptr, y, w, dot, unused);
  if (partial) {
    const double t = block_sum_serial(dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

// r = b - A x (partials of r.r and b.b)
__global__ void __launch_bounds__(kSpmvThreads, 5)
k_residual(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
           const double* __restrict__ val, const double* __restrict__ x, const double* __restrict__ b,
           double* __restrict__ r_out, double* __restrict__ partial_rr, double* __restrict__ partial_bb) {
  __shared__ double sh[kSpmvThreads + kSpmvThreads / 32];
  double rr = 0.0, bb = 0.0;
  csr_rows<1>(n, rowptr, col, val, x, b, r_out, nullptr, rr, bb);
  double t = block_sum_serial(rr, sh);
  if (threadIdx.x == 0) partial_rr[blockIdx.x] = t;
  t = block_sum_serial(bb, sh);
  if (threadIdx.x == 0) partial_bb[blockIdx.x] = t;
}

// ---------------------------------------------------------------------------------
// Sliced ELL (short rows): one thread per row, the warp's 32 rows read their k-th entries
// as one coalesced 256-byte line, with no shared-memory staging and no block barrier, so
// the blocks stay resident at full occupancy and the FP64 FMAs overlap the HBM stream.
// ---------------------------------------------------------------------------------
constexpr int kSellThreads = 256;

// stored entries per row (the non-zeros) and each 32-row slice's longest row
__global__ void k_sell_len(int64_t n, const int64_t* __restrict__ rowptr, const double* __restrict__ val,
                           int32_t* __restrict__ len, int32_t* __restrict__ width) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0;
  if (r < n) {
    for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) c += val[e] != 0.0;
    len[r] = c;
  }
  int m = c;
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0 && r < n) width[r >> 5] = m;   // lane 0 holds the slice's first row
}

__global__ void k_sell_fill(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                            const double* __restrict__ val, const int64_t* __restrict__ off, double* __restrict__ sval,
                            int32_t* __restrict__ scol) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t base = 32 * off[r >> 5] + (r & 31);
  int64_t k = 0;
  for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) {
    const double v = val[e];
    if (v != 0.0) {
      sval[base + 32 * k] = v;
      scol[base + 32 * k] = col[e];
      ++k;
    }
  }
}

// MODE 0: y = A x with the partial of y.w per block (w may be null); MODE 1: r = b - A x
// (r may be null) with the partials of r.r and b.b.  A row's products are summed in CSR
// order, four loads of the row in flight at a time.
template <int MODE>
__global__ void __launch_bounds__(kSellThreads)
k_sell_rows(int64_t n, const int64_t* __restrict__ off, const int32_t* __restrict__ len,
            const double* __restrict__ sval, const int32_t* __restrict__ scol, const double* __restrict__ x,
            const double* __restrict__ b, double* __restrict__ out, const double* __restrict__ w,
            double* __restrict__ p1, double* __restrict__ p2) {
  __shared__ double sh[32];
  double s1 = 0.0, s2 = 0.0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t base = 32 * off[r >> 5] + (r & 31);
    const double* pv = sval + base;
    const int32_t* pc = scol + base;
    const int L = len[r];
    double acc = 0.0;
    int k = 0;
    for (; k + 4 <= L; k += 4) {
      double v[4], xv[4];
      int32_t c[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        v[u] = __ldcs(pv + 32 * (k + u));
        c[u] = __ldcs(pc + 32 * (k + u));
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
      for (int u = 0; u < 4; ++u) acc = fma(v[u], xv[u], acc);
    }
    for (; k < L; ++k) acc = fma(__ldcs(pv + 32 * k), __ldg(x + __ldcs(pc + 32 * k)), acc);
    if (MODE == 0) {
      out[r] = acc;
      if (w) s1 = fma(acc, w[r], s1);
    } else {
      const double bv = b[r];
      const double rv = bv - acc;
      if (out) out[r] = rv;
      s1 = fma(rv, rv, s1);
      s2 = fma(bv, bv, s2);
    }
  }
  if (p1) {
    const double t = block_sum(s1, sh);
    if (threadIdx.x == 0) p1[blockIdx.x] = t;
  }
  if (MODE == 1 && p2) {
    const double t = block_sum(s2, sh);
    if (threadIdx.x == 0) p2[blockIdx.x] = t;
  }
}

// grid-stride over the rows with only as many blocks as are resident at once (and at most
// kMaxPartials, the partial sums the scalar kernels read)
static int sell_grid(int64_t n) {
  static int resident[64] = {0};
  int64_t b = std::max<int64_t>(1, std::min<int64_t>((n + kSellThreads - 1) / kSellThreads, kMaxPartials));
  int dev = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
    if (!resident[dev]) {
      int sms = 0, per_sm = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sell_rows<1>, kSellThreads, 0);
      cudaGetLastError();
      resident[dev] = sms * per_sm > 0 ? sms * per_sm : kMaxPartials;
    }
    if (b > resident[dev]) b = resident[dev];
  }
  return (int)b;
}

// Long rows (vector and high-order systems: 81 to 375 entries): G lanes per row, each lane
// a strided share of the row's entries (coalesced across the group), then a log2(G)
// shuffle tree.  Thread-per-row staging leaves most lanes idle there, because a chunk of
// staged entries covers only a few rows.
template <int MODE, int G>
__device__ __forceinline__ void csr_rows_g(int64_t n, const int64_t* __restrict__ rowptr,
                                           const int32_t* __restrict__ col, const double* __restrict__ val,
                                           const double* __restrict__ x, const double* __restrict__ b,
                                           double* __restrict__ out, const double* __restrict__ w, double& s1,
                                           double& s2) {
  constexpr int RPW = 32 / G;
  const int lane = threadIdx.x & 31, sub = lane / G, gl = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t rb = warp * RPW; rb < n; rb += nw * RPW) {   // warp-uniform trip count
    const int64_t r = rb + sub;
    const bool valid = r < n;
    double acc = 0.0;
    if (valid) {
      const int64_t e1 = rowptr[r + 1];
      int64_t e = rowptr[r] + gl;
      for (; e + 3 * G < e1; e += 4 * G) {   // 4 independent entries in flight per lane
        int32_t c[4];
        double v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          c[u] = col[e + u * G];
          v[u] = val[e + u * G];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) xv[u] = __ldg(x + c[u]);
#pragma unroll
        for (int u = 0; u < 4; ++u) acc = fma(v[u], xv[u], acc);
      }
      for (; e < e1; e += G) acc = fma(val[e], __ldg(x + col[e]), acc);
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (valid && gl == 0) {
      if (MODE == 0) {
        out[r] = acc;
        if (w) s1 = fma(acc, w[r], s1);
      } else {
        const double bv = b[r];
        const double rv = bv - acc;
        if (out) out[r] = rv;
        s1 = fma(rv, rv, s1);
        s2 = fma(bv, bv, s2);
      }
    }
  }
}

template <int G>
__global__ void __launch_bounds__(kSpmvThreads)
k_spmv_g(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
         const double* __restrict__ val, const double* __restrict__ x, double* __restrict__ y,
         const double* __restrict__ w, double* __restrict__ partial) {
  __shared__ double sh[kSpmvThreads + kSpmvThreads / 32];
  double dot = 0.0, unused = 0.0;
  csr_rows_g<0, G>(n, rowptr, col, val, x, nullptr, y, w, dot, unused);
  if (partial) {
    const double t = block_sum_serial(dot, sh);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
  }
}

template <int G>
__global__ void __launch_bounds__(kSpmvThreads)
k_residual_g(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
             const double* __restrict__ val, const double* __restrict__ x, const double* __restrict__ b,
             double* __restrict__ r_out, double* __restrict__ partial_rr, double* __restrict__ partial_bb) {
  __shared__ double sh[kSpmvThreads + kSpmvThreads / 32];
  double rr = 0.0, bb = 0.0;
  csr_rows_g<1, G>(n, rowptr, col, val, x, b, r_out, nullptr, rr, bb);
  double t = block_sum_serial(rr, sh);
  if (threadIdx.x == 0) partial_rr[blockIdx.x] = t;
  t = block_sum_serial(bb, sh);
  if (threadIdx.x == 0) partial_bb[blockIdx.x] = t;
}

__global__ void k_dinv(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ col,
                       const double* __restrict__ val, double* __restrict__ dinv, int32_t* __restrict__ bad) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  double d = 0.0;
  for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e)
    if (col[e] == r) d = val[e];
  if (!(d > 0.0) || !isfinite(d)) {
    atomicAdd(bad, 1);
    dinv[r] = 0.0;
  } else {
    dinv[r] = 1.0 / d;
  }
}

// z = dinv*r, p = z, partial of r.z and r.r
__global__ void k_pcg_init(int64_t n, const double* __restrict__ dinv, const double* __restrict__ r,
                           double* __restrict__ z, double* __restrict__ p, double* __restrict__ prz,
                           double* __restrict__ prr) {
  __shared__ double sh[kVecThreads / 32];
  double a = 0.0, b = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double zi = dinv[i] * r[i];
    z[i] = zi;
    p[i] = zi;
    a += r[i] * zi;
    b += r[i] * r[i];
  }
  double t = block_sum(a, sh);
  if (threadIdx.x == 0) prz[blockIdx.x] = t;
  t = block_sum(b, sh);
  if (threadIdx.x == 0) prr[blockIdx.x] = t;
}

// x += alpha p; r -= alpha q; z = dinv r; partials r.z, r.r
__global__ void k_pcg_update(int64_t n, const Scalars* __restrict__ sc, double* __restrict__ x,
                             double* __restrict__ r, double* __restrict__ z, const double* __restrict__ p,
                             const double* __restrict__ q, const double* __restrict__ dinv,
                             double* __restrict__ prz, double* __restrict__ prr) {
  __shared__ double sh[kVecThreads / 32];
  const double alpha = sc->alpha;
  double a = 0.0, b = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    x[i] += alpha * p[i];
    double ri = r[i] - alpha * q[i];
    r[i] = ri;
    double zi = dinv[i] * ri;
    z[i] = zi;
    a += ri * zi;
    b += ri * ri;
  }
  double t = block_sum(a, sh);
  if (threadIdx.x == 0) prz[blockIdx.x] = t;
  t = block_sum(b, sh);
  if (threadIdx.x == 0) prr[blockIdx.x] = t;
}

__global__ void k_pcg_pupdate(int64_t n, const Scalars* __restrict__ sc, const double* __restrict__ z,
                              double* __restrict__ p) {
  const double beta = sc->beta;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    p[i] = z[i] + beta * p[i];
}

// one block: fixed-order sums of partials and the CG scalars
// mode 0: init (rz, rr); 1: alpha from pq; 2: beta from rz_new, rr
__global__ void k_pcg_scalars(int mode, int nb, const double* __restrict__ pa, const double* __restrict__ pb,
                              Scalars* __restrict__ sc) {
  __shared__ double sh[kVecThreads / 32];
  double a = 0.0, b = 0.0;
  for (int i = threadIdx.x; i < nb; i += blockDim.x) {
    a += pa[i];
    if (pb) b += pb[i];
  }
  double sa = block_sum(a, sh);
  double sb = block_sum(b, sh);
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    sc->rz = sa;
    sc->rr = sb;
  } else if (mode == 1) {
    sc->pq = sa;
    sc->alpha = (!sc->done && sa != 0.0) ? sc->rz / sa : 0.0;
  } else {
    sc->beta = sc->rz != 0.0 ? sa / sc->rz : 0.0;
    sc->rz = sa;
    sc->rr = sb;
    if (!sc->done) {
      ++sc->iters;
      if (sb <= sc->tol2) sc->done = 1;
    }
  }
}

// Starts a CG cycle: no step taken yet, stop at r.r <= tol2.
__global__ void k_pcg_arm(Scalars* __restrict__ sc, double tol2) {
  sc->tol2 = tol2;
  sc->done = 0;
  sc->iters = 0;
}

__global__ void k_gather_local(int64_t n, const int64_t* __restrict__ lid_gid, const double* __restrict__ xg,
                               double* __restrict__ xl) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) xl[i] = xg[lid_gid[i]];
}

static int grid_for(int64_t n, int per_block);
int gather_local_vec(const gd_space* S, int part, const double* xg, double* xl, cudaStream_t st);

// FP64 residual r = b - A x with per-block partials of r.r and b.b; returns the block count
int residual_fp64(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, const double* x,
                  const double* b, double* r, double* prr, double* pbb, cudaStream_t st, int* nblocks) {
  const int gs = grid_for(n, kRowsPerSpmvBlock);
  k_residual<<<gs, kSpmvThreads, 0, st>>>(n, rowptr, col, val, x, b, r, prr, pbb);
  GD_CUDA_TRY(cudaGetLastError());
  *nblocks = gs;
  return GD_OK;
}

int sell_build(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, SellMat& S, int64_t version,
               cudaStream_t st) {
  if (version >= 0 && S.version == version && S.n == n) return GD_OK;
  S.version = -1;
  if (n <= 0) {
    S.n = n;
    S.version = version;
    return GD_OK;
  }
  const int64_t ns = (n + 31) / 32;
  if (S.len.n < (size_t)n) GD_TRY(dalloc(S.len, n));
  if (S.width.n < (size_t)ns) GD_TRY(dalloc(S.width, ns));
  if (S.off.n < (size_t)(ns + 1)) GD_TRY(dalloc(S.off, ns + 1));
  const unsigned gb = (unsigned)((n + kSellThreads - 1) / kSellThreads);
  k_sell_len<<<gb, kSellThreads, 0, st>>>(n, rowptr, val, S.len.p, S.width.p);
  GD_CUDA_TRY(cudaGetLastError());
  GD_TRY(exclusive_scan_i32(S.width.p, S.off.p, ns, st));
  int64_t total = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&total, S.off.p + ns, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const size_t ne = (size_t)std::max<int64_t>(32 * total, 1);
  if (S.val.n < ne) GD_TRY(dalloc(S.val, ne));
  if (S.col.n < ne) GD_TRY(dalloc(S.col, ne));
  k_sell_fill<<<gb, kSellThreads, 0, st>>>(n, rowptr, col, val, S.off.p, S.val.p, S.col.p);
  GD_CUDA_TRY(cudaGetLastError());
  S.n = n;
  S.version = version;
  return GD_OK;
}

static int grid_for(int64_t n, int per_block) {
  int64_t b = (n + per_block - 1) / per_block;
  if (b > kMaxPartials) b = kMaxPartials;
  if (b < 1) b = 1;
  if (per_block == kRowsPerSpmvBlock) {
    // the SpMV grid-strides over row groups: launch only what is resident at once
    static int resident[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < 64) {
      if (!resident[dev]) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_residual, kSpmvThreads, 0);
        resident[dev] = sms * per_sm > 0 ? sms * per_sm : kMaxPartials;
      }
      if (b > resident[dev]) b = resident[dev];
    }
  }
  return (int)b;
}

int residual_fp64_asm(gd_asm* A, const double* x, const double* b, double* r, double* prr, double* pbb,
                      cudaStream_t st, int* nblocks) {
  const int64_t n = A->ngdofs;
  if (!sell_suits(n, A->nnz_own))
    return residual_fp64(n, A->rowptr.p, A->colgid.p, A->vals.p, x, b, r, prr, pbb, st, nblocks);
  GD_TRY(sell_build(n, A->rowptr.p, A->colgid.p, A->vals.p, A->sell, A->numeric_epoch, st));
  const int gs = sell_grid(n);
  k_sell_rows<1><<<gs, kSellThreads, 0, st>>>(n, A->sell.off.p, A->sell.len.p, A->sell.val.p, A->sell.col.p, x, b, r,
                                              nullptr, prr, pbb);
  GD_CUDA_TRY(cudaGetLastError());
  *nblocks = gs;
  return GD_OK;
}

}  // namespace gd

using namespace gd;

static int check_ready(const gd_asm* A, const char* fn) {
  if (!A) return fail(GD_ERR_ARG, std::string(fn) + ": null assembler");
  if (!A->numeric_done) return fail(GD_ERR_STATE, std::string(fn) + ": run gd_assemble_numeric first");
  return GD_OK;
}

extern "C" int gd_spmv(gd_asm* A, const double* x, double* y, int where) {
  GD_TRY(check_ready(A, "gd_spmv"));
  if (!x || !y) return fail(GD_ERR_ARG, "gd_spmv: null vector");
  cudaStream_t st = A->test->model->ctx->stream;
  const int64_t n = A->ngdofs;
  const double* dx = x;
  double* dy = y;
  DBuf<double> tx, ty;
  if (where == GD_HOST) {
    GD_TRY(dalloc(tx, n));
    GD_TRY(dalloc(ty, n));
    GD_CUDA_TRY(cudaMemcpyAsync(tx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    dx = tx.p;
    dy = ty.p;
  }
  if (sell_suits(n, A->nnz_own)) {   // the solver's sliced-ELL copy (built once per numeric assembly)
    GD_TRY(sell_build(n, A->rowptr.p, A->colgid.p, A->vals.p, A->sell, A->numeric_epoch, st));
    k_sell_rows<0><<<sell_grid(n), kSellThreads, 0, st>>>(n, A->sell.off.p, A->sell.len.p, A->sell.val.p,
                                                          A->sell.col.p, dx, nullptr, dy, nullptr, nullptr, nullptr);
  } else if (n > 0) {   // long rows: lane groups on the CSR, as in the solver
    const int64_t avg = A->nnz_own / n;
    const int G = avg >= 256 ? 32 : avg >= 96 ? 16 : 8;
    const int gs = (int)std::max<int64_t>(1, std::min<int64_t>((n * G + kSpmvThreads - 1) / kSpmvThreads, kMaxPartials));
    const int64_t* rp = A->rowptr.p;
    const int32_t* cg = A->colgid.p;
    const double* v = A->vals.p;
    switch (G) {
      case 32: k_spmv_g<32><<<gs, kSpmvThreads, 0, st>>>(n, rp, cg, v, dx, dy, nullptr, nullptr); break;
      case 16: k_spmv_g<16><<<gs, kSpmvThreads, 0, st>>>(n, rp, cg, v, dx, dy, nullptr, nullptr); break;
      default: k_spmv_g<8><<<gs, kSpmvThreads, 0, st>>>(n, rp, cg, v, dx, dy, nullptr, nullptr);
    }
  }
  GD_CUDA_TRY(cudaGetLastError());
  if (where == GD_HOST) GD_CUDA_TRY(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(tx);
  dfreeb(ty);
  return GD_OK;
}

extern "C" int gd_solve(gd_asm* A, int method, double rtol, int maxit, double* x, int where, gd_solve_stats* stats) {
  GD_TRY(check_ready(A, "gd_solve"));
  if (method == GD_SOLVE_MIXED_IR) {
    if (!x || !(rtol > 0.0) || maxit < 0) return fail(GD_ERR_ARG, "gd_solve: bad argument");
    return mixed_solve(A, rtol, maxit, x, where, stats, nullptr);
  }
  if (method != GD_SOLVE_JACOBI_PCG) return fail(GD_ERR_UNSUPPORTED, "gd_solve: unknown method");
  if (!x || !(rtol > 0.0) || maxit < 0) return fail(GD_ERR_ARG, "gd_solve: bad argument");
  return jacobi_pcg_csr(A->ngdofs, A->rowptr.p, A->colgid.p, A->vals.p, A->rhs_override ? A->rhs_override : A->rhs.p,
                        A->w, A->dinv, A->dred, A->test->model->ctx->stream, rtol, maxit, x, where, stats, &A->sell,
                        A->numeric_epoch);
}

namespace gd {

// Device buffers of one FP64 Jacobi-PCG: five vectors, the inverse diagonal, two arrays of
// per-block partial sums, the scalars and the bad-diagonal counter.
struct PcgBufs {
  double *x, *r, *z, *p, *q, *dinv, *pa, *pb;
  Scalars* sc;
  int32_t* bad;
};

// Every DOF is a Dirichlet DOF: nothing to solve.
static int pcg_empty(gd_solve_stats* stats, std::chrono::steady_clock::time_point t0) {
  if (stats) {
    stats->iterations = 0;
    stats->converged = 1;
    stats->rel_residual = 0.0;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  return GD_OK;
}

// The FP64 Jacobi-PCG iteration shared by gd_solve and gd_solve_noalloc; `spmv` (y = A p
// with partials of p.y) and `residual` (r = b - A x with partials of r.r and b.b) launch
// the matrix kernels on gs blocks, the vector kernels run on gv.  CG checks the recursive
// residual every few steps on the host; when it meets the tolerance but the true residual
// (recomputed in FP64) does not -- rounding makes the two drift apart near tight
// tolerances -- CG restarts from the true residual, at most kMaxRestarts times.
template <typename SpmvF, typename ResidF>
static int pcg_run(const char* fn, int64_t n, const int64_t* rowptr, const int32_t* colgid, const double* vals,
                   const PcgBufs& B, int gs, int gv, SpmvF& spmv, ResidF& residual, cudaStream_t st, double rtol,
                   int maxit, double* x, int where, gd_solve_stats* stats,
                   std::chrono::steady_clock::time_point t0) {
  const std::string name(fn);
  GD_CUDA_TRY(cudaMemsetAsync(B.bad, 0, sizeof(int32_t), st));
  GD_CUDA_TRY(cudaMemsetAsync(B.x, 0, sizeof(double) * n, st));
  k_dinv<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, rowptr, colgid, vals, B.dinv, B.bad);
  GD_CUDA_TRY(cudaGetLastError());
  // r = b - A*0 = b ; bb
  residual(B.x, B.r, B.pa, B.pb);
  k_pcg_scalars<<<1, kVecThreads, 0, st>>>(0, gs, B.pb, B.pa, B.sc);   // rz <- bb (temp), rr <- rr
  GD_CUDA_TRY(cudaGetLastError());
  Scalars h{};
  int32_t hbad = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&h, B.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&hbad, B.bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (hbad)
    return fail(GD_ERR_NUMERIC, name + ": non-positive or missing diagonal in " + std::to_string(hbad) + " rows");
  const double bnorm = std::sqrt(h.rz);
  const double tol2 = (rtol * bnorm) * (rtol * bnorm);
  k_pcg_init<<<gv, kVecThreads, 0, st>>>(n, B.dinv, B.r, B.z, B.p, B.pa, B.pb);
  k_pcg_scalars<<<1, kVecThreads, 0, st>>>(0, gv, B.pa, B.pb, B.sc);
  k_pcg_arm<<<1, 1, 0, st>>>(B.sc, tol2);
  GD_CUDA_TRY(cudaGetLastError());
  int launched = 0, taken = 0;
  bool conv = bnorm == 0.0;
  const int check_every = 8;
  constexpr int kMaxRestarts = 3;
  for (int restart = 0;; ++restart) {
    int cycle = 0;
    while (!conv && launched < maxit) {
      const int nstep = std::min(check_every, maxit - launched);
      for (int s = 0; s < nstep; ++s) {
        spmv(B.p, B.q, B.p, B.pa);
        k_pcg_scalars<<<1, kVecThreads, 0, st>>>(1, gs, B.pa, nullptr, B.sc);
        k_pcg_update<<<gv, kVecThreads, 0, st>>>(n, B.sc, B.x, B.r, B.z, B.p, B.q, B.dinv, B.pa, B.pb);
        k_pcg_scalars<<<1, kVecThreads, 0, st>>>(2, gv, B.pa, B.pb, B.sc);
        k_pcg_pupdate<<<gv, kVecThreads, 0, st>>>(n, B.sc, B.z, B.p);
      }
      GD_CUDA_TRY(cudaGetLastError());
      launched += nstep;
      GD_CUDA_TRY(cudaMemcpyAsync(&h, B.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
      cycle = h.iters;
      if (!std::isfinite(h.rr)) break;
      if (h.done) conv = true;
    }
    taken += cycle;
    // true FP64 residual (kept in r for a restart)
    residual(B.x, B.r, B.pa, B.pb);
    k_pcg_scalars<<<1, kVecThreads, 0, st>>>(0, gs, B.pa, B.pb, B.sc);
    GD_CUDA_TRY(cudaGetLastError());
    GD_CUDA_TRY(cudaMemcpyAsync(&h, B.sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    const double rel_true = bnorm > 0.0 ? std::sqrt(h.rz) / bnorm : 0.0;
    if (!conv || rel_true <= rtol || !std::isfinite(rel_true) || launched >= maxit || restart >= kMaxRestarts) break;
    conv = false;
    k_pcg_init<<<gv, kVecThreads, 0, st>>>(n, B.dinv, B.r, B.z, B.p, B.pa, B.pb);
    k_pcg_scalars<<<1, kVecThreads, 0, st>>>(0, gv, B.pa, B.pb, B.sc);
    k_pcg_arm<<<1, 1, 0, st>>>(B.sc, tol2);
    GD_CUDA_TRY(cudaGetLastError());
  }
  GD_CUDA_TRY(cudaMemcpyAsync(x, B.x, sizeof(double) * n,
                              where == GD_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const double rel = bnorm > 0.0 ? std::sqrt(h.rz) / bnorm : 0.0;
  if (stats) {
    stats->iterations = taken;
    stats->converged = rel <= rtol;
    stats->rel_residual = rel;
    stats->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  if (!std::isfinite(rel)) return fail(GD_ERR_NUMERIC, name + ": residual is not finite");
  if (rel > rtol)
    return fail(GD_ERR_NOTCONVERGED, name + ": tolerance not reached in " + std::to_string(taken) + " iterations");
  return GD_OK;
}

}  // namespace gd

// FP64 Jacobi-PCG on the owned rows of a CSR (global column ids); workspace buffers are
// (re)allocated as needed: w (5 n: x r z p q), dinv (n), dred (partials and scalars).
int gd::jacobi_pcg_csr(int64_t n, const int64_t* rowptr, const int32_t* colgid, const double* vals, const double* rhs,
                   DBuf<double>& w, DBuf<double>& dinvb, DBuf<double>& dred, cudaStream_t st, double rtol, int maxit,
                   double* x, int where, gd_solve_stats* stats, SellMat* sell, int64_t version) {
  auto t0 = std::chrono::steady_clock::now();
  if (n == 0) return pcg_empty(stats, t0);
  // rows per lane group from the average row length; below 48 entries one thread per row
  // on the sliced-ELL copy (the caller's cached one, else a temporary freed on return)
  int64_t nnz = 0;
  if (n) {
    GD_CUDA_TRY(cudaMemcpyAsync(&nnz, rowptr + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
  }
  const int64_t avg = n ? nnz / n : 0;
  const int G = avg >= 256 ? 32 : avg >= 96 ? 16 : avg >= 48 ? 8 : 1;
  SellMat local;
  struct Release {
    SellMat* m;
    ~Release() {
      if (m) m->release();
    }
  } release_local{sell ? nullptr : &local};
  SellMat* S = sell ? sell : &local;
  if (G == 1) GD_TRY(sell_build(n, rowptr, colgid, vals, *S, sell ? version : -1, st));
  const int gsg = G == 1 ? sell_grid(n)
                         : (int)std::max<int64_t>(1, std::min<int64_t>((n * G + kSpmvThreads - 1) / kSpmvThreads,
                                                                       kMaxPartials));
  auto spmv = [&](const double* xin, double* yout, const double* wdot, double* part) {
    switch (G) {
      case 32: k_spmv_g<32><<<gsg, kSpmvThreads, 0, st>>>(n, rowptr, colgid, vals, xin, yout, wdot, part); break;
      case 16: k_spmv_g<16><<<gsg, kSpmvThreads, 0, st>>>(n, rowptr, colgid, vals, xin, yout, wdot, part); break;
      case 8: k_spmv_g<8><<<gsg, kSpmvThreads, 0, st>>>(n, rowptr, colgid, vals, xin, yout, wdot, part); break;
      default:
        k_sell_rows<0><<<gsg, kSellThreads, 0, st>>>(n, S->off.p, S->len.p, S->val.p, S->col.p, xin, nullptr, yout,
                                                     wdot, part, nullptr);
    }
  };
  auto residual = [&](const double* xin, double* rout, double* prr, double* pbb) {
    switch (G) {
      case 32: k_residual_g<32><<<gsg, kSpmvThreads, 0, st>>>(n, rowptr, colgid, vals, xin, rhs, rout, prr, pbb); break;
      case 16: k_residual_g<16><<<gsg, kSpmvThreads, 0, st>>>(n, rowptr, colgid, vals, xin, rhs, rout, prr, pbb); break;
      case 8: k_residual_g<8><<<gsg, kSpmvThreads, 0, st>>>(n, rowptr, colgid, vals, xin, rhs, rout, prr, pbb); break;
      default:
        k_sell_rows<1><<<gsg, kSellThreads, 0, st>>>(n, S->off.p, S->len.p, S->val.p, S->col.p, xin, rhs, rout,
                                                     nullptr, prr, pbb);
    }
  };
  if (w.n < (size_t)(5 * n)) GD_TRY(dalloc(w, 5 * std::max<int64_t>(n, 1)));
  if (dinvb.n < (size_t)n) GD_TRY(dalloc(dinvb, std::max<int64_t>(n, 1)));
  if (!dred.p) GD_TRY(dalloc(dred, 4096));
  PcgBufs B;
  B.x = w.p;
  B.r = B.x + n;
  B.z = B.r + n;
  B.p = B.z + n;
  B.q = B.p + n;
  B.dinv = dinvb.p;
  B.pa = dred.p + 16;
  B.pb = B.pa + kMaxPartials;
  B.sc = (Scalars*)(dred.p + 16 + 2 * kMaxPartials);
  B.bad = (int32_t*)dred.p;
  return pcg_run("gd_solve", n, rowptr, colgid, vals, B, gsg, grid_for(n, kVecThreads), spmv, residual, st, rtol, maxit,
                 x, where, stats, t0);
}

extern "C" int gd_fe_function_local(const gd_space* S, int part, const double* x_global, int where, double* x_local) {
  if (!S || part < 0 || part >= S->geom.nparts || !x_global || !x_local)
    return fail(GD_ERR_ARG, "gd_fe_function_local: bad argument");
  cudaStream_t st = S->model->ctx->stream;
  const DevPart& P = S->parts[part];
  const int bs = S->ncomp;
  const int64_t n = P.nfree * bs, ng = S->ngdofs * bs;
  DBuf<double> xg, xl;
  const double* dxg = x_global;
  if (where == GD_HOST) {
    GD_TRY(dalloc(xg, std::max<int64_t>(ng, 1)));
    GD_CUDA_TRY(cudaMemcpyAsync(xg.p, x_global, sizeof(double) * ng, cudaMemcpyHostToDevice, st));
    dxg = xg.p;
    GD_TRY(dalloc(xl, std::max<int64_t>(n, 1)));
  }
  double* dxl = where == GD_HOST ? xl.p : x_local;
  if (bs > 1) {
    GD_TRY(gather_local_vec(S, part, dxg, dxl, st));
  } else if (n > 0) {
    k_gather_local<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, S->lid_gid.p + P.lid_off, dxg, dxl);
    GD_CUDA_TRY(cudaGetLastError());
  }
  if (where == GD_HOST && n > 0)
    GD_CUDA_TRY(cudaMemcpyAsync(x_local, dxl, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(xg);
  dfreeb(xl);
  return GD_OK;
}

// ---------------------------------------------------------------------------------
// Allocation-free solve
//
// Some callers of this library cannot allocate device memory while they run: an
// application whose device memory is owned by its own pool allocator (every byte
// reserved up front, so a cudaMalloc behind its back fails or evicts), or a control
// or time-stepping loop in which a cudaMalloc -- which may synchronise the whole
// device, or fail part-way through a run -- is not acceptable.  gd_solve allocates
// its Jacobi-PCG workspace on first use; gd_solve_noalloc runs the same iteration
// (pcg_run: the same steps, restarts from the true FP64 residual and stopping rule)
// with every scratch vector, partial sum and scalar in one file-scope device array
// instead, so it calls no cudaMalloc/cudaFree at all.  Its matrix kernel is the CSR
// one (k_spmv / k_residual: one thread per row, entries staged through shared memory),
// since the sliced-ELL copy that gd_solve builds for short rows would need memory.
//
// Limits and rules (also stated in gdgpu.h):
//  * at most kNoAllocMaxDofs global DOFs; larger systems are rejected with GD_ERR_ARG;
//  * the array (about 12.6 MB) is held by every device that loads the library, until
//    the process exits;
//  * every call looks the array's device address up (cudaGetSymbolAddress, which
//    allocates nothing) with the assembler's device current, and puts the caller's
//    current device back before it returns;
//  * every call shares the one array and it keeps the last call's contents: each call
//    clears what must start at zero, and calls that overlap on the GPU (other streams,
//    other host threads) race on it.
// ---------------------------------------------------------------------------------
namespace gd {

constexpr int64_t kNoAllocMaxDofs = (int64_t)1 << 18;   // 262,144 global DOFs
constexpr int64_t kNoAllocDoubles = 6 * kNoAllocMaxDofs + 2 * kMaxPartials + 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocDoubles];

// Makes `dev` current for the lifetime of the guard, then restores the caller's device.
struct DeviceGuard {
  int prev = -1;
  bool changed = false;
  int set(int dev) {
    GD_CUDA_TRY(cudaGetDevice(&prev));
    if (prev != dev) {
      GD_CUDA_TRY(cudaSetDevice(dev));
      changed = true;
    }
    return GD_OK;
  }
  ~DeviceGuard() {
    if (changed) cudaSetDevice(prev);
  }
};

// Device address of the scratch array on the current device.
static int noalloc_scratch(double** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(GD_ERR_CUDA, std::string("gd_solve_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
  *out = static_cast<double*>(p);
  return GD_OK;
}

}  // namespace gd

extern "C" int gd_solve_noalloc(gd_asm* A, double rtol, int maxit, double* x, int where, gd_solve_stats* stats) {
  GD_TRY(check_ready(A, "gd_solve_noalloc"));
  if (!x || !(rtol > 0.0) || maxit < 0) return fail(GD_ERR_ARG, "gd_solve_noalloc: bad argument");
  const int64_t n = A->ngdofs;
  if (n > kNoAllocMaxDofs)
    return fail(GD_ERR_ARG, "gd_solve_noalloc: " + std::to_string(n) + " DOFs exceed the static scratch limit of " +
                                std::to_string(kNoAllocMaxDofs) + " (use gd_solve)");
  auto t0 = std::chrono::steady_clock::now();
  if (n == 0) return pcg_empty(stats, t0);
  DeviceGuard guard;
  GD_TRY(guard.set(A->test->model->ctx->device));
  double* base = nullptr;
  GD_TRY(noalloc_scratch(&base));
  cudaStream_t st = A->test->model->ctx->stream;
  PcgBufs B;
  B.x = base;
  B.r = base + 1 * kNoAllocMaxDofs;
  B.z = base + 2 * kNoAllocMaxDofs;
  B.p = base + 3 * kNoAllocMaxDofs;
  B.q = base + 4 * kNoAllocMaxDofs;
  B.dinv = base + 5 * kNoAllocMaxDofs;
  B.pa = base + 6 * kNoAllocMaxDofs;
  B.pb = B.pa + kMaxPartials;
  B.sc = reinterpret_cast<Scalars*>(B.pb + kMaxPartials);          // a 16-double slot
  B.bad = reinterpret_cast<int32_t*>(B.pb + kMaxPartials + 16);   // after it
  const int64_t* rowptr = A->rowptr.p;
  const int32_t* col = A->colgid.p;
  const double* val = A->vals.p;
  const double* rhs = A->rhs.p;
  const int gs = grid_for(n, kRowsPerSpmvBlock);
  auto spmv = [&](const double* xin, double* yout, const double* wdot, double* part) {
    k_spmv<<<gs, kSpmvThreads, 0, st>>>(n, rowptr, col, val, xin, yout, wdot, part);
  };
  auto residual = [&](const double* xin, double* rout, double* prr, double* pbb) {
    k_residual<<<gs, kSpmvThreads, 0, st>>>(n, rowptr, col, val, xin, rhs, rout, prr, pbb);
  };
  return pcg_run("gd_solve_noalloc", n, rowptr, col, val, B, gs, grid_for(n, kVecThreads), spmv, residual, st, rtol,
                 maxit, x, where, stats, t0);
}

// x = A \ b for a caller-given right-hand side (device or host), same methods as gd_solve.
extern "C" int gd_solve_rhs(gd_asm* A, int method, double rtol, int maxit, const double* b, double* x, int where,
                            gd_solve_stats* stats) {
  GD_TRY(check_ready(A, "gd_solve_rhs"));
  if (!b || !x) return fail(GD_ERR_ARG, "gd_solve_rhs: null vector");
  cudaStream_t st = A->test->model->ctx->stream;
  const int64_t n = A->ngdofs;
  DBuf<double> tb;
  const double* db = b;
  if (where == GD_HOST) {
    GD_TRY(dalloc(tb, std::max<int64_t>(n, 1)));
    GD_CUDA_TRY(cudaMemcpyAsync(tb.p, b, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    db = tb.p;
  }
  A->rhs_override = db;
  const int rc = gd_solve(A, method, rtol, maxit, x, where, stats);
  A->rhs_override = nullptr;
  dfreeb(tb);
  return rc;
}
