// A7/A8/A10/A12 numeric phase: element integrals and the deterministic assembly of
// matrix values and right-hand side into the symbolic pattern.
//
// CellData integrate (src/CellData.jl:234-259) evaluates per cell
//   K_e[i,j] = sum_q w_q |J| kappa_c grad(phi_i).grad(phi_j),
//   b_e[i]   = sum_q w_q |J| f phi_i  - K_e[i,D] u_D          (Dirichlet lifting).
// A CartesianDiscreteModel cell is an axis-aligned box of the same size everywhere,
// so with a cell-constant kappa, K_e = kappa_c * Khat where Khat is integrated once
// on the device from the 1D shape tables (k_reference_element).  The assembly then
// gathers, for every stored entry (row node X, column node Y = X + offset), the
// cells that hold both nodes: value = sum_c kappa_c Khat[X in c, Y in c].  Each
// entry is produced by exactly one thread in a fixed cell order -- the sum of
// duplicates of Algebra.jl's COO + sparse() without atomics -- and written once,
// coalesced, in CSR order.  Ghost rows (SubAssembledRows) hold explicit zeros
// (Algebra.jl:1084): their range is cleared with a memset.
#include <cmath>
#include <string>
#include <vector>

#include "gd_internal.h"

namespace gd {

// ---- 1D Gauss-Legendre rule on [0,1] (Newton on the Legendre recurrence) -------
static void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
  x.assign(n, 0.0);
  w.assign(n, 0.0);
  const double pi = 3.14159265358979323846;
  for (int i = 0; i < n; ++i) {
    double z = std::cos(pi * (i + 0.75) / (n + 0.5));
    double pp = 0.0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1.0);
      double dz = p1 / pp;
      z -= dz;
      if (std::fabs(dz) < 1e-16) break;
    }
    // recompute derivative at the converged root
    double p1 = 1.0, p2 = 0.0;
    for (int j = 1; j <= n; ++j) {
      double p3 = p2;
      p2 = p1;
      p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j;
    }
    pp = n * (z * p1 - p2) / (z * z - 1.0);
    x[n - 1 - i] = 0.5 * (z + 1.0);
    w[n - 1 - i] = 1.0 / ((1.0 - z * z) * pp * pp);   // 2/((1-z^2)p'^2) scaled by 1/2
  }
}

// Equispaced Lagrange basis of order k on [0,1]: values and derivatives at x.
static void lagrange01(int k, double x, double* v, double* dv) {
  for (int a = 0; a <= k; ++a) {
    double xa = (double)a / k, den = 1.0, val = 1.0, der = 0.0;
    for (int b = 0; b <= k; ++b) {
      if (b == a) continue;
      double xb = (double)b / k;
      den *= (xa - xb);
    }
    for (int b = 0; b <= k; ++b) {
      if (b == a) continue;
      double xb = (double)b / k;
      val *= (x - xb);
      double t = 1.0;
      for (int c = 0; c <= k; ++c) {
        if (c == a || c == b) continue;
        t *= (x - (double)c / k);
      }
      der += t;
    }
    v[a] = val / den;
    dv[a] = der / den;
  }
}

// One block: Khat/Mhat/Fhat in lexicographic cell-local node order.
// tab layout: [nq][k+1] values, then [nq][k+1] derivatives, then [nq] weights.
__global__ void k_reference_element(int dim, int k, int nq, const double* __restrict__ tab, double h0, double h1,
                                    double h2, double* __restrict__ Kh, double* __restrict__ Mh,
                                    double* __restrict__ Fh) {
  extern __shared__ double s_tab[];
  const int kp1 = k + 1;
  const int ntab = 2 * nq * kp1 + nq;
  for (int i = threadIdx.x; i < ntab; i += blockDim.x) s_tab[i] = tab[i];
  __syncthreads();
  const double* V = s_tab;
  const double* D = s_tab + nq * kp1;
  const double* W = s_tab + 2 * nq * kp1;
  const double h[3] = {h0, h1, h2};
  int nn = 1, nqt = 1;
  for (int d = 0; d < dim; ++d) {
    nn *= kp1;
    nqt *= nq;
  }
  double detJ = 1.0;
  for (int d = 0; d < dim; ++d) detJ *= h[d];
  for (int ij = threadIdx.x; ij < nn * nn; ij += blockDim.x) {
    int i = ij / nn, j = ij % nn;
    int oi[3] = {0, 0, 0}, oj[3] = {0, 0, 0};
    for (int d = 0, ri = i, rj = j; d < dim; ++d) {
      oi[d] = ri % kp1;
      ri /= kp1;
      oj[d] = rj % kp1;
      rj /= kp1;
    }
    double ks = 0.0, ms = 0.0, fs = 0.0;
    for (int q = 0; q < nqt; ++q) {
      int qi[3] = {0, 0, 0};
      for (int d = 0, r = q; d < dim; ++d) {
        qi[d] = r % nq;
        r /= nq;
      }
      double w = detJ;
      double vi = 1.0, vj = 1.0;
      for (int d = 0; d < dim; ++d) {
        w *= W[qi[d]];
        vi *= V[qi[d] * kp1 + oi[d]];
        vj *= V[qi[d] * kp1 + oj[d]];
      }
      double gg = 0.0;
      for (int d = 0; d < dim; ++d) {
        double gi = D[qi[d] * kp1 + oi[d]] / h[d], gj = D[qi[d] * kp1 + oj[d]] / h[d];
        for (int e = 0; e < dim; ++e) {
          if (e == d) continue;
          gi *= V[qi[e] * kp1 + oi[e]];
          gj *= V[qi[e] * kp1 + oj[e]];
        }
        gg += gi * gj;
      }
      ks += w * gg;
      ms += w * vi * vj;
      if (j == 0) fs += w * vi;
    }
    Kh[ij] = ks;
    Mh[ij] = ms;
    if (j == 0) Fh[i] = fs;
  }
}

int reference_element(gd_asm* A, int degree) {
  const Geom& g = A->test->geom;
  cudaStream_t st = A->test->model->ctx->stream;
  if (A->ref_degree == degree && A->Khat.p) return GD_OK;
  int nq = (degree + 2) / 2;
  if (nq < 1 || nq > 16) return fail(GD_ERR_ARG, "quadrature degree out of range");
  std::vector<double> xq, wq;
  gauss_legendre01(nq, xq, wq);
  const int kp1 = g.k + 1;
  std::vector<double> tab(2 * nq * kp1 + nq);
  for (int q = 0; q < nq; ++q) {
    lagrange01(g.k, xq[q], &tab[q * kp1], &tab[nq * kp1 + q * kp1]);
    tab[2 * nq * kp1 + q] = wq[q];
  }
  int nn = 1;
  for (int d = 0; d < g.dim; ++d) nn *= kp1;
  GD_TRY(dalloc(A->Khat, nn * nn));
  GD_TRY(dalloc(A->Mhat, nn * nn));
  GD_TRY(dalloc(A->Fhat, nn));
  DBuf<double> dtab;
  GD_TRY(dalloc(dtab, tab.size()));
  GD_CUDA_TRY(cudaMemcpyAsync(dtab.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st));
  k_reference_element<<<1, 256, sizeof(double) * tab.size(), st>>>(g.dim, g.k, nq, dtab.p, g.h[0], g.h[1],
                                                                   g.dim == 3 ? g.h[2] : 1.0, A->Khat.p, A->Mhat.p,
                                                                   A->Fhat.p);
  GD_CUDA_TRY(cudaGetLastError());
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(dtab);
  A->ref_degree = degree;
  return GD_OK;
}

// ---- matrix values ------------------------------------------------------------------
template <int DIM, int K>
struct Lat {
  static constexpr int KP1 = K + 1;
  static constexpr int NN = DIM == 2 ? KP1 * KP1 : KP1 * KP1 * KP1;
  static constexpr int W = 2 * K + 1;
};

constexpr int kRowsPerBlock = 128;
constexpr int kNumericThreads = 256;

template <int DIM, int K, typename CodeT>
__global__ void __launch_bounds__(kNumericThreads)
k_numeric_matrix(Geom g, int64_t nrows_own, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ row_node,
                 const CodeT* __restrict__ code, const double* __restrict__ kappa, const double* __restrict__ Khat,
                 double* __restrict__ vals) {
  using L = Lat<DIM, K>;
  __shared__ double s_K[L::NN * L::NN];
  __shared__ int64_t s_rp[kRowsPerBlock + 1];
  __shared__ int32_t s_node[kRowsPerBlock];
  const int64_t r0 = (int64_t)blockIdx.x * kRowsPerBlock;
  const int nr = (int)((nrows_own - r0) < kRowsPerBlock ? (nrows_own - r0) : kRowsPerBlock);
  for (int i = threadIdx.x; i < L::NN * L::NN; i += blockDim.x) s_K[i] = Khat[i];
  for (int i = threadIdx.x; i <= nr; i += blockDim.x) s_rp[i] = rowptr[r0 + i];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) s_node[i] = row_node[r0 + i];
  __syncthreads();
  const int64_t e0 = s_rp[0], e1 = s_rp[nr];
  const int64_t N0 = g.N[0], N1 = g.N[1];
  const int64_t n0 = g.n[0], n1 = g.n[1];
  for (int64_t e = e0 + threadIdx.x; e < e1; e += blockDim.x) {
    int lo = 0, hi = nr - 1;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (s_rp[mid] <= e) lo = mid; else hi = mid - 1;
    }
    const int64_t lin = s_node[lo];
    int64_t X[3], Y[3];
    X[0] = lin % N0;
    if (DIM == 2) {
      X[1] = lin / N0;
    } else {
      int64_t t = lin / N0;
      X[1] = t % N1;
      X[2] = t / N1;
    }
    int c = (int)code[e];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      Y[d] = X[d] + (c % L::W) - K;
      c /= L::W;
    }
    int64_t clo[3], chi[3];
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      int64_t mn = X[d] < Y[d] ? X[d] : Y[d];
      int64_t mx = X[d] < Y[d] ? Y[d] : X[d];
      int64_t lo_c = mx <= K ? 0 : (mx - 1) / K;
      int64_t hi_c = mn / K;
      const int64_t nd = d == 0 ? n0 : (d == 1 ? n1 : g.n[2]);
      if (hi_c > nd - 1) hi_c = nd - 1;
      clo[d] = lo_c;
      chi[d] = hi_c;
    }
    double v = 0.0;
    if (DIM == 2) {
      for (int64_t cy = clo[1]; cy <= chi[1]; ++cy)
        for (int64_t cx = clo[0]; cx <= chi[0]; ++cx) {
          const int li = (int)(X[0] - K * cx) + L::KP1 * (int)(X[1] - K * cy);
          const int lj = (int)(Y[0] - K * cx) + L::KP1 * (int)(Y[1] - K * cy);
          v += __ldg(kappa + cx + n0 * cy) * s_K[li * L::NN + lj];
        }
    } else {
      for (int64_t cz = clo[2]; cz <= chi[2]; ++cz)
        for (int64_t cy = clo[1]; cy <= chi[1]; ++cy)
          for (int64_t cx = clo[0]; cx <= chi[0]; ++cx) {
            const int li = (int)(X[0] - K * cx) + L::KP1 * ((int)(X[1] - K * cy) + L::KP1 * (int)(X[2] - K * cz));
            const int lj = (int)(Y[0] - K * cx) + L::KP1 * ((int)(Y[1] - K * cy) + L::KP1 * (int)(Y[2] - K * cz));
            v += __ldg(kappa + cx + n0 * (cy + n1 * cz)) * s_K[li * L::NN + lj];
          }
    }
    vals[e] = v;
  }
}

// ---- right-hand side: f-term and Dirichlet lifting, one thread per owned row -----------
template <int DIM, int K>
__global__ void k_numeric_rhs(Geom g, int64_t nrows_own, const int32_t* __restrict__ row_node,
                              const double* __restrict__ kappa, const double* __restrict__ Khat,
                              const double* __restrict__ Mhat, const double* __restrict__ Fhat, double f_const,
                              const double* __restrict__ f_nodal, const double* __restrict__ u_dir,
                              double* __restrict__ rhs, int32_t* __restrict__ bad) {
  using L = Lat<DIM, K>;
  // The element tables are small and read through the read-only cache.
  const double* __restrict__ s_K = Khat;
  const double* __restrict__ s_M = Mhat;
  const double* __restrict__ s_F = Fhat;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows_own) return;
  int64_t lin = row_node[r];
  int64_t X[3] = {0, 0, 0};
  for (int d = 0; d < DIM; ++d) {
    X[d] = lin % g.N[d];
    lin /= g.N[d];
  }
  int64_t clo[3] = {0, 0, 0}, chi[3] = {0, 0, 0};
  for (int d = 0; d < DIM; ++d) {
    int64_t c = X[d] / K;
    if (X[d] % K == 0) {
      clo[d] = c - 1 < 0 ? 0 : c - 1;
      chi[d] = c > g.n[d] - 1 ? g.n[d] - 1 : c;
    } else {
      clo[d] = chi[d] = c;
    }
  }
  double b = 0.0;
  int nbad = 0;
  for (int64_t cz = clo[2]; cz <= chi[2]; ++cz)
    for (int64_t cy = clo[1]; cy <= chi[1]; ++cy)
      for (int64_t cx = clo[0]; cx <= chi[0]; ++cx) {
        const int64_t cc[3] = {cx, cy, cz};
        const double kap = kappa ? __ldg(kappa + cell_lin(g, cc)) : 1.0;
        if (!(kap > 0.0) || !isfinite(kap)) ++nbad;
        int li = 0;
        for (int d = DIM - 1; d >= 0; --d) li = li * L::KP1 + (int)(X[d] - K * cc[d]);
        if (!f_nodal) b += f_const * s_F[li];
        if (f_nodal || u_dir) {
          for (int lj = 0; lj < L::NN; ++lj) {
            int64_t Y[3] = {0, 0, 0};
            for (int d = 0, rest = lj; d < DIM; ++d) {
              Y[d] = K * cc[d] + rest % L::KP1;
              rest /= L::KP1;
            }
            const int64_t ylin = lattice_lin(g, Y);
            if (f_nodal) b += s_M[li * L::NN + lj] * __ldg(f_nodal + ylin);
            if (u_dir && node_is_dirichlet(g, Y)) b -= kap * s_K[li * L::NN + lj] * __ldg(u_dir + ylin);
          }
        }
      }
  rhs[r] = b;
  if (nbad) atomicAdd(bad, nbad);
}


// ---- Q1 fast path: one thread per owned row, values staged in shared memory ----------------
// Each thread loads the kappa of the 2^DIM cells around its node once and forms the
// whole 3^DIM stencil in registers (64 FMAs in 3D, unrolled at compile time); the row's
// pattern id gives the CSR position of every neighbour.  A 128-row chunk of values
// is contiguous in the CSR value array; it is written into a shared-memory buffer and
// streamed to global memory with one TMA bulk store (cp.async.bulk), double-buffered
// so the store of one chunk overlaps the computation of the next.  The right-hand side
// (source term and Dirichlet lifting) is fused.  Per row the kernel reads 4 bytes of
// node id and 2 bytes of pattern id; per entry it only writes the value.
constexpr int kQ1Rows = 128;

__device__ __forceinline__ void bulk_store_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  const uint32_t saddr = (uint32_t)__cvta_generic_to_shared(ssrc);
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(saddr), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory");
}
template <int N>
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

template <int DIM>
struct Q1 {
  static constexpr int S = DIM == 3 ? 27 : 9;   // stencil neighbours
  static constexpr int NC = 1 << DIM;           // cells around a node = nodes of a cell
  static constexpr int BUF = kQ1Rows * S + 2;   // doubles per staging buffer (even)
  static constexpr int TAB = 2 * NC * NC + NC + (NC & 1) + 4;   // Khat, Mhat, Fhat, warp sums
  static constexpr size_t SMEM = sizeof(double) * (TAB + 2 * BUF);
};

template <int DIM, bool FN, bool UD>
__global__ void __launch_bounds__(kQ1Rows)
k_numeric_q1(Geom g, int64_t nrows, int64_t nchunks, const int64_t* __restrict__ rowptr,
             const int32_t* __restrict__ row_node, const uint16_t* __restrict__ row_pat,
             const uint8_t* __restrict__ pat, const double* __restrict__ kappa, const double* __restrict__ Khat,
             const double* __restrict__ Mhat, const double* __restrict__ Fhat, double f_const,
             const double* __restrict__ f_nodal, const double* __restrict__ u_dir, double* __restrict__ vals,
             double* __restrict__ rhs, int32_t* __restrict__ bad) {
  using Q = Q1<DIM>;
  constexpr int S = Q::S, NC = Q::NC;
  extern __shared__ __align__(128) double smem[];
  double* sK = smem;
  double* sM = sK + NC * NC;
  double* sF = sM + NC * NC;
  int* s_wsum = (int*)(sF + NC + (NC & 1));
  double* buf0 = smem + Q::TAB;
  double* buf1 = buf0 + Q::BUF;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int i = tid; i < NC * NC; i += blockDim.x) {
    sK[i] = Khat[i];
    sM[i] = Mhat[i];
  }
  if (tid < NC) sF[tid] = Fhat[tid];
  __syncthreads();
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
  const int64_t n0 = g.n[0], n1 = g.n[1], n2 = DIM == 3 ? g.n[2] : 1;
  int nbad = 0;
  int b = 0;
  for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
    const int64_t r0 = c * kQ1Rows;
    const int64_t r = r0 + tid;
    const bool valid = r < nrows;
    double v[S];
    uint32_t pw[8];
    int len = 0;
    if (valid) {
      const uint32_t lin = (uint32_t)row_node[r];
      int64_t X[3];
      X[0] = lin % N0;
      if (DIM == 3) {
        const uint32_t t = lin / N0;
        X[1] = t % N1;
        X[2] = t / N1;
      } else {
        X[1] = lin / N0;
        X[2] = 0;
      }
      const uint4* pp = reinterpret_cast<const uint4*>(pat + (int64_t)row_pat[r] * 32);
      const uint4 p0 = __ldg(pp), p1 = __ldg(pp + 1);
      pw[0] = p0.x; pw[1] = p0.y; pw[2] = p0.z; pw[3] = p0.w;
      pw[4] = p1.x; pw[5] = p1.y; pw[6] = p1.z; pw[7] = p1.w;
      len = (int)(pw[7] >> 24);
      // kappa of the cells around X; slot a: cell X - 1 + bit_d(a) per direction
      double kap[NC];
      bool cin[NC];
#pragma unroll
      for (int a = 0; a < NC; ++a) {
        const int64_t cx = X[0] - 1 + (a & 1), cy = X[1] - 1 + ((a >> 1) & 1);
        const int64_t cz = DIM == 3 ? X[2] - 1 + ((a >> 2) & 1) : 0;
        cin[a] = cx >= 0 && cx < n0 && cy >= 0 && cy < n1 && (DIM == 2 || (cz >= 0 && cz < n2));
        kap[a] = cin[a] ? __ldg(kappa + cx + n0 * (cy + n1 * cz)) : 0.0;
        if (cin[a] && !(kap[a] > 0.0 && kap[a] < INFINITY)) ++nbad;
      }
      double bval = 0.0;
#pragma unroll
      for (int a = 0; a < NC; ++a)
        if (cin[a]) bval += f_const * sF[(NC - 1) - a];   // local index of X in slot a is (1-bit_d(a))
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const int o0 = s % 3 - 1, o1 = (s / 3) % 3 - 1, o2 = DIM == 3 ? s / 9 - 1 : 0;
        double acc = 0.0, macc = 0.0;
#pragma unroll
        for (int a = 0; a < NC; ++a) {
          const int a0 = a & 1, a1 = (a >> 1) & 1, a2 = DIM == 3 ? (a >> 2) & 1 : 0;
          const bool ok = (o0 == 0 || (o0 < 0) == (a0 == 0)) && (o1 == 0 || (o1 < 0) == (a1 == 0)) &&
                          (DIM == 2 || o2 == 0 || (o2 < 0) == (a2 == 0));
          if (ok) {
            const int lx = (1 - a0) + 2 * (1 - a1) + (DIM == 3 ? 4 * (1 - a2) : 0);
            const int ly = (1 - a0 + o0) + 2 * (1 - a1 + o1) + (DIM == 3 ? 4 * (1 - a2 + o2) : 0);
            acc += kap[a] * sK[lx * NC + ly];
            if (FN && cin[a]) macc += sM[lx * NC + ly];
          }
        }
        v[s] = acc;
        if (FN || UD) {
          const int64_t Y0 = X[0] + o0, Y1 = X[1] + o1, Y2 = X[2] + o2;
          const bool in = Y0 >= 0 && Y0 < g.N[0] && Y1 >= 0 && Y1 < g.N[1] && (DIM == 2 || (Y2 >= 0 && Y2 < g.N[2]));
          if (in) {
            const int64_t ylin = Y0 + g.N[0] * (Y1 + g.N[1] * Y2);
            if (FN) bval += macc * __ldg(f_nodal + ylin);
            if (UD) {
              const int64_t Yv[3] = {Y0, Y1, Y2};
              if (node_is_dirichlet(g, Yv)) bval -= acc * __ldg(u_dir + ylin);
            }
          }
        }
      }
      rhs[r] = bval;
    }
    // block-wide exclusive scan of the row lengths
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (tid == 0) bulk_wait_read<1>();   // the store that last read this buffer is done
    __syncthreads();
    if (lane == 31) s_wsum[wid] = incl;
    __syncthreads();
    int woff = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kQ1Rows / 32; ++w) {
      const int t = s_wsum[w];
      woff += w < wid ? t : 0;
      total += t;
    }
    const int off = woff + incl - len;
    const int64_t e0 = rowptr[r0];
    const int ofs = (int)(e0 & 1);   // keeps shared and global addresses congruent mod 16 bytes
    double* buf = b ? buf1 : buf0;
    if (valid) {
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const uint32_t pos = (pw[s >> 2] >> (8 * (s & 3))) & 0xFFu;
        if (pos != 0xFFu) buf[ofs + off + (int)pos] = v[s];
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0 && total > 0) {
      const int64_t e1 = e0 + total;
      if (ofs) vals[e0] = buf[1];                                   // unaligned head
      const int64_t ja = e0 + ofs, jb = e1 - (e1 & 1);
      if ((e1 & 1) && e1 - 1 >= ja) vals[e1 - 1] = buf[ofs + total - 1];   // unaligned tail
      if (jb > ja) bulk_store_s2g(vals + ja, buf + ofs + (ja - e0), (uint32_t)((jb - ja) * sizeof(double)));
    }
    if (tid == 0) bulk_commit();
    b ^= 1;
  }
  if (tid == 0) bulk_wait_all<0>();
  if (nbad) atomicAdd(bad, nbad);
}

template <int DIM, bool FN, bool UD>
static int launch_q1_inst(gd_asm* A, const double* kappa, const double* f_nodal, double f_const, const double* udir,
                          int32_t* bad, cudaStream_t st) {
  using Q = Q1<DIM>;
  static int blocks_per_sm = -1;
  static int num_sms = 0;
  auto kern = k_numeric_q1<DIM, FN, UD>;
  if (blocks_per_sm < 0) {
    GD_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q::SMEM));
    GD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, kQ1Rows, Q::SMEM));
    int dev = 0;
    GD_CUDA_TRY(cudaGetDevice(&dev));
    GD_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  const int64_t n = A->ngdofs;
  const int64_t nchunks = (n + kQ1Rows - 1) / kQ1Rows;
  int64_t grid = (int64_t)blocks_per_sm * num_sms;
  if (grid > nchunks) grid = nchunks;
  A->q1_grid = (int)grid;
  kern<<<(unsigned)grid, kQ1Rows, Q::SMEM, st>>>(A->test->geom, n, nchunks, A->rowptr.p, A->row_node.p,
                                                  A->row_pat.p, A->pat.p, kappa, A->Khat.p, A->Mhat.p, A->Fhat.p,
                                                  f_const, f_nodal, udir, A->vals.p, A->rhs.p, bad);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

template <int DIM>
static int launch_q1(gd_asm* A, const double* kappa, const double* f_nodal, double f_const, int32_t* bad,
                     cudaStream_t st) {
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  if (A->ngdofs == 0) return GD_OK;
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[1], st));
  int s;
  if (f_nodal && udir) s = launch_q1_inst<DIM, true, true>(A, kappa, f_nodal, 0.0, udir, bad, st);
  else if (f_nodal) s = launch_q1_inst<DIM, true, false>(A, kappa, f_nodal, 0.0, nullptr, bad, st);
  else if (udir) s = launch_q1_inst<DIM, false, true>(A, kappa, nullptr, f_const, udir, bad, st);
  else s = launch_q1_inst<DIM, false, false>(A, kappa, nullptr, f_const, nullptr, bad, st);
  if (s != GD_OK) return s;
  if (A->profiling) {   // one fused kernel: the rhs phase is empty
    GD_CUDA_TRY(cudaEventRecord(A->ev[2], st));
    GD_CUDA_TRY(cudaEventRecord(A->ev[3], st));
  }
  return GD_OK;
}

template <int DIM, int K>
static int launch_numeric(gd_asm* A, const double* kappa, const double* f_nodal, double f_const,
                          int32_t* bad, cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  if (R == 0) return GD_OK;
  const unsigned nb = (unsigned)((R + kRowsPerBlock - 1) / kRowsPerBlock);
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[1], st));
  if (A->code_bytes == 1)
    k_numeric_matrix<DIM, K, uint8_t><<<nb, kNumericThreads, 0, st>>>(g, R, A->rowptr.p, A->row_node.p, A->code.p,
                                                                       kappa, A->Khat.p, A->vals.p);
  else
    k_numeric_matrix<DIM, K, uint16_t><<<nb, kNumericThreads, 0, st>>>(g, R, A->rowptr.p, A->row_node.p,
                                                                        (const uint16_t*)A->code.p, kappa,
                                                                        A->Khat.p, A->vals.p);
  GD_CUDA_TRY(cudaGetLastError());
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[2], st));
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  k_numeric_rhs<DIM, K><<<(unsigned)((R + 127) / 128), 128, 0, st>>>(g, R, A->row_node.p, kappa, A->Khat.p,
                                                                     A->Mhat.p, A->Fhat.p, f_const, f_nodal, udir,
                                                                     A->rhs.p, bad);
  GD_CUDA_TRY(cudaGetLastError());
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[3], st));
  return GD_OK;
}

int numeric_impl(gd_asm* A, const gd_coeffs* c, bool sync) {
  if (!A || !c) return fail(GD_ERR_ARG, "gd_assemble_numeric: null argument");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_assemble_numeric: run gd_assemble_symbolic first");
  const Geom& g = A->test->geom;
  cudaStream_t st = A->test->model->ctx->stream;
  GD_TRY(reference_element(A, c->degree));
  int64_t ncells = 1, nnodes = 1;
  for (int d = 0; d < g.dim; ++d) {
    ncells *= g.n[d];
    nnodes *= g.N[d];
  }
  const double* kappa = c->kappa;
  const double* fn = c->f_nodal;
  if (c->where == GD_HOST) {
    if (kappa) {
      if (A->kappa_dev.n != (size_t)ncells) GD_TRY(dalloc(A->kappa_dev, ncells));
      GD_CUDA_TRY(cudaMemcpyAsync(A->kappa_dev.p, kappa, sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
      kappa = A->kappa_dev.p;
    }
    if (fn) {
      if (A->f_dev.n != (size_t)nnodes) GD_TRY(dalloc(A->f_dev, nnodes));
      GD_CUDA_TRY(cudaMemcpyAsync(A->f_dev.p, fn, sizeof(double) * nnodes, cudaMemcpyHostToDevice, st));
      fn = A->f_dev.p;
    }
  }
  if (!kappa) {   // kappa = 1
    if (A->kappa_dev.n != (size_t)ncells) GD_TRY(dalloc(A->kappa_dev, ncells));
    std::vector<double> ones(ncells, 1.0);
    GD_CUDA_TRY(cudaMemcpyAsync(A->kappa_dev.p, ones.data(), sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    kappa = A->kappa_dev.p;
  }
  // reduction/flag scratch lives in dred[0] (as int)
  if (!A->dred.p) GD_TRY(dalloc(A->dred, 4096));
  int32_t* bad = (int32_t*)A->dred.p;
  GD_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
  // Ghost rows (SubAssembledRows) hold explicit zeros: they were cleared by the symbolic
  // phase and no numeric kernel writes them.
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[0], st));
  int s = GD_ERR_UNSUPPORTED;
  if (A->fast_q1 && g.dim == 3) s = launch_q1<3>(A, kappa, fn, c->f_const, bad, st);
  else if (A->fast_q1 && g.dim == 2) s = launch_q1<2>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 2 && g.k == 1) s = launch_numeric<2, 1>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 2 && g.k == 2) s = launch_numeric<2, 2>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 2 && g.k == 3) s = launch_numeric<2, 3>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 3 && g.k == 1) s = launch_numeric<3, 1>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 3 && g.k == 2) s = launch_numeric<3, 2>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 3 && g.k == 3) s = launch_numeric<3, 3>(A, kappa, fn, c->f_const, bad, st);
  if (s != GD_OK) return s == GD_ERR_UNSUPPORTED ? fail(s, "numeric: unsupported dim/order") : s;
  if (sync) {
    int32_t hbad = 0;
    GD_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    if (hbad) return fail(GD_ERR_NUMERIC, "numeric: kappa is not finite and positive in " + std::to_string(hbad) +
                                              " cell visits");
  }
  A->numeric_done = true;
  return GD_OK;
}

}  // namespace gd

extern "C" int gd_assembler_set_profiling(gd_asm* A, int on) {
  if (!A) return gd::fail(GD_ERR_ARG, "gd_assembler_set_profiling: null assembler");
  if (on && !A->ev[0])
    for (int i = 0; i < 4; ++i) GD_CUDA_TRY(cudaEventCreate(&A->ev[i]));
  A->profiling = on != 0;
  return GD_OK;
}

extern "C" int gd_assembler_phase_times(const gd_asm* A, double* ms0, double* ms1, double* ms2) {
  if (!A || !A->ev[0]) return gd::fail(GD_ERR_STATE, "gd_assembler_phase_times: profiling was not enabled");
  GD_CUDA_TRY(cudaEventSynchronize(A->ev[3]));
  float t[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i) GD_CUDA_TRY(cudaEventElapsedTime(&t[i], A->ev[i], A->ev[i + 1]));
  if (ms0) *ms0 = t[0];
  if (ms1) *ms1 = t[1];
  if (ms2) *ms2 = t[2];
  return GD_OK;
}

extern "C" int gd_assembler_counts(const gd_asm* A, int64_t* ngdofs, int64_t* nnz_owned, int64_t* nnz_total,
                                   int32_t* kernels) {
  if (!A || !A->symbolic_done) return gd::fail(GD_ERR_STATE, "gd_assembler_counts: run gd_assemble_symbolic first");
  if (ngdofs) *ngdofs = A->ngdofs;
  if (nnz_owned) *nnz_owned = A->nnz_own;
  if (nnz_total) *nnz_total = A->nnz_total;
  if (kernels) *kernels = A->fast_q1 ? 1 : 2;   // fused Q1 kernel, or k_numeric_matrix + k_numeric_rhs
  return GD_OK;
}

extern "C" int gd_assemble_numeric(gd_asm* A, const gd_coeffs* c) { return gd::numeric_impl(A, c, true); }
extern "C" int gd_assemble_numeric_async(gd_asm* A, const gd_coeffs* c) { return gd::numeric_impl(A, c, false); }
