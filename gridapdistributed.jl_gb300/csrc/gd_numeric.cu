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
#include <cstring>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_rows.cuh"

namespace gd {

// ---- 1D Gauss-Legendre rule on [0,1] (Newton on the Legendre recurrence) -------
void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w) {
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
void lagrange01(int k, double x, double* v, double* dv) {
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

// ---- Q_k values and right-hand side (row bodies in gd_rows.cuh) ---------------------------
// Lane groups of a warp take owned rows; the reference stiffness table is staged in
// shared memory.
template <int DIM, int K, typename CodeT>
__global__ void __launch_bounds__(256)
k_numeric_qk_rows(Geom g, int64_t nrows_own, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ row_node,
                  const CodeT* __restrict__ code, const double* __restrict__ kappa, const double* __restrict__ Khat,
                  double* __restrict__ vals) {
  using L = Lat<DIM, K>;
  constexpr int RPW = RowLanes<DIM, K>::RPW;
  __shared__ double s_K[L::NN * L::NN];
  __shared__ double s_kap[8][32];
  __shared__ int s_lx[8][32];
  __shared__ uint16_t s_tab[EntryTab<DIM, K>::SIZE];
  for (int i = threadIdx.x; i < L::NN * L::NN; i += blockDim.x) s_K[i] = Khat[i];
  build_entry_tab<DIM, K>(s_tab);
  __syncthreads();
  const int wl = threadIdx.x >> 5;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t rb = warp * RPW; rb < nrows_own; rb += nwarps * RPW)
    qk_matrix_rows<DIM, K, CodeT>(g, rb, nrows_own, rowptr, row_node, code, kappa, s_K, s_tab, vals, s_kap[wl],
                                  s_lx[wl]);
}

// one thread per owned row
template <int DIM, int K>
__global__ void k_numeric_rhs(Geom g, int64_t nrows_own, const int32_t* __restrict__ row_node,
                              const double* __restrict__ kappa, const double* __restrict__ Khat,
                              const double* __restrict__ Mhat, const double* __restrict__ Fhat, double f_const,
                              const double* __restrict__ f_nodal, const double* __restrict__ u_dir,
                              double* __restrict__ rhs, int32_t* __restrict__ bad) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows_own) return;
  const int nbad = qk_rhs_row<DIM, K>(g, r, row_node, kappa, Khat, Mhat, Fhat, f_const, f_nodal, u_dir, rhs);
  if (nbad) atomicAdd(bad, nbad);
}


// ---- Q1 fast path: one thread per owned row, values staged in shared memory ----------------
// Each thread loads the coefficients of the 2^DIM cells around its node once and forms
// the whole 3^DIM stencil in registers from class sums (q1_row_values: on cube cells
// about 16 FP64 operations per 3D row, a separable subset-sum tree on other boxes); the
// row's pattern id gives the CSR position of every neighbour.  A chunk of consecutive
// rows (64, 128 or 256, the launch shape the autotuner picks, with one or two staging
// buffers) is contiguous in the CSR value array; it is written into a shared-memory
// buffer and streamed to global memory with one TMA bulk store (cp.async.bulk), the
// unaligned first and last entries by plain stores, double-buffered so that the store of
// one chunk overlaps the computation of the next.  The row ids, patterns and coefficients
// of the next chunk are prefetched while the current one is stored.  The right-hand side
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

template <int DIM, int ROWS = kQ1Rows, int NBUF = 2>
struct Q1 {
  static constexpr int S = DIM == 3 ? 27 : 9;   // stencil neighbours
  static constexpr int NC = 1 << DIM;           // cells around a node = nodes of a cell
  static constexpr int BUF = ROWS * S + 2;      // doubles per staging buffer (even)
  static constexpr int HEAD = 8 + 72;           // warp sums, mass table
  static constexpr size_t SMEM = sizeof(double) * (HEAD + NBUF * BUF);
};

// Launch shapes the autotuner chooses from: rows per chunk (= threads per CTA) and
// staging buffers per CTA (2 overlaps a chunk's bulk store with the next chunk; 1
// halves shared memory so twice as many CTAs fit on an SM).
struct Q1Shape {
  int rows, nbuf;
};
constexpr Q1Shape kQ1Shapes[] = {{128, 2}, {128, 1}, {64, 2}, {64, 1}, {256, 1}};
constexpr int kNumQ1Shapes = 5;

// Element-matrix classes of an axis-aligned Q1 cell.  With exact (degree >= 2)
// quadrature, K_e[i][j] depends only on which coordinates of nodes i and j differ
// (class bits x=1, y=2, z=4), and so does M_e; the load int(phi_i) is the same for
// every node.  So the value of the entry (X, X+o) is K[class(o)] * (sum of kappa over
// the valid cells that hold both nodes).
struct Q1Const {
  double Kc[8];        // stiffness per class
  double Mtab[8][9];   // mass per class times the number of valid shared cells
  double btab[9];      // f * load per node times the number of valid cells
  double ratio;        // Kc[0] / Kc[3] (cube mode)
  int kzero[8];        // class whose stiffness vanishes exactly in exact arithmetic
};

// The kappa of a cell is a finite positive double: checked on the bits (integer pipe).
__device__ __forceinline__ bool bad_coefficient(double k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(k);
  return (b >> 63) != 0ull || ((b >> 52) & 0x7FFull) == 0x7FFull || b == 0ull;
}

// Cube cells: w_c = Kc[3] * kappa_c once per cell (validated here), so a 3D row needs
// 12 adds for the face diagonals, 3 adds + 1 multiply for the diagonal, and nothing
// for the corners (w itself) and the edge neighbours (exactly 0 on a cube).
// w = scale * kappa per cell with the coefficient check; 16-byte accesses, four of them in
// flight per thread (8 cells), kappa read with streaming loads (not reused) so that w,
// which the matrix kernel reads next, keeps the L2.  kappa must be 16-byte aligned (w
// always is), otherwise k_prescale_scalar runs.
__global__ void __launch_bounds__(256)
k_prescale(int64_t ncells, const double* __restrict__ kappa, double scale, double* __restrict__ w,
           int32_t* __restrict__ bad) {
  int nbad = 0;
  const int64_t n2 = ncells >> 1;   // double2 units
  const double2* k2 = reinterpret_cast<const double2*>(kappa);
  double2* w2 = reinterpret_cast<double2*>(w);
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i0 < n2; i0 += 4 * stride) {
    double2 a[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t i = i0 + u * stride;
      a[u] = i < n2 ? __ldcs(k2 + i) : make_double2(1.0, 1.0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t i = i0 + u * stride;
      if (i >= n2) break;
      nbad += bad_coefficient(a[u].x) + bad_coefficient(a[u].y);
      w2[i] = make_double2(scale * a[u].x, scale * a[u].y);
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && (ncells & 1)) {   // tail
    const double k = kappa[ncells - 1];
    nbad += bad_coefficient(k);
    w[ncells - 1] = scale * k;
  }
  if (nbad) atomicAdd(bad, nbad);
}

__global__ void k_prescale_scalar(int64_t ncells, const double* __restrict__ kappa, double scale,
                                  double* __restrict__ w, int32_t* __restrict__ bad) {
  int nbad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ncells; i += (int64_t)gridDim.x * blockDim.x) {
    const double k = kappa[i];
    nbad += bad_coefficient(k);
    w[i] = scale * k;
  }
  if (nbad) atomicAdd(bad, nbad);
}

// values of one row in canonical neighbour order (offsets lexicographic, x fastest)
template <int DIM, bool CUBE>
__device__ __forceinline__ void q1_row_values(const double* kap, const Q1Const& q, double* v) {
  if (CUBE) {   // DIM == 3; kap holds w = Kc[3] * kappa
    double P[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) P[a] = kap[a] + kap[a + 4];   // z pairs at (a0, a1)
#pragma unroll
    for (int s = 0; s < 27; ++s) {
      const int o0 = s % 3 - 1, o1 = (s / 3) % 3 - 1, o2 = s / 9 - 1;
      const int nz = (o0 != 0) + (o1 != 0) + (o2 != 0);
      const int a0 = (o0 + 1) >> 1, a1 = (o1 + 1) >> 1, a2 = (o2 + 1) >> 1;
      if (nz == 0) {
        v[s] = q.ratio * ((P[0] + P[1]) + (P[2] + P[3]));
      } else if (nz == 1) {
        v[s] = 0.0;
      } else if (nz == 3) {
        v[s] = kap[a0 + 2 * a1 + 4 * a2];
      } else if (o2 == 0) {
        v[s] = P[a0 + 2 * a1];
      } else if (o1 == 0) {
        v[s] = kap[a0 + 4 * a2] + kap[a0 + 2 + 4 * a2];
      } else {
        v[s] = kap[2 * a1 + 4 * a2] + kap[1 + 2 * a1 + 4 * a2];
      }
    }
    return;
  }
  // general axis-aligned box: subset sums by a separable tree (x, then y, then z)
  // sx[ch][a1][a2]: ch 0 -> cell a0=0, 1 -> a0=1, 2 -> both
  constexpr int NZ = DIM == 3 ? 2 : 1;
  double sx[3][2][NZ];
#pragma unroll
  for (int a1 = 0; a1 < 2; ++a1)
#pragma unroll
    for (int a2 = 0; a2 < NZ; ++a2) {
      const double k0 = kap[2 * a1 + 4 * a2], k1 = kap[1 + 2 * a1 + 4 * a2];
      sx[0][a1][a2] = k0;
      sx[1][a1][a2] = k1;
      sx[2][a1][a2] = k0 + k1;
    }
  double sxy[3][3][NZ];
#pragma unroll
  for (int cx = 0; cx < 3; ++cx)
#pragma unroll
    for (int a2 = 0; a2 < NZ; ++a2) {
      sxy[cx][0][a2] = sx[cx][0][a2];
      sxy[cx][1][a2] = sx[cx][1][a2];
      sxy[cx][2][a2] = sx[cx][0][a2] + sx[cx][1][a2];
    }
#pragma unroll
  for (int s = 0; s < Q1<DIM>::S; ++s) {
    const int o0 = s % 3 - 1, o1 = (s / 3) % 3 - 1, o2 = DIM == 3 ? s / 9 - 1 : 0;
    const int c0 = o0 == 0 ? 2 : (o0 + 1) >> 1, c1 = o1 == 0 ? 2 : (o1 + 1) >> 1;
    double S;
    if (DIM == 2) {
      S = sxy[c0][c1][0];
    } else {
      const int c2 = o2 == 0 ? 2 : (o2 + 1) >> 1;
      S = c2 == 2 ? sxy[c0][c1][0] + sxy[c0][c1][NZ - 1] : sxy[c0][c1][c2 == 2 ? 0 : c2];
    }
    const int cls = (o0 != 0) | ((o1 != 0) << 1) | ((o2 != 0) << 2);
    v[s] = q.kzero[cls] ? 0.0 : q.Kc[cls] * S;
  }
}

// Per-row inputs of one chunk, loaded one chunk ahead (software pipeline): the
// row ids are fetched two chunks ahead, the coefficients and pattern one chunk ahead,
// so their latency overlaps the staging and bulk store of the current chunk.
template <int DIM>
struct Q1Row {
  int64_t X[3];
  uint32_t pw[8];
  double kap[1 << DIM];
  int ncell;
  uint32_t cmask;   // cells inside the mesh
  bool valid;
};

template <int DIM, bool CUBE>
__device__ __forceinline__ void q1_load_row(const Geom& g, int64_t r, int64_t nrows, uint32_t lin, uint32_t pid,
                                            const uint8_t* __restrict__ pat, const double* __restrict__ kappa,
                                            Q1Row<DIM>& R) {
  constexpr int NC = 1 << DIM;
  R.valid = r < nrows;
  R.ncell = 0;
  R.cmask = 0;
  if (!R.valid) {
    for (int i = 0; i < 8; ++i) R.pw[i] = 0xFFFFFFFFu;
    R.pw[7] = 0x00FFFFFFu;   // length 0
    return;
  }
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
  R.X[0] = lin % N0;
  if (DIM == 3) {
    const uint32_t t = lin / N0;
    R.X[1] = t % N1;
    R.X[2] = t / N1;
  } else {
    R.X[1] = lin / N0;
    R.X[2] = 0;
  }
  const uint4* pp = reinterpret_cast<const uint4*>(pat + (int64_t)pid * 32);
  const uint4 p0 = __ldg(pp), p1 = __ldg(pp + 1);
  R.pw[0] = p0.x; R.pw[1] = p0.y; R.pw[2] = p0.z; R.pw[3] = p0.w;
  R.pw[4] = p1.x; R.pw[5] = p1.y; R.pw[6] = p1.z; R.pw[7] = p1.w;
  const int64_t n0 = g.n[0], n1 = g.n[1], n2 = DIM == 3 ? g.n[2] : 1;
#pragma unroll
  for (int a = 0; a < NC; ++a) {
    const int64_t cx = R.X[0] - 1 + (a & 1), cy = R.X[1] - 1 + ((a >> 1) & 1);
    const int64_t cz = DIM == 3 ? R.X[2] - 1 + ((a >> 2) & 1) : 0;
    const bool cin = cx >= 0 && cx < n0 && cy >= 0 && cy < n1 && (DIM == 2 || (cz >= 0 && cz < n2));
    R.kap[a] = cin ? __ldg(kappa + cx + n0 * (cy + n1 * cz)) : 0.0;
    R.ncell += cin;
    R.cmask |= (uint32_t)cin << a;
  }
}

template <int DIM, bool CUBE, bool FN, bool UD, int ROWS, int NBUF>
__global__ void __launch_bounds__(ROWS)
k_numeric_q1(Geom g, Q1Const q, int64_t nrows, int64_t nchunks, const int64_t* __restrict__ rowptr,
             const int32_t* __restrict__ row_node, const uint16_t* __restrict__ row_pat,
             const uint8_t* __restrict__ pat, const double* __restrict__ kappa, const double* __restrict__ f_nodal,
             const double* __restrict__ u_dir, double* __restrict__ vals, double* __restrict__ rhs,
             int32_t* __restrict__ bad) {
  using Q = Q1<DIM, ROWS, NBUF>;
  constexpr int S = Q::S, NC = Q::NC;
  extern __shared__ __align__(128) double smem[];
  int* s_wsum = (int*)smem;
  double* s_mtab = smem + 8;   // mass per class and shared-cell count (kernel parameters
                               // are not indexed dynamically: that would go to local memory)
  double* buf0 = smem + Q::HEAD;
  double* buf1 = NBUF == 2 ? buf0 + Q::BUF : buf0;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (FN)
    for (int i = tid; i < 72; i += blockDim.x) s_mtab[i] = q.Mtab[i / 9][i % 9];
  if (FN) __syncthreads();
  const int64_t G = gridDim.x;
  int nbad = 0;
  int b = 0;
  // pipeline prologue: data of the first chunk, ids of the second
  int64_t c = blockIdx.x;
  Q1Row<DIM> cur;
  int64_t e0_cur = c < nchunks ? rowptr[c * ROWS] : 0;
  {
    const int64_t r = c * ROWS + tid;
    const bool ok = c < nchunks && r < nrows;
    const uint32_t lin = ok ? (uint32_t)row_node[r] : 0u;
    const uint32_t pid = ok ? (uint32_t)row_pat[r] : 0u;
    q1_load_row<DIM, CUBE>(g, ok ? r : nrows, nrows, lin, pid, pat, kappa, cur);
  }
  uint32_t nlin = 0, npid = 0;
  int64_t e0_next = c + G < nchunks ? rowptr[(c + G) * ROWS] : 0;
  {
    const int64_t r = (c + G) * ROWS + tid;
    if (c + G < nchunks && r < nrows) {
      nlin = (uint32_t)row_node[r];
      npid = (uint32_t)row_pat[r];
    }
  }
  for (; c < nchunks; c += G) {
    const int64_t r0 = c * ROWS;
    const int64_t r = r0 + tid;
    const int len = (int)(cur.pw[7] >> 24);
    // block-wide exclusive scan of the row lengths
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    if (tid == 0) bulk_wait_read<NBUF - 1>();   // the store that last read this buffer is done
    __syncthreads();
    if (lane == 31) s_wsum[wid] = incl;
    __syncthreads();
    int woff = 0, total = 0;
#pragma unroll
    for (int w = 0; w < ROWS / 32; ++w) {
      const int t = s_wsum[w];
      woff += w < wid ? t : 0;
      total += t;
    }
    const int off = woff + incl - len;
    const int64_t e0 = e0_cur;
    const int ofs = (int)(e0 & 1);   // keeps shared and global addresses congruent mod 16 bytes
    double* buf = b ? buf1 : buf0;
    if (cur.valid) {
      if (!CUBE)
#pragma unroll
        for (int a = 0; a < NC; ++a) nbad += ((cur.cmask >> a) & 1u) && bad_coefficient(cur.kap[a]);
      double v[S];
      q1_row_values<DIM, CUBE>(cur.kap, q, v);
      double* dst = buf + ofs + off;
#pragma unroll
      for (int s = 0; s < S; ++s) {
        const uint32_t pos = (cur.pw[s >> 2] >> (8 * (s & 3))) & 0xFFu;
        if (pos != 0xFFu) dst[pos] = v[s];
      }
      double bval = 0.0;
      if (!FN) {
#pragma unroll
        for (int n = 0; n <= NC; ++n) bval = cur.ncell == n ? q.btab[n] : bval;
      }
      if (FN || UD) {
        const int64_t n0 = g.n[0], n1 = g.n[1], n2 = DIM == 3 ? g.n[2] : 1;
#pragma unroll
        for (int s = 0; s < S; ++s) {
          const int o0 = s % 3 - 1, o1 = (s / 3) % 3 - 1, o2 = DIM == 3 ? s / 9 - 1 : 0;
          const int64_t Y0 = cur.X[0] + o0, Y1 = cur.X[1] + o1, Y2 = cur.X[2] + o2;
          const bool in = Y0 >= 0 && Y0 < g.N[0] && Y1 >= 0 && Y1 < g.N[1] && (DIM == 2 || (Y2 >= 0 && Y2 < g.N[2]));
          if (!in) continue;
          const int64_t ylin = Y0 + g.N[0] * (Y1 + g.N[1] * Y2);
          if (FN) {   // number of valid cells shared by X and Y
            int cnt = 0;
#pragma unroll
            for (int a = 0; a < NC; ++a) {
              const int a0 = a & 1, a1 = (a >> 1) & 1, a2 = (a >> 2) & 1;
              const bool sh = (o0 == 0 || (o0 < 0) == (a0 == 0)) && (o1 == 0 || (o1 < 0) == (a1 == 0)) &&
                              (DIM == 2 || o2 == 0 || (o2 < 0) == (a2 == 0));
              const int64_t cx = cur.X[0] - 1 + a0, cy = cur.X[1] - 1 + a1, cz = DIM == 3 ? cur.X[2] - 1 + a2 : 0;
              cnt += sh && cx >= 0 && cx < n0 && cy >= 0 && cy < n1 && (DIM == 2 || (cz >= 0 && cz < n2));
            }
            const int cls = (o0 != 0) | ((o1 != 0) << 1) | ((o2 != 0) << 2);
            bval += s_mtab[cls * 9 + cnt] * __ldg(f_nodal + ylin);
          }
          if (UD && Y0 >= 0) {
            const bool dir = (g.dsides[0] && Y0 == 0) || (g.dsides[1] && Y0 == g.N[0] - 1) ||
                             (g.dsides[2] && Y1 == 0) || (g.dsides[3] && Y1 == g.N[1] - 1) ||
                             (DIM == 3 && ((g.dsides[4] && Y2 == 0) || (g.dsides[5] && Y2 == g.N[2] - 1)));
            if (dir) bval -= v[s] * __ldg(u_dir + ylin);
          }
        }
      }
      rhs[r] = bval;
    }
    // prefetch: data of the next chunk (its ids arrived one iteration ago), ids of the one after
    {
      const int64_t cn = c + G;
      const int64_t rn = cn * ROWS + tid;
      const bool okn = cn < nchunks && rn < nrows;
      q1_load_row<DIM, CUBE>(g, okn ? rn : nrows, nrows, nlin, npid, pat, kappa, cur);
      e0_cur = e0_next;
      e0_next = c + 2 * G < nchunks ? rowptr[(c + 2 * G) * ROWS] : 0;
      const int64_t r2 = (c + 2 * G) * ROWS + tid;
      nlin = 0;
      npid = 0;
      if (c + 2 * G < nchunks && r2 < nrows) {
        nlin = (uint32_t)row_node[r2];
        npid = (uint32_t)row_pat[r2];
      }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0 && total > 0) {
      const int64_t e1 = e0 + total;
      if (ofs) vals[e0] = buf[1];                                          // unaligned head
      const int64_t ja = e0 + ofs, jb = e1 - (e1 & 1);
      if ((e1 & 1) && e1 - 1 >= ja) vals[e1 - 1] = buf[ofs + total - 1];   // unaligned tail
      if (jb > ja) bulk_store_s2g(vals + ja, buf + ofs + (ja - e0), (uint32_t)((jb - ja) * sizeof(double)));
    }
    if (tid == 0) bulk_commit();
    if (NBUF == 2) b ^= 1;
  }
  if (tid == 0) bulk_wait_all<0>();
  if (nbad) atomicAdd(bad, nbad);
}

// Class constants from the device reference element (lexicographic local nodes).
static int q1_constants(gd_asm* A, double f_const, Q1Const& q, bool& cube) {
  const Geom& g = A->test->geom;
  cudaStream_t st = A->test->model->ctx->stream;
  const int NC = 1 << g.dim;
  if (A->q1c_degree == A->ref_degree) {   // cached for this reference element
    q = *reinterpret_cast<const Q1Const*>(A->q1c_blob.data());
    for (int n = 0; n <= 8; ++n) q.btab[n] = f_const * A->q1c_f0 * n;
    cube = A->q1c_cube;
    return GD_OK;
  }
  std::vector<double> K(NC * NC), M(NC * NC), F(NC);
  GD_CUDA_TRY(cudaMemcpyAsync(K.data(), A->Khat.p, sizeof(double) * NC * NC, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(M.data(), A->Mhat.p, sizeof(double) * NC * NC, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(F.data(), A->Fhat.p, sizeof(double) * NC, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  memset(&q, 0, sizeof(q));
  // node 0 is (0,0,0); node cls has the coordinate bits of the class
  for (int cls = 0; cls < 8; ++cls) {
    if (cls >= NC) continue;
    q.Kc[cls] = K[0 * NC + cls];
    for (int n = 0; n <= 8; ++n) q.Mtab[cls][n] = M[0 * NC + cls] * n;
  }
  for (int n = 0; n <= 8; ++n) q.btab[n] = f_const * F[0] * n;
  const double k0 = std::fabs(q.Kc[0]);
  // the class rule holds only if every entry equals its class representative
  bool classes_ok = true;
  for (int i = 0; i < NC; ++i)
    for (int j = 0; j < NC; ++j) {
      const int cls = (i ^ j);
      if (std::fabs(K[i * NC + j] - q.Kc[cls]) > 1e-14 * k0 || std::fabs(M[i * NC + j] - M[cls]) > 1e-14 * std::fabs(M[0]))
        classes_ok = false;
    }
  for (int i = 0; i < NC; ++i)
    if (std::fabs(F[i] - F[0]) > 1e-14 * std::fabs(F[0])) classes_ok = false;
  if (!classes_ok) return fail(GD_ERR_UNSUPPORTED, "Q1 element matrix does not have the box-cell class structure");
  for (int cls = 0; cls < NC; ++cls) q.kzero[cls] = std::fabs(q.Kc[cls]) <= 1e-14 * k0;
  cube = g.dim == 3 && q.kzero[1] && q.kzero[2] && q.kzero[4] &&
         std::fabs(q.Kc[3] - q.Kc[7]) <= 1e-14 * k0 && std::fabs(q.Kc[5] - q.Kc[7]) <= 1e-14 * k0 &&
         std::fabs(q.Kc[6] - q.Kc[7]) <= 1e-14 * k0 && q.Kc[3] != 0.0;
  q.ratio = cube ? q.Kc[0] / q.Kc[3] : 0.0;
  A->q1c_blob.assign(reinterpret_cast<const char*>(&q), reinterpret_cast<const char*>(&q) + sizeof(q));
  A->q1c_f0 = F[0];
  A->q1c_cube = cube;
  A->q1c_degree = A->ref_degree;
  return GD_OK;
}

template <int DIM, bool CUBE, bool FN, bool UD, int ROWS, int NBUF>
static int launch_q1_inst(gd_asm* A, const Q1Const& q, const double* kappa, const double* f_nodal,
                          const double* udir, int32_t* bad, cudaStream_t st) {
  using Q = Q1<DIM, ROWS, NBUF>;
  static int blocks_per_sm = -1;
  static int num_sms = 0;
  auto kern = k_numeric_q1<DIM, CUBE, FN, UD, ROWS, NBUF>;
  if (blocks_per_sm < 0) {
    GD_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)Q::SMEM));
    GD_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks_per_sm, kern, ROWS, Q::SMEM));
    int dev = 0;
    GD_CUDA_TRY(cudaGetDevice(&dev));
    GD_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    if (blocks_per_sm < 1) blocks_per_sm = 1;
  }
  // owned rows r0 .. r1-1: the row-indexed arrays are offset; rowptr holds absolute
  // positions in vals, so the kernel needs no row offset of its own
  const int64_t r0 = A->q1_rows[0], r1 = A->q1_rows[1] >= 0 ? A->q1_rows[1] : A->ngdofs;
  const int64_t n = r1 - r0;
  if (n <= 0) return GD_OK;
  const int64_t nchunks = (n + ROWS - 1) / ROWS;
  int64_t grid = (int64_t)blocks_per_sm * num_sms;   // persistent: one wave of resident CTAs
  if (grid > nchunks) grid = nchunks;
  A->q1_grid = (int)grid;
  kern<<<(unsigned)grid, ROWS, Q::SMEM, st>>>(A->test->geom, q, n, nchunks, A->rowptr.p + r0, A->row_node.p + r0,
                                               A->row_pat.p + r0, A->pat.p, kappa, f_nodal, udir, A->vals.p,
                                               A->rhs.p + r0, bad);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

template <int DIM, bool CUBE, bool FN, bool UD>
static int launch_q1_shape(gd_asm* A, int shape, const Q1Const& q, const double* kappa, const double* f_nodal,
                           const double* udir, int32_t* bad, cudaStream_t st) {
  switch (shape) {
    case 1: return launch_q1_inst<DIM, CUBE, FN, UD, 128, 1>(A, q, kappa, f_nodal, udir, bad, st);
    case 2: return launch_q1_inst<DIM, CUBE, FN, UD, 64, 2>(A, q, kappa, f_nodal, udir, bad, st);
    case 3: return launch_q1_inst<DIM, CUBE, FN, UD, 64, 1>(A, q, kappa, f_nodal, udir, bad, st);
    case 4: return launch_q1_inst<DIM, CUBE, FN, UD, 256, 1>(A, q, kappa, f_nodal, udir, bad, st);
    default: return launch_q1_inst<DIM, CUBE, FN, UD, 128, 2>(A, q, kappa, f_nodal, udir, bad, st);
  }
}

template <int DIM, bool CUBE>
static int launch_q1_mode(gd_asm* A, int shape, const Q1Const& q, const double* kappa, const double* f_nodal,
                          const double* udir, int32_t* bad, cudaStream_t st) {
  if (f_nodal && udir) return launch_q1_shape<DIM, CUBE, true, true>(A, shape, q, kappa, f_nodal, udir, bad, st);
  if (f_nodal) return launch_q1_shape<DIM, CUBE, true, false>(A, shape, q, kappa, f_nodal, nullptr, bad, st);
  if (udir) return launch_q1_shape<DIM, CUBE, false, true>(A, shape, q, kappa, nullptr, udir, bad, st);
  return launch_q1_shape<DIM, CUBE, false, false>(A, shape, q, kappa, nullptr, nullptr, bad, st);
}

template <int DIM>
static int launch_q1(gd_asm* A, const double* kappa, const double* f_nodal, double f_const, int32_t* bad,
                     cudaStream_t st) {
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  if (A->ngdofs == 0) return GD_OK;
  Q1Const q;
  bool cube = false;
  GD_TRY(q1_constants(A, f_nodal ? 0.0 : f_const, q, cube));
  A->mf_ratio = q.ratio;
  A->mf_k2 = q.Kc[3];
  int64_t ncells = 1;
  for (int d = 0; d < DIM; ++d) ncells *= A->test->geom.n[d];
  const double* coef = kappa;
  if (cube) {   // w = Kc[3] * kappa, validated on the way
    if (A->w_cells.n != (size_t)ncells) GD_TRY(dalloc(A->w_cells, ncells));
    if (((uintptr_t)kappa & 15) == 0) {
      const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((ncells / 8 + 255) / 256, 152 * 8));
      k_prescale<<<blocks, 256, 0, st>>>(ncells, kappa, q.Kc[3], A->w_cells.p, bad);
    } else {
      const int blocks = (int)std::min<int64_t>((ncells + 255) / 256, 4096);
      k_prescale_scalar<<<blocks, 256, 0, st>>>(ncells, kappa, q.Kc[3], A->w_cells.p, bad);
    }
    GD_CUDA_TRY(cudaGetLastError());
    coef = A->w_cells.p;
  }
  // autotune the launch shape once per assembler: time every shape with CUDA events
  // (each run writes the same values), the shapes in turn over several rounds so that a
  // drift of the clocks or the memory state does not favour one of them, and keep the
  // fastest by its best time (the first round only warms up)
  if (A->q1_shape < 0) {
    constexpr int kRounds = 6;
    cudaEvent_t e0, e1;
    GD_CUDA_TRY(cudaEventCreate(&e0));
    GD_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms[kNumQ1Shapes];
    for (int sh = 0; sh < kNumQ1Shapes; ++sh) best_ms[sh] = 1e30f;
    for (int rep = 0; rep < kRounds; ++rep) {
      for (int sh = 0; sh < kNumQ1Shapes; ++sh) {
        GD_CUDA_TRY(cudaEventRecord(e0, st));
        int s2 = cube ? launch_q1_mode<DIM, true>(A, sh, q, coef, f_nodal, udir, bad, st)
                      : launch_q1_mode<DIM, false>(A, sh, q, coef, f_nodal, udir, bad, st);
        if (s2 != GD_OK) return s2;
        GD_CUDA_TRY(cudaEventRecord(e1, st));
        GD_CUDA_TRY(cudaEventSynchronize(e1));
        float ms = 0.f;
        GD_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        if (rep > 0) best_ms[sh] = std::min(best_ms[sh], ms);
      }
    }
    int best_shape = 0;
    for (int sh = 0; sh < kNumQ1Shapes; ++sh) {
      A->q1_shape_ms[sh] = best_ms[sh];
      if (best_ms[sh] < best_ms[best_shape]) best_shape = sh;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    A->q1_shape = best_shape;
  }
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[1], st));
  if (A->dl_active) {
    // pipelined download: one launch per row range; the copy stream takes each range's
    // values and rhs to the host while the next range is assembled
    const size_t nr = A->dl_rows.size() - 1;
    for (size_t k = 0; k < nr; ++k) {
      A->q1_rows[0] = A->dl_rows[k];
      A->q1_rows[1] = A->dl_rows[k + 1];
      const int s2 = cube ? launch_q1_mode<DIM, true>(A, A->q1_shape, q, coef, f_nodal, udir, bad, st)
                          : launch_q1_mode<DIM, false>(A, A->q1_shape, q, coef, f_nodal, udir, bad, st);
      A->q1_rows[0] = 0;
      A->q1_rows[1] = -1;
      if (s2 != GD_OK) return s2;
      GD_CUDA_TRY(cudaEventRecord(A->dl_events[k], st));
      GD_CUDA_TRY(cudaStreamWaitEvent(A->dl_stream, A->dl_events[k], 0));
      const int64_t e0 = A->dl_nnz[k], e1 = A->dl_nnz[k + 1];
      const int64_t q0 = A->dl_rows[k], q1 = A->dl_rows[k + 1];
      if (A->dl_vals && e1 > e0)
        GD_CUDA_TRY(cudaMemcpyAsync(A->dl_vals + e0, A->vals.p + e0, sizeof(double) * (e1 - e0),
                                    cudaMemcpyDeviceToHost, A->dl_stream));
      if (A->dl_rhs && q1 > q0)
        GD_CUDA_TRY(cudaMemcpyAsync(A->dl_rhs + q0, A->rhs.p + q0, sizeof(double) * (q1 - q0),
                                    cudaMemcpyDeviceToHost, A->dl_stream));
    }
  } else {
    const int s = cube ? launch_q1_mode<DIM, true>(A, A->q1_shape, q, coef, f_nodal, udir, bad, st)
                       : launch_q1_mode<DIM, false>(A, A->q1_shape, q, coef, f_nodal, udir, bad, st);
    if (s != GD_OK) return s;
  }
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
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[1], st));
  // one warp per row; grid sized for a few waves of resident blocks
  const unsigned nbw = (unsigned)std::min<int64_t>((R + 7) / 8, 152 * 64);
  if (A->code_bytes == 1)
    k_numeric_qk_rows<DIM, K, uint8_t><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p, A->code.p, kappa,
                                                            A->Khat.p, A->vals.p);
  else
    k_numeric_qk_rows<DIM, K, uint16_t><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p,
                                                             (const uint16_t*)A->code.p, kappa, A->Khat.p, A->vals.p);
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

// ---- 2D Q_k (k = 2, 3): values and right-hand side in one kernel, a lane pair per row ----
// lanes per row of k_rows2d_fused (1, 2 or 4; on the 128^2 Q2 case 2 lanes took 14.3 us,
// 1 lane 16.8 us and 4 lanes 16.0 us)
constexpr int kR2dLanes = 2;

// A 2D row has at most (2k+1)^2 entries (25 for Q2), so kR2dLanes lanes form a whole row:
// each decodes the node's (at most 4) cells, takes every kR2dLanes-th CSR entry (the
// stencil code of each entry gives the offset and the cells that hold both nodes through
// the shared-memory entry table, as in qk_matrix_rows) and a share of the node's cells
// for the right-hand side (source term and Dirichlet lifting, only in cells on a Dirichlet
// side), summed over the lanes by shuffles.  Consecutive lane groups own consecutive rows,
// so a warp's values are one contiguous range of the CSR value array.
// CS (class sums): when the reference tables are invariant under the square's reflections
// (checked on the host), the cells that hold both nodes of an entry are reflections of
// one another across the node's cell boundaries and give the same table value, so the
// entry is that value times the sum of their coefficients: the row's lanes form the 9
// subset sums of the (at most 4) cell coefficients once (left, right or both cells per
// direction: five sums of two or four coefficients, split over a lane pair so that each
// lane executes three FP64 additions) and an entry costs one FP64 multiply, where the
// exact per-cell form costs one FMA per cell (up to 4).  GB300 issues FP64 at a small fraction
// of its FP32 rate (the per-cell form kept its FP64 pipe 56 % busy, the class sums 36 %).
// Memory order: the row's node and CSR range are loaded before the block's tables are set
// up, and its stencil codes and cell coefficients together right after, so a row waits for
// two memory round trips instead of a chain of five (tables, node, coefficients, CSR range,
// codes).
// Source table: s_Fn[5 l + n] = f_const F[l] n, the load of local node l summed over n valid
// cells, formed on the host (no FP64 work per block).
struct R2dFn {
  double v[16 * 5];   // NN * 5 for K <= 3
};

template <int K, typename CodeT, bool FN, bool UD, bool CS>
__global__ void __launch_bounds__(128)
k_rows2d_fused(Geom g, int64_t nrows_own, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ row_node,
               const CodeT* __restrict__ code, const double* __restrict__ kappa, const double* __restrict__ Khat,
               const double* __restrict__ Mhat, const double* __restrict__ Fhat, double f_const, const R2dFn fn,
               const double* __restrict__ f_nodal, const double* __restrict__ u_dir, double* __restrict__ vals,
               double* __restrict__ rhs, int32_t* __restrict__ bad) {
  using L = Lat<2, K>;
  constexpr int NN = L::NN;
  __shared__ double s_K[NN * NN];
  __shared__ double s_M[FN ? NN * NN : 1];
  __shared__ double s_F[NN];
  __shared__ double s_Fn[CS && !FN ? NN * 5 : 1];   // f_const F[l] n for n = 0..4 valid cells
  __shared__ uint16_t s_tab[EntryTab<2, K>::SIZE];
  __shared__ double s_kap[4][128];   // per thread: coefficient and local index of its 4 slots
  __shared__ int s_lx[4][128];       // (shared, not local, memory: they are indexed at run time)
  __shared__ double s_S[CS ? 9 : 1][128];   // per thread: subset sums, index ox + 3 oy (0 left, 1 right, 2 both)
  // kR2dLanes lanes per row: all decode the row's cells, each forms every kR2dLanes-th
  // entry and a share of the node's cells for the rhs (more warps than one lane per row,
  // to hide latency)
  constexpr int LPR = kR2dLanes;
  const int t = threadIdx.x, sub = t % LPR;
  const int64_t r = ((int64_t)blockIdx.x * blockDim.x + t) / LPR;
  const bool live = r < nrows_own;
  const uint32_t lin = live ? (uint32_t)row_node[r] : 0u;
  const int64_t e0 = live ? rowptr[r] : 0;
  const int len = live ? (int)(rowptr[r + 1] - e0) : 0;
  for (int i = t; i < NN * NN; i += blockDim.x) {
    s_K[i] = Khat[i];
    if (FN) s_M[i] = Mhat[i];
  }
  for (int i = t; i < NN; i += blockDim.x) s_F[i] = Fhat[i];
  if (CS && !FN)
    for (int i = t; i < NN * 5; i += blockDim.x) s_Fn[i] = fn.v[i];
  build_entry_tab<2, K>(s_tab);
  // all stencil codes of the row (independent loads), then the cell coefficients; a 2D
  // row has at most MAXE entries
  constexpr int MAXE = (2 * K + 1) * (2 * K + 1);
  constexpr int MAXH = (MAXE + LPR - 1) / LPR;   // entries of one lane
  int cv[MAXH];
#pragma unroll
  for (int h = 0; h < MAXH; ++h) {
    const int i = LPR * h + sub;
    cv[h] = i < len ? (int)__ldg(code + e0 + i) : 0;
  }
  int nbad = 0;
  const uint32_t N0 = (uint32_t)g.N[0];
  const int X0 = (int)(lin % N0), X1 = (int)(lin / N0);
  const int rm0 = X0 % K, rm1 = X1 % K;
  const int onb = (rm0 == 0 ? 1 : 0) | (rm1 == 0 ? 2 : 0);
  uint32_t vmask = 0;
#pragma unroll
  for (int a = 0; a < 4; ++a) {
    const int s0 = a & 1, s1 = (a >> 1) & 1;
    const int c0 = s0 ? X0 / K : X0 / K - 1, c1 = s1 ? X1 / K : X1 / K - 1;
    const bool ok = live && (s0 || rm0 == 0) && (s1 || rm1 == 0) && c0 >= 0 && c0 < (int)g.n[0] && c1 >= 0 &&
                    c1 < (int)g.n[1];
    const double k = ok ? __ldg(kappa + (int64_t)c1 * g.n[0] + c0) : 0.0;
    if (ok && sub == 0) {   // finite and positive, tested on the bits (integer pipe, not GB300's scarce FP64 one)
      const unsigned long long bits = (unsigned long long)__double_as_longlong(k);
      nbad += (bits >> 63) != 0ull || ((bits >> 52) & 0x7FFull) == 0x7FFull || bits == 0ull;
    }
    s_kap[a][t] = k;
    s_lx[a][t] = (s0 ? rm0 : K) + L::KP1 * (s1 ? rm1 : K);
    vmask |= (uint32_t)ok << a;
  }
  __syncthreads();
  if (!live) return;
  const unsigned gmask = ((1u << LPR) - 1u) << ((t & 31) & ~(LPR - 1));   // the row's lanes
  if (CS) {   // slot a = s0 | 2 s1 (s = 1: the cell on the upper side of the node)
    const double k00 = s_kap[0][t], k10 = s_kap[1][t], k01 = s_kap[2][t], k11 = s_kap[3][t];
    double lo2, hi2, s6, s7;
    if (LPR == 2) {
      // the lane pair splits the four two-cell sums (lane 0: k00 + k10 and k00 + k01,
      // lane 1: k01 + k11 and k10 + k11; the same operands in the same order, so the same
      // bits) and swaps them: two FP64 additions per lane instead of four
      const double xa = sub ? k01 : k00, xb = sub ? k11 : k10;
      const double ya = sub ? k10 : k00, yb = sub ? k11 : k01;
      const double x = xa + xb, y = ya + yb;
      const double xo = __shfl_xor_sync(gmask, x, 1), yo = __shfl_xor_sync(gmask, y, 1);
      lo2 = sub ? xo : x;
      hi2 = sub ? x : xo;
      s6 = sub ? yo : y;
      s7 = sub ? y : yo;
    } else {
      lo2 = k00 + k10;
      hi2 = k01 + k11;
      s6 = k00 + k01;
      s7 = k10 + k11;
    }
    s_S[0][t] = k00;
    s_S[1][t] = k10;
    s_S[2][t] = lo2;
    s_S[3][t] = k01;
    s_S[4][t] = k11;
    s_S[5][t] = hi2;
    s_S[6][t] = s6;
    s_S[7][t] = s7;
    s_S[8][t] = lo2 + hi2;
  }
  const uint16_t* et = s_tab + onb * EntryTab<2, K>::E;
#pragma unroll
  for (int h = 0; h < MAXH; ++h) {
    const int i = LPR * h + sub;
    if (i >= len) break;
    const int info = et[cv[h]];
    const int off = (info & 255) - 128;
    const int fixed = (info >> 8) & 7, both = (info >> 11) & 7;
    double v = 0.0;
    if (CS) {
      const int ox = (both & 1) ? 2 : (fixed & 1), oy = (both & 2) ? 2 : ((fixed >> 1) & 1);
      v = s_K[s_lx[fixed][t] * (NN + 1) + off] * s_S[ox + 3 * oy][t];
    } else {
      int sb = both;
      while (true) {
        const int a = fixed | sb;
        if ((vmask >> a) & 1u) v = fma(s_kap[a][t], s_K[s_lx[a][t] * (NN + 1) + off], v);
        if (sb == 0) break;
        sb = (sb - 1) & both;
      }
    }
    vals[e0 + i] = v;
  }
  // right-hand side: source over the node's cells minus the lifting of the Dirichlet values;
  // the lanes take 4 / LPR cells each and add their parts (CS: the source value of the
  // node's local position is the same in all its cells; slot 3, the cell on the upper side
  // in both directions, always holds the node)
  double b = CS && !FN && sub == 0 ? s_Fn[s_lx[3][t] * 5 + __popc(vmask)] : 0.0;
#pragma unroll
  for (int h = 0; h < 4 / LPR; ++h) {
    const int a = (4 / LPR) * sub + h;
    if (!((vmask >> a) & 1u)) continue;
    const int la = s_lx[a][t];
    if (!FN && !CS) b += f_const * s_F[la];
    const int64_t c0 = (a & 1) ? X0 / K : X0 / K - 1, c1 = (a & 2) ? X1 / K : X1 / K - 1;
    // Dirichlet nodes of a cell lie on its sides that are Dirichlet sides of the domain:
    // cells away from them have nothing to lift (most rows)
    const bool lift = UD && ((g.dsides[0] && c0 == 0) || (g.dsides[1] && c0 == g.n[0] - 1) ||
                             (g.dsides[2] && c1 == 0) || (g.dsides[3] && c1 == g.n[1] - 1));
    if (FN || lift) {
      const double ka = s_kap[a][t];
      for (int lj = 0; lj < NN; ++lj) {
        const int64_t Y0 = (int64_t)K * c0 + lj % L::KP1, Y1 = (int64_t)K * c1 + lj / L::KP1;
        const int64_t ylin = Y1 * g.N[0] + Y0;
        if (FN) b += s_M[la * NN + lj] * __ldg(f_nodal + ylin);
        if (lift) {
          const bool dir = (g.dsides[0] && Y0 == 0) || (g.dsides[1] && Y0 == g.N[0] - 1) ||
                           (g.dsides[2] && Y1 == 0) || (g.dsides[3] && Y1 == g.N[1] - 1);
          if (dir) b -= ka * s_K[la * NN + lj] * __ldg(u_dir + ylin);
        }
      }
    }
  }
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) b += __shfl_xor_sync(gmask, b, o);
  if (sub == 0) rhs[r] = b;
  if (nbad) atomicAdd(bad, nbad);
}

// True when the 2D Q_k reference stiffness and load tables are invariant under the
// reflections of the square (K[R(i)][R(j)] = K[i][j], F[R(i)] = F[i] to 1e-14 relative for
// the reflection of x and the reflection of y), the condition of the class-sum rows.
// Cached per reference element.
static int rows2d_symmetric(gd_asm* A, int K, bool* sym) {
  if (A->r2d_sym_degree == A->ref_degree) {
    *sym = A->r2d_sym;
    return GD_OK;
  }
  const int KP1 = K + 1, NN = KP1 * KP1;
  cudaStream_t st = A->test->model->ctx->stream;
  std::vector<double> Kh(NN * NN), Fh(NN);
  GD_CUDA_TRY(cudaMemcpyAsync(Kh.data(), A->Khat.p, sizeof(double) * NN * NN, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(Fh.data(), A->Fhat.p, sizeof(double) * NN, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  double kmax = 0.0, fmax = 0.0;
  for (double v : Kh) kmax = std::max(kmax, std::fabs(v));
  for (double v : Fh) fmax = std::max(fmax, std::fabs(v));
  bool ok = true;
  for (int refl = 0; refl < 2 && ok; ++refl) {
    auto R = [&](int i) {
      const int x = i % KP1, y = i / KP1;
      return refl == 0 ? (K - x) + KP1 * y : x + KP1 * (K - y);
    };
    for (int i = 0; i < NN && ok; ++i) {
      if (std::fabs(Fh[R(i)] - Fh[i]) > 1e-14 * fmax) ok = false;
      for (int j = 0; j < NN && ok; ++j)
        if (std::fabs(Kh[R(i) * NN + R(j)] - Kh[i * NN + j]) > 1e-14 * kmax) ok = false;
    }
  }
  A->r2d_sym = ok;
  A->r2d_sym_degree = A->ref_degree;
  A->r2d_F = Fh;
  *sym = ok;
  return GD_OK;
}

template <int K, typename CodeT>
static int launch_rows2d_code(gd_asm* A, const double* kappa, const double* f_nodal, double f_const, int32_t* bad,
                              cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  const unsigned nb = (unsigned)((kR2dLanes * R + 127) / 128);
  const CodeT* code = reinterpret_cast<const CodeT*>(A->code.p);
  bool cs = false;
  GD_TRY(rows2d_symmetric(A, K, &cs));
  cs = cs && A->r2d_class_sums;
  constexpr int NN = (K + 1) * (K + 1);
  static_assert(NN * 5 <= (int)(sizeof(R2dFn::v) / sizeof(double)), "source table size");
  R2dFn fn = {};
  if (cs && !f_nodal) {   // the same products, in the same order, as f_const * F[l] * n on the device
    if (A->r2d_F.size() != (size_t)NN) return fail(GD_ERR_STATE, "2D reference load table not cached");
    for (int i = 0; i < NN * 5; ++i) fn.v[i] = f_const * A->r2d_F[i / 5] * (double)(i % 5);
  }
#define GD_R2D(FNV, UDV, CSV)                                                                                     \
  k_rows2d_fused<K, CodeT, FNV, UDV, CSV><<<nb, 128, 0, st>>>(g, R, A->rowptr.p, A->row_node.p, code, kappa,      \
                                                              A->Khat.p, A->Mhat.p, A->Fhat.p, f_const, fn,       \
                                                              f_nodal, udir, A->vals.p, A->rhs.p, bad)
  if (cs) {
    if (f_nodal && udir) GD_R2D(true, true, true);
    else if (f_nodal) GD_R2D(true, false, true);
    else if (udir) GD_R2D(false, true, true);
    else GD_R2D(false, false, true);
  } else {
    if (f_nodal && udir) GD_R2D(true, true, false);
    else if (f_nodal) GD_R2D(true, false, false);
    else if (udir) GD_R2D(false, true, false);
    else GD_R2D(false, false, false);
  }
#undef GD_R2D
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

template <int K>
static int launch_rows2d(gd_asm* A, const double* kappa, const double* f_nodal, double f_const, int32_t* bad,
                         cudaStream_t st) {
  if (A->ngdofs == 0) return GD_OK;
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[1], st));
  const int s = A->code_bytes == 1 ? launch_rows2d_code<K, uint8_t>(A, kappa, f_nodal, f_const, bad, st)
                                   : launch_rows2d_code<K, uint16_t>(A, kappa, f_nodal, f_const, bad, st);
  if (s != GD_OK) return s;
  if (A->profiling) {   // one fused kernel: the rhs phase is empty
    GD_CUDA_TRY(cudaEventRecord(A->ev[2], st));
    GD_CUDA_TRY(cudaEventRecord(A->ev[3], st));
  }
  return GD_OK;
}

// Values of the owned rows with an arbitrary reference element table (a linear
// combination of the stiffness and mass tables), kappa per cell: the generic row
// kernel over the assembler's pattern, into `vals` (multi-field blocks).
template <int DIM, int K>
static int launch_rows_table_t(gd_asm* A, const double* kappa, const double* table, double* vals, cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  if (R == 0) return GD_OK;
  const unsigned nbw = (unsigned)std::min<int64_t>((R + 7) / 8, 152 * 64);
  if (A->code_bytes == 1)
    k_numeric_qk_rows<DIM, K, uint8_t><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p, A->code.p, kappa, table,
                                                            vals);
  else
    k_numeric_qk_rows<DIM, K, uint16_t><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p,
                                                             (const uint16_t*)A->code.p, kappa, table, vals);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// Right-hand side of the owned rows: f_const * (int v) minus the Dirichlet lifting with
// `table` (kappa per cell), into `rhs`.
template <int DIM, int K>
static int launch_rhs_table_t(gd_asm* A, const double* kappa, const double* table, double f_const, double* rhs,
                              int32_t* bad, cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  if (R == 0) return GD_OK;
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  k_numeric_rhs<DIM, K><<<(unsigned)((R + 127) / 128), 128, 0, st>>>(g, R, A->row_node.p, kappa, table, A->Mhat.p,
                                                                     A->Fhat.p, f_const, nullptr, udir, rhs, bad);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

int launch_rows_table(gd_asm* A, const double* kappa, const double* table, double* vals, cudaStream_t st) {
  const Geom& g = A->test->geom;
  if (g.dim == 2 && g.k == 1) return launch_rows_table_t<2, 1>(A, kappa, table, vals, st);
  if (g.dim == 2 && g.k == 2) return launch_rows_table_t<2, 2>(A, kappa, table, vals, st);
  if (g.dim == 2 && g.k == 3) return launch_rows_table_t<2, 3>(A, kappa, table, vals, st);
  if (g.dim == 3 && g.k == 1) return launch_rows_table_t<3, 1>(A, kappa, table, vals, st);
  if (g.dim == 3 && g.k == 2) return launch_rows_table_t<3, 2>(A, kappa, table, vals, st);
  if (g.dim == 3 && g.k == 3) return launch_rows_table_t<3, 3>(A, kappa, table, vals, st);
  return fail(GD_ERR_UNSUPPORTED, "numeric: unsupported dim/order");
}

int launch_rhs_table(gd_asm* A, const double* kappa, const double* table, double f_const, double* rhs, int32_t* bad,
                     cudaStream_t st) {
  const Geom& g = A->test->geom;
  if (g.dim == 2 && g.k == 1) return launch_rhs_table_t<2, 1>(A, kappa, table, f_const, rhs, bad, st);
  if (g.dim == 2 && g.k == 2) return launch_rhs_table_t<2, 2>(A, kappa, table, f_const, rhs, bad, st);
  if (g.dim == 2 && g.k == 3) return launch_rhs_table_t<2, 3>(A, kappa, table, f_const, rhs, bad, st);
  if (g.dim == 3 && g.k == 1) return launch_rhs_table_t<3, 1>(A, kappa, table, f_const, rhs, bad, st);
  if (g.dim == 3 && g.k == 2) return launch_rhs_table_t<3, 2>(A, kappa, table, f_const, rhs, bad, st);
  if (g.dim == 3 && g.k == 3) return launch_rhs_table_t<3, 3>(A, kappa, table, f_const, rhs, bad, st);
  return fail(GD_ERR_UNSUPPORTED, "numeric: unsupported dim/order");
}

// Reads the coefficient-check count after the stream's work; a failure is reported once
// (the count is reset).
static int numeric_report(gd_asm* A, cudaStream_t st) {
  int32_t hbad = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&hbad, A->nbad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (!hbad) return GD_OK;
  GD_CUDA_TRY(cudaMemsetAsync(A->nbad.p, 0, sizeof(int32_t), st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return fail(GD_ERR_NUMERIC, "numeric: kappa is not finite and positive in " + std::to_string(hbad) + " cell visits");
}

int numeric_impl(gd_asm* A, const gd_coeffs* c, bool sync) {
  if (!A || !c) return fail(GD_ERR_ARG, "gd_assemble_numeric: null argument");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_assemble_numeric: run gd_assemble_symbolic first");
  if (A->bs > 1)
    return fail(GD_ERR_UNSUPPORTED, "gd_assemble_numeric: vector-valued space; use gd_assemble_elasticity");
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
  // the coefficient-check count: zeroed when allocated and after a reported failure, so a
  // numeric assembly is its kernels alone
  if (!A->nbad.p) {
    GD_TRY(dalloc(A->nbad, 1));
    GD_CUDA_TRY(cudaMemsetAsync(A->nbad.p, 0, sizeof(int32_t), st));
  }
  int32_t* bad = A->nbad.p;
  // Ghost rows (SubAssembledRows) hold explicit zeros: they were cleared by the symbolic
  // phase and no numeric kernel writes them.
  if (A->profiling) GD_CUDA_TRY(cudaEventRecord(A->ev[0], st));
  int s = GD_ERR_UNSUPPORTED;
  if (A->fast_q1 && g.dim == 3) s = launch_q1<3>(A, kappa, fn, c->f_const, bad, st);
  else if (A->fast_q1 && g.dim == 2) s = launch_q1<2>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 2 && g.k == 1) s = launch_numeric<2, 1>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 2 && g.k == 2) s = launch_rows2d<2>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 2 && g.k == 3) s = launch_rows2d<3>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 3 && g.k == 1) s = launch_numeric<3, 1>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 3 && g.k == 2) s = launch_numeric<3, 2>(A, kappa, fn, c->f_const, bad, st);
  else if (g.dim == 3 && g.k == 3) s = launch_numeric<3, 3>(A, kappa, fn, c->f_const, bad, st);
  if (s != GD_OK) return s == GD_ERR_UNSUPPORTED ? fail(s, "numeric: unsupported dim/order") : s;
  if (sync) GD_TRY(numeric_report(A, st));
  A->numeric_done = true;
  A->qp_values = false;
  ++A->numeric_epoch;
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
  if (!A) return gd::fail(GD_ERR_ARG, "gd_assembler_phase_times: null assembler");
  if (!A->ev[0]) return gd::fail(GD_ERR_STATE, "gd_assembler_phase_times: profiling was not enabled");
  GD_CUDA_TRY(cudaEventSynchronize(A->ev[3]));
  float t[3] = {0, 0, 0};
  for (int i = 0; i < 3; ++i) GD_CUDA_TRY(cudaEventElapsedTime(&t[i], A->ev[i], A->ev[i + 1]));
  if (ms0) *ms0 = t[0];
  if (ms1) *ms1 = t[1];
  if (ms2) *ms2 = t[2];
  return GD_OK;
}

extern "C" int gd_assembler_tuning(const gd_asm* A, int32_t* shape, int32_t* rows, int32_t* nbuf, float* ms,
                                   int32_t* nshapes) {
  if (!A) return gd::fail(GD_ERR_ARG, "gd_assembler_tuning: null assembler");
  const int sh = A->fast_q1 ? A->q1_shape : -1;
  if (shape) *shape = sh;
  if (rows) *rows = sh >= 0 ? gd::kQ1Shapes[sh].rows : 0;
  if (nbuf) *nbuf = sh >= 0 ? gd::kQ1Shapes[sh].nbuf : 0;
  if (ms)
    for (int i = 0; i < gd::kNumQ1Shapes; ++i) ms[i] = A->q1_shape_ms[i];
  if (nshapes) *nshapes = gd::kNumQ1Shapes;
  return GD_OK;
}

extern "C" int gd_assembler_set_shape(gd_asm* A, int shape) {
  if (!A) return gd::fail(GD_ERR_ARG, "gd_assembler_set_shape: null assembler");
  if (!A->symbolic_done) return gd::fail(GD_ERR_STATE, "gd_assembler_set_shape: run gd_assemble_symbolic first");
  if (!A->fast_q1) return gd::fail(GD_ERR_UNSUPPORTED, "gd_assembler_set_shape: the assembler does not use the Q1 kernel");
  if (shape < -1 || shape >= gd::kNumQ1Shapes) return gd::fail(GD_ERR_ARG, "gd_assembler_set_shape: shape out of range");
  A->q1_shape = shape;   // -1: the next numeric assembly times every shape again
  return GD_OK;
}

extern "C" int gd_assembler_set_class_sums(gd_asm* A, int on) {
  if (!A) return gd::fail(GD_ERR_ARG, "gd_assembler_set_class_sums: null assembler");
  A->r2d_class_sums = on != 0;
  return GD_OK;
}

extern "C" int gd_assembler_counts(const gd_asm* A, int64_t* ngdofs, int64_t* nnz_owned, int64_t* nnz_total,
                                   int32_t* kernels) {
  if (!A) return gd::fail(GD_ERR_ARG, "gd_assembler_counts: null assembler");
  if (!A->symbolic_done) return gd::fail(GD_ERR_STATE, "gd_assembler_counts: run gd_assemble_symbolic first");
  if (ngdofs) *ngdofs = A->ngdofs;
  if (nnz_owned) *nnz_owned = A->nnz_own;
  if (nnz_total) *nnz_total = A->nnz_total;
  // cube Q1: k_prescale + k_numeric_q1; other Q1: k_numeric_q1; 2D Q2/Q3: k_rows2d_fused;
  // 3D Q_k: k_numeric_qk_rows + k_numeric_rhs
  const bool fused2d = !A->fast_q1 && A->test->geom.dim == 2 && A->test->geom.k >= 2 && A->bs == 1;
  if (kernels) *kernels = A->fast_q1 ? (A->q1c_cube ? 2 : 1) : (fused2d ? 1 : 2);
  return GD_OK;
}

// assemble_vector(assem, collect_cell_vector(V, l)) for l(v) = int(v f): the load vector
// alone (no Dirichlet lifting, which Gridap applies only with a cell matrix), over the
// owned rows in global order, into a caller buffer; the assembler's matrix values and
// right-hand side are left as they are.
extern "C" int gd_assemble_vector(gd_asm* A, const gd_coeffs* c, double* b, int where_b) {
  using namespace gd;
  if (!A || !c || !b) return fail(GD_ERR_ARG, "gd_assemble_vector: null argument");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_assemble_vector: run gd_assemble_symbolic first");
  if (A->bs > 1) return fail(GD_ERR_UNSUPPORTED, "gd_assemble_vector: scalar spaces only");
  const Geom& g = A->test->geom;
  cudaStream_t st = A->test->model->ctx->stream;
  GD_TRY(reference_element(A, c->degree));
  const int64_t R = A->ngdofs;
  int64_t nnodes = 1;
  for (int d = 0; d < g.dim; ++d) nnodes *= g.N[d];
  const double* fn = c->f_nodal;
  if (fn && c->where == GD_HOST) {
    if (A->f_dev.n != (size_t)nnodes) GD_TRY(dalloc(A->f_dev, nnodes));
    GD_CUDA_TRY(cudaMemcpyAsync(A->f_dev.p, fn, sizeof(double) * nnodes, cudaMemcpyHostToDevice, st));
    fn = A->f_dev.p;
  }
  if (R == 0) return GD_OK;
  DBuf<double> tmp;
  double* out = b;
  if (where_b == GD_HOST) {
    GD_TRY(dalloc(tmp, R));
    out = tmp.p;
  }
  if (!A->dred.p) GD_TRY(dalloc(A->dred, 4096));
  int32_t* bad = (int32_t*)A->dred.p;
  GD_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
  const unsigned nb = (unsigned)((R + 127) / 128);
  const int sel = g.dim * 10 + g.k;
#define GD_VEC_LAUNCH(D, K)                                                                                    \
  k_numeric_rhs<D, K><<<nb, 128, 0, st>>>(g, R, A->row_node.p, nullptr, A->Khat.p, A->Mhat.p, A->Fhat.p, c->f_const, \
                                          fn, nullptr, out, bad)
  switch (sel) {
    case 21: GD_VEC_LAUNCH(2, 1); break;
    case 22: GD_VEC_LAUNCH(2, 2); break;
    case 23: GD_VEC_LAUNCH(2, 3); break;
    case 31: GD_VEC_LAUNCH(3, 1); break;
    case 32: GD_VEC_LAUNCH(3, 2); break;
    case 33: GD_VEC_LAUNCH(3, 3); break;
    default:
      dfreeb(tmp);
      return fail(GD_ERR_UNSUPPORTED, "gd_assemble_vector: unsupported dim/order");
  }
#undef GD_VEC_LAUNCH
  GD_CUDA_TRY(cudaGetLastError());
  if (where_b == GD_HOST) GD_CUDA_TRY(cudaMemcpyAsync(b, out, sizeof(double) * R, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(tmp);
  return GD_OK;
}

extern "C" int gd_assemble_numeric(gd_asm* A, const gd_coeffs* c) { return gd::numeric_impl(A, c, true); }

// Numeric assembly followed by the download of the rhs and the owned-row values, with
// the download overlapped with the assembly on the Q1 path: the owned rows are assembled
// in kDownloadRanges launches, and each range's values and rhs go to the host on a second
// stream while the next range is assembled.  Other paths assemble, then download.
extern "C" int gd_assemble_download(gd_asm* A, const gd_coeffs* c, double* rhs, double* owned_vals) {
  using namespace gd;
  constexpr int kDownloadRanges = 8;
  if (!A || !c) return fail(GD_ERR_ARG, "gd_assemble_download: null argument");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_assemble_download: run gd_assemble_symbolic first");
  if (!A->fast_q1 || A->bs > 1 || A->ngdofs == 0) {
    GD_TRY(numeric_impl(A, c, true));
    return gd_system_download(A, rhs, owned_vals);
  }
  cudaStream_t st = A->test->model->ctx->stream;
  if (!A->dl_stream) GD_CUDA_TRY(cudaStreamCreateWithFlags(&A->dl_stream, cudaStreamNonBlocking));
  if (A->dl_rows.empty()) {   // row ranges and their first entries, once per assembler
    const int64_t n = A->ngdofs;
    std::vector<int64_t> rows(kDownloadRanges + 1), nnz(kDownloadRanges + 1);
    for (int k = 0; k <= kDownloadRanges; ++k) rows[k] = n * k / kDownloadRanges;
    for (int k = 0; k <= kDownloadRanges; ++k)
      GD_CUDA_TRY(cudaMemcpyAsync(&nnz[k], A->rowptr.p + rows[k], sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    for (int k = 0; k < kDownloadRanges; ++k) {
      cudaEvent_t e;
      GD_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      A->dl_events.push_back(e);
    }
    A->dl_rows = rows;
    A->dl_nnz = nnz;
  }
  // the copies of a previous call are done (that call synchronised), so the values may be
  // rewritten
  A->dl_active = true;
  A->dl_rhs = rhs;
  A->dl_vals = owned_vals;
  const int s = numeric_impl(A, c, false);
  A->dl_active = false;
  A->dl_rhs = A->dl_vals = nullptr;
  const cudaError_t e1 = cudaStreamSynchronize(A->dl_stream);
  if (s != GD_OK) return s;
  if (e1 != cudaSuccess) return fail(GD_ERR_CUDA, std::string("gd_assemble_download: ") + cudaGetErrorString(e1));
  return numeric_report(A, st);
}
extern "C" int gd_assemble_numeric_async(gd_asm* A, const gd_coeffs* c) { return gd::numeric_impl(A, c, false); }
