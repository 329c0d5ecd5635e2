// Vector-valued Lagrangian spaces (ReferenceFE(lagrangian, VectorValue{D,Float64}, k),
// k <= 2) and linear elasticity.
//
// Gridap numbers the DOFs of a vector space face by face with the face's own nodes
// component-major (FESpaces.jl:570-614 through Gridap's Lagrangian reffe).  For k <= 2
// every vertex, edge, face and cell owns exactly one node, so when all components share
// the Dirichlet sides the vector numbering is the scalar node numbering interleaved:
// dof(node, c) = bs * dof(node) + c for local ids, gids and owners alike (checked
// against the oracle's own restatement).  The space therefore keeps its scalar node
// arrays and the assembler expands its sparsity into bs x bs blocks after the scalar
// symbolic phase.  One ordering is not interleaved: SubAssembledRows numbers ghost
// columns by first appearance while visiting owned cells and their cell DOFs, and a
// vector cell lists its DOFs component-major, so the ghost columns first seen in one
// cell appear as [all of them, component 0][component 1]...; the expansion permutes
// ghost columns group by group (a group = the scalar ghost columns sharing a first
// cell) to match.
//
// Elasticity: a(u,v) = int C(E) eps(u):eps(v) with isotropic C, E per cell, Poisson
// ratio nu; l(v) = int v.force.  On an axis-aligned cell with constant E the element
// matrix is E_c * Kel (Kel the E = 1 matrix of the reference cell, computed once on the
// host by tensor Gauss quadrature), so the numeric kernel has the structure of the
// scalar Q_k row kernel with a component pair per entry.
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_rows.cuh"

namespace gd {

int reference_element(gd_asm* A, int degree);

static inline unsigned vblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

static int vlaunch_ok(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return GD_OK;
}

__device__ inline int part_by_gcol(const DevPart* parts, int nparts, int64_t j) {
  int lo = 0, hi = nparts - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (parts[mid].gcol_off <= j) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ---- ghost-column groups ------------------------------------------------------------------
// skey[gcol_off_p + rank] = key of the part's ghost column of that rank (keys sorted)
__global__ void k_gcol_sorted_keys(const DevPart* __restrict__ parts, int nparts, int64_t ncand,
                                   const unsigned long long* __restrict__ ckey, const int32_t* __restrict__ rank,
                                   unsigned long long* __restrict__ skey) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncand) return;
  const int p = part_by_gcol(parts, nparts, i);
  skey[parts[p].gcol_off + rank[i]] = ckey[i];
}

// group of a sorted ghost column: SubAssembledRows keys share (tier, sender, first cell)
// in bits 16..63 within a group; FullyAssembledRows columns are groups of one
__global__ void k_gcol_groups(const DevPart* __restrict__ parts, int nparts, int64_t ncand, int by_cell,
                              const unsigned long long* __restrict__ skey, int32_t* __restrict__ gstart,
                              int32_t* __restrict__ gsize) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncand) return;
  const int p = part_by_gcol(parts, nparts, j);
  const int64_t a = parts[p].gcol_off, b = a + parts[p].n_gcol;
  int64_t s = j, e = j + 1;
  if (by_cell) {
    const unsigned long long gk = skey[j] >> 16;
    while (s > a && (skey[s - 1] >> 16) == gk) --s;
    while (e < b && (skey[e] >> 16) == gk) ++e;
  }
  gstart[j] = (int32_t)(s - a);
  gsize[j] = (int32_t)(e - s);
}

// ---- CSR expansion into bs x bs blocks ------------------------------------------------------
__global__ void k_vec_rowptr(int64_t R, int bs, const int64_t* __restrict__ rp, int64_t* __restrict__ rpv) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= R) return;
  const int64_t len = rp[r + 1] - rp[r];
  for (int c = 0; c < bs; ++c) rpv[bs * r + c] = (int64_t)bs * bs * rp[r] + (int64_t)c * bs * len;
  if (r == R - 1) rpv[bs * R] = (int64_t)bs * bs * rp[R];
}

// vector row (r, c): owned-column entries interleaved by component, then the ghost
// columns group by group, component-major inside a group
__global__ void k_vec_fill(int64_t R, int bs, const DevPart* __restrict__ parts, const int64_t* __restrict__ rp,
                           const int32_t* __restrict__ row_part, const int32_t* __restrict__ ci,
                           const int32_t* __restrict__ cg, const uint8_t* __restrict__ cd,
                           const int32_t* __restrict__ gstart, const int32_t* __restrict__ gsize,
                           const int64_t* __restrict__ rpv, int32_t* __restrict__ civ, int32_t* __restrict__ cgv,
                           uint16_t* __restrict__ cdv) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= bs * R) return;
  const int64_t r = v / bs;
  const int p = row_part[r];
  const int64_t nown = parts[p].n_own, goff = parts[p].gcol_off;
  const int64_t e0 = rp[r], e1 = rp[r + 1];
  int64_t o = rpv[v];
  int64_t e = e0;
  for (; e < e1 && ci[e] < nown; ++e)
    for (int c2 = 0; c2 < bs; ++c2) {
      civ[o] = bs * ci[e] + c2;
      cgv[o] = bs * cg[e] + c2;
      cdv[o] = (uint16_t)(cd[e] * bs + c2);
      ++o;
    }
  while (e < e1) {
    const int64_t g0 = ci[e] - nown;
    const int64_t s0 = gstart[goff + g0], m = gsize[goff + g0];
    int64_t f = e;
    while (f < e1 && gstart[goff + (ci[f] - nown)] == s0) ++f;
    for (int c2 = 0; c2 < bs; ++c2)
      for (int64_t x = e; x < f; ++x) {
        const int64_t g = ci[x] - nown;
        civ[o] = (int32_t)(bs * nown + bs * s0 + c2 * m + (g - s0));
        cgv[o] = bs * cg[x] + c2;
        cdv[o] = (uint16_t)(cd[x] * bs + c2);
        ++o;
      }
    e = f;
  }
}

__global__ void k_vec_rows(int64_t R, int bs, const int32_t* __restrict__ rn, const int32_t* __restrict__ rpart,
                           int32_t* __restrict__ rnv, int32_t* __restrict__ rpartv) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= bs * R) return;
  rnv[v] = rn[v / bs];
  rpartv[v] = rpart[v / bs];
}

__global__ void k_vec_lids(int64_t n, int bs, const int32_t* __restrict__ lid, int32_t* __restrict__ lidv) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= bs * n) return;
  lidv[v] = bs * lid[v / bs] + (int32_t)(v % bs);
}

__global__ void k_vec_gcol_lids(const DevPart* __restrict__ parts, int nparts, int64_t ncand, int bs,
                                const int32_t* __restrict__ lid, const int32_t* __restrict__ gstart,
                                const int32_t* __restrict__ gsize, int32_t* __restrict__ lidv) {
  const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= ncand) return;
  const int p = part_by_gcol(parts, nparts, j);
  const int64_t goff = parts[p].gcol_off, g = j - goff;
  const int64_t s0 = gstart[j], m = gsize[j];
  for (int c = 0; c < bs; ++c) lidv[bs * goff + bs * s0 + c * m + (g - s0)] = bs * lid[j] + c;
}

int gcol_groups(gd_asm* A, const unsigned long long* ckey, const int32_t* rank, int64_t ncand) {
  cudaStream_t st = A->test->model->ctx->stream;
  const int np = (int)A->parts.size();
  GD_TRY(dalloc(A->gcol_gstart, std::max<int64_t>(ncand, 1)));
  GD_TRY(dalloc(A->gcol_gsize, std::max<int64_t>(ncand, 1)));
  if (ncand == 0) return GD_OK;
  DBuf<unsigned long long> skey;
  GD_TRY(dalloc(skey, ncand));
  k_gcol_sorted_keys<<<vblk(ncand, 256), 256, 0, st>>>(A->d_parts.p, np, ncand, ckey, rank, skey.p);
  GD_TRY(vlaunch_ok("k_gcol_sorted_keys"));
  k_gcol_groups<<<vblk(ncand, 256), 256, 0, st>>>(A->d_parts.p, np, ncand,
                                                  A->strategy == GD_SUB_ASSEMBLED_ROWS ? 1 : 0, skey.p,
                                                  A->gcol_gstart.p, A->gcol_gsize.p);
  GD_TRY(vlaunch_ok("k_gcol_groups"));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(skey);
  return GD_OK;
}

int vector_expand(gd_asm* A) {
  gd_space* S = A->test;
  cudaStream_t st = S->model->ctx->stream;
  const int bs = S->ncomp;
  const int np = (int)A->parts.size();
  const int64_t R = A->nrows_total, nnz = A->nnz_total, ncand = A->total_gcols;
  int64_t ngrow = 0;
  for (const DevPart& P : A->parts) ngrow += P.n_grow;
  const int64_t Rv = bs * R, nnzv = (int64_t)bs * bs * nnz;
  if (A->code_bytes != 1) return fail(GD_ERR_UNSUPPORTED, "vector space: stencil codes wider than one byte");
  if (nnzv >= ((int64_t)1 << 40)) return fail(GD_ERR_UNSUPPORTED, "vector space: too many entries");
  DBuf<int64_t> rpv;
  DBuf<int32_t> civ, cgv, rnv, rpartv, growv, gcolv;
  DBuf<uint16_t> cdv;
  GD_TRY(dalloc(rpv, Rv + 1));
  GD_TRY(dalloc(civ, std::max<int64_t>(nnzv, 1)));
  GD_TRY(dalloc(cgv, std::max<int64_t>(nnzv, 1)));
  GD_TRY(dalloc(cdv, std::max<int64_t>(nnzv, 1)));
  GD_TRY(dalloc(rnv, std::max<int64_t>(Rv, 1)));
  GD_TRY(dalloc(rpartv, std::max<int64_t>(Rv, 1)));
  GD_TRY(dalloc(growv, std::max<int64_t>(bs * ngrow, 1)));
  GD_TRY(dalloc(gcolv, std::max<int64_t>(bs * ncand, 1)));
  if (R > 0) {
    k_vec_rowptr<<<vblk(R, 256), 256, 0, st>>>(R, bs, A->rowptr.p, rpv.p);
    GD_TRY(vlaunch_ok("k_vec_rowptr"));
    k_vec_fill<<<vblk(Rv, 128), 128, 0, st>>>(R, bs, A->d_parts.p, A->rowptr.p, A->row_part.p, A->colidx.p,
                                               A->colgid.p, A->code.p, A->gcol_gstart.p, A->gcol_gsize.p, rpv.p,
                                               civ.p, cgv.p, cdv.p);
    GD_TRY(vlaunch_ok("k_vec_fill"));
    k_vec_rows<<<vblk(Rv, 256), 256, 0, st>>>(R, bs, A->row_node.p, A->row_part.p, rnv.p, rpartv.p);
    GD_TRY(vlaunch_ok("k_vec_rows"));
  } else {
    GD_CUDA_TRY(cudaMemsetAsync(rpv.p, 0, sizeof(int64_t), st));
  }
  if (ngrow > 0) {
    k_vec_lids<<<vblk(bs * ngrow, 256), 256, 0, st>>>(ngrow, bs, A->grow_lid.p, growv.p);
    GD_TRY(vlaunch_ok("k_vec_lids"));
  }
  if (ncand > 0) {
    k_vec_gcol_lids<<<vblk(ncand, 256), 256, 0, st>>>(A->d_parts.p, np, ncand, bs, A->gcol_lid.p,
                                                      A->gcol_gstart.p, A->gcol_gsize.p, gcolv.p);
    GD_TRY(vlaunch_ok("k_vec_gcol_lids"));
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  // swap in the vector arrays
  std::swap(A->rowptr, rpv);
  std::swap(A->colidx, civ);
  std::swap(A->colgid, cgv);
  std::swap(A->row_node, rnv);
  std::swap(A->row_part, rpartv);
  std::swap(A->grow_lid, growv);
  std::swap(A->gcol_lid, gcolv);
  dfreeb(A->code);
  A->code.p = reinterpret_cast<uint8_t*>(cdv.p);
  A->code.n = (size_t)std::max<int64_t>(nnzv, 1) * 2;
  cdv.p = nullptr;
  cdv.n = 0;
  for (DBuf<int64_t>* b : {&rpv}) dfreeb(*b);
  for (DBuf<int32_t>* b : {&civ, &cgv, &rnv, &rpartv, &growv, &gcolv}) dfreeb(*b);
  dfreeb(A->gcol_gstart);
  dfreeb(A->gcol_gsize);
  dfreeb(A->row_pat);
  dfreeb(A->pat);
  A->fast_q1 = false;
  A->code_bytes = 2;
  A->bs = bs;
  A->ngdofs *= bs;
  A->nrows_total = Rv;
  A->nnz_total = nnzv;
  A->nnz_own *= (int64_t)bs * bs;
  A->total_gcols *= bs;
  for (DevPart& P : A->parts) {
    P.n_own *= bs;
    P.first_gdof *= bs;
    P.grow_off *= bs;
    P.n_grow *= bs;
    P.gcol_off *= bs;
    P.n_gcol *= bs;
  }
  GD_CUDA_TRY(cudaMemcpyAsync(A->d_parts.p, A->parts.data(), sizeof(DevPart) * np, cudaMemcpyHostToDevice, st));
  GD_TRY(dalloc(A->vals, std::max<int64_t>(nnzv, 1)));
  GD_TRY(dalloc(A->rhs, std::max<int64_t>(Rv, 1)));
  GD_CUDA_TRY(cudaMemsetAsync(A->vals.p, 0, sizeof(double) * std::max<int64_t>(nnzv, 1), st));
  GD_CUDA_TRY(cudaMemsetAsync(A->rhs.p, 0, sizeof(double) * std::max<int64_t>(Rv, 1), st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

// ---- elasticity reference matrix (host) ------------------------------------------------------
// Kel[(c*NN + i) * (bs*NN) + d*NN + j] = int lam d_c(phi_i) d_d(phi_j)
//   + mu (delta_cd grad(phi_i).grad(phi_j) + d_d(phi_i) d_c(phi_j)),  E = 1,
// local nodes i, j lexicographic (x fastest), lam = nu/((1+nu)(1-2nu)), mu = 1/(2(1+nu)).
static void elasticity_reference(int dim, int k, const double* h, int degree, double nu, std::vector<double>& K) {
  const int nq = (degree + 2) / 2, kp1 = k + 1;
  std::vector<double> xq, wq;
  gauss_legendre01(nq, xq, wq);
  std::vector<double> V(nq * kp1), D(nq * kp1);
  for (int q = 0; q < nq; ++q) lagrange01(k, xq[q], &V[q * kp1], &D[q * kp1]);
  int nn = 1, nqt = 1;
  for (int d = 0; d < dim; ++d) {
    nn *= kp1;
    nqt *= nq;
  }
  double detJ = 1.0;
  for (int d = 0; d < dim; ++d) detJ *= h[d];
  // gradients at the quadrature points: G[q][i][d]
  std::vector<double> G((size_t)nqt * nn * dim), W(nqt);
  for (int q = 0; q < nqt; ++q) {
    int qi[3] = {0, 0, 0};
    for (int d = 0, r = q; d < dim; ++d) {
      qi[d] = r % nq;
      r /= nq;
    }
    double w = detJ;
    for (int d = 0; d < dim; ++d) w *= wq[qi[d]];
    W[q] = w;
    for (int i = 0; i < nn; ++i) {
      int oi[3] = {0, 0, 0};
      for (int d = 0, r = i; d < dim; ++d) {
        oi[d] = r % kp1;
        r /= kp1;
      }
      for (int d = 0; d < dim; ++d) {
        double gv = D[qi[d] * kp1 + oi[d]] / h[d];
        for (int e = 0; e < dim; ++e)
          if (e != d) gv *= V[qi[e] * kp1 + oi[e]];
        G[((size_t)q * nn + i) * dim + d] = gv;
      }
    }
  }
  const double lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = 1.0 / (2.0 * (1.0 + nu));
  const int M = dim * nn;
  K.assign((size_t)M * M, 0.0);
  for (int c = 0; c < dim; ++c)
    for (int i = 0; i < nn; ++i)
      for (int d = 0; d < dim; ++d)
        for (int j = 0; j < nn; ++j) {
          double s = 0.0;
          for (int q = 0; q < nqt; ++q) {
            const double* gi = &G[((size_t)q * nn + i) * dim];
            const double* gj = &G[((size_t)q * nn + j) * dim];
            double lap = 0.0;
            for (int e = 0; e < dim; ++e) lap += gi[e] * gj[e];
            s += W[q] * (lam * gi[c] * gj[d] + mu * ((c == d ? lap : 0.0) + gi[d] * gj[c]));
          }
          K[(size_t)(c * nn + i) * M + d * nn + j] = s;
        }
}

// ---- elasticity numeric kernel ---------------------------------------------------------------
template <int DIM, int K>
struct VecLanes {
  static constexpr int W = 2 * K + 1;
  static constexpr int E = DIM * (DIM == 3 ? W * W * W : W * W);   // entries of a vector row
  static constexpr int G = E <= 32 ? 8 : (E <= 128 ? 16 : 32);
  static constexpr int RPW = 32 / G;
};

// Owned vector rows, lane groups as in qk_matrix_rows; row (node, c), entry (node+o, d):
// sum over the cells holding both nodes of E_cell * Kel[(c NN + lx) (bs NN) + d NN + lx + off].
template <int DIM, int K>
__global__ void __launch_bounds__(256)
k_numeric_elasticity(Geom g, int64_t nrows_own, const int64_t* __restrict__ rowptr,
                     const int32_t* __restrict__ row_node, const uint16_t* __restrict__ code,
                     const double* __restrict__ E, const double* __restrict__ Kel, double* __restrict__ vals) {
  using L = Lat<DIM, K>;
  using VL = VecLanes<DIM, K>;
  constexpr int NC = 1 << DIM;
  constexpr int G = VL::G;
  constexpr int M = DIM * L::NN;
  extern __shared__ double sKel[];   // M * M
  __shared__ uint16_t s_tab[EntryTab<DIM, K>::SIZE];
  __shared__ double s_kap[8][32];
  __shared__ int s_lx[8][32];
  for (int i = threadIdx.x; i < M * M; i += blockDim.x) sKel[i] = Kel[i];
  build_entry_tab<DIM, K>(s_tab);
  __syncthreads();
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5, sub = lane / G, gl = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double* skap = s_kap[wl];
  int* slx = s_lx[wl];
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
  for (int64_t rb = warp * VL::RPW; rb < nrows_own; rb += nwarps * VL::RPW) {
    const int64_t r = rb + sub;
    const bool live = r < nrows_own;
    const int c = (int)(r % DIM);
    const uint32_t lin = live ? (uint32_t)row_node[r] : 0u;
    int X[3], rm[3];
    X[0] = (int)(lin % N0);
    if (DIM == 3) {
      const uint32_t t = lin / N0;
      X[1] = (int)(t % N1);
      X[2] = (int)(t / N1);
    } else {
      X[1] = (int)(lin / N0);
      X[2] = 0;
    }
    int onb = 0;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      rm[d] = X[d] % K;
      if (rm[d] == 0) onb |= 1 << d;
    }
    bool slot_ok = false;
    if (live && gl < NC) {
      bool ok = true;
      int cl = 0, stride = 1, lx = 0, mul = 1;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int sd = (gl >> d) & 1;
        const int cc = sd ? X[d] / K : X[d] / K - 1;
        if (!sd && rm[d] != 0) ok = false;
        if (cc < 0 || cc >= (int)g.n[d]) ok = false;
        cl += stride * cc;
        stride *= (int)g.n[d];
        lx += mul * (sd ? rm[d] : K);
        mul *= L::KP1;
      }
      skap[sub * NC + gl] = ok ? __ldg(E + cl) : 0.0;
      slx[sub * NC + gl] = (c * L::NN + lx) * M + lx;
      slot_ok = ok;
    }
    const uint32_t vmask = (__ballot_sync(0xffffffffu, slot_ok) >> (sub * G)) & ((1u << NC) - 1);
    __syncwarp();
    if (live) {
      const double* sk = skap + sub * NC;
      const int* sl = slx + sub * NC;
      const uint16_t* et = s_tab + onb * EntryTab<DIM, K>::E;
      const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
      for (int64_t e = e0 + gl; e < e1; e += G) {
        const int cv = (int)code[e];
        const int d2 = cv % DIM;
        const int info = et[cv / DIM];
        const int off = (info & 255) - 128 + d2 * L::NN;
        const int fixed = (info >> 8) & 7, both = (info >> 11) & 7;
        double v = 0.0;
        int sb = both;
        while (true) {
          const int a = fixed | sb;
          if ((vmask >> a) & 1u) v = fma(sk[a], sKel[sl[a] + off], v);
          if (sb == 0) break;
          sb = (sb - 1) & both;
        }
        vals[e] = v;
      }
    }
    __syncwarp();
  }
}

// Dirichlet lifting of owned vector row (node X, component c): minus the sum over the
// node's cells of E_cell * Kel[(c NN + li) M + d NN + lj] * u_D(node lj, d) over the
// cell's Dirichlet nodes lj and all components d (FESpaces.jl:703-715: b_e -= K_e[:,D] u_D).
template <int DIM, int K>
__device__ double elasticity_lifting(const Geom& g, int64_t lin, int c, const double* __restrict__ E,
                                     const double* __restrict__ Kel, const double* __restrict__ u_dir) {
  using L = Lat<DIM, K>;
  constexpr int M = DIM * L::NN;
  int64_t X[3] = {0, 0, 0};
  for (int d = 0; d < DIM; ++d) {
    X[d] = lin % g.N[d];
    lin /= g.N[d];
  }
  int64_t clo[3] = {0, 0, 0}, chi[3] = {0, 0, 0};
  for (int d = 0; d < DIM; ++d) {
    const int64_t cc = X[d] / K;
    if (X[d] % K == 0) {
      clo[d] = cc - 1 < 0 ? 0 : cc - 1;
      chi[d] = cc > g.n[d] - 1 ? g.n[d] - 1 : cc;
    } else {
      clo[d] = chi[d] = cc;
    }
  }
  double b = 0.0;
  for (int64_t cz = clo[2]; cz <= chi[2]; ++cz)
    for (int64_t cy = clo[1]; cy <= chi[1]; ++cy)
      for (int64_t cx = clo[0]; cx <= chi[0]; ++cx) {
        const int64_t cc[3] = {cx, cy, cz};
        const double e = __ldg(E + cell_lin(g, cc));
        int li = 0;
        for (int d = DIM - 1; d >= 0; --d) li = li * L::KP1 + (int)(X[d] - K * cc[d]);
        const double* krow = Kel + (size_t)(c * L::NN + li) * M;
        for (int lj = 0; lj < L::NN; ++lj) {
          int64_t Y[3] = {0, 0, 0};
          for (int d = 0, rest = lj; d < DIM; ++d) {
            Y[d] = K * cc[d] + rest % L::KP1;
            rest /= L::KP1;
          }
          if (!node_is_dirichlet(g, Y)) continue;
          const int64_t ylin = lattice_lin(g, Y);
          for (int d = 0; d < DIM; ++d) b -= e * __ldg(krow + d * L::NN + lj) * __ldg(u_dir + DIM * ylin + d);
        }
      }
  return b;
}

// rhs of owned vector row r = (node, c): force_c * int phi_node over the node's cells,
// minus the Dirichlet lifting when the trial space has values (u_dir non-null)
template <int DIM, int K>
__global__ void k_rhs_elasticity(Geom g, int64_t nrows_own, const int32_t* __restrict__ row_node,
                                 const double* __restrict__ E, const double* __restrict__ Khat,
                                 const double* __restrict__ Mhat, const double* __restrict__ Fhat, double f0,
                                 double f1, double f2, const double* __restrict__ Kel,
                                 const double* __restrict__ u_dir, double* __restrict__ rhs,
                                 int32_t* __restrict__ bad) {
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows_own) return;
  const int c = (int)(r % DIM);
  const double f = c == 0 ? f0 : (c == 1 ? f1 : f2);
  const int nbad = qk_rhs_row<DIM, K>(g, r, row_node, E, Khat, Mhat, Fhat, f, nullptr, nullptr, rhs);
  if (u_dir) rhs[r] += elasticity_lifting<DIM, K>(g, row_node[r], c, E, Kel, u_dir);
  if (nbad) atomicAdd(bad, nbad);
}

template <int DIM, int K>
static int launch_elasticity(gd_asm* A, const double* E, const double* force, int32_t* bad, cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  if (R == 0) return GD_OK;
  constexpr int M = DIM * Lat<DIM, K>::NN;
  const size_t smem = sizeof(double) * M * M;
  auto kern = k_numeric_elasticity<DIM, K>;
  if (smem > 48 * 1024) GD_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const unsigned nbw = (unsigned)std::min<int64_t>((R + 7) / 8, 152 * 16);
  kern<<<nbw, 256, smem, st>>>(g, R, A->rowptr.p, A->row_node.p, reinterpret_cast<const uint16_t*>(A->code.p), E,
                               A->Kel.p, A->vals.p);
  GD_CUDA_TRY(cudaGetLastError());
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  k_rhs_elasticity<DIM, K><<<(unsigned)((R + 127) / 128), 128, 0, st>>>(
      g, R, A->row_node.p, E, A->Khat.p, A->Mhat.p, A->Fhat.p, force[0], force[1], DIM == 3 ? force[2] : 0.0,
      A->Kel.p, udir, A->rhs.p, bad);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

__global__ void k_gather_local_vec(int64_t n, int bs, const int64_t* __restrict__ lid_gid,
                                   const double* __restrict__ xg, double* __restrict__ xl) {
  const int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (v < bs * n) xl[v] = xg[bs * lid_gid[v / bs] + v % bs];
}

int gather_local_vec(const gd_space* S, int part, const double* xg, double* xl, cudaStream_t st) {
  const DevPart& P = S->parts[part];
  const int64_t n = P.nfree;
  if (n == 0) return GD_OK;
  k_gather_local_vec<<<vblk(S->ncomp * n, 256), 256, 0, st>>>(n, S->ncomp, S->lid_gid.p + P.lid_off, xg, xl);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

}  // namespace gd

using namespace gd;

extern "C" int gd_assemble_elasticity(gd_asm* A, const gd_elasticity* c) {
  if (!A || !c) return fail(GD_ERR_ARG, "gd_assemble_elasticity: null argument");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_assemble_elasticity: run gd_assemble_symbolic first");
  const Geom& g = A->test->geom;
  if (A->bs != g.dim) return fail(GD_ERR_UNSUPPORTED, "gd_assemble_elasticity: needs a vector space with dim components");
  if (!(c->nu > -1.0 && c->nu < 0.5)) return fail(GD_ERR_ARG, "gd_assemble_elasticity: Poisson ratio outside (-1, 0.5)");
  cudaStream_t st = A->test->model->ctx->stream;
  GD_TRY(reference_element(A, c->degree));
  if (A->el_degree != c->degree || A->el_nu != c->nu || !A->Kel.p) {
    std::vector<double> K;
    elasticity_reference(g.dim, g.k, g.h, c->degree, c->nu, K);
    GD_TRY(dalloc(A->Kel, K.size()));
    GD_CUDA_TRY(cudaMemcpyAsync(A->Kel.p, K.data(), sizeof(double) * K.size(), cudaMemcpyHostToDevice, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    A->el_degree = c->degree;
    A->el_nu = c->nu;
  }
  int64_t ncells = 1;
  for (int d = 0; d < g.dim; ++d) ncells *= g.n[d];
  const double* E = c->E;
  if (!E || c->where == GD_HOST) {
    if (A->E_dev.n != (size_t)ncells) GD_TRY(dalloc(A->E_dev, ncells));
    if (E) {
      GD_CUDA_TRY(cudaMemcpyAsync(A->E_dev.p, E, sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
    } else {
      std::vector<double> ones(ncells, 1.0);
      GD_CUDA_TRY(cudaMemcpyAsync(A->E_dev.p, ones.data(), sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
    }
    E = A->E_dev.p;
  }
  if (!A->dred.p) GD_TRY(dalloc(A->dred, 4096));
  int32_t* bad = (int32_t*)A->dred.p;
  GD_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int32_t), st));
  int s = GD_ERR_UNSUPPORTED;
  if (g.dim == 3 && g.k == 1) s = launch_elasticity<3, 1>(A, E, c->force, bad, st);
  else if (g.dim == 3 && g.k == 2) s = launch_elasticity<3, 2>(A, E, c->force, bad, st);
  else if (g.dim == 2 && g.k == 1) s = launch_elasticity<2, 1>(A, E, c->force, bad, st);
  else if (g.dim == 2 && g.k == 2) s = launch_elasticity<2, 2>(A, E, c->force, bad, st);
  if (s != GD_OK) return s == GD_ERR_UNSUPPORTED ? fail(s, "gd_assemble_elasticity: unsupported dim/order") : s;
  int32_t hbad = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&hbad, bad, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (hbad) return fail(GD_ERR_NUMERIC, "gd_assemble_elasticity: E is not finite and positive in " +
                                            std::to_string(hbad) + " cell visits");
  A->numeric_done = true;
  A->qp_values = false;
  ++A->numeric_epoch;
  return GD_OK;
}
