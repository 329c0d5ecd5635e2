// Batched assembly and solve of many independent problems (uneven sizes and orders).
//
// No counterpart in the reference, which assembles one problem per call.  A batch holds
// assemblers whose symbolic phase is done; one numeric assembly of the whole batch is a
// single persistent kernel launch: a grid of resident CTAs pulls row tasks (a fixed
// number of consecutive owned rows of one problem) from an atomic counter, problems of
// higher order (costlier rows) and more rows first, so uneven problems balance without
// per-problem launches.  A task runs the same row bodies as the single-problem Q_k
// kernels (gd_rows.cuh: lane groups of a warp per matrix row, one thread per right-hand-side row), so
// every problem's values equal what its own assembler would compute.  The launch shape
// (rows per task, CTAs per SM) is chosen by timing candidates on the first call; the
// counter reset and the launch are then captured in a CUDA graph and replayed.
//
// The batched Jacobi-PCG (FP64) advances all unconverged problems together: every CG
// step is one launch over the row tasks of all problems, with per-problem scalars formed
// from per-task partials summed in task order (deterministic); problems that reached the
// tolerance drop out of the work.  Sixteen CG steps are captured in a CUDA graph and
// replayed until every problem has converged.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_rows.cuh"
#include "gd_solve_mixed.h"

namespace gd {

int reference_element(gd_asm* A, int degree);

struct BatchProb {
  Geom g;
  int k, code_bytes;
  int64_t nrows;   // owned rows
  const int64_t* rowptr;
  const int32_t* row_node;
  const void* code;
  const int32_t* colgid;
  const double* kappa;
  const double* Khat;
  const double* Mhat;
  const double* Fhat;
  double f_const;
  const double* f_nodal;
  const double* u_dir;
  double* vals;
  double* rhs;
  int64_t voff;              // offset of the problem's vectors in the batch solve vectors
  int64_t stask0, nstasks;   // solve tasks
};

struct BScal {
  double rz, pq, alpha, beta, rr, bb, tol2;
  int32_t conv, it;
};

constexpr int kBatchThreads = 256;
constexpr int kBatchMaxKhat = 64 * 64;    // doubles of the largest reference stiffness table (3D Q3)
constexpr int kBatchMaxEtab = 8 * 343;    // entries of the largest entry table (3D Q3)
constexpr size_t kBatchSmem = sizeof(double) * kBatchMaxKhat + sizeof(uint16_t) * kBatchMaxEtab;
constexpr int kSolveRows = 128;   // rows per solve task
constexpr int kSolveStepsPerGraph = 16;

struct BatchShape {
  int rows, per_sm;
};
constexpr BatchShape kBatchShapes[] = {{32, 3}, {64, 3}, {128, 3}, {256, 3}, {64, 2}, {128, 2}, {256, 2}, {128, 4}};
constexpr int kNumBatchShapes = 8;

// ---- assembly -------------------------------------------------------------------------
template <int DIM, int K, typename CodeT>
__device__ __forceinline__ void batch_task(const BatchProb& P, int64_t r0, int64_t r1, const double* sK,
                                           const uint16_t* etab, double* skap, int* slx, int& nbad) {
  constexpr int RPW = RowLanes<DIM, K>::RPW;
  const int warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t rb = r0 + warp * RPW; rb < r1; rb += nw * RPW)
    qk_matrix_rows<DIM, K, CodeT>(P.g, rb, r1, P.rowptr, P.row_node, (const CodeT*)P.code, P.kappa, sK, etab,
                                  P.vals, skap + 32 * warp, slx + 32 * warp);
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x)
    nbad += qk_rhs_row<DIM, K>(P.g, r, P.row_node, P.kappa, P.Khat, P.Mhat, P.Fhat, P.f_const, P.f_nodal, P.u_dir,
                               P.rhs);
}

// tstart[j] = first task of the j-th problem in schedule order ord[j]; tstart[nprobs] = total
__global__ void __launch_bounds__(kBatchThreads, 3)
k_batch_numeric(const BatchProb* __restrict__ probs, const int32_t* __restrict__ ord,
                const int64_t* __restrict__ tstart, int nprobs, int rows_per_task, unsigned long long* next,
                int32_t* bad) {
  extern __shared__ double sK[];   // reference stiffness table of the current problem, then its entry table
  __shared__ long long s_task;
  __shared__ int s_prob;
  __shared__ double s_kap[kBatchThreads / 32 * 32];
  __shared__ int s_lx[kBatchThreads / 32 * 32];
  int nbad = 0;
  const int64_t total = tstart[nprobs];
  if (threadIdx.x == 0) s_prob = -1;
  while (true) {
    __syncthreads();   // every thread has read the previous task id
    if (threadIdx.x == 0) s_task = (long long)atomicAdd(next, 1ull);
    __syncthreads();
    const int64_t t = s_task;
    if (t >= total) break;
    int lo = 0, hi = nprobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (tstart[mid] <= t) lo = mid;
      else hi = mid - 1;
    }
    const int pid = ord[lo];
    const BatchProb& P = probs[pid];
    uint16_t* etab = reinterpret_cast<uint16_t*>(sK + kBatchMaxKhat);
    if (pid != s_prob) {   // uniform across the block
      __syncthreads();      // the previous problem's tables are no longer read
      int nn = 1;
      for (int d = 0; d < P.g.dim; ++d) nn *= P.k + 1;
      for (int i = threadIdx.x; i < nn * nn; i += blockDim.x) sK[i] = P.Khat[i];
      switch (P.g.dim * 10 + P.k) {
        case 31: build_entry_tab<3, 1>(etab); break;
        case 32: build_entry_tab<3, 2>(etab); break;
        case 33: build_entry_tab<3, 3>(etab); break;
        case 21: build_entry_tab<2, 1>(etab); break;
        case 22: build_entry_tab<2, 2>(etab); break;
        case 23: build_entry_tab<2, 3>(etab); break;
        default: break;
      }
      __syncthreads();
      if (threadIdx.x == 0) s_prob = pid;
    }
    const int64_t r0 = (t - tstart[lo]) * rows_per_task;
    const int64_t r1 = r0 + rows_per_task < P.nrows ? r0 + rows_per_task : P.nrows;
    switch (P.g.dim * 10 + P.k) {
      case 31: batch_task<3, 1, uint8_t>(P, r0, r1, sK, etab, s_kap, s_lx, nbad); break;
      case 32: batch_task<3, 2, uint8_t>(P, r0, r1, sK, etab, s_kap, s_lx, nbad); break;
      case 33: batch_task<3, 3, uint16_t>(P, r0, r1, sK, etab, s_kap, s_lx, nbad); break;
      case 21: batch_task<2, 1, uint8_t>(P, r0, r1, sK, etab, s_kap, s_lx, nbad); break;
      case 22: batch_task<2, 2, uint8_t>(P, r0, r1, sK, etab, s_kap, s_lx, nbad); break;
      case 23: batch_task<2, 3, uint8_t>(P, r0, r1, sK, etab, s_kap, s_lx, nbad); break;
      default: break;
    }
  }
  if (nbad) atomicAdd(bad, nbad);
}

// ---- batched Jacobi-PCG (FP64) ---------------------------------------------------------
// solve task t -> (problem p, rows [r0, r1)); stask0 is ascending in problem order
__device__ __forceinline__ int stask_problem(const BatchProb* probs, int nprobs, int64_t t) {
  int lo = 0, hi = nprobs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (probs[mid].stask0 <= t) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ double bsum(double v, double* sh) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
  __syncthreads();
  return s;   // valid in thread 0
}

// d = 1/diag, x = 0, r = b, z = d r, p = z; partials r.z, r.r
__global__ void __launch_bounds__(kBatchThreads)
k_bpcg_init(const BatchProb* __restrict__ probs, int nprobs, int64_t ntasks, double* __restrict__ X,
            double* __restrict__ Rv, double* __restrict__ Z, double* __restrict__ Pv, double* __restrict__ D,
            double* __restrict__ part, int32_t* __restrict__ bad) {
  __shared__ double sh[kBatchThreads / 32];
  for (int64_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const int p = stask_problem(probs, nprobs, t);
    const BatchProb& P = probs[p];
    const int64_t r0 = (t - P.stask0) * kSolveRows;
    const int64_t r1 = r0 + kSolveRows < P.nrows ? r0 + kSolveRows : P.nrows;
    double a = 0.0, b2 = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      double dg = 0.0;
      for (int64_t e = P.rowptr[r]; e < P.rowptr[r + 1]; ++e)
        if (P.colgid[e] == r) dg = P.vals[e];
      if (!(dg > 0.0) || !isfinite(dg)) atomicAdd(bad, 1);
      const double di = dg > 0.0 ? 1.0 / dg : 0.0;
      const int64_t i = P.voff + r;
      const double bv = P.rhs[r];
      D[i] = di;
      X[i] = 0.0;
      Rv[i] = bv;
      const double zi = di * bv;
      Z[i] = zi;
      Pv[i] = zi;
      a += bv * zi;
      b2 += bv * bv;
    }
    const double sa = bsum(a, sh), sb = bsum(b2, sh);
    if (threadIdx.x == 0) {
      part[2 * t] = sa;
      part[2 * t + 1] = sb;
    }
  }
}

// q = A p (one warp per row), partial p.q
__global__ void __launch_bounds__(kBatchThreads)
k_bpcg_spmv(const BatchProb* __restrict__ probs, int nprobs, int64_t ntasks, const BScal* __restrict__ sc,
            const double* __restrict__ Pv, double* __restrict__ Q, double* __restrict__ part) {
  __shared__ double sh[kBatchThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int64_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const int p = stask_problem(probs, nprobs, t);
    if (sc[p].conv) continue;   // uniform across the block
    const BatchProb& P = probs[p];
    const int64_t r0 = (t - P.stask0) * kSolveRows;
    const int64_t r1 = r0 + kSolveRows < P.nrows ? r0 + kSolveRows : P.nrows;
    const double* pp = Pv + P.voff;
    double dot = 0.0;
    for (int64_t r = r0 + warp; r < r1; r += nw) {
      double s = 0.0;
      for (int64_t e = P.rowptr[r] + lane; e < P.rowptr[r + 1]; e += 32) s = fma(P.vals[e], pp[P.colgid[e]], s);
      for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
      if (lane == 0) {
        Q[P.voff + r] = s;
        dot = fma(s, pp[r], dot);
      }
    }
    const double sd = bsum(dot, sh);
    if (threadIdx.x == 0) part[2 * t] = sd;
  }
}

// per problem (one CTA each): sums of its task partials in task order
// mode 0: rz, rr (= bb at start); 1: alpha = rz / pq; 2: beta, convergence
__global__ void __launch_bounds__(kBatchThreads)
k_bpcg_scalars(const BatchProb* __restrict__ probs, int mode, const double* __restrict__ part, BScal* __restrict__ sc,
               double rtol) {
  __shared__ double sh[kBatchThreads / 32];
  const int p = blockIdx.x;
  const BatchProb& P = probs[p];
  BScal& S = sc[p];
  if (mode != 0 && S.conv) return;   // uniform across the block
  double a = 0.0, b = 0.0;
  for (int64_t t = P.stask0 + threadIdx.x; t < P.stask0 + P.nstasks; t += blockDim.x) {
    a += part[2 * t];
    if (mode != 1) b += part[2 * t + 1];
  }
  const double sa = bsum(a, sh), sb = bsum(b, sh);
  if (threadIdx.x != 0) return;
  if (mode == 0) {
    S.rz = sa;
    S.rr = sb;
    S.bb = sb;
    S.tol2 = rtol * rtol * sb;
    S.it = 0;
    S.beta = 0.0;
    S.conv = (sb == 0.0 || P.nrows == 0) ? 1 : 0;
  } else if (mode == 1) {
    S.pq = sa;
    S.alpha = sa != 0.0 ? S.rz / sa : 0.0;
  } else {
    S.beta = S.rz != 0.0 ? sa / S.rz : 0.0;
    S.rz = sa;
    S.rr = sb;
    S.it += 1;
    if (!(sb > S.tol2)) S.conv = 1;   // also stops on a non-finite residual
  }
}

// x += alpha p, r -= alpha q, z = d r; partials r.z, r.r
__global__ void __launch_bounds__(kBatchThreads)
k_bpcg_update(const BatchProb* __restrict__ probs, int nprobs, int64_t ntasks, const BScal* __restrict__ sc,
              double* __restrict__ X, double* __restrict__ Rv, double* __restrict__ Z, const double* __restrict__ Pv,
              const double* __restrict__ Q, const double* __restrict__ D, double* __restrict__ part) {
  __shared__ double sh[kBatchThreads / 32];
  for (int64_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const int p = stask_problem(probs, nprobs, t);
    if (sc[p].conv) continue;
    const BatchProb& P = probs[p];
    const double alpha = sc[p].alpha;
    const int64_t r0 = (t - P.stask0) * kSolveRows;
    const int64_t r1 = r0 + kSolveRows < P.nrows ? r0 + kSolveRows : P.nrows;
    double a = 0.0, b = 0.0;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const int64_t i = P.voff + r;
      X[i] += alpha * Pv[i];
      const double ri = Rv[i] - alpha * Q[i];
      Rv[i] = ri;
      const double zi = D[i] * ri;
      Z[i] = zi;
      a += ri * zi;
      b += ri * ri;
    }
    const double sa = bsum(a, sh), sb = bsum(b, sh);
    if (threadIdx.x == 0) {
      part[2 * t] = sa;
      part[2 * t + 1] = sb;
    }
  }
}

// p = z + beta p
__global__ void __launch_bounds__(kBatchThreads)
k_bpcg_pupdate(const BatchProb* __restrict__ probs, int nprobs, int64_t ntasks, const BScal* __restrict__ sc,
               const double* __restrict__ Z, double* __restrict__ Pv) {
  for (int64_t t = blockIdx.x; t < ntasks; t += gridDim.x) {
    const int p = stask_problem(probs, nprobs, t);
    if (sc[p].conv) continue;
    const BatchProb& P = probs[p];
    const double beta = sc[p].beta;
    const int64_t r0 = (t - P.stask0) * kSolveRows;
    const int64_t r1 = r0 + kSolveRows < P.nrows ? r0 + kSolveRows : P.nrows;
    for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
      const int64_t i = P.voff + r;
      Pv[i] = Z[i] + beta * Pv[i];
    }
  }
}

}  // namespace gd

using namespace gd;

struct gd_batch {
  std::vector<gd_asm*> asms;
  std::vector<BatchProb> hp;
  std::vector<int32_t> ord;   // schedule order (problem indices)
  DBuf<BatchProb> probs;
  DBuf<int32_t> d_ord;
  DBuf<int64_t> tstart;
  DBuf<unsigned long long> counter;
  DBuf<int32_t> bad;
  int64_t rows = 0, nnz = 0;
  int shape = -1;
  float shape_ms[kNumBatchShapes] = {0};
  int grid = 0;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  // solve
  DBuf<double> vec;   // x r z p q d (6 * rows)
  DBuf<double> part;
  DBuf<BScal> sc;
  int64_t nstasks = 0;
  cudaGraph_t sgraph = nullptr;
  cudaGraphExec_t sexec = nullptr;
  double solve_rtol = -1.0;
};

namespace gd {

static int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 152;
}

// task prefix for a rows-per-task value, in schedule order
static int upload_tasks(gd_batch* B, int rows_per_task, cudaStream_t st) {
  const int np = (int)B->hp.size();
  std::vector<int64_t> ts(np + 1, 0);
  for (int j = 0; j < np; ++j) {
    const BatchProb& P = B->hp[B->ord[j]];
    ts[j + 1] = ts[j] + (P.nrows + rows_per_task - 1) / rows_per_task;
  }
  GD_CUDA_TRY(cudaMemcpyAsync(B->tstart.p, ts.data(), sizeof(int64_t) * (np + 1), cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

static int launch_batch(gd_batch* B, int shape, cudaStream_t st) {
  const BatchShape s = kBatchShapes[shape];
  GD_CUDA_TRY(cudaMemsetAsync(B->counter.p, 0, sizeof(unsigned long long), st));
  k_batch_numeric<<<sm_count() * s.per_sm, kBatchThreads, kBatchSmem, st>>>(B->probs.p, B->d_ord.p, B->tstart.p,
                                                                          (int)B->hp.size(), s.rows, B->counter.p,
                                                                          B->bad.p);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

// time every candidate shape once (after one untimed launch), keep the fastest, capture it
static int tune_and_capture(gd_batch* B, cudaStream_t st) {
  cudaEvent_t e0, e1;
  GD_CUDA_TRY(cudaEventCreate(&e0));
  GD_CUDA_TRY(cudaEventCreate(&e1));
  int best = 0;
  for (int s = 0; s < kNumBatchShapes; ++s) {
    GD_TRY(upload_tasks(B, kBatchShapes[s].rows, st));
    if (s == 0) GD_TRY(launch_batch(B, s, st));   // first launch pays module loading
    GD_CUDA_TRY(cudaEventRecord(e0, st));
    GD_TRY(launch_batch(B, s, st));
    GD_CUDA_TRY(cudaEventRecord(e1, st));
    GD_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    GD_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
    B->shape_ms[s] = ms;
    if (ms < B->shape_ms[best]) best = s;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  B->shape = best;
  GD_TRY(upload_tasks(B, kBatchShapes[best].rows, st));
  GD_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  const int rc = launch_batch(B, best, st);
  cudaGraph_t g = nullptr;
  const cudaError_t ce = cudaStreamEndCapture(st, &g);
  if (rc != GD_OK) return rc;
  GD_CUDA_TRY(ce);
  B->graph = g;
  GD_CUDA_TRY(cudaGraphInstantiate(&B->exec, g, 0));
  return GD_OK;
}

static int stage_coeffs(gd_asm* A, const gd_coeffs* c, const double** kappa, const double** fn, cudaStream_t st) {
  const Geom& g = A->test->geom;
  int64_t ncells = 1, nnodes = 1;
  for (int d = 0; d < g.dim; ++d) {
    ncells *= g.n[d];
    nnodes *= g.N[d];
  }
  *kappa = c->kappa;
  *fn = c->f_nodal;
  if (c->where == GD_HOST || !c->kappa) {
    if (A->kappa_dev.n != (size_t)ncells) GD_TRY(dalloc(A->kappa_dev, ncells));
    if (c->kappa) {
      GD_CUDA_TRY(cudaMemcpyAsync(A->kappa_dev.p, c->kappa, sizeof(double) * ncells,
                                  c->where == GD_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice, st));
    } else {
      std::vector<double> ones(ncells, 1.0);
      GD_CUDA_TRY(cudaMemcpyAsync(A->kappa_dev.p, ones.data(), sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
    }
    *kappa = A->kappa_dev.p;
  }
  if (c->f_nodal && c->where == GD_HOST) {
    if (A->f_dev.n != (size_t)nnodes) GD_TRY(dalloc(A->f_dev, nnodes));
    GD_CUDA_TRY(cudaMemcpyAsync(A->f_dev.p, c->f_nodal, sizeof(double) * nnodes, cudaMemcpyHostToDevice, st));
    *fn = A->f_dev.p;
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

}  // namespace gd

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" int gd_batch_create(gd_asm* const* asms, const gd_coeffs* coeffs, int nprobs, gd_batch** out) {
  if (!asms || !coeffs || nprobs < 1 || !out) return fail(GD_ERR_ARG, "gd_batch_create: bad argument");
  gd_ctx* ctx = nullptr;
  for (int p = 0; p < nprobs; ++p) {
    gd_asm* A = asms[p];
    if (!A) return fail(GD_ERR_ARG, "gd_batch_create: null assembler");
    if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_batch_create: every assembler needs its symbolic phase");
    if (A->test->geom.k < 1 || A->test->geom.k > 3) return fail(GD_ERR_UNSUPPORTED, "gd_batch_create: order 1..3");
    if (A->bs != 1) return fail(GD_ERR_UNSUPPORTED, "gd_batch_create: scalar spaces only");
    const Geom& g = A->test->geom;
    const int W = 2 * g.k + 1;
    const int want = (W * W * (g.dim == 3 ? W : 1)) <= 256 ? 1 : 2;
    if (A->code_bytes != want) return fail(GD_ERR_STATE, "gd_batch_create: unexpected stencil code width");
    if (!ctx) ctx = A->test->model->ctx;
    else if (A->test->model->ctx != ctx)
      return fail(GD_ERR_ARG, "gd_batch_create: all problems must share one context");
    for (int q = 0; q < p; ++q)
      if (asms[q] == A) return fail(GD_ERR_ARG, "gd_batch_create: an assembler appears twice");
  }
  cudaStream_t st = ctx->stream;
  gd_batch* B = new gd_batch();
  auto bail = [&](int s) {
    std::string msg = gd_last_error();
    gd_batch_destroy(B);
    return fail(s, msg);
  };
  int s = GD_OK;
  int64_t voff = 0, st0 = 0;
  for (int p = 0; p < nprobs; ++p) {
    gd_asm* A = asms[p];
    const gd_coeffs* c = coeffs + p;
    if ((s = reference_element(A, c->degree)) != GD_OK) return bail(s);
    const double* kappa = nullptr;
    const double* fn = nullptr;
    if ((s = stage_coeffs(A, c, &kappa, &fn, st)) != GD_OK) return bail(s);
    BatchProb P{};
    P.g = A->test->geom;
    P.k = P.g.k;
    P.code_bytes = A->code_bytes;
    P.nrows = A->ngdofs;
    P.rowptr = A->rowptr.p;
    P.row_node = A->row_node.p;
    P.code = A->code.p;
    P.colgid = A->colgid.p;
    P.kappa = kappa;
    P.Khat = A->Khat.p;
    P.Mhat = A->Mhat.p;
    P.Fhat = A->Fhat.p;
    P.f_const = c->f_const;
    P.f_nodal = fn;
    P.u_dir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
    P.vals = A->vals.p;
    P.rhs = A->rhs.p;
    P.voff = voff;
    P.stask0 = st0;
    P.nstasks = (P.nrows + kSolveRows - 1) / kSolveRows;
    voff += P.nrows;
    st0 += P.nstasks;
    B->rows += P.nrows;
    B->nnz += A->nnz_own;
    B->asms.push_back(A);
    B->hp.push_back(P);
  }
  B->nstasks = st0;
  B->ord.resize(nprobs);
  std::iota(B->ord.begin(), B->ord.end(), 0);
  std::stable_sort(B->ord.begin(), B->ord.end(), [&](int a, int b) {
    if (B->hp[a].k != B->hp[b].k) return B->hp[a].k > B->hp[b].k;
    return B->hp[a].nrows > B->hp[b].nrows;
  });
  if ((s = dalloc(B->probs, nprobs)) != GD_OK) return bail(s);
  if ((s = dalloc(B->d_ord, nprobs)) != GD_OK) return bail(s);
  if ((s = dalloc(B->tstart, nprobs + 1)) != GD_OK) return bail(s);
  if ((s = dalloc(B->counter, 1)) != GD_OK) return bail(s);
  if ((s = dalloc(B->bad, 1)) != GD_OK) return bail(s);
  cudaError_t e = cudaMemcpyAsync(B->probs.p, B->hp.data(), sizeof(BatchProb) * nprobs, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(B->d_ord.p, B->ord.data(), sizeof(int32_t) * nprobs, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(B->bad.p, 0, sizeof(int32_t), st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) {
    fail(GD_ERR_CUDA, std::string("gd_batch_create: ") + cudaGetErrorString(e));
    return bail(GD_ERR_CUDA);
  }
  *out = B;
  return GD_OK;
}

extern "C" int gd_batch_destroy(gd_batch* B) {
  if (!B) return GD_OK;
  if (B->exec) cudaGraphExecDestroy(B->exec);
  if (B->graph) cudaGraphDestroy(B->graph);
  if (B->sexec) cudaGraphExecDestroy(B->sexec);
  if (B->sgraph) cudaGraphDestroy(B->sgraph);
  dfreeb(B->probs);
  dfreeb(B->d_ord);
  dfreeb(B->tstart);
  dfreeb(B->counter);
  dfreeb(B->bad);
  dfreeb(B->vec);
  dfreeb(B->part);
  dfreeb(B->sc);
  delete B;
  return GD_OK;
}

static int batch_stream(const gd_batch* B, cudaStream_t* st) {
  *st = B->asms[0]->test->model->ctx->stream;
  return GD_OK;
}

// One numeric assembly of every problem: a single persistent launch (graph replay).
// The first call autotunes the launch shape and captures the graph.
static int batch_assemble(gd_batch* B, bool sync) {
  if (!B) return fail(GD_ERR_ARG, "gd_batch_assemble: null batch");
  cudaStream_t st;
  batch_stream(B, &st);
  if (!B->exec) {
    GD_CUDA_TRY(cudaMemsetAsync(B->bad.p, 0, sizeof(int32_t), st));
    GD_TRY(tune_and_capture(B, st));
  }
  GD_CUDA_TRY(cudaMemsetAsync(B->bad.p, 0, sizeof(int32_t), st));
  GD_CUDA_TRY(cudaGraphLaunch(B->exec, st));
  for (gd_asm* A : B->asms) {
    A->numeric_done = true;
    ++A->numeric_epoch;
  }
  if (sync) {
    int32_t hbad = 0;
    GD_CUDA_TRY(cudaMemcpyAsync(&hbad, B->bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    if (hbad) return fail(GD_ERR_NUMERIC, "gd_batch_assemble: kappa is not finite and positive in " +
                                              std::to_string(hbad) + " cell visits");
  }
  return GD_OK;
}

extern "C" int gd_batch_assemble(gd_batch* B) { return batch_assemble(B, true); }
extern "C" int gd_batch_assemble_async(gd_batch* B) { return batch_assemble(B, false); }

extern "C" int gd_batch_counts(const gd_batch* B, int32_t* nprobs, int64_t* rows, int64_t* nnz_owned) {
  if (!B) return fail(GD_ERR_ARG, "gd_batch_counts: null batch");
  if (nprobs) *nprobs = (int32_t)B->asms.size();
  if (rows) *rows = B->rows;
  if (nnz_owned) *nnz_owned = B->nnz;
  return GD_OK;
}

extern "C" int gd_batch_tuning(const gd_batch* B, int32_t* shape, int32_t* rows_per_task, int32_t* ctas_per_sm,
                               float* ms_per_shape, int32_t* nshapes) {
  if (!B) return fail(GD_ERR_ARG, "gd_batch_tuning: null batch");
  if (shape) *shape = B->shape;
  if (rows_per_task) *rows_per_task = B->shape >= 0 ? kBatchShapes[B->shape].rows : -1;
  if (ctas_per_sm) *ctas_per_sm = B->shape >= 0 ? kBatchShapes[B->shape].per_sm : -1;
  if (ms_per_shape)
    for (int s = 0; s < kNumBatchShapes; ++s) ms_per_shape[s] = B->shape_ms[s];
  if (nshapes) *nshapes = kNumBatchShapes;
  return GD_OK;
}

// Batched Jacobi-PCG (FP64) of every problem to the relative residual rtol.
// stats (optional) receives one entry per problem; the residual there is recomputed in
// FP64 from the assembled matrix at exit.
extern "C" int gd_batch_solve(gd_batch* B, double rtol, int maxit, gd_solve_stats* stats) {
  if (!B || !(rtol > 0.0) || maxit < 1) return fail(GD_ERR_ARG, "gd_batch_solve: bad argument");
  for (gd_asm* A : B->asms)
    if (!A->numeric_done) return fail(GD_ERR_STATE, "gd_batch_solve: assemble the batch first");
  cudaStream_t st;
  batch_stream(B, &st);
  const int np = (int)B->hp.size();
  const int64_t N = std::max<int64_t>(B->rows, 1);
  auto t0 = std::chrono::steady_clock::now();
  if (B->vec.n < (size_t)(6 * N)) GD_TRY(dalloc(B->vec, 6 * N));
  if (B->part.n < (size_t)(2 * std::max<int64_t>(B->nstasks, 1))) GD_TRY(dalloc(B->part, 2 * std::max<int64_t>(B->nstasks, 1)));
  if (B->sc.n < (size_t)np) GD_TRY(dalloc(B->sc, np));
  double* X = B->vec.p;
  double* Rv = X + N;
  double* Z = Rv + N;
  double* Pv = Z + N;
  double* Q = Pv + N;
  double* D = Q + N;
  const int grid = (int)std::min<int64_t>(std::max<int64_t>(B->nstasks, 1), (int64_t)sm_count() * 8);
  GD_CUDA_TRY(cudaMemsetAsync(B->bad.p, 0, sizeof(int32_t), st));
  k_bpcg_init<<<grid, kBatchThreads, 0, st>>>(B->probs.p, np, B->nstasks, X, Rv, Z, Pv, D, B->part.p, B->bad.p);
  k_bpcg_scalars<<<np, kBatchThreads, 0, st>>>(B->probs.p, 0, B->part.p, B->sc.p, rtol);
  GD_CUDA_TRY(cudaGetLastError());
  int32_t hbad = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&hbad, B->bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (hbad) return fail(GD_ERR_NUMERIC, "gd_batch_solve: a diagonal entry is not positive");
  // sixteen CG steps as one graph (the scalars live on the device)
  if (!B->sexec || B->solve_rtol != rtol) {
    if (B->sexec) {
      cudaGraphExecDestroy(B->sexec);
      cudaGraphDestroy(B->sgraph);
      B->sexec = nullptr;
      B->sgraph = nullptr;
    }
    GD_CUDA_TRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < kSolveStepsPerGraph; ++k) {
      k_bpcg_spmv<<<grid, kBatchThreads, 0, st>>>(B->probs.p, np, B->nstasks, B->sc.p, Pv, Q, B->part.p);
      k_bpcg_scalars<<<np, kBatchThreads, 0, st>>>(B->probs.p, 1, B->part.p, B->sc.p, rtol);
      k_bpcg_update<<<grid, kBatchThreads, 0, st>>>(B->probs.p, np, B->nstasks, B->sc.p, X, Rv, Z, Pv, Q, D,
                                                     B->part.p);
      k_bpcg_scalars<<<np, kBatchThreads, 0, st>>>(B->probs.p, 2, B->part.p, B->sc.p, rtol);
      k_bpcg_pupdate<<<grid, kBatchThreads, 0, st>>>(B->probs.p, np, B->nstasks, B->sc.p, Z, Pv);
    }
    cudaGraph_t g = nullptr;
    const cudaError_t le = cudaGetLastError();
    const cudaError_t ce = cudaStreamEndCapture(st, &g);
    GD_CUDA_TRY(le);
    GD_CUDA_TRY(ce);
    B->sgraph = g;
    GD_CUDA_TRY(cudaGraphInstantiate(&B->sexec, g, 0));
    B->solve_rtol = rtol;
  }
  std::vector<BScal> hs(np);
  int done_steps = 0;
  while (true) {
    GD_CUDA_TRY(cudaMemcpyAsync(hs.data(), B->sc.p, sizeof(BScal) * np, cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    bool all = true;
    for (int p = 0; p < np; ++p) all = all && hs[p].conv;
    if (all || done_steps >= maxit) break;
    GD_CUDA_TRY(cudaGraphLaunch(B->sexec, st));
    done_steps += kSolveStepsPerGraph;
  }
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  bool all_conv = true;
  for (int p = 0; p < np; ++p) {
    const BatchProb& P = B->hp[p];
    gd_asm* A = B->asms[p];
    double rel = 0.0;
    if (P.nrows > 0) {
      DBuf<double>& w = A->dred;
      if (!w.p || w.n < 4096) GD_TRY(dalloc(w, 4096));
      int gr = 0;
      GD_TRY(residual_fp64(P.nrows, A->rowptr.p, A->colgid.p, A->vals.p, X + P.voff, A->rhs.p, nullptr, w.p,
                           w.p + 2048, st, &gr));
      std::vector<double> h(2 * (size_t)gr);
      GD_CUDA_TRY(cudaMemcpyAsync(h.data(), w.p, sizeof(double) * gr, cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaMemcpyAsync(h.data() + gr, w.p + 2048, sizeof(double) * gr, cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
      double rr = 0.0, bb = 0.0;
      for (int i = 0; i < gr; ++i) {
        rr += h[i];
        bb += h[gr + i];
      }
      rel = bb > 0.0 ? std::sqrt(rr / bb) : 0.0;
    }
    const bool conv = hs[p].conv && rel <= 10.0 * rtol;
    all_conv = all_conv && conv;
    if (stats) {
      stats[p].iterations = hs[p].it;
      stats[p].converged = conv;
      stats[p].rel_residual = rel;
      stats[p].seconds = secs;
    }
  }
  if (!all_conv) return fail(GD_ERR_NOTCONVERGED, "gd_batch_solve: not every problem reached the tolerance");
  return GD_OK;
}

extern "C" int gd_batch_solution(const gd_batch* B, int p, double* x, int where) {
  if (!B || p < 0 || p >= (int)B->hp.size() || !x) return fail(GD_ERR_ARG, "gd_batch_solution: bad argument");
  if (!B->vec.p) return fail(GD_ERR_STATE, "gd_batch_solution: run gd_batch_solve first");
  cudaStream_t st;
  batch_stream(B, &st);
  const BatchProb& P = B->hp[p];
  const int64_t N = std::max<int64_t>(B->rows, 1);
  (void)N;
  GD_CUDA_TRY(cudaMemcpyAsync(x, B->vec.p + P.voff, sizeof(double) * P.nrows,
                              where == GD_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}
