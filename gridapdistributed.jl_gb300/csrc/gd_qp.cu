// Coefficients that vary inside a cell: a(u,v) = int kappa(x) grad(v).grad(u) dOmega, and
// linear elasticity with E(x), where kappa (or E) is known at the tensor Gauss points of
// every cell -- CellData's integrate of an integrand built from a CellField that is not
// constant per cell (src/CellData.jl:234-259, `*(Integrand, Measure)` at :255-259).
//
// Every cell of a CartesianDiscreteModel is the same axis-aligned box, so
//   K_e(cell) = sum_q kappa(cell, q) H_q,
//   H_q[i][j] = w_q |J| grad(phi_i)(x_q) . grad(phi_j)(x_q)            (scalar)
//   H_q[(c,i)][(d,j)] = w_q |J| (lam d_c phi_i d_d phi_j + mu d_d phi_i d_c phi_j
//                              + delta_cd mu grad(phi_i) . grad(phi_j))  (elasticity, E = 1)
// with the same H_q for all cells.  Over all cells that is one matrix product,
//   Ke[cell][n] = sum_q H[n][q] C[cell][q]   (n: element-matrix entry, q: point),
// with K = 8 .. 64 points and 64 .. 6561 entries: the contraction runs on the tensor cores
// (tcgen05.mma kind::f16, BF16 operands, FP32 accumulators in TMEM).  BF16 keeps 8
// mantissa bits; each FP32 operand is split into 1, 2 or 3 BF16 terms and the products of
// the terms whose orders add up to less than the split count are accumulated, which gives
// about 2^-9, 2^-17 or 2^-24 relative accuracy (GD_QP_BF16 / _BF16X3 / _BF16X6).  The
// element matrices go to HBM in FP32, cell-major, and a row kernel then sums each CSR entry
// over the cells that hold both of its nodes in a fixed order (deterministic, no atomics),
// as the cell-constant path does with kappa_c Khat.  GD_QP_FP64 forms Ke in FP64 on the
// CUDA cores instead (the exact mode, same row kernels).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gd_internal.h"
#include "gd_rows.cuh"
#include "gd_tc.cuh"

namespace gd {

// ---------------------------------------------------------------------------------------
// Workspace
// ---------------------------------------------------------------------------------------
struct QpState {
  // reference tables of the current (degree, ncomp, nu): H[q][n] in FP64
  int degree = -1, ncomp = 0;
  double nu = 0.0;
  int nqt = 0, nne = 0, nnep = 0, kp = 0;
  DBuf<double> H64;
  // A operand tiles of H^T per split count (index S-1): [entry tile][split][128 x KP] BF16
  DBuf<__nv_bfloat16> At[3];
  int n_etiles = 0;
  // B operand tiles of the coefficients: [cell tile][split][NCT x KP] BF16
  DBuf<__nv_bfloat16> Bt;
  // element matrices, cell-major with row stride nnep
  DBuf<float> Ke32;
  DBuf<double> Ke64;
  DBuf<double> kq_dev;   // staging of host coefficients
  DBuf<int32_t> flags;   // [0] bad coefficients, [1] tensor-kernel error
  int last_precision = -1;
  double ms_ke = 0.0, ms_rows = 0.0;   // event-timed phases of the last call
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
};

void qp_release(QpState* q) {
  if (!q) return;
  dfreeb(q->H64);
  for (auto& a : q->At) dfreeb(a);
  dfreeb(q->Bt);
  dfreeb(q->Ke32);
  dfreeb(q->Ke64);
  dfreeb(q->kq_dev);
  dfreeb(q->flags);
  for (auto& e : q->ev)
    if (e) cudaEventDestroy(e);
  delete q;
}

// ---------------------------------------------------------------------------------------
// Host: per-point tables, BF16 splitting, operand tiles
// ---------------------------------------------------------------------------------------
static uint16_t f2bf_bits(float f) {   // round to nearest even (finite inputs)
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7FFFFFFFu) > 0x7F800000u) return 0x7FC0u;
  const uint32_t r = u + 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(r >> 16);
}
static float bf_bits2f(uint16_t b) {
  const uint32_t u = (uint32_t)b << 16;
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

// H[q][n] of one reference cell (lexicographic local nodes, points x fastest).
static void qp_tables(int dim, int k, const double* h, int degree, int ncomp, double nu, std::vector<double>& H,
                      int& nqt, int& nne) {
  const int nq = (degree + 2) / 2, kp1 = k + 1;
  std::vector<double> xq, wq;
  gauss_legendre01(nq, xq, wq);
  std::vector<double> V(nq * kp1), D(nq * kp1);
  for (int q = 0; q < nq; ++q) lagrange01(k, xq[q], &V[q * kp1], &D[q * kp1]);
  int nn = 1;
  nqt = 1;
  for (int d = 0; d < dim; ++d) {
    nn *= kp1;
    nqt *= nq;
  }
  double detJ = 1.0;
  for (int d = 0; d < dim; ++d) detJ *= h[d];
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
  auto grad = [&](int q, int i, int d) { return G[((size_t)q * nn + i) * dim + d]; };
  if (ncomp == 1) {
    nne = nn * nn;
    H.assign((size_t)nqt * nne, 0.0);
    for (int q = 0; q < nqt; ++q)
      for (int i = 0; i < nn; ++i)
        for (int j = 0; j < nn; ++j) {
          double s = 0.0;
          for (int d = 0; d < dim; ++d) s += grad(q, i, d) * grad(q, j, d);
          H[(size_t)q * nne + i * nn + j] = W[q] * s;
        }
    return;
  }
  const double lam = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), mu = 1.0 / (2.0 * (1.0 + nu));
  const int M = dim * nn;
  nne = M * M;
  H.assign((size_t)nqt * nne, 0.0);
  for (int q = 0; q < nqt; ++q)
    for (int c = 0; c < dim; ++c)
      for (int i = 0; i < nn; ++i)
        for (int d = 0; d < dim; ++d)
          for (int j = 0; j < nn; ++j) {
            double lap = 0.0;
            for (int e = 0; e < dim; ++e) lap += grad(q, i, e) * grad(q, j, e);
            double s = lam * grad(q, i, c) * grad(q, j, d) + mu * grad(q, i, d) * grad(q, j, c);
            if (c == d) s += mu * lap;
            H[(size_t)q * nne + (size_t)(c * nn + i) * M + d * nn + j] = W[q] * s;
          }
}

static int kp_for(int nqt) { return nqt <= 16 ? 16 : (nqt <= 32 ? 32 : 64); }

// Tiles of H^T (entries x points) for S-term splitting.
static void build_a_tiles(const std::vector<double>& H, int nqt, int nne, int kp, int S, std::vector<uint16_t>& out,
                          int& n_etiles) {
  n_etiles = (nne + 127) / 128;
  const size_t tile = (size_t)128 * kp;
  out.assign((size_t)n_etiles * S * tile, 0);
  for (int et = 0; et < n_etiles; ++et)
    for (int r = 0; r < 128; ++r) {
      const int n = et * 128 + r;
      if (n >= nne) continue;
      for (int k = 0; k < nqt; ++k) {
        float x = (float)H[(size_t)k * nne + n];
        for (int s = 0; s < S; ++s) {
          const uint16_t b = f2bf_bits(x);
          out[((size_t)et * S + s) * tile + tc::tile_off(r, k, kp)] = b;
          x -= bf_bits2f(b);
        }
      }
    }
}

// ---------------------------------------------------------------------------------------
// Device: coefficient split and check, FP64 element matrices
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ bool bad_value(double k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(k);
  return (b >> 63) != 0ull || ((b >> 52) & 0x7FFull) == 0x7FFull || b == 0ull;
}

// Coefficients at the points -> B operand tiles ([cell tile][split][NCT x KP], BF16) and
// the count of values that are not finite and positive.
template <int KP, int S, int NCT>
__global__ void k_qp_split(int64_t ncells, int nqt, int64_t n_ctiles, const double* __restrict__ kq,
                           __nv_bfloat16* __restrict__ Bt, int32_t* __restrict__ bad) {
  int nbad = 0;
  const int64_t total = n_ctiles * NCT * KP;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = i / KP;
    const int k = (int)(i % KP);
    double x = 0.0;
    if (cell < ncells && k < nqt) {
      x = __ldg(kq + cell * nqt + k);
      nbad += bad_value(x);
    }
    const int64_t ct = cell / NCT;
    const int row = (int)(cell % NCT);
    float r = (float)x;
    __nv_bfloat16* t = Bt + ct * S * NCT * KP + tc::tile_off(row, k, KP);
#pragma unroll
    for (int s = 0; s < S; ++s) {
      const __nv_bfloat16 b = __float2bfloat16_rn(r);
      t[(int64_t)s * NCT * KP] = b;
      r -= __bfloat162float(b);
    }
  }
  if (nbad) atomicAdd(bad, nbad);
}

__global__ void k_qp_check(int64_t n, const double* __restrict__ kq, int32_t* __restrict__ bad) {
  int nbad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    nbad += bad_value(__ldg(kq + i));
  if (nbad) atomicAdd(bad, nbad);
}

// Ke[cell][n] = sum_q kq[cell][q] H[q][n] in FP64 (n < nne; padding entries 0).
__global__ void k_qp_ke_fp64(int64_t ncells, int nqt, int nne, int nnep, const double* __restrict__ kq,
                             const double* __restrict__ H, double* __restrict__ Ke) {
  const int64_t total = ncells * nnep;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t cell = i / nnep;
    const int n = (int)(i % nnep);
    double v = 0.0;
    if (n < nne)
      for (int q = 0; q < nqt; ++q) v = fma(__ldg(kq + cell * nqt + q), __ldg(H + (int64_t)q * nne + n), v);
    Ke[i] = v;
  }
}

// ---------------------------------------------------------------------------------------
// Device: the tensor-core contraction
//
// One CTA per SM, persistent over work items (cell tile of NCT cells, entry tile of 128
// element-matrix entries), entry tile fastest.  Warp 0 (one thread) loads each item's
// operand tiles -- the S splits of the entry tile of H^T (A, 128 x KP) and of the cell
// tile of coefficients (B, NCT x KP), both stored in global memory already in the
// tensor cores' K-major core-matrix layout -- with two bulk copies into a ring of NST
// shared-memory stages.  Warp 1 (one thread) issues the MMAs of an item into one of two
// TMEM accumulators (128 lanes x NCT columns, FP32) and commits them to mbarriers that
// free the stage and hand the accumulator to the epilogue.  Warps 2-9 drain an
// accumulator (tcgen05.ld) while the next item's MMAs fill the other one: thread l of a
// warp holds entry n = 32 (warp % 4) + l for 32 cells at a time and stores them as
// Ke[cell][n], so each store instruction of a warp writes 128 contiguous bytes.
// Every wait is bounded; on a timeout the kernel records an error, the other warps leave
// their loops, the MMA thread waits for its own MMAs, and the TMEM is freed.
// ---------------------------------------------------------------------------------------
template <int KP, int S, int NCT>
struct QpGemm {
  static constexpr int A_BYTES = 128 * KP * 2;
  static constexpr int B_BYTES = NCT * KP * 2;
  static constexpr int STAGE = S * (A_BYTES + B_BYTES);
  static constexpr int NST = (4 * STAGE <= 192 * 1024) ? 4 : ((3 * STAGE <= 192 * 1024) ? 3 : 2);
  static constexpr int TMEM_COLS = 2 * NCT;
  static constexpr int THREADS = 320;
  static constexpr int EPI_WARPS = 8;
  static constexpr size_t SMEM = (size_t)NST * STAGE + 256 + 1024;
  static_assert(NCT % 64 == 0 && NCT <= 256, "cell tile");
  static_assert(KP % 16 == 0, "K step");
};

template <int KP, int S, int NCT>
__global__ void __launch_bounds__(320, 1)
k_qp_gemm(const __nv_bfloat16* __restrict__ At, const __nv_bfloat16* __restrict__ Bt, int n_etiles, int64_t n_ctiles,
          int64_t ncells, int nnep, float* __restrict__ Ke, int32_t* __restrict__ err) {
  using Q = QpGemm<KP, S, NCT>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + (size_t)Q::NST * Q::STAGE);
  uint64_t* empty = full + Q::NST;
  uint64_t* accf = empty + Q::NST;
  uint64_t* acce = accf + 2;
  uint64_t* fin = acce + 2;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(fin + 1);
  int* abort_flag = reinterpret_cast<int*>(tslot + 1);
  volatile int* abrt = abort_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < Q::NST; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&accf[b], 1);
      tc::mbar_init(&acce[b], Q::EPI_WARPS);
    }
    tc::mbar_init(fin, 1);
    *abort_flag = 0;
    tc::mbar_fence_init();
  }
  if (warp == 1) tc::tmem_alloc(tslot, Q::TMEM_COLS);
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const int64_t nitems = (int64_t)n_etiles * n_ctiles;

  if (warp == 0) {
    if (lane == 0) {
      int last_parity[Q::NST];
      for (int s = 0; s < Q::NST; ++s) last_parity[s] = -1;
      int it = 0;
      for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x, ++it) {
        const int st = it % Q::NST;
        const uint32_t ph = (uint32_t)(it / Q::NST) & 1u;
        if (!tc::mbar_wait(&empty[st], ph ^ 1u, abrt)) {
          atomicExch(err, 1);
          *abrt = 1;
          break;
        }
        const int64_t ct = item / n_etiles;
        const int et = (int)(item % n_etiles);
        uint8_t* sA = base + (size_t)st * Q::STAGE;
        uint8_t* sB = sA + S * Q::A_BYTES;
        tc::mbar_arrive_expect_tx(&full[st], (uint32_t)Q::STAGE);
        tc::bulk_g2s(sA, At + (int64_t)et * S * (Q::A_BYTES / 2), S * Q::A_BYTES, &full[st]);
        tc::bulk_g2s(sB, Bt + ct * S * (Q::B_BYTES / 2), S * Q::B_BYTES, &full[st]);
        last_parity[st] = (int)ph;
      }
      // the copies issued last on every stage have landed before the CTA exits
      int zero = 0;
      for (int s = 0; s < Q::NST; ++s)
        if (last_parity[s] >= 0 && !tc::mbar_wait(&full[s], (uint32_t)last_parity[s], &zero)) atomicExch(err, 2);
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16_f32(128, NCT);
      int it = 0;
      for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x, ++it) {
        const int st = it % Q::NST;
        const uint32_t ph = (uint32_t)(it / Q::NST) & 1u;
        const int b = it & 1;
        const uint32_t bph = (uint32_t)(it >> 1) & 1u;
        if (!tc::mbar_wait(&acce[b], bph ^ 1u, abrt) || !tc::mbar_wait(&full[st], ph, abrt)) {
          atomicExch(err, 3);
          *abrt = 1;
          break;
        }
        tc::fence_after_sync();
        const uint32_t sA = tc::smem_u32(base + (size_t)st * Q::STAGE);
        const uint32_t sB = sA + S * Q::A_BYTES;
        const uint32_t d = tmem + (uint32_t)(b * NCT);
        uint32_t acc = 0;
#pragma unroll
        for (int pa = 0; pa < S; ++pa)
#pragma unroll
          for (int pb = 0; pb + pa < S; ++pb)
#pragma unroll
            for (int ks = 0; ks < KP / 16; ++ks) {
              const uint64_t ad = tc::smem_desc(sA + pa * Q::A_BYTES + ks * 256, 128, KP * 16);
              const uint64_t bd = tc::smem_desc(sB + pb * Q::B_BYTES + ks * 256, 128, KP * 16);
              tc::mma_bf16(d, ad, bd, idesc, acc);
              acc = 1;
            }
        tc::mma_commit(&empty[st]);
        tc::mma_commit(&accf[b]);
      }
      // every MMA issued above has completed before the TMEM is freed
      tc::mma_commit(fin);
      int zero = 0;
      if (!tc::mbar_wait(fin, 0, &zero)) atomicExch(err, 4);
    }
  } else {
    const int q = warp & 3;              // TMEM lane quarter this warp may access
    const int half = (warp - 2) >> 2;    // which half of the columns
    int it = 0;
    for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x, ++it) {
      const int b = it & 1;
      const uint32_t bph = (uint32_t)(it >> 1) & 1u;
      // every lane waits; the warp leaves together if any lane gave up (tcgen05.ld is
      // a warp-wide instruction)
      const bool ready = __all_sync(0xffffffffu, tc::mbar_wait(&accf[b], bph, abrt));
      if (!ready) {
        if (lane == 0) {
          atomicExch(err, 5);
          *abrt = 1;
        }
        break;
      }
      tc::fence_after_sync();
      const int64_t ct = item / n_etiles;
      const int et = (int)(item % n_etiles);
      const int nbase = et * 128 + q * 32;
      const bool nok = nbase < nnep;   // whole warp: nnep is a multiple of 32
      float* dst = Ke + (int64_t)nbase + lane;
#pragma unroll 1
      for (int c0 = half * (NCT / 2); c0 < (half + 1) * (NCT / 2); c0 += 32) {
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * NCT + c0), v);
        if (nok) {
          const int64_t cell0 = ct * NCT + c0;
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (cell0 + j < ncells) __stcs(dst + (cell0 + j) * nnep, v[j]);
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&acce[b]);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, Q::TMEM_COLS);
  }
}

// ---------------------------------------------------------------------------------------
// Device: CSR entries from the element matrices
// ---------------------------------------------------------------------------------------
// Scalar rows (lane groups as in qk_matrix_rows): entry (X, X+o) = sum over the slots a
// whose cell holds both nodes of Ke[cell_a][lx(a) NN + lx(a) + off(o)], slots in the
// fixed order of the entry table.
template <int DIM, int K, typename CodeT, typename KeT>
__global__ void __launch_bounds__(256)
k_qp_rows(Geom g, int64_t nrows_own, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ row_node,
          const CodeT* __restrict__ code, const KeT* __restrict__ Ke, int nnep, double* __restrict__ vals) {
  using L = Lat<DIM, K>;
  using RL = RowLanes<DIM, K>;
  constexpr int NC = 1 << DIM;
  constexpr int G = RL::G;
  __shared__ int64_t s_cell[8][32];
  __shared__ int s_lx[8][32];
  __shared__ uint16_t s_tab[EntryTab<DIM, K>::SIZE];
  build_entry_tab<DIM, K>(s_tab);
  __syncthreads();
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = lane / G, gl = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
  for (int64_t rb = warp * RL::RPW; rb < nrows_own; rb += nwarps * RL::RPW) {
    const int64_t r = rb + sub;
    const bool live = r < nrows_own;
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
      int64_t cl = 0, stride = 1;
      int lx = 0, mul = 1;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int sd = (gl >> d) & 1;
        const int c = sd ? X[d] / K : X[d] / K - 1;
        if (!sd && rm[d] != 0) ok = false;
        if (c < 0 || c >= (int)g.n[d]) ok = false;
        cl += stride * c;
        stride *= g.n[d];
        lx += mul * (sd ? rm[d] : K);
        mul *= L::KP1;
      }
      s_cell[wl][sub * NC + gl] = ok ? cl * nnep : 0;
      s_lx[wl][sub * NC + gl] = lx * (L::NN + 1);
      slot_ok = ok;
    }
    const uint32_t vmask = (__ballot_sync(0xffffffffu, slot_ok) >> (sub * G)) & ((1u << NC) - 1);
    __syncwarp();
    if (live) {
      const int64_t* sc = s_cell[wl] + sub * NC;
      const int* sl = s_lx[wl] + sub * NC;
      const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
      const uint16_t* et = s_tab + onb * EntryTab<DIM, K>::E;
      for (int64_t e = e0 + gl; e < e1; e += G) {
        const int info = et[(int)code[e]];
        const int off = (info & 255) - 128;
        const int fixed = (info >> 8) & 7, both = (info >> 11) & 7;
        KeT v = 0;
        int sb = both;
        while (true) {
          const int a = fixed | sb;
          if ((vmask >> a) & 1u) v += __ldg(Ke + sc[a] + sl[a] + off);
          if (sb == 0) break;
          sb = (sb - 1) & both;
        }
        vals[e] = (double)v;
      }
    }
    __syncwarp();
  }
}

template <int DIM, int K>
struct QpVecLanes {
  static constexpr int W = 2 * K + 1;
  static constexpr int E = DIM * (DIM == 3 ? W * W * W : W * W);
  static constexpr int G = E <= 32 ? 8 : (E <= 128 ? 16 : 32);
  static constexpr int RPW = 32 / G;
};

// Vector rows (dof = DIM * node dof + component, 16-bit codes = stencil * DIM + component):
// row (X, c), entry (X+o, d) sums Ke[cell][(c NN + lx) M + d NN + lx + off].
template <int DIM, int K, typename KeT>
__global__ void __launch_bounds__(256)
k_qp_rows_vec(Geom g, int64_t nrows_own, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ row_node,
              const uint16_t* __restrict__ code, const KeT* __restrict__ Ke, int nnep, double* __restrict__ vals) {
  using L = Lat<DIM, K>;
  using VL = QpVecLanes<DIM, K>;
  constexpr int NC = 1 << DIM;
  constexpr int G = VL::G;
  constexpr int M = DIM * L::NN;
  __shared__ int64_t s_cell[8][32];
  __shared__ int s_lx[8][32];
  __shared__ uint16_t s_tab[EntryTab<DIM, K>::SIZE];
  build_entry_tab<DIM, K>(s_tab);
  __syncthreads();
  const int wl = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = lane / G, gl = lane % G;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
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
      int64_t cl = 0, stride = 1;
      int lx = 0, mul = 1;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int sd = (gl >> d) & 1;
        const int cc = sd ? X[d] / K : X[d] / K - 1;
        if (!sd && rm[d] != 0) ok = false;
        if (cc < 0 || cc >= (int)g.n[d]) ok = false;
        cl += stride * cc;
        stride *= g.n[d];
        lx += mul * (sd ? rm[d] : K);
        mul *= L::KP1;
      }
      s_cell[wl][sub * NC + gl] = ok ? cl * nnep : 0;
      s_lx[wl][sub * NC + gl] = (c * L::NN + lx) * M + lx;
      slot_ok = ok;
    }
    const uint32_t vmask = (__ballot_sync(0xffffffffu, slot_ok) >> (sub * G)) & ((1u << NC) - 1);
    __syncwarp();
    if (live) {
      const int64_t* sc = s_cell[wl] + sub * NC;
      const int* sl = s_lx[wl] + sub * NC;
      const uint16_t* et = s_tab + onb * EntryTab<DIM, K>::E;
      const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
      for (int64_t e = e0 + gl; e < e1; e += G) {
        const int cv = (int)code[e];
        const int d2 = cv % DIM;
        const int info = et[cv / DIM];
        const int off = (info & 255) - 128 + d2 * L::NN;
        const int fixed = (info >> 8) & 7, both = (info >> 11) & 7;
        KeT v = 0;
        int sb = both;
        while (true) {
          const int a = fixed | sb;
          if ((vmask >> a) & 1u) v += __ldg(Ke + sc[a] + sl[a] + off);
          if (sb == 0) break;
          sb = (sb - 1) & both;
        }
        vals[e] = (double)v;
      }
    }
    __syncwarp();
  }
}

// Right-hand side of owned row r: the source term (f_const int(phi), the nodal load M f,
// or the body force component) minus the Dirichlet lifting with the element matrices.
// NCOMP = 1: scalar rows; NCOMP = DIM: vector rows (component r % DIM).
template <int DIM, int K, int NCOMP, typename KeT>
__global__ void k_qp_rhs(Geom g, int64_t nrows_own, const int32_t* __restrict__ row_node, const KeT* __restrict__ Ke,
                         int nnep, const double* __restrict__ Mhat, const double* __restrict__ Fhat, double f0,
                         double f1, double f2, const double* __restrict__ f_nodal, const double* __restrict__ u_dir,
                         double* __restrict__ rhs) {
  using L = Lat<DIM, K>;
  constexpr int M = NCOMP * L::NN;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows_own) return;
  const int c = NCOMP == 1 ? 0 : (int)(r % NCOMP);
  const double f = c == 0 ? f0 : (c == 1 ? f1 : f2);
  int64_t lin = row_node[r];
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
        int li = 0;
        for (int d = DIM - 1; d >= 0; --d) li = li * L::KP1 + (int)(X[d] - K * cc[d]);
        if (!f_nodal) b += f * __ldg(Fhat + li);
        if (f_nodal || u_dir) {
          const KeT* kr = Ke + cell_lin(g, cc) * nnep + (int64_t)(c * L::NN + li) * M;
          for (int lj = 0; lj < L::NN; ++lj) {
            int64_t Y[3] = {0, 0, 0};
            for (int d = 0, rest = lj; d < DIM; ++d) {
              Y[d] = K * cc[d] + rest % L::KP1;
              rest /= L::KP1;
            }
            const int64_t ylin = lattice_lin(g, Y);
            if (f_nodal) b += __ldg(Mhat + li * L::NN + lj) * __ldg(f_nodal + ylin);
            if (u_dir && node_is_dirichlet(g, Y))
              for (int d = 0; d < NCOMP; ++d)
                b -= (double)__ldg(kr + d * L::NN + lj) * __ldg(u_dir + ylin * NCOMP + d);
          }
        }
      }
  rhs[r] = b;
}

// ---------------------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------------------
static int grid_sm(int64_t work, int per_block) {
  const int64_t b = (work + per_block - 1) / per_block;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

template <int KP, int S, int NCT>
static int launch_gemm_t(gd_asm* A, QpState* Q, const double* kq, int64_t ncells, cudaStream_t st) {
  using G = QpGemm<KP, S, NCT>;
  const int64_t n_ctiles = (ncells + NCT - 1) / NCT;
  const size_t bt_elems = (size_t)n_ctiles * S * NCT * KP;
  if (Q->Bt.n < bt_elems) GD_TRY(dalloc(Q->Bt, bt_elems));
  k_qp_split<KP, S, NCT><<<grid_sm(bt_elems, 256), 256, 0, st>>>(ncells, Q->nqt, n_ctiles, kq, Q->Bt.p, Q->flags.p);
  GD_CUDA_TRY(cudaGetLastError());
  static int num_sms = 0;
  auto kern = k_qp_gemm<KP, S, NCT>;
  if (num_sms == 0) {
    int dev = 0;
    GD_CUDA_TRY(cudaGetDevice(&dev));
    GD_CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev));
    GD_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)G::SMEM));
  }
  const int64_t nitems = (int64_t)Q->n_etiles * n_ctiles;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(nitems, num_sms));
  if (Q->ev[0]) GD_CUDA_TRY(cudaEventRecord(Q->ev[0], st));
  kern<<<grid, G::THREADS, G::SMEM, st>>>(Q->At[S - 1].p, Q->Bt.p, Q->n_etiles, n_ctiles, ncells, Q->nnep, Q->Ke32.p,
                                          Q->flags.p + 1);
  GD_CUDA_TRY(cudaGetLastError());
  if (Q->ev[1]) GD_CUDA_TRY(cudaEventRecord(Q->ev[1], st));
  return GD_OK;
}

template <int KP>
static int launch_gemm_kp(gd_asm* A, QpState* Q, const double* kq, int64_t ncells, int S, cudaStream_t st) {
  constexpr int NCT = KP >= 64 ? 128 : 256;
  switch (S) {
    case 1: return launch_gemm_t<KP, 1, NCT>(A, Q, kq, ncells, st);
    case 2: return launch_gemm_t<KP, 2, NCT>(A, Q, kq, ncells, st);
    default: return launch_gemm_t<KP, 3, NCT>(A, Q, kq, ncells, st);
  }
}

template <int DIM, int K, typename KeT>
static int launch_rows_t(gd_asm* A, QpState* Q, const KeT* Ke, cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  if (R == 0) return GD_OK;
  if (A->bs == 1) {
    const unsigned nbw = (unsigned)std::min<int64_t>((R + 7) / 8, 152 * 64);
    if (A->code_bytes == 1)
      k_qp_rows<DIM, K, uint8_t, KeT><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p, A->code.p, Ke, Q->nnep,
                                                           A->vals.p);
    else
      k_qp_rows<DIM, K, uint16_t, KeT><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p,
                                                            reinterpret_cast<const uint16_t*>(A->code.p), Ke, Q->nnep,
                                                            A->vals.p);
  } else {
    const unsigned nbw = (unsigned)std::min<int64_t>((R + 7) / 8, 152 * 64);
    k_qp_rows_vec<DIM, K, KeT><<<nbw, 256, 0, st>>>(g, R, A->rowptr.p, A->row_node.p,
                                                    reinterpret_cast<const uint16_t*>(A->code.p), Ke, Q->nnep,
                                                    A->vals.p);
  }
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

template <int DIM, int K, typename KeT>
static int launch_rhs_t(gd_asm* A, QpState* Q, const KeT* Ke, const double* force, const double* f_nodal,
                        cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int64_t R = A->ngdofs;
  if (R == 0) return GD_OK;
  const double* udir = A->trial->has_dirichlet_values ? A->trial->u_dir.p : nullptr;
  const unsigned nb = (unsigned)((R + 127) / 128);
  if (A->bs == 1)
    k_qp_rhs<DIM, K, 1, KeT><<<nb, 128, 0, st>>>(g, R, A->row_node.p, Ke, Q->nnep, A->Mhat.p, A->Fhat.p, force[0], 0.0,
                                                 0.0, f_nodal, udir, A->rhs.p);
  else
    k_qp_rhs<DIM, K, DIM, KeT><<<nb, 128, 0, st>>>(g, R, A->row_node.p, Ke, Q->nnep, A->Mhat.p, A->Fhat.p, force[0],
                                                   force[1], DIM == 3 ? force[2] : 0.0, nullptr, udir, A->rhs.p);
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

template <typename KeT>
static int launch_rows_rhs(gd_asm* A, QpState* Q, const KeT* Ke, const double* force, const double* f_nodal,
                           cudaStream_t st) {
  const Geom& g = A->test->geom;
  const int sel = g.dim * 10 + g.k;
#define GD_QP_CASE(D, KK)                                            \
  case D * 10 + KK:                                                  \
    GD_TRY((launch_rows_t<D, KK, KeT>(A, Q, Ke, st)));               \
    if (Q->ev[2]) GD_CUDA_TRY(cudaEventRecord(Q->ev[2], st));        \
    return launch_rhs_t<D, KK, KeT>(A, Q, Ke, force, f_nodal, st);
  switch (sel) {
    GD_QP_CASE(2, 1)
    GD_QP_CASE(2, 2)
    GD_QP_CASE(2, 3)
    GD_QP_CASE(3, 1)
    GD_QP_CASE(3, 2)
    GD_QP_CASE(3, 3)
    default: return fail(GD_ERR_UNSUPPORTED, "quadrature-point assembly: unsupported dim/order");
  }
#undef GD_QP_CASE
}

// Reference tables and operand tiles for (degree, ncomp, nu, split count).
static int qp_prepare(gd_asm* A, QpState* Q, int degree, int ncomp, double nu, int S, cudaStream_t st) {
  const Geom& g = A->test->geom;
  if (Q->degree != degree || Q->ncomp != ncomp || (ncomp > 1 && Q->nu != nu)) {
    std::vector<double> H;
    int nqt = 0, nne = 0;
    qp_tables(g.dim, g.k, g.h, degree, ncomp, nu, H, nqt, nne);
    if (nqt > 64) return fail(GD_ERR_UNSUPPORTED, "quadrature-point assembly: at most 64 points per cell");
    Q->nqt = nqt;
    Q->nne = nne;
    Q->nnep = (nne + 31) / 32 * 32;
    Q->kp = kp_for(nqt);
    GD_TRY(dalloc(Q->H64, H.size()));
    GD_CUDA_TRY(cudaMemcpyAsync(Q->H64.p, H.data(), sizeof(double) * H.size(), cudaMemcpyHostToDevice, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    for (auto& a : Q->At) dfreeb(a);
    Q->degree = degree;
    Q->ncomp = ncomp;
    Q->nu = nu;
  }
  if (S > 0 && !Q->At[S - 1].p) {
    std::vector<double> H((size_t)Q->nqt * Q->nne);
    GD_CUDA_TRY(cudaMemcpy(H.data(), Q->H64.p, sizeof(double) * H.size(), cudaMemcpyDeviceToHost));
    std::vector<uint16_t> tiles;
    build_a_tiles(H, Q->nqt, Q->nne, Q->kp, S, tiles, Q->n_etiles);
    GD_TRY(dalloc(Q->At[S - 1], tiles.size()));
    GD_CUDA_TRY(cudaMemcpyAsync(Q->At[S - 1].p, tiles.data(), sizeof(uint16_t) * tiles.size(),
                                cudaMemcpyHostToDevice, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return GD_OK;
}

// The whole quadrature-point assembly of matrix values and right-hand side.
static int qp_assemble(gd_asm* A, const double* kq_in, int where, int degree, int precision, int ncomp, double nu,
                       const double* force, const double* f_nodal_in, const char* fn) {
  const std::string name(fn);
  if (!A->symbolic_done) return fail(GD_ERR_STATE, name + ": run gd_assemble_symbolic first");
  if (!kq_in) return fail(GD_ERR_ARG, name + ": null coefficient array");
  if (precision < GD_QP_FP64 || precision > GD_QP_BF16X6) return fail(GD_ERR_ARG, name + ": unknown precision");
  const Geom& g = A->test->geom;
  cudaStream_t st = A->test->model->ctx->stream;
  GD_TRY(reference_element(A, degree));
  if (!A->qp) A->qp = new QpState();
  QpState* Q = A->qp;
  const int S = precision == GD_QP_FP64 ? 0 : (precision == GD_QP_BF16 ? 1 : (precision == GD_QP_BF16X3 ? 2 : 3));
  GD_TRY(qp_prepare(A, Q, degree, ncomp, nu, S, st));
  int64_t ncells = 1, nnodes = 1;
  for (int d = 0; d < g.dim; ++d) {
    ncells *= g.n[d];
    nnodes *= g.N[d];
  }
  const int64_t nkq = ncells * Q->nqt;
  const double* kq = kq_in;
  if (where == GD_HOST) {
    if (Q->kq_dev.n < (size_t)nkq) GD_TRY(dalloc(Q->kq_dev, nkq));
    GD_CUDA_TRY(cudaMemcpyAsync(Q->kq_dev.p, kq_in, sizeof(double) * nkq, cudaMemcpyHostToDevice, st));
    kq = Q->kq_dev.p;
  }
  const double* fn_dev = f_nodal_in;
  if (f_nodal_in && where == GD_HOST) {
    if (A->f_dev.n != (size_t)nnodes) GD_TRY(dalloc(A->f_dev, nnodes));
    GD_CUDA_TRY(cudaMemcpyAsync(A->f_dev.p, f_nodal_in, sizeof(double) * nnodes, cudaMemcpyHostToDevice, st));
    fn_dev = A->f_dev.p;
  }
  if (!Q->flags.p) GD_TRY(dalloc(Q->flags, 2));
  GD_CUDA_TRY(cudaMemsetAsync(Q->flags.p, 0, 2 * sizeof(int32_t), st));
  if (A->profiling && !Q->ev[0])
    for (auto& e : Q->ev) GD_CUDA_TRY(cudaEventCreate(&e));
  cudaEvent_t saved[3] = {Q->ev[0], Q->ev[1], Q->ev[2]};
  if (!A->profiling)
    for (auto& e : Q->ev) e = nullptr;
  const size_t ke_elems = (size_t)ncells * Q->nnep;
  int s = GD_OK;
  if (S == 0) {
    dfreeb(Q->Ke32);
    if (Q->Ke64.n < ke_elems) s = dalloc(Q->Ke64, ke_elems);
    if (s == GD_OK) {
      k_qp_check<<<grid_sm(nkq, 256), 256, 0, st>>>(nkq, kq, Q->flags.p);
      if (Q->ev[0]) cudaEventRecord(Q->ev[0], st);
      k_qp_ke_fp64<<<grid_sm((int64_t)ke_elems, 256), 256, 0, st>>>(ncells, Q->nqt, Q->nne, Q->nnep, kq, Q->H64.p,
                                                                    Q->Ke64.p);
      s = cudaGetLastError() == cudaSuccess ? GD_OK : fail(GD_ERR_CUDA, name + ": FP64 element kernel launch failed");
      if (Q->ev[1]) cudaEventRecord(Q->ev[1], st);
      if (s == GD_OK) s = launch_rows_rhs<double>(A, Q, Q->Ke64.p, force, fn_dev, st);
    }
  } else {
    dfreeb(Q->Ke64);
    if (Q->Ke32.n < ke_elems) s = dalloc(Q->Ke32, ke_elems);
    if (s == GD_OK) {
      if (Q->kp == 16) s = launch_gemm_kp<16>(A, Q, kq, ncells, S, st);
      else if (Q->kp == 32) s = launch_gemm_kp<32>(A, Q, kq, ncells, S, st);
      else s = launch_gemm_kp<64>(A, Q, kq, ncells, S, st);
      if (s == GD_OK) s = launch_rows_rhs<float>(A, Q, Q->Ke32.p, force, fn_dev, st);
    }
  }
  for (int i = 0; i < 3; ++i) Q->ev[i] = saved[i];
  if (s != GD_OK) return s;
  int32_t hf[2] = {0, 0};
  GD_CUDA_TRY(cudaMemcpyAsync(hf, Q->flags.p, sizeof(hf), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (hf[1]) return fail(GD_ERR_TIMEOUT, name + ": a bounded wait of the tensor-core kernel ran out (code " +
                                             std::to_string(hf[1]) + ")");
  if (hf[0]) return fail(GD_ERR_NUMERIC, name + ": coefficient is not finite and positive at " +
                                             std::to_string(hf[0]) + " quadrature points");
  if (A->profiling && Q->ev[0]) {
    float t0 = 0.f, t1 = 0.f;
    GD_CUDA_TRY(cudaEventElapsedTime(&t0, Q->ev[0], Q->ev[1]));
    GD_CUDA_TRY(cudaEventElapsedTime(&t1, Q->ev[1], Q->ev[2]));
    Q->ms_ke = t0;
    Q->ms_rows = t1;
  }
  Q->last_precision = precision;
  A->qp_values = true;
  A->numeric_done = true;
  ++A->numeric_epoch;
  return GD_OK;
}

}  // namespace gd

using namespace gd;

extern "C" int gd_assemble_qp(gd_asm* A, const gd_qp_coeffs* c) {
  if (!A || !c) return fail(GD_ERR_ARG, "gd_assemble_qp: null argument");
  if (A->bs != 1) return fail(GD_ERR_UNSUPPORTED, "gd_assemble_qp: scalar spaces (use gd_assemble_elasticity_qp)");
  const double force[3] = {c->f_const, 0.0, 0.0};
  return qp_assemble(A, c->kappa_qp, c->where, c->degree, c->precision, 1, 0.0, force, c->f_nodal,
                     "gd_assemble_qp");
}

extern "C" int gd_assemble_elasticity_qp(gd_asm* A, const gd_elasticity_qp* c) {
  if (!A || !c) return fail(GD_ERR_ARG, "gd_assemble_elasticity_qp: null argument");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_assemble_elasticity_qp: run gd_assemble_symbolic first");
  const Geom& g = A->test->geom;
  if (A->bs != g.dim) return fail(GD_ERR_UNSUPPORTED, "gd_assemble_elasticity_qp: needs a vector space with dim components");
  if (!(c->nu > -1.0 && c->nu < 0.5)) return fail(GD_ERR_ARG, "gd_assemble_elasticity_qp: Poisson ratio outside (-1, 0.5)");
  if (g.k > 2) return fail(GD_ERR_UNSUPPORTED, "gd_assemble_elasticity_qp: vector spaces of order 1-2");
  return qp_assemble(A, c->E_qp, c->where, c->degree, c->precision, g.dim, c->nu, c->force, nullptr,
                     "gd_assemble_elasticity_qp");
}

extern "C" int gd_qp_info(const gd_asm* A, int32_t* points, int32_t* entries, int32_t* kpad, int32_t* etiles,
                          double* ms_element, double* ms_rows) {
  if (!A) return fail(GD_ERR_ARG, "gd_qp_info: null assembler");
  if (!A->qp) return fail(GD_ERR_STATE, "gd_qp_info: no quadrature-point assembly has run");
  const QpState* Q = A->qp;
  if (points) *points = Q->nqt;
  if (entries) *entries = Q->nne;
  if (kpad) *kpad = Q->kp;
  if (etiles) *etiles = Q->n_etiles;
  if (ms_element) *ms_element = Q->ms_ke;
  if (ms_rows) *ms_rows = Q->ms_rows;
  return GD_OK;
}
