// Row bodies of the generic Q_k numeric assembly, shared by the single-problem kernels
// (gd_numeric.cu) and the batched persistent kernel (gd_batch.cu).
#pragma once
#include "gd_internal.h"

namespace gd {

template <int DIM, int K>
struct Lat {
  static constexpr int KP1 = K + 1;
  static constexpr int NN = DIM == 2 ? KP1 * KP1 : KP1 * KP1 * KP1;
  static constexpr int W = 2 * K + 1;
};

// Lanes per matrix row: a row of a Q_k stencil has at most (2k+1)^DIM entries, so a
// warp takes 4 rows of at most 32 entries (8 lanes each), 2 rows of at most 128 (16
// lanes each) or one longer row; the per-row decoding below is then shared by 4, 2 or
// 1 rows per warp instruction.
// Entry table of a (DIM, K) stencil: for every stencil code (W-ary digits o_d + K) and
// every set of directions in which the row's node sits on a cell boundary (3 bits), the
// packed entry: bits 0-7 off(o) + 128, bits 8-10 slot bits forced to 1, bits 11-13
// slot bits that take both values.  One shared-memory lookup then replaces the digit
// decoding of every entry.
template <int DIM, int K>
struct EntryTab {
  static constexpr int W = 2 * K + 1;
  static constexpr int E = DIM == 3 ? W * W * W : W * W;
  static constexpr int SIZE = 8 * E;
};

template <int DIM, int K>
__device__ __forceinline__ void build_entry_tab(uint16_t* tab) {
  using T = EntryTab<DIM, K>;
  constexpr int KP1 = K + 1;
  for (int i = threadIdx.x; i < T::SIZE; i += blockDim.x) {
    const int onb = i / T::E;
    int cv = i % T::E;
    int off = 0, fixed = 0, both = 0, mul = 1;
    for (int d = 0; d < DIM; ++d) {
      const int od = cv % T::W - K;
      cv /= T::W;
      off += od * mul;
      mul *= KP1;
      if (od > 0 || !((onb >> d) & 1)) fixed |= 1 << d;
      else if (od == 0) both |= 1 << d;
    }
    tab[i] = (uint16_t)((off + 128) | (fixed << 8) | (both << 11));
  }
}

template <int DIM, int K>
struct RowLanes {
  static constexpr int W = 2 * K + 1;
  static constexpr int E = DIM == 3 ? W * W * W : W * W;
  static constexpr int G = E <= 32 ? 8 : (E <= 128 ? 16 : 32);
  static constexpr int RPW = 32 / G;   // rows per warp
};

// Matrix values of owned rows rbase .. rbase+RPW-1 (those < rend), one lane group of G
// lanes per row; all 32 lanes of the warp call it.
// Along each direction the row's node X sits either on a cell boundary (X % K == 0:
// cells "below" = slot bit 0 and "above" = slot bit 1) or inside one cell (bit 1).
// Entry (X, X+o) sums kappa_c * Khat[X in c][X+o in c] over the slots whose cell holds
// both nodes: per direction o_d < 0 -> bit 0, o_d > 0 -> bit 1, o_d = 0 -> both when X
// is on a cell boundary, bit 1 inside a cell.  With lx(a) the local index of X in slot
// a's cell, the local index of X+o there is lx(a) + off(o), off = sum o_d (K+1)^d, so an
// entry is sum over its (usually one) slots of kap[a] * Khat[lx(a) (NN + 1) + off].
// The first 2^DIM lanes of a group decode the slots (coefficient, lx, validity) into
// the warp's shared-memory slot tables (skap: 32 doubles, slx: 32 ints); the group then
// walks its row's entries (coalesced stencil codes in, coalesced values out), each
// entry's offset and slots read from the entry table etab (build_entry_tab).  Kt is
// the reference stiffness table (shared or global memory).
template <int DIM, int K, typename CodeT>
__device__ __forceinline__ void qk_matrix_rows(const Geom& g, int64_t rbase, int64_t rend,
                                               const int64_t* __restrict__ rowptr,
                                               const int32_t* __restrict__ row_node, const CodeT* __restrict__ code,
                                               const double* __restrict__ kappa, const double* Kt,
                                               const uint16_t* etab, double* __restrict__ vals, double* skap,
                                               int* slx) {
  using L = Lat<DIM, K>;
  using RL = RowLanes<DIM, K>;
  constexpr int NC = 1 << DIM;
  constexpr int G = RL::G;
  const int lane = threadIdx.x & 31, sub = lane / G, gl = lane % G;
  const int64_t r = rbase + sub;
  const bool live = r < rend;
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
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
  int onb = 0;   // bit d: X on a cell boundary along d
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    rm[d] = X[d] % K;
    if (rm[d] == 0) onb |= 1 << d;
  }
  bool slot_ok = false;
  if (live && gl < NC) {
    bool ok = true;
    int cl = 0, stride = 1;   // cell ids stay below 2^31 (checked when the space is created)
    int lx = 0, mul = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int sd = (gl >> d) & 1;
      const int c = sd ? X[d] / K : X[d] / K - 1;
      if (!sd && rm[d] != 0) ok = false;
      if (c < 0 || c >= (int)g.n[d]) ok = false;
      cl += stride * c;
      stride *= (int)g.n[d];
      lx += mul * (sd ? rm[d] : K);
      mul *= L::KP1;
    }
    skap[sub * NC + gl] = ok ? __ldg(kappa + cl) : 0.0;
    slx[sub * NC + gl] = lx * (L::NN + 1);
    slot_ok = ok;
  }
  const uint32_t vmask = (__ballot_sync(0xffffffffu, slot_ok) >> (sub * G)) & ((1u << NC) - 1);   // valid slots
  __syncwarp();
  if (live) {
    const double* sk = skap + sub * NC;
    const int* sl = slx + sub * NC;
    const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
    const uint16_t* et = etab + onb * EntryTab<DIM, K>::E;
    for (int64_t e = e0 + gl; e < e1; e += G) {
      const int info = et[(int)code[e]];
      const int off = (info & 255) - 128;
      const int fixed = (info >> 8) & 7;   // only the cell above
      const int both = (info >> 11) & 7;   // both cells (node on a boundary, o_d = 0)
      double v = 0.0;
      int sb = both;
      while (true) {
        const int a = fixed | sb;
        if ((vmask >> a) & 1u) v = fma(sk[a], Kt[sl[a] + off], v);
        if (sb == 0) break;
        sb = (sb - 1) & both;
      }
      vals[e] = v;
    }
  }
  __syncwarp();
}

// Right-hand side of owned row r (source term and Dirichlet lifting), one thread.
// Returns the number of cell visits whose kappa is not finite and positive.
template <int DIM, int K>
__device__ __forceinline__ int qk_rhs_row(const Geom& g, int64_t r, const int32_t* __restrict__ row_node,
                                          const double* __restrict__ kappa, const double* __restrict__ Khat,
                                          const double* __restrict__ Mhat, const double* __restrict__ Fhat,
                                          double f_const, const double* __restrict__ f_nodal,
                                          const double* __restrict__ u_dir, double* __restrict__ rhs) {
  using L = Lat<DIM, K>;
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
        if (!f_nodal) b += f_const * __ldg(Fhat + li);
        if (f_nodal || u_dir) {
          for (int lj = 0; lj < L::NN; ++lj) {
            int64_t Y[3] = {0, 0, 0};
            for (int d = 0, rest = lj; d < DIM; ++d) {
              Y[d] = K * cc[d] + rest % L::KP1;
              rest /= L::KP1;
            }
            const int64_t ylin = lattice_lin(g, Y);
            if (f_nodal) b += __ldg(Mhat + li * L::NN + lj) * __ldg(f_nodal + ylin);
            if (u_dir && node_is_dirichlet(g, Y)) b -= kap * __ldg(Khat + li * L::NN + lj) * __ldg(u_dir + ylin);
          }
        }
      }
  rhs[r] = b;
  return nbad;
}

}  // namespace gd
