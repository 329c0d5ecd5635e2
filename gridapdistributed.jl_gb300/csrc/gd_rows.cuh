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

// Matrix values of owned row r, computed by one warp (all 32 lanes call it).
// The row's node X and the coefficients of the (up to 2^DIM) cells around it are decoded
// once per warp; the lanes then walk the row's entries (coalesced stencil codes in,
// coalesced values out).  Along each direction the node sits either on a cell boundary
// (X % K == 0: cells "below" = slot 0 and "above" = slot 1) or inside one cell (slot 1);
// entry (X, X+o) sums kappa_c * Khat[X in c][X+o in c] over the slots whose cell holds
// both nodes: o_d < 0 -> slot 0, o_d > 0 -> slot 1, o_d = 0 -> both.  Kt is the
// reference stiffness table (shared or global memory).
template <int DIM, int K, typename CodeT>
__device__ __forceinline__ void qk_matrix_row(const Geom& g, int64_t r, const int64_t* __restrict__ rowptr,
                                              const int32_t* __restrict__ row_node, const CodeT* __restrict__ code,
                                              const double* __restrict__ kappa, const double* Kt,
                                              double* __restrict__ vals) {
  using L = Lat<DIM, K>;
  constexpr int NC = 1 << DIM;
  const int lane = threadIdx.x & 31;
  const uint32_t N0 = (uint32_t)g.N[0], N1 = (uint32_t)g.N[1];
  const uint32_t lin = (uint32_t)row_node[r];
  int X[3], q[3], rm[3];
  X[0] = (int)(lin % N0);
  if (DIM == 3) {
    const uint32_t t = lin / N0;
    X[1] = (int)(t % N1);
    X[2] = (int)(t / N1);
  } else {
    X[1] = (int)(lin / N0);
    X[2] = 0;
  }
#pragma unroll
  for (int d = 0; d < DIM; ++d) {
    q[d] = X[d] / K;
    rm[d] = X[d] % K;
  }
  // coefficient of slot a (lane a loads it, then broadcast)
  double kv = 0.0;
  bool slot_ok = false;
  if (lane < NC) {
    bool ok = true;
    int64_t cl = 0, stride = 1;
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      const int sd = (lane >> d) & 1;
      const int c = sd ? q[d] : q[d] - 1;
      if (!sd && rm[d] != 0) ok = false;
      if (c < 0 || c >= g.n[d]) ok = false;
      cl += stride * c;
      stride *= g.n[d];
    }
    kv = ok ? __ldg(kappa + cl) : 0.0;
    slot_ok = ok;
  }
  const uint32_t vmask = __ballot_sync(0xffffffffu, slot_ok);   // valid slots (integer test, not FP64)
  double kap[NC];
#pragma unroll
  for (int a = 0; a < NC; ++a) kap[a] = __shfl_sync(0xffffffffu, kv, a);
  const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
  for (int64_t e = e0 + lane; e < e1; e += 32) {
    int cv = (int)code[e];
    int o[3] = {0, 0, 0};
#pragma unroll
    for (int d = 0; d < DIM; ++d) {
      o[d] = cv % L::W - K;
      cv /= L::W;
    }
    double v = 0.0;
#pragma unroll
    for (int a = 0; a < NC; ++a) {
      bool ok = (vmask >> a) & 1u;
      int lx = 0, ly = 0, mul = 1;
#pragma unroll
      for (int d = 0; d < DIM; ++d) {
        const int sd = (a >> d) & 1;
        if (sd == 0 && (rm[d] != 0 || o[d] > 0)) ok = false;
        if (sd == 1 && rm[d] == 0 && o[d] < 0) ok = false;
        const int lxd = sd ? rm[d] : K;
        lx += mul * lxd;
        ly += mul * (lxd + o[d]);
        mul *= L::KP1;
      }
      if (ok) v = fma(kap[a], Kt[lx * L::NN + ly], v);
    }
    vals[e] = v;
  }
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
