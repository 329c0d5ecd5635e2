// Discontinuous Galerkin: Q_k spaces with conformity L2 on the Cartesian model and the
// symmetric interior penalty form of test/PoissonTests.jl:47-77,
//   a(u,v) = int grad(v).grad(u) dOmega
//          + sum_{Gamma_d} int( (gamma/h) v u - v (n.grad u) - (n.grad v) u )
//          + sum_{Lambda}  int( (gamma/h) [[v n]].[[u n]] - [[v n]].{grad u} - {grad v}.[[u n]] )
//   l(v) = int f v dOmega + sum_{Gamma_n} int g v + sum_{Gamma_d} int( (gamma/h) v u_D - (n.grad v) u_D )
// with [[w n]] = (w+ - w-) n+ and {q} = (q+ + q-) / 2 on an interior face (both terms are
// unchanged when the sides swap, so no orientation convention enters the values).
//
// Numbering (Gridap's L2 spaces): every cell holds its (k+1)^dim dofs in the reference
// element's node order; a part owns the dofs of its owned cells and numbers them cell by
// cell in lexicographic cell order, parts one after another; its local dofs are those of
// every local cell (owned and ghost layer), cell by cell in the local box's order.
//
// On a uniform Cartesian mesh every term is one of a few constant tables: the volume
// stiffness, and per cell face f (direction d, side s) the Dirichlet-boundary matrix, the
// interior-face self matrix and the interior-face neighbour matrix (the neighbour's basis
// evaluated at the same face points), plus the face value / normal-derivative rows for
// the right-hand side.  The tables are built once in FP64 on the host; a row of the
// matrix (owned dof a of cell X) is table entries for X's own dofs (volume + its faces)
// and for each face neighbour's dofs.  Every owned row is summed completely (the global
// operator the reference assembles, whichever the strategy).  The local parts follow the
// strategy:
//  * FullyAssembledRows: owned rows only; columns: the owned dofs, then the touched ghost
//    dofs (the face-neighbour cells in the ghost layer) in local-id order;
//  * SubAssembledRows (the reference's default): a part integrates the interior faces
//    whose cell with the larger global id it owns (src/Geometry.jl:864-882) -- with
//    lexicographic cell ids those are the faces to the ghost cells just below its owned
//    box -- so the dofs of those ghost cells are touched ghost rows (local-id order, their
//    entries explicit zeros: the triplets went to their owners, Algebra.jl:1048-1131);
//    ghost columns come in order of first appearance in the local COO and then the
//    received triplets (Algebra.jl:1210-1238): the cells below the owned box by local id
//    (each meets its one owned neighbour at a face that Gridap's face numbering reaches
//    at the lower cell, plus side = lower local id, block columns walked plus first),
//    then the cells just above it, owner by owner (receives in ascending sender order),
//    lexicographic within an owner.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "gd_internal.h"

namespace gd {
namespace {

struct DgPart {
  int64_t own_lo[kMaxDim], own_hi[kMaxDim];
  int64_t loc_lo[kMaxDim], loc_hi[kMaxDim];
  int64_t first;      // first owned gid
  int64_t ncell_own;
  int64_t nloc_cells;
  int64_t gc_off, n_gc;   // touched ghost cells (local-box lexicographic ids, sorted)
  int64_t gr_off, n_gr;   // ghost-row cells (SubAssembledRows: the cells just below the owned box)
};

struct DgGeo {
  int dim, k, nn, np;
  int64_t n[kMaxDim];
  Geom g;   // the model's (for cell owners)
};

__host__ __device__ inline int64_t box_lex(const int64_t* lo, const int64_t* hi, const int64_t* X, int dim) {
  int64_t l = 0, stride = 1;
  for (int d = 0; d < dim; ++d) {
    l += (X[d] - lo[d]) * stride;
    stride *= hi[d] - lo[d];
  }
  return l;
}

__host__ __device__ inline bool in_box(const int64_t* lo, const int64_t* hi, const int64_t* X, int dim) {
  for (int d = 0; d < dim; ++d)
    if (X[d] < lo[d] || X[d] >= hi[d]) return false;
  return true;
}

// gid of dof 0 of cell X
__device__ inline int64_t dg_cell_gid0(const DgGeo& G, const DgPart* parts, const int64_t* X) {
  const int q = cell_owner(G.g, X);
  const DgPart& Q = parts[q];
  return Q.first + (int64_t)G.nn * box_lex(Q.own_lo, Q.own_hi, X, G.dim);
}

__device__ inline int dg_find_part(const DgPart* parts, int np, int64_t r) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (parts[mid].first <= r) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// owned row r -> part, cell X (global coordinates), local dof a
__device__ inline void dg_row(const DgGeo& G, const DgPart* parts, int64_t r, int& p, int64_t* X, int& a) {
  p = dg_find_part(parts, G.np, r);
  const DgPart& P = parts[p];
  const int64_t o = r - P.first;
  int64_t c = o / G.nn;
  a = (int)(o - c * G.nn);
  for (int d = 0; d < kMaxDim; ++d) X[d] = 0;
  for (int d = 0; d < G.dim; ++d) {
    const int64_t w = P.own_hi[d] - P.own_lo[d];
    X[d] = P.own_lo[d] + c % w;
    c /= w;
  }
}

struct RowCell {
  int64_t colbase;   // local column of the cell's dof 0
  int64_t gid0;      // global column of the cell's dof 0
  int face;          // -1: the row's own cell, else the face of the row cell it lies across
};

// the row cell and its face neighbours, in local column order
__device__ inline int dg_row_cells(const DgGeo& G, const DgPart* parts, const int64_t* __restrict__ gcells,
                                   const int32_t* __restrict__ gperm, int p, const int64_t* X, RowCell* rc) {
  const DgPart& P = parts[p];
  int m = 0;
  for (int f = -1; f < 2 * G.dim; ++f) {
    int64_t Y[kMaxDim] = {X[0], X[1], X[2]};
    if (f >= 0) {
      const int d = f >> 1;
      Y[d] += (f & 1) ? 1 : -1;
      if (Y[d] < 0 || Y[d] >= G.n[d]) continue;
    }
    RowCell c;
    c.face = f;
    c.gid0 = dg_cell_gid0(G, parts, Y);
    if (in_box(P.own_lo, P.own_hi, Y, G.dim)) {
      c.colbase = (int64_t)G.nn * box_lex(P.own_lo, P.own_hi, Y, G.dim);
    } else {
      const int64_t key = box_lex(P.loc_lo, P.loc_hi, Y, G.dim);
      int64_t lo = 0, hi = P.n_gc - 1;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (gcells[P.gc_off + mid] < key) lo = mid + 1;
        else hi = mid;
      }
      c.colbase = (int64_t)G.nn * (P.ncell_own + gperm[P.gc_off + lo]);
    }
    int j = m++;
    while (j > 0 && rc[j - 1].colbase > c.colbase) {
      rc[j] = rc[j - 1];
      --j;
    }
    rc[j] = c;
  }
  return m;
}

__global__ void k_dg_rowlen(DgGeo G, const DgPart* __restrict__ parts, int64_t nrows, int32_t* __restrict__ len) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int p, a;
    int64_t X[kMaxDim];
    dg_row(G, parts, r, p, X, a);
    int m = 1;
    for (int d = 0; d < G.dim; ++d) m += (X[d] > 0) + (X[d] < G.n[d] - 1);
    len[r] = m * G.nn;
  }
}

// Tables (FP64): K[nn*nn] | F[nn] | per face f: Bd[nn*nn] S[nn*nn] N[nn*nn] Rd[nqf*nn] Rn[nqf*nn]
struct DgTabs {
  int nn, nqf;
  __host__ __device__ int64_t face_base(int f) const {
    return (int64_t)nn * nn + nn + (int64_t)f * (3 * nn * nn + 2 * nqf * nn);
  }
};

// warp per owned row; lanes over the row's entries
__global__ void __launch_bounds__(256)
k_dg_fill(DgGeo G, DgTabs T, const DgPart* __restrict__ parts, const int64_t* __restrict__ gcells,
          const int32_t* __restrict__ gperm, int64_t nrows, int dmask, const double* __restrict__ tab,
          const int64_t* __restrict__ rowptr, int32_t* __restrict__ colidx, int32_t* __restrict__ colgid,
          double* __restrict__ vals) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const int nn = G.nn;
  for (int64_t r = warp; r < nrows; r += nw) {
    int p, a;
    int64_t X[kMaxDim];
    dg_row(G, parts, r, p, X, a);
    RowCell rc[2 * kMaxDim + 1];
    const int m = dg_row_cells(G, parts, gcells, gperm, p, X, rc);
    // which faces of X are interior / Dirichlet boundary
    int interior = 0, dir = 0;
    for (int f = 0; f < 2 * G.dim; ++f) {
      const int d = f >> 1;
      const bool bnd = (f & 1) ? X[d] == G.n[d] - 1 : X[d] == 0;
      if (!bnd) interior |= 1 << f;
      else if ((dmask >> f) & 1) dir |= 1 << f;
    }
    const int64_t e0 = rowptr[r];
    for (int e = lane; e < m * nn; e += 32) {
      const RowCell& c = rc[e / nn];
      const int b = e - (e / nn) * nn;
      double v;
      if (c.face < 0) {
        v = tab[a * nn + b];
        for (int f = 0; f < 2 * G.dim; ++f) {
          const double* fb = tab + T.face_base(f);
          if ((dir >> f) & 1) v += fb[a * nn + b];
          else if ((interior >> f) & 1) v += fb[nn * nn + a * nn + b];
        }
      } else {
        v = tab[T.face_base(c.face) + 2 * nn * nn + a * nn + b];
      }
      colidx[e0 + e] = (int32_t)(c.colbase + b);
      colgid[e0 + e] = (int32_t)(c.gid0 + b);
      vals[e0 + e] = v;
    }
  }
}

// SubAssembledRows ghost rows (rows nown_total + i): the dofs of a ghost cell X' just below
// the owned box, whose one owned neighbour is X' + e_d.  Columns sorted by local id: the
// neighbour's dofs (owned), then X''s dofs (a ghost column); values explicit zeros.
// Mode 0: row lengths; mode 1: columns and values.
__global__ void k_dg_ghost_rows(DgGeo G, const DgPart* __restrict__ parts, const int64_t* __restrict__ grcells,
                                const int64_t* __restrict__ gcells, const int32_t* __restrict__ gperm, int64_t n_own,
                                int64_t nghost, int mode, int32_t* __restrict__ len,
                                const int64_t* __restrict__ rowptr, int32_t* __restrict__ colidx,
                                int32_t* __restrict__ colgid, double* __restrict__ vals) {
  const int nn = G.nn;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nghost; i += (int64_t)gridDim.x * blockDim.x) {
    if (mode == 0) {
      len[n_own + i] = 2 * nn;
      continue;
    }
    const int64_t gc = i / nn;   // ghost-row cell (all parts concatenated)
    int p = 0;
    while (p + 1 < G.np && parts[p + 1].gr_off <= gc) ++p;
    const DgPart& P = parts[p];
    const int64_t key = grcells[gc];
    int64_t X[kMaxDim] = {0, 0, 0}, Y[kMaxDim] = {0, 0, 0}, rest = key;
    for (int d = 0; d < G.dim; ++d) {
      const int64_t w = P.loc_hi[d] - P.loc_lo[d];
      X[d] = P.loc_lo[d] + rest % w;
      rest /= w;
    }
    for (int d = 0; d < G.dim; ++d) Y[d] = X[d] + (X[d] == P.own_lo[d] - 1 ? 1 : 0);
    int64_t lo = 0, hi = P.n_gc - 1;   // X' among the part's ghost columns
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (gcells[P.gc_off + mid] < key) lo = mid + 1;
      else hi = mid;
    }
    const int64_t cown = (int64_t)nn * box_lex(P.own_lo, P.own_hi, Y, G.dim);
    const int64_t cgh = (int64_t)nn * (P.ncell_own + gperm[P.gc_off + lo]);
    const int64_t gY = dg_cell_gid0(G, parts, Y), gX = dg_cell_gid0(G, parts, X);
    const int64_t e0 = rowptr[n_own + i];
    for (int b = 0; b < nn; ++b) {
      colidx[e0 + b] = (int32_t)(cown + b);
      colgid[e0 + b] = (int32_t)(gY + b);
      vals[e0 + b] = 0.0;
      colidx[e0 + nn + b] = (int32_t)(cgh + b);
      colgid[e0 + nn + b] = (int32_t)(gX + b);
      vals[e0 + nn + b] = 0.0;
    }
  }
}

// thread per owned row: f (constant or at the cell Gauss points) + Neumann g + Dirichlet u_D
__global__ void k_dg_rhs(DgGeo G, DgTabs T, const DgPart* __restrict__ parts, int64_t nrows, const double* __restrict__ tab,
                         double f_const, const double* __restrict__ f_qp, const double* __restrict__ vtab, int nqt,
                         int dmask, const int64_t* __restrict__ doff, const double* __restrict__ ud_qp, int nmask,
                         const int64_t* __restrict__ noff, const double* __restrict__ g_qp, double* __restrict__ rhs) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += (int64_t)gridDim.x * blockDim.x) {
    int p, a;
    int64_t X[kMaxDim];
    dg_row(G, parts, r, p, X, a);
    const int nn = G.nn;
    double b = 0.0;
    if (f_qp) {
      const int64_t zero[kMaxDim] = {0, 0, 0};
      const int64_t cl = box_lex(zero, G.n, X, G.dim);
      for (int q = 0; q < nqt; ++q) b = fma(vtab[q * nn + a], f_qp[cl * nqt + q], b);
    } else {
      b = f_const * tab[nn * nn + a];
    }
    for (int f = 0; f < 2 * G.dim; ++f) {
      const int d = f >> 1;
      const bool bnd = (f & 1) ? X[d] == G.n[d] - 1 : X[d] == 0;
      if (!bnd) continue;
      const bool isd = (dmask >> f) & 1, isn = (nmask >> f) & 1;
      if (!isd && !isn) continue;
      // the face's index on its side: lexicographic over the tangential cells, lowest first
      int64_t fi = 0, stride = 1;
      for (int t = 0; t < G.dim; ++t) {
        if (t == d) continue;
        fi += X[t] * stride;
        stride *= G.n[t];
      }
      const double* fb = tab + T.face_base(f) + 3 * nn * nn;
      if (isd) {
        const double* u = ud_qp + (doff[f] + fi) * T.nqf;
        for (int q = 0; q < T.nqf; ++q) b = fma(fb[q * nn + a], u[q], b);
      }
      if (isn) {
        const double* gq = g_qp + (noff[f] + fi) * T.nqf;
        for (int q = 0; q < T.nqf; ++q) b = fma(fb[T.nqf * nn + q * nn + a], gq[q], b);
      }
    }
    rhs[r] = b;
  }
}

// per-cell squared L2 error sum_q w_q (u_q - uh(x_q))^2 |J|, block partials
__global__ void k_dg_l2(DgGeo G, const DgPart* __restrict__ parts, int64_t ncells, const double* __restrict__ x,
                        const double* __restrict__ vtab, int nqt, const double* __restrict__ u_qp,
                        double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncells; c += (int64_t)gridDim.x * blockDim.x) {
    int64_t X[kMaxDim] = {0, 0, 0}, rest = c;
    for (int d = 0; d < G.dim; ++d) {
      X[d] = rest % G.n[d];
      rest /= G.n[d];
    }
    const int64_t g0 = dg_cell_gid0(G, parts, X);
    for (int q = 0; q < nqt; ++q) {
      double uh = 0.0;
      for (int a = 0; a < G.nn; ++a) uh = fma(vtab[q * G.nn + a], x[g0 + a], uh);
      const double e = u_qp[c * nqt + q] - uh;
      s = fma(vtab[nqt * G.nn + q], e * e, s);   // weight row: w_q |J|
    }
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)blockDim.x; ++i) t += sh[i];
    part[blockIdx.x] = t;
  }
}

// y = A x over the owned rows (global columns)
__global__ void k_dg_spmv(int64_t n, const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colgid,
                          const double* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t e = rowptr[r]; e < rowptr[r + 1]; ++e) s = fma(vals[e], x[colgid[e]], s);
    y[r] = s;
  }
}

unsigned dg_grid(int64_t n, int per) {
  const int64_t b = (n + per - 1) / per;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

// 1D Lagrange values / derivatives of the k+1 equispaced nodes at x
void basis1d(int k, double x, std::vector<double>& v, std::vector<double>& dv) {
  v.assign(k + 1, 0.0);
  dv.assign(k + 1, 0.0);
  lagrange01(k, x, v.data(), dv.data());
}

}  // namespace
}  // namespace gd

struct gd_dgspace {
  gd_model* model = nullptr;
  int k = 1, nn = 1, dim = 2;
  std::vector<gd::DgPart> parts;
  gd::DBuf<gd::DgPart> d_parts;
  std::vector<int64_t> h_gcells;
  gd::DBuf<int64_t> gcells;
  int strategy = GD_SUB_ASSEMBLED_ROWS;
  std::vector<int32_t> h_gperm;    // per ghost column (sorted by local id): its position in the column order
  gd::DBuf<int32_t> gperm;
  std::vector<int64_t> h_grcells;  // ghost-row cells per part (local-box ids, sorted)
  gd::DBuf<int64_t> grcells;
  int64_t nghost_rows = 0;         // ghost rows of all parts (dofs)
  std::vector<int> dofpos;   // 3 per local dof
  int64_t ndofs = 0, nnz = 0;
  bool assembled = false;
  gd::DBuf<int64_t> rowptr;
  gd::DBuf<int32_t> colidx, colgid;
  gd::DBuf<double> vals, rhs, tabs;
  gd::DBuf<double> w, dinv, dred;
  ~gd_dgspace() {
    gd::dfreeb(d_parts);
    gd::dfreeb(gcells);
    gd::dfreeb(gperm);
    gd::dfreeb(grcells);
    gd::dfreeb(rowptr);
    gd::dfreeb(colidx);
    gd::dfreeb(colgid);
    gd::dfreeb(vals);
    gd::dfreeb(rhs);
    gd::dfreeb(tabs);
    gd::dfreeb(w);
    gd::dfreeb(dinv);
    gd::dfreeb(dred);
  }
};

using namespace gd;

static DgGeo dg_geo(const gd_dgspace* S) {
  DgGeo G{};
  G.dim = S->dim;
  G.k = S->k;
  G.nn = S->nn;
  G.np = (int)S->parts.size();
  G.g = S->model->geom;
  for (int d = 0; d < kMaxDim; ++d) G.n[d] = d < S->dim ? S->model->geom.n[d] : 1;
  return G;
}

extern "C" int gd_dg_space_create(gd_model* m, int order, gd_dgspace** out) {
  if (!m || !out) return fail(GD_ERR_ARG, "gd_dg_space_create: null argument");
  if (order < 1 || order > 3) return fail(GD_ERR_UNSUPPORTED, "gd_dg_space_create: order 1 to 3");
  const Geom& g = m->geom;
  gd_dgspace* S = new gd_dgspace();
  S->model = m;
  S->k = order;
  S->dim = g.dim;
  S->nn = 1;
  for (int d = 0; d < g.dim; ++d) S->nn *= order + 1;
  cell_dof_positions(g.dim, order, S->dofpos);
  int64_t first = 0;
  for (const DevPart& P : m->parts) {
    DgPart D{};
    D.ncell_own = 1;
    D.nloc_cells = 1;
    for (int d = 0; d < kMaxDim; ++d) {
      D.own_lo[d] = d < g.dim ? P.own_lo[d] : 0;
      D.own_hi[d] = d < g.dim ? P.own_hi[d] : 1;
      D.loc_lo[d] = d < g.dim ? P.loc_lo[d] : 0;
      D.loc_hi[d] = d < g.dim ? P.loc_hi[d] : 1;
      D.ncell_own *= D.own_hi[d] - D.own_lo[d];
      D.nloc_cells *= D.loc_hi[d] - D.loc_lo[d];
    }
    D.first = first;
    first += (int64_t)S->nn * D.ncell_own;
    // ghost cells that share a face with an owned cell, in local-box order
    D.gc_off = (int64_t)S->h_gcells.size();
    for (int64_t l = 0; l < D.nloc_cells; ++l) {
      int64_t X[kMaxDim] = {0, 0, 0}, rest = l;
      for (int d = 0; d < g.dim; ++d) {
        const int64_t w = D.loc_hi[d] - D.loc_lo[d];
        X[d] = D.loc_lo[d] + rest % w;
        rest /= w;
      }
      if (in_box(D.own_lo, D.own_hi, X, g.dim)) continue;
      int out_dirs = 0;
      bool adjacent = true;
      for (int d = 0; d < g.dim; ++d) {
        if (X[d] < D.own_lo[d] || X[d] >= D.own_hi[d]) {
          ++out_dirs;
          if (X[d] != D.own_lo[d] - 1 && X[d] != D.own_hi[d]) adjacent = false;
        }
      }
      if (out_dirs == 1 && adjacent) S->h_gcells.push_back(l);
    }
    D.n_gc = (int64_t)S->h_gcells.size() - D.gc_off;
    S->parts.push_back(D);
  }
  S->ndofs = first;
  cudaStream_t st = m->ctx->stream;
  int s = dalloc(S->d_parts, S->parts.size());
  if (s == GD_OK) s = dalloc(S->gcells, std::max<size_t>(S->h_gcells.size(), 1));
  if (s == GD_OK &&
      (cudaMemcpyAsync(S->d_parts.p, S->parts.data(), sizeof(DgPart) * S->parts.size(), cudaMemcpyHostToDevice, st) !=
           cudaSuccess ||
       (S->h_gcells.size() && cudaMemcpyAsync(S->gcells.p, S->h_gcells.data(), sizeof(int64_t) * S->h_gcells.size(),
                                              cudaMemcpyHostToDevice, st) != cudaSuccess) ||
       cudaStreamSynchronize(st) != cudaSuccess))
    s = fail(GD_ERR_CUDA, "gd_dg_space_create: copy");
  if (s != GD_OK) {
    delete S;
    return s;
  }
  *out = S;
  return GD_OK;
}

extern "C" int gd_dg_space_destroy(gd_dgspace* S) {
  delete S;
  return GD_OK;
}

extern "C" int gd_dg_num_free_dofs(const gd_dgspace* S, int64_t* n) {
  if (!S || !n) return fail(GD_ERR_ARG, "gd_dg_num_free_dofs: null argument");
  *n = S->ndofs;
  return GD_OK;
}

extern "C" int gd_dg_local_sizes(const gd_dgspace* S, int part, int64_t* nlocal, int64_t* nown, int64_t* first) {
  if (!S || part < 0 || part >= (int)S->parts.size()) return fail(GD_ERR_ARG, "gd_dg_local_sizes: bad part");
  const DgPart& P = S->parts[part];
  if (nlocal) *nlocal = (int64_t)S->nn * P.nloc_cells;
  if (nown) *nown = (int64_t)S->nn * P.ncell_own;
  if (first) *first = P.first;
  return GD_OK;
}

// gids / owners of the part's local dofs (local cells in local-box order, nn dofs each)
extern "C" int gd_dg_get_gids(const gd_dgspace* S, int part, int64_t* gid, int32_t* owner) {
  if (!S || part < 0 || part >= (int)S->parts.size()) return fail(GD_ERR_ARG, "gd_dg_get_gids: bad part");
  const DgPart& P = S->parts[part];
  const Geom& g = S->model->geom;
  for (int64_t l = 0; l < P.nloc_cells; ++l) {
    int64_t X[kMaxDim] = {0, 0, 0}, rest = l;
    for (int d = 0; d < S->dim; ++d) {
      const int64_t w = P.loc_hi[d] - P.loc_lo[d];
      X[d] = P.loc_lo[d] + rest % w;
      rest /= w;
    }
    const int q = cell_owner(g, X);
    const DgPart& Q = S->parts[q];
    const int64_t g0 = Q.first + (int64_t)S->nn * box_lex(Q.own_lo, Q.own_hi, X, S->dim);
    for (int a = 0; a < S->nn; ++a) {
      if (gid) gid[l * S->nn + a] = g0 + a;
      if (owner) owner[l * S->nn + a] = q;
    }
  }
  return GD_OK;
}

// Ghost-column order and ghost-row cells of every part for the space's strategy (see the
// file comment), uploaded with the part table.
static int dg_layout(gd_dgspace* S) {
  const Geom& g = S->model->geom;
  S->h_gperm.assign(std::max<size_t>(S->h_gcells.size(), 1), 0);
  S->h_grcells.clear();
  for (DgPart& P : S->parts) {
    struct Item {
      int cls, owner;
      int64_t key;
      int64_t idx;
    };
    std::vector<Item> items;
    P.gr_off = (int64_t)S->h_grcells.size();
    for (int64_t i = 0; i < P.n_gc; ++i) {
      const int64_t key = S->h_gcells[P.gc_off + i];
      int64_t X[kMaxDim] = {0, 0, 0}, rest = key;
      for (int d = 0; d < S->dim; ++d) {
        const int64_t w = P.loc_hi[d] - P.loc_lo[d];
        X[d] = P.loc_lo[d] + rest % w;
        rest /= w;
      }
      bool lower = false;
      for (int d = 0; d < S->dim; ++d) lower = lower || X[d] == P.own_lo[d] - 1;
      if (S->strategy == GD_FULLY_ASSEMBLED_ROWS) {
        items.push_back({0, 0, key, i});
      } else if (lower) {
        items.push_back({0, 0, key, i});
        S->h_grcells.push_back(key);
      } else {
        items.push_back({1, cell_owner(g, X), cell_lin(g, X), i});
      }
    }
    std::stable_sort(items.begin(), items.end(), [](const Item& a, const Item& b) {
      if (a.cls != b.cls) return a.cls < b.cls;
      if (a.owner != b.owner) return a.owner < b.owner;
      return a.key < b.key;
    });
    for (size_t pos = 0; pos < items.size(); ++pos) S->h_gperm[P.gc_off + items[pos].idx] = (int32_t)pos;
    P.n_gr = (int64_t)S->h_grcells.size() - P.gr_off;
  }
  S->nghost_rows = (int64_t)S->nn * (int64_t)S->h_grcells.size();
  cudaStream_t st = S->model->ctx->stream;
  GD_TRY(dalloc(S->gperm, S->h_gperm.size()));
  GD_TRY(dalloc(S->grcells, std::max<size_t>(S->h_grcells.size(), 1)));
  GD_CUDA_TRY(cudaMemcpyAsync(S->d_parts.p, S->parts.data(), sizeof(DgPart) * S->parts.size(), cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaMemcpyAsync(S->gperm.p, S->h_gperm.data(), sizeof(int32_t) * S->h_gperm.size(),
                              cudaMemcpyHostToDevice, st));
  if (!S->h_grcells.empty())
    GD_CUDA_TRY(cudaMemcpyAsync(S->grcells.p, S->h_grcells.data(), sizeof(int64_t) * S->h_grcells.size(),
                                cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

extern "C" int gd_dg_set_strategy(gd_dgspace* S, int strategy) {
  if (!S) return fail(GD_ERR_ARG, "gd_dg_set_strategy: null space");
  if (strategy != GD_SUB_ASSEMBLED_ROWS && strategy != GD_FULLY_ASSEMBLED_ROWS)
    return fail(GD_ERR_ARG, "gd_dg_set_strategy: unknown strategy");
  if (S->rowptr.p && strategy != S->strategy)
    return fail(GD_ERR_STATE, "gd_dg_set_strategy: the pattern of the other strategy is built already");
  S->strategy = strategy;
  return GD_OK;
}

// Host tables of the SIPG form on the model's cells (see the file comment).
static void dg_tables(const gd_dgspace* S, double gamma, double hpen, int degree, std::vector<double>& tab,
                      std::vector<double>& vtab, int& nq, int& nqf, int& nqt) {
  const int dim = S->dim, k = S->k, nn = S->nn;
  const Geom& g = S->model->geom;
  nq = (degree + 2) / 2;
  std::vector<double> xq, wq;
  gauss_legendre01(nq, xq, wq);
  nqf = 1;
  for (int d = 0; d + 1 < dim; ++d) nqf *= nq;
  nqt = nqf * nq;
  double h[kMaxDim] = {1, 1, 1}, det = 1.0;
  for (int d = 0; d < dim; ++d) {
    h[d] = g.h[d];
    det *= h[d];
  }
  // shape value and gradient (physical) of dof a at reference point xi
  auto shape = [&](int a, const double* xi, double& v, double* grad) {
    std::vector<double> bv, bd;
    double vals[kMaxDim], ders[kMaxDim];
    for (int d = 0; d < dim; ++d) {
      basis1d(k, xi[d], bv, bd);
      vals[d] = bv[S->dofpos[3 * a + d]];
      ders[d] = bd[S->dofpos[3 * a + d]];
    }
    v = 1.0;
    for (int d = 0; d < dim; ++d) v *= vals[d];
    for (int e = 0; e < dim; ++e) {
      double t = ders[e] / h[e];
      for (int d = 0; d < dim; ++d)
        if (d != e) t *= vals[d];
      grad[e] = t;
    }
  };
  const DgTabs T{nn, nqf};
  tab.assign(T.face_base(2 * dim), 0.0);
  vtab.assign((size_t)nqt * nn + nqt, 0.0);
  // volume: stiffness, load and the values at the Gauss points (with w |J| as a last row)
  for (int q = 0; q < nqt; ++q) {
    double xi[kMaxDim] = {0, 0, 0}, wt = det;
    for (int d = 0, r = q; d < dim; ++d) {
      xi[d] = xq[r % nq];
      wt *= wq[r % nq];
      r /= nq;
    }
    std::vector<double> v(nn), gr(nn * kMaxDim);
    for (int a = 0; a < nn; ++a) shape(a, xi, v[a], &gr[a * kMaxDim]);
    for (int a = 0; a < nn; ++a) {
      tab[nn * nn + a] += wt * v[a];
      vtab[q * nn + a] = v[a];
      for (int b = 0; b < nn; ++b) {
        double s = 0.0;
        for (int e = 0; e < dim; ++e) s += gr[a * kMaxDim + e] * gr[b * kMaxDim + e];
        tab[a * nn + b] += wt * s;
      }
    }
    vtab[(size_t)nqt * nn + q] = wt;
  }
  const double pen = gamma / hpen;
  for (int f = 0; f < 2 * dim; ++f) {
    const int d = f >> 1, sd = f & 1;
    const double sgn = sd ? 1.0 : -1.0;
    double fm = 1.0;
    for (int e = 0; e < dim; ++e)
      if (e != d) fm *= h[e];
    double* Bd = tab.data() + T.face_base(f);
    double* Sm = Bd + nn * nn;
    double* Nb = Sm + nn * nn;
    double* Rd = Nb + nn * nn;
    double* Rn = Rd + (size_t)nqf * nn;
    for (int q = 0; q < nqf; ++q) {
      double xi[kMaxDim] = {0, 0, 0}, xo[kMaxDim] = {0, 0, 0}, wt = fm;
      for (int e = 0, r = q; e < dim; ++e) {
        if (e == d) continue;
        xi[e] = xo[e] = xq[r % nq];
        wt *= wq[r % nq];
        r /= nq;
      }
      xi[d] = sd;          // this cell's face
      xo[d] = 1.0 - sd;    // the same point seen from the neighbour across the face
      std::vector<double> v(nn), dn(nn), vo(nn), dno(nn);
      double gr[kMaxDim];
      for (int a = 0; a < nn; ++a) {
        shape(a, xi, v[a], gr);
        dn[a] = sgn * gr[d];
        shape(a, xo, vo[a], gr);
        dno[a] = sgn * gr[d];
      }
      for (int a = 0; a < nn; ++a) {
        Rd[q * nn + a] = wt * (pen * v[a] - dn[a]);
        Rn[q * nn + a] = wt * v[a];
        for (int b = 0; b < nn; ++b) {
          Bd[a * nn + b] += wt * (pen * v[a] * v[b] - v[a] * dn[b] - dn[a] * v[b]);
          Sm[a * nn + b] += wt * (pen * v[a] * v[b] - 0.5 * v[a] * dn[b] - 0.5 * dn[a] * v[b]);
          Nb[a * nn + b] += wt * (-pen * v[a] * vo[b] - 0.5 * v[a] * dno[b] + 0.5 * dn[a] * vo[b]);
        }
      }
    }
  }
}

// Side offsets (in faces) of the flagged sides in the face Gauss-point arrays.
static int64_t side_offsets(const Geom& g, const int32_t* sides, std::vector<int64_t>& off, int& mask) {
  off.assign(2 * kMaxDim, 0);
  mask = 0;
  int64_t nf = 0;
  for (int s = 0; s < 2 * g.dim; ++s) {
    off[s] = nf;
    if (!sides || !sides[s]) continue;
    mask |= 1 << s;
    int64_t c = 1;
    for (int t = 0; t < g.dim; ++t)
      if (t != s / 2) c *= g.n[t];
    nf += c;
  }
  return nf;
}

// Assemble the SIPG system (matrix and right-hand side, FullyAssembledRows).
extern "C" int gd_dg_assemble(gd_dgspace* S, const gd_dg_form* F) {
  if (!S || !F) return fail(GD_ERR_ARG, "gd_dg_assemble: null argument");
  if (!(F->gamma >= 0.0) || !(F->h > 0.0)) return fail(GD_ERR_ARG, "gd_dg_assemble: gamma >= 0 and h > 0");
  const Geom& g = S->model->geom;
  cudaStream_t st = S->model->ctx->stream;
  std::vector<double> tab, vtab;
  int nq, nqf, nqt;
  dg_tables(S, F->gamma, F->h, F->degree, tab, vtab, nq, nqf, nqt);
  if (nq < 1 || nq > 16) return fail(GD_ERR_ARG, "gd_dg_assemble: quadrature degree out of range");
  std::vector<int64_t> doff, noff;
  int dmask = 0, nmask = 0;
  const int64_t ndf = side_offsets(g, F->dirichlet_sides, doff, dmask);
  const int64_t nnf = side_offsets(g, F->neumann_sides, noff, nmask);
  if (dmask & nmask) return fail(GD_ERR_ARG, "gd_dg_assemble: a side is both Dirichlet and Neumann");
  if ((dmask && !F->ud_qp) || (nmask && !F->g_qp)) return fail(GD_ERR_ARG, "gd_dg_assemble: missing boundary values");
  int64_t ncells = 1;
  for (int d = 0; d < g.dim; ++d) ncells *= g.n[d];
  const int64_t n = S->ndofs;
  const DgGeo G = dg_geo(S);
  const DgTabs T{S->nn, nqf};
  DBuf<double> dvt, dud, dg, dfq;
  DBuf<int64_t> ddoff, dnoff;
  DBuf<int32_t> len;
  auto done = [&](int s) {
    dfreeb(dvt);
    dfreeb(dud);
    dfreeb(dg);
    dfreeb(dfq);
    dfreeb(ddoff);
    dfreeb(dnoff);
    dfreeb(len);
    return s;
  };
  int s = GD_OK;
  if (S->tabs.n != tab.size()) s = dalloc(S->tabs, tab.size());
  if (s == GD_OK) s = dalloc(dvt, vtab.size());
  if (s == GD_OK) s = dalloc(ddoff, doff.size());
  if (s == GD_OK) s = dalloc(dnoff, noff.size());
  if (s != GD_OK) return done(s);
  const double* ud = F->ud_qp;
  const double* gq = F->g_qp;
  const double* fq = F->f_qp;
  cudaError_t e = cudaMemcpyAsync(S->tabs.p, tab.data(), sizeof(double) * tab.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dvt.p, vtab.data(), sizeof(double) * vtab.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(ddoff.p, doff.data(), sizeof(int64_t) * doff.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dnoff.p, noff.data(), sizeof(int64_t) * noff.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && F->where == GD_HOST) {
    if (dmask) {
      if ((s = dalloc(dud, ndf * nqf)) != GD_OK) return done(s);
      e = cudaMemcpyAsync(dud.p, F->ud_qp, sizeof(double) * ndf * nqf, cudaMemcpyHostToDevice, st);
      ud = dud.p;
    }
    if (e == cudaSuccess && nmask) {
      if ((s = dalloc(dg, nnf * nqf)) != GD_OK) return done(s);
      e = cudaMemcpyAsync(dg.p, F->g_qp, sizeof(double) * nnf * nqf, cudaMemcpyHostToDevice, st);
      gq = dg.p;
    }
    if (e == cudaSuccess && F->f_qp) {
      if ((s = dalloc(dfq, ncells * nqt)) != GD_OK) return done(s);
      e = cudaMemcpyAsync(dfq.p, F->f_qp, sizeof(double) * ncells * nqt, cudaMemcpyHostToDevice, st);
      fq = dfq.p;
    }
  }
  if (e != cudaSuccess) return done(fail(GD_ERR_CUDA, "gd_dg_assemble: copy"));
  // pattern (once): ghost layout of the strategy, row lengths of the owned rows and then of
  // the ghost rows (SubAssembledRows), offsets; the ghost rows' columns and their explicit
  // zeros are written here once
  if (!S->rowptr.p) {
    if ((s = dg_layout(S)) != GD_OK) return done(s);
    const int64_t nt = n + S->nghost_rows;
    if ((s = dalloc(len, std::max<int64_t>(nt, 1))) != GD_OK) return done(s);
    if ((s = dalloc(S->rowptr, nt + 1)) != GD_OK) return done(s);
    if (n) k_dg_rowlen<<<dg_grid(n, 256), 256, 0, st>>>(G, S->d_parts.p, n, len.p);
    if (S->nghost_rows)
      k_dg_ghost_rows<<<dg_grid(S->nghost_rows, 256), 256, 0, st>>>(G, S->d_parts.p, S->grcells.p, S->gcells.p,
                                                                     S->gperm.p, n, S->nghost_rows, 0, len.p,
                                                                     nullptr, nullptr, nullptr, nullptr);
    if (cudaGetLastError() != cudaSuccess) return done(fail(GD_ERR_CUDA, "gd_dg_assemble: row lengths"));
    if ((s = exclusive_scan_i32(len.p, S->rowptr.p, nt, st)) != GD_OK) return done(s);
    int64_t nz_all = 0;
    if (cudaMemcpyAsync(&S->nnz, S->rowptr.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(&nz_all, S->rowptr.p + nt, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return done(fail(GD_ERR_CUDA, "gd_dg_assemble: entry count"));
    if (nz_all >= ((int64_t)1 << 31) || nt >= ((int64_t)1 << 31))
      return done(fail(GD_ERR_UNSUPPORTED, "gd_dg_assemble: more than 2^31 entries"));
    const size_t nz = (size_t)std::max<int64_t>(nz_all, 1);
    if ((s = dalloc(S->colidx, nz)) != GD_OK || (s = dalloc(S->colgid, nz)) != GD_OK ||
        (s = dalloc(S->vals, nz)) != GD_OK || (s = dalloc(S->rhs, std::max<int64_t>(n, 1))) != GD_OK)
      return done(s);
    if (S->nghost_rows) {
      k_dg_ghost_rows<<<dg_grid(S->nghost_rows, 256), 256, 0, st>>>(G, S->d_parts.p, S->grcells.p, S->gcells.p,
                                                                     S->gperm.p, n, S->nghost_rows, 1, nullptr,
                                                                     S->rowptr.p, S->colidx.p, S->colgid.p, S->vals.p);
      if (cudaGetLastError() != cudaSuccess) return done(fail(GD_ERR_CUDA, "gd_dg_assemble: ghost rows"));
    }
  }
  if (n) {
    k_dg_fill<<<dg_grid(n * 32, 256), 256, 0, st>>>(G, T, S->d_parts.p, S->gcells.p, S->gperm.p, n, dmask, S->tabs.p,
                                                     S->rowptr.p, S->colidx.p, S->colgid.p, S->vals.p);
    k_dg_rhs<<<dg_grid(n, 128), 128, 0, st>>>(G, T, S->d_parts.p, n, S->tabs.p, F->f_const, fq, dvt.p, nqt, dmask,
                                              ddoff.p, ud, nmask, dnoff.p, gq, S->rhs.p);
  }
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return done(fail(GD_ERR_CUDA, "gd_dg_assemble: kernels"));
  S->assembled = true;
  return done(GD_OK);
}

extern "C" int gd_dg_matrix_sizes(const gd_dgspace* S, int part, int64_t* nrows, int64_t* ncols, int64_t* nnz,
                                  int64_t* n_ghost_rows, int64_t* n_ghost_cols) {
  if (!S) return fail(GD_ERR_ARG, "gd_dg_matrix_sizes: null DG space");
  if (!S->assembled) return fail(GD_ERR_STATE, "gd_dg_matrix_sizes: assemble first");
  if (part < 0 || part >= (int)S->parts.size()) return fail(GD_ERR_ARG, "gd_dg_matrix_sizes: bad part");
  const DgPart& P = S->parts[part];
  cudaStream_t st = S->model->ctx->stream;
  const int64_t r0 = P.first, r1 = P.first + (int64_t)S->nn * P.ncell_own;
  const int64_t g0 = S->ndofs + (int64_t)S->nn * P.gr_off, g1 = g0 + (int64_t)S->nn * P.n_gr;
  int64_t b[4];
  GD_CUDA_TRY(cudaMemcpyAsync(&b[0], S->rowptr.p + r0, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[1], S->rowptr.p + r1, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[2], S->rowptr.p + g0, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[3], S->rowptr.p + g1, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (nrows) *nrows = (r1 - r0) + (g1 - g0);
  if (ncols) *ncols = (int64_t)S->nn * (P.ncell_own + P.n_gc);
  if (nnz) *nnz = (b[1] - b[0]) + (b[3] - b[2]);
  if (n_ghost_rows) *n_ghost_rows = g1 - g0;
  if (n_ghost_cols) *n_ghost_cols = (int64_t)S->nn * P.n_gc;
  return GD_OK;
}

// gid and owner of dof a of the cell with local-box id `key` of part P
static void dg_local_cell_gid(const gd_dgspace* S, const DgPart& P, int64_t key, int64_t* gid0, int32_t* owner) {
  const Geom& g = S->model->geom;
  int64_t X[kMaxDim] = {0, 0, 0}, rest = key;
  for (int d = 0; d < S->dim; ++d) {
    const int64_t w = P.loc_hi[d] - P.loc_lo[d];
    X[d] = P.loc_lo[d] + rest % w;
    rest /= w;
  }
  const int q = cell_owner(g, X);
  const DgPart& Q = S->parts[q];
  *gid0 = Q.first + (int64_t)S->nn * box_lex(Q.own_lo, Q.own_hi, X, S->dim);
  *owner = q;
}

// One part: local CSR over the owned rows and then the ghost rows, the ghost rows' and
// ghost columns' gids / owners (in the strategy's order), the right-hand side (ghost rows 0).
extern "C" int gd_dg_matrix_export(const gd_dgspace* S, int part, int64_t* rowptr, int32_t* colidx, double* vals,
                                   int64_t* ghost_row_gids, int32_t* ghost_row_owners, int64_t* ghost_col_gids,
                                   int32_t* ghost_col_owners, double* rhs) {
  if (!S) return fail(GD_ERR_ARG, "gd_dg_matrix_export: null DG space");
  if (!S->assembled) return fail(GD_ERR_STATE, "gd_dg_matrix_export: assemble first");
  if (part < 0 || part >= (int)S->parts.size()) return fail(GD_ERR_ARG, "gd_dg_matrix_export: bad part");
  const DgPart& P = S->parts[part];
  cudaStream_t st = S->model->ctx->stream;
  const int nn = S->nn;
  const int64_t r0 = P.first, nr = (int64_t)nn * P.ncell_own;
  const int64_t g0 = S->ndofs + (int64_t)nn * P.gr_off, ng = (int64_t)nn * P.n_gr;
  std::vector<int64_t> rp(nr + 1), gp(ng + 1);
  GD_CUDA_TRY(cudaMemcpyAsync(rp.data(), S->rowptr.p + r0, sizeof(int64_t) * (nr + 1), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(gp.data(), S->rowptr.p + g0, sizeof(int64_t) * (ng + 1), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const int64_t nz = rp[nr] - rp[0], nzg = gp[ng] - gp[0];
  if (rowptr) {
    for (int64_t i = 0; i <= nr; ++i) rowptr[i] = rp[i] - rp[0];
    for (int64_t i = 1; i <= ng; ++i) rowptr[nr + i] = nz + gp[i] - gp[0];
  }
  if (colidx && nz) GD_CUDA_TRY(cudaMemcpyAsync(colidx, S->colidx.p + rp[0], sizeof(int32_t) * nz, cudaMemcpyDeviceToHost, st));
  if (colidx && nzg)
    GD_CUDA_TRY(cudaMemcpyAsync(colidx + nz, S->colidx.p + gp[0], sizeof(int32_t) * nzg, cudaMemcpyDeviceToHost, st));
  if (vals && nz) GD_CUDA_TRY(cudaMemcpyAsync(vals, S->vals.p + rp[0], sizeof(double) * nz, cudaMemcpyDeviceToHost, st));
  if (vals && nzg)
    GD_CUDA_TRY(cudaMemcpyAsync(vals + nz, S->vals.p + gp[0], sizeof(double) * nzg, cudaMemcpyDeviceToHost, st));
  if (rhs && nr) GD_CUDA_TRY(cudaMemcpyAsync(rhs, S->rhs.p + r0, sizeof(double) * nr, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (rhs)
    for (int64_t i = 0; i < ng; ++i) rhs[nr + i] = 0.0;
  for (int64_t i = 0; i < P.n_gr; ++i) {
    int64_t gid0;
    int32_t q;
    dg_local_cell_gid(S, P, S->h_grcells[P.gr_off + i], &gid0, &q);
    for (int a = 0; a < nn; ++a) {
      if (ghost_row_gids) ghost_row_gids[i * nn + a] = gid0 + a;
      if (ghost_row_owners) ghost_row_owners[i * nn + a] = q;
    }
  }
  for (int64_t i = 0; i < P.n_gc; ++i) {
    int64_t gid0;
    int32_t q;
    dg_local_cell_gid(S, P, S->h_gcells[P.gc_off + i], &gid0, &q);
    const int64_t pos = S->h_gperm[P.gc_off + i];
    for (int a = 0; a < nn; ++a) {
      if (ghost_col_gids) ghost_col_gids[pos * nn + a] = gid0 + a;
      if (ghost_col_owners) ghost_col_owners[pos * nn + a] = q;
    }
  }
  return GD_OK;
}

extern "C" int gd_dg_spmv(const gd_dgspace* S, const double* x, double* y, int where) {
  if (!S || !S->assembled || !x || !y) return fail(GD_ERR_ARG, "gd_dg_spmv: assemble first; non-null vectors");
  cudaStream_t st = S->model->ctx->stream;
  const int64_t n = S->ndofs;
  DBuf<double> bx, by;
  const double* dx = x;
  double* dy = y;
  int s = GD_OK;
  if (where == GD_HOST) {
    s = dalloc(bx, std::max<int64_t>(n, 1));
    if (s == GD_OK) s = dalloc(by, std::max<int64_t>(n, 1));
    if (s == GD_OK && n && cudaMemcpyAsync(bx.p, x, sizeof(double) * n, cudaMemcpyHostToDevice, st) != cudaSuccess)
      s = fail(GD_ERR_CUDA, "gd_dg_spmv: copy");
    dx = bx.p;
    dy = by.p;
  }
  if (s == GD_OK && n) {
    k_dg_spmv<<<dg_grid(n, 256), 256, 0, st>>>(n, S->rowptr.p, S->colgid.p, S->vals.p, dx, dy);
    if (cudaGetLastError() != cudaSuccess) s = fail(GD_ERR_CUDA, "gd_dg_spmv: launch");
  }
  if (s == GD_OK && where == GD_HOST && n &&
      cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
    s = fail(GD_ERR_CUDA, "gd_dg_spmv: copy");
  if (s == GD_OK && cudaStreamSynchronize(st) != cudaSuccess) s = fail(GD_ERR_CUDA, "gd_dg_spmv: sync");
  dfreeb(bx);
  dfreeb(by);
  return s;
}

// x = A \ b: FP64 Jacobi-PCG (the SIPG matrix is SPD for a large enough penalty)
extern "C" int gd_dg_solve(gd_dgspace* S, double rtol, int maxit, double* x, int where, gd_solve_stats* stats) {
  if (!S || !S->assembled || !x) return fail(GD_ERR_ARG, "gd_dg_solve: assemble first; non-null x");
  if (!(rtol > 0.0) || maxit < 0) return fail(GD_ERR_ARG, "gd_dg_solve: bad argument");
  return jacobi_pcg_csr(S->ndofs, S->rowptr.p, S->colgid.p, S->vals.p, S->rhs.p, S->w, S->dinv, S->dred,
                        S->model->ctx->stream, rtol, maxit, x, where, stats);
}

// sqrt(sum over cells int (u - uh)^2): x the global dof values, u at the cells' Gauss
// points (cells lexicographic, nq^dim points x fastest, nq = (degree + 2) / 2)
extern "C" int gd_dg_l2_error(const gd_dgspace* S, const double* x, const double* u_qp, int degree, int where,
                              double* err) {
  if (!S || !x || !u_qp || !err) return fail(GD_ERR_ARG, "gd_dg_l2_error: null argument");
  cudaStream_t st = S->model->ctx->stream;
  std::vector<double> tab, vtab;
  int nq, nqf, nqt;
  dg_tables(S, 0.0, 1.0, degree, tab, vtab, nq, nqf, nqt);
  const Geom& g = S->model->geom;
  int64_t ncells = 1;
  for (int d = 0; d < g.dim; ++d) ncells *= g.n[d];
  const unsigned nb = dg_grid(ncells, 256);
  DBuf<double> dvt, bx, bu, part;
  int s = dalloc(dvt, vtab.size());
  if (s == GD_OK) s = dalloc(part, nb);
  const double* dx = x;
  const double* du = u_qp;
  cudaError_t e = cudaSuccess;
  if (s == GD_OK) e = cudaMemcpyAsync(dvt.p, vtab.data(), sizeof(double) * vtab.size(), cudaMemcpyHostToDevice, st);
  if (s == GD_OK && e == cudaSuccess && where == GD_HOST) {
    s = dalloc(bx, std::max<int64_t>(S->ndofs, 1));
    if (s == GD_OK) s = dalloc(bu, std::max<int64_t>(ncells * nqt, 1));
    if (s == GD_OK) e = cudaMemcpyAsync(bx.p, x, sizeof(double) * S->ndofs, cudaMemcpyHostToDevice, st);
    if (s == GD_OK && e == cudaSuccess) e = cudaMemcpyAsync(bu.p, u_qp, sizeof(double) * ncells * nqt, cudaMemcpyHostToDevice, st);
    dx = bx.p;
    du = bu.p;
  }
  std::vector<double> hp(nb);
  if (s == GD_OK && e == cudaSuccess) {
    k_dg_l2<<<nb, 256, 0, st>>>(dg_geo(S), S->d_parts.p, ncells, dx, dvt.p, nqt, du, part.p);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  dfreeb(dvt);
  dfreeb(bx);
  dfreeb(bu);
  dfreeb(part);
  if (s != GD_OK) return s;
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, "gd_dg_l2_error: kernel");
  double t = 0.0;
  for (double v : hp) t += v;
  *err = std::sqrt(t);
  return GD_OK;
}
