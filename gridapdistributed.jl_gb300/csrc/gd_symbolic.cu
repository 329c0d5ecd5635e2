// A9-A11 symbolic phase: row and column index sets of every part and the local CSR
// patterns, built on the device without a COO.
//
// The reference builds a COO per part (cells in order, columns outer, rows inner),
// sends ghost-row triplets to their owners and compresses with sparse()
// (Algebra.jl:593-646, 1048-1131).  On a Cartesian mesh every quantity that
// process produces has a closed form per DOF:
//  * ghost rows (SubAssembledRows): non-owned free DOFs on the part's owned cells,
//    sorted by local DOF id (Algebra.jl:931-962, 919-928);
//  * ghost columns: SubAssembledRows orders them by first appearance in the COO
//    after the exchange (Algebra.jl:1210-1238): local triplets first (key: first
//    owned cell holding the DOF, then its cell-local position), then triplets
//    received from each sender in ascending part order (key: sender, sender's cell,
//    cell-local position).  FullyAssembledRows sorts them by local DOF id
//    (Algebra.jl:1245-1257);
//  * the entries of a row are the free nodes of the cells that contribute to it,
//    which on a structured grid form a box; the local CSR sorts them by column id.
// Every entry also gets a stencil code (lattice offset of its column relative to
// its row) so the numeric phase needs no cell->entry position map.
#include <algorithm>
#include <string>

#include "gd_internal.h"

namespace gd {

static inline unsigned nblk(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

static int launch_ok(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return GD_OK;
}

__device__ inline int part_by_lid(const DevPart* parts, int nparts, int64_t t) {
  int lo = 0, hi = nparts - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (parts[mid].lid_off <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ inline int part_by_gid(const DevPart* parts, int nparts, int64_t gid) {
  int lo = 0, hi = nparts - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (parts[mid].first_gdof <= gid) lo = mid; else hi = mid - 1;
  }
  return lo;
}
__device__ inline int part_by_grow(const DevPart* parts, int nparts, int64_t t) {
  int lo = 0, hi = nparts - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (parts[mid].grow_off <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ inline void lid_coords(const Geom& g, const DevPart& P, int32_t lnode, int64_t* X) {
  int64_t li = lnode;
  for (int d = 0; d < g.dim; ++d) {
    X[d] = g.k * P.loc_lo[d] + li % P.nb[d];
    li /= P.nb[d];
  }
}

// local node index of lattice node X in part P's box, or -1
__device__ inline int64_t box_index(const Geom& g, const DevPart& P, const int64_t* X) {
  int64_t r = 0;
  for (int d = g.dim - 1; d >= 0; --d) {
    int64_t y = X[d] - g.k * P.loc_lo[d];
    if (y < 0 || y >= P.nb[d]) return -1;
    r = r * P.nb[d] + y;
  }
  return r;
}

// Cells along d that hold lattice coordinate x: [lo, hi] (global, clamped).
__device__ inline void cells_of(const Geom& g, int d, int64_t x, int64_t* lo, int64_t* hi) {
  int64_t c = x / g.k;
  if (x % g.k == 0) {
    *lo = c - 1 < 0 ? 0 : c - 1;
    *hi = c > g.n[d] - 1 ? g.n[d] - 1 : c;
  } else {
    *lo = c;
    *hi = c;
  }
}

// Does cell c (global coords) contain a free node owned by part p?
__device__ bool cell_has_owned_free(const Geom& g, const int64_t* c, int p) {
  const int kp1 = g.k + 1;
  int nn = 1;
  for (int d = 0; d < g.dim; ++d) nn *= kp1;
  for (int a = 0; a < nn; ++a) {
    int64_t X[kMaxDim] = {0, 0, 0};
    int rest = a;
    for (int d = 0; d < g.dim; ++d) {
      X[d] = g.k * c[d] + rest % kp1;
      rest /= kp1;
    }
    if (!node_is_dirichlet(g, X) && node_owner(g, X) == p) return true;
  }
  return false;
}

__device__ inline int lex_local(const Geom& g, const int64_t* X, const int64_t* c) {
  int r = 0;
  for (int d = g.dim - 1; d >= 0; --d) r = r * (g.k + 1) + (int)(X[d] - g.k * c[d]);
  return r;
}

// ---- ghost rows -----------------------------------------------------------------
__global__ void k_ghost_row_flag(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                                 const int32_t* __restrict__ lid_node, const int32_t* __restrict__ lid_owner,
                                 int32_t* __restrict__ flag) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int p = part_by_lid(parts, g.nparts, t);
  const DevPart& P = parts[p];
  int f = 0;
  if (lid_owner[t] != p) {
    int64_t X[kMaxDim];
    lid_coords(g, P, lid_node[t], X);
    f = 1;
    for (int d = 0; d < g.dim; ++d)
      if (X[d] < g.k * P.own_lo[d] || X[d] > g.k * P.own_hi[d]) f = 0;
  }
  flag[t] = f;
}

__global__ void k_ghost_row_fill(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                                 const int32_t* __restrict__ flag, const int64_t* __restrict__ scan,
                                 int32_t* __restrict__ grow_lid) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  if (!flag[t]) return;
  int p = part_by_lid(parts, g.nparts, t);
  const DevPart& P = parts[p];
  // scan is global; the part's ghost rows start at grow_off
  grow_lid[scan[t]] = (int32_t)(t - P.lid_off);
  (void)P;
}

// ---- ghost columns ------------------------------------------------------------------
// key = ~0 when the DOF is not a ghost column of its part.
__global__ void k_ghost_col_key(Geom g, const DevPart* __restrict__ parts, int64_t total_lids, int strategy,
                                const int32_t* __restrict__ lid_node, const int32_t* __restrict__ lid_owner,
                                const int* __restrict__ lex2gridap, unsigned long long* __restrict__ key,
                                int32_t* __restrict__ flag) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int p = part_by_lid(parts, g.nparts, t);
  const DevPart& P = parts[p];
  unsigned long long best = ~0ull;
  if (lid_owner[t] != p) {
    int64_t X[kMaxDim] = {0, 0, 0};
    lid_coords(g, P, lid_node[t], X);
    int64_t clo[kMaxDim] = {0, 0, 0}, chi[kMaxDim] = {0, 0, 0};
    for (int d = 0; d < g.dim; ++d) cells_of(g, d, X[d], &clo[d], &chi[d]);
    if (strategy == GD_FULLY_ASSEMBLED_ROWS) {
      // touched iff a local cell around it holds a free DOF owned by p; order = local id
      bool touched = false;
      int ncomb = 1 << g.dim;
      for (int cb = 0; cb < ncomb && !touched; ++cb) {
        int64_t c[kMaxDim] = {0, 0, 0};
        bool ok = true;
        for (int d = 0; d < g.dim; ++d) {
          c[d] = ((cb >> d) & 1) ? chi[d] : clo[d];
          if (((cb >> d) & 1) && chi[d] == clo[d]) ok = false;   // avoid duplicates
          if (c[d] < P.loc_lo[d] || c[d] >= P.loc_hi[d]) ok = false;
        }
        if (ok && cell_has_owned_free(g, c, p)) touched = true;
      }
      if (touched) best = (unsigned long long)(t - P.lid_off);
    } else {
      // first owned cell of p holding X (lexicographic = smallest index per direction)
      bool in_own = true;
      int64_t c0[kMaxDim] = {0, 0, 0};
      for (int d = 0; d < g.dim; ++d) {
        int64_t lo = clo[d] > P.own_lo[d] ? clo[d] : P.own_lo[d];
        int64_t hi = chi[d] < P.own_hi[d] - 1 ? chi[d] : P.own_hi[d] - 1;
        if (lo > hi) in_own = false;
        c0[d] = lo;
      }
      if (in_own) {
        int64_t rho = 0;
        for (int d = g.dim - 1; d >= 0; --d) rho = rho * (P.own_hi[d] - P.own_lo[d]) + (c0[d] - P.own_lo[d]);
        int jpos = lex2gridap[lex_local(g, X, c0)];
        best = ((unsigned long long)rho << 16) | (unsigned long long)jpos;
      } else {
        // received triplets only: sender q's cells around X that hold a row owned by p
        int ncomb = 1 << g.dim;
        for (int cb = 0; cb < ncomb; ++cb) {
          int64_t c[kMaxDim] = {0, 0, 0};
          bool ok = true;
          for (int d = 0; d < g.dim; ++d) {
            c[d] = ((cb >> d) & 1) ? chi[d] : clo[d];
            if (((cb >> d) & 1) && chi[d] == clo[d]) ok = false;
          }
          if (!ok) continue;
          if (!cell_has_owned_free(g, c, p)) continue;
          int q = cell_owner(g, c);
          const DevPart& Q = parts[q];
          int64_t rho = 0;
          for (int d = g.dim - 1; d >= 0; --d) rho = rho * (Q.own_hi[d] - Q.own_lo[d]) + (c[d] - Q.own_lo[d]);
          int jpos = lex2gridap[lex_local(g, X, c)];
          unsigned long long kk = (1ull << 63) | ((unsigned long long)q << 48) | ((unsigned long long)rho << 16) |
                                  (unsigned long long)jpos;
          if (kk < best) best = kk;
        }
      }
    }
  }
  key[t] = best;
  flag[t] = best != ~0ull;
}

__global__ void k_compact_candidates(int64_t total_lids, const int32_t* __restrict__ flag,
                                     const int64_t* __restrict__ scan, const unsigned long long* __restrict__ key,
                                     unsigned long long* __restrict__ ckey, int32_t* __restrict__ clid_concat) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  if (!flag[t]) return;
  ckey[scan[t]] = key[t];
  clid_concat[scan[t]] = (int32_t)t;
}

// rank of each candidate among the candidates of the same part (keys are unique)
constexpr int kRankTile = 1024;
__global__ void k_rank_candidates(int64_t off, int64_t n, const unsigned long long* __restrict__ ckey,
                                  int32_t* __restrict__ rank) {
  __shared__ unsigned long long tile[kRankTile];
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long mine = i < n ? ckey[off + i] : 0;
  int64_t r = 0;
  for (int64_t base = 0; base < n; base += kRankTile) {
    int64_t m = n - base < kRankTile ? n - base : kRankTile;
    for (int j = threadIdx.x; j < m; j += blockDim.x) tile[j] = ckey[off + base + j];
    __syncthreads();
    if (i < n)
      for (int j = 0; j < m; ++j) r += tile[j] < mine;
    __syncthreads();
  }
  if (i < n) rank[off + i] = (int32_t)r;
}

__global__ void k_assign_cols(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                              const int32_t* __restrict__ lid_owner, const int32_t* __restrict__ lid_ownidx,
                              int32_t* __restrict__ lid_col) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int p = part_by_lid(parts, g.nparts, t);
  lid_col[t] = lid_owner[t] == p ? lid_ownidx[t] : -1;
}

__global__ void k_assign_ghost_cols(Geom g, const DevPart* __restrict__ parts, int64_t ncand,
                                    const int32_t* __restrict__ clid_concat, const int32_t* __restrict__ rank,
                                    int32_t* __restrict__ lid_col, int32_t* __restrict__ gcol_lid) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ncand) return;
  int64_t t = clid_concat[i];
  int p = part_by_lid(parts, g.nparts, t);
  const DevPart& P = parts[p];
  lid_col[t] = (int32_t)(P.n_own + rank[i]);
  gcol_lid[P.gcol_off + rank[i]] = (int32_t)(t - P.lid_off);
}

// ---- rows: location, node, contributing cell box ----------------------------------------
struct RowInfo {
  int p;
  int64_t lid;          // local lid in part p
  int64_t X[kMaxDim];
  int64_t Ilo[kMaxDim], Ihi[kMaxDim];   // lattice node box of the contributing cells
};

__device__ inline void row_info(const Geom& g, const DevPart* parts, int64_t ngdofs, int64_t r,
                                const int32_t* own_lid, const int32_t* grow_lid, const int32_t* lid_node,
                                RowInfo& ri) {
  bool ghost = r >= ngdofs;
  if (!ghost) {
    ri.p = part_by_gid(parts, g.nparts, r);
    ri.lid = own_lid[r];
  } else {
    int64_t t = r - ngdofs;
    ri.p = part_by_grow(parts, g.nparts, t);
    ri.lid = grow_lid[t];
  }
  const DevPart& P = parts[ri.p];
  lid_coords(g, P, lid_node[P.lid_off + ri.lid], ri.X);
  for (int d = 0; d < kMaxDim; ++d) {
    ri.Ilo[d] = 0;
    ri.Ihi[d] = 0;
  }
  for (int d = 0; d < g.dim; ++d) {
    int64_t lo, hi;
    cells_of(g, d, ri.X[d], &lo, &hi);
    if (ghost) {   // SubAssembledRows ghost row: only the part's owned cells contribute
      if (lo < P.own_lo[d]) lo = P.own_lo[d];
      if (hi > P.own_hi[d] - 1) hi = P.own_hi[d] - 1;
    }
    ri.Ilo[d] = g.k * lo;
    ri.Ihi[d] = g.k * (hi + 1);
  }
}

__global__ void k_own_lid(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                          const int32_t* __restrict__ lid_owner, const int32_t* __restrict__ lid_ownidx,
                          int32_t* __restrict__ own_lid) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int p = part_by_lid(parts, g.nparts, t);
  if (lid_owner[t] == p) own_lid[parts[p].first_gdof + lid_ownidx[t]] = (int32_t)(t - parts[p].lid_off);
}

__global__ void k_row_len(Geom g, const DevPart* __restrict__ parts, int64_t ngdofs, int64_t nrows,
                          const int32_t* __restrict__ own_lid, const int32_t* __restrict__ grow_lid,
                          const int32_t* __restrict__ lid_node, int32_t* __restrict__ len,
                          int32_t* __restrict__ row_node, int32_t* __restrict__ row_part) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  RowInfo ri;
  row_info(g, parts, ngdofs, r, own_lid, grow_lid, lid_node, ri);
  int64_t L = 1;
  for (int d = 0; d < g.dim; ++d) {
    int64_t c = ri.Ihi[d] - ri.Ilo[d] + 1;
    if (g.dsides[2 * d] && ri.Ilo[d] == 0) --c;
    if (g.dsides[2 * d + 1] && ri.Ihi[d] == g.N[d] - 1) --c;
    L *= c;
  }
  len[r] = (int32_t)L;
  row_node[r] = (int32_t)lattice_lin(g, ri.X);
  row_part[r] = ri.p;
}

constexpr int kMaxRow = 343;   // (2k+1)^3 for k = 3

template <typename CodeT>
__global__ void k_row_fill(Geom g, const DevPart* __restrict__ parts, int64_t ngdofs, int64_t nrows,
                           const int32_t* __restrict__ own_lid, const int32_t* __restrict__ grow_lid,
                           const int32_t* __restrict__ lid_node, const int32_t* __restrict__ node_lid,
                           const int32_t* __restrict__ lid_col, const int64_t* __restrict__ lid_gid,
                           const int64_t* __restrict__ rowptr, int32_t* __restrict__ colidx,
                           int32_t* __restrict__ colgid, CodeT* __restrict__ code, int32_t* __restrict__ err) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  RowInfo ri;
  row_info(g, parts, ngdofs, r, own_lid, grow_lid, lid_node, ri);
  const DevPart& P = parts[ri.p];
  int32_t cols[kMaxRow];
  int32_t gids[kMaxRow];
  int32_t cds[kMaxRow];
  int n = 0;
  const int64_t w = 2 * g.k + 1;
  int64_t ext[kMaxDim] = {1, 1, 1};
  for (int d = 0; d < g.dim; ++d) ext[d] = ri.Ihi[d] - ri.Ilo[d] + 1;
  int64_t tot = ext[0] * ext[1] * ext[2];
  for (int64_t a = 0; a < tot; ++a) {
    int64_t Y[kMaxDim] = {0, 0, 0};
    int64_t rest = a;
    for (int d = 0; d < g.dim; ++d) {
      Y[d] = ri.Ilo[d] + rest % ext[d];
      rest /= ext[d];
    }
    if (node_is_dirichlet(g, Y)) continue;
    int64_t bi = box_index(g, P, Y);
    int32_t lid = bi >= 0 ? node_lid[P.node_off + bi] : -1;
    int32_t col = lid >= 0 ? lid_col[P.lid_off + lid] : -1;
    if (col < 0 || n >= kMaxRow) {
      atomicExch(err, 1);
      return;
    }
    int64_t cd = 0;
    for (int d = g.dim - 1; d >= 0; --d) cd = cd * w + (Y[d] - ri.X[d] + g.k);
    // insertion into sorted position
    int j = n;
    while (j > 0 && cols[j - 1] > col) {
      cols[j] = cols[j - 1];
      gids[j] = gids[j - 1];
      cds[j] = cds[j - 1];
      --j;
    }
    cols[j] = col;
    gids[j] = (int32_t)lid_gid[P.lid_off + lid];
    cds[j] = (int32_t)cd;
    ++n;
  }
  int64_t e0 = rowptr[r];
  if (rowptr[r + 1] - e0 != n) {
    atomicExch(err, 2);
    return;
  }
  for (int j = 0; j < n; ++j) {
    colidx[e0 + j] = cols[j];
    colgid[e0 + j] = gids[j];
    code[e0 + j] = (CodeT)cds[j];
  }
}


// ---- Q1 row patterns ---------------------------------------------------------------------
// For an owned Q1 row every lattice neighbour within +-1 that is free shares a cell with
// it.  perm[s] = CSR position of canonical neighbour s (offsets lexicographic, x
// fastest), 0xFF if absent.  Rows with equal perm share a pattern id, so the numeric
// kernel reads 2 bytes per row instead of a code per entry.
template <int DIM>
__global__ void k_row_perm_q1(Geom g, const DevPart* __restrict__ parts, int64_t nrows_own,
                              const int32_t* __restrict__ row_node, const int32_t* __restrict__ row_part,
                              const int32_t* __restrict__ node_lid, const int32_t* __restrict__ lid_col,
                              const int64_t* __restrict__ rowptr, uint8_t* __restrict__ rec,
                              unsigned long long* __restrict__ hash, int32_t* __restrict__ err) {
  constexpr int S = DIM == 3 ? 27 : 9;
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows_own) return;
  const DevPart& P = parts[row_part[r]];
  int64_t X[kMaxDim] = {0, 0, 0};
  lattice_coords(g, row_node[r], X);
  int32_t col[S];
  int n = 0;
#pragma unroll
  for (int s = 0; s < S; ++s) {
    int64_t Y[kMaxDim] = {X[0] + (s % 3) - 1, X[1] + (s / 3) % 3 - 1, DIM == 3 ? X[2] + s / 9 - 1 : 0};
    bool in = true;
    for (int d = 0; d < DIM; ++d) in = in && Y[d] >= 0 && Y[d] < g.N[d];
    col[s] = -1;
    if (in && !node_is_dirichlet(g, Y)) {
      int64_t bi = box_index(g, P, Y);
      int32_t lid = bi >= 0 ? node_lid[P.node_off + bi] : -1;
      col[s] = lid >= 0 ? lid_col[P.lid_off + lid] : -2;
      if (col[s] < 0) atomicExch(err, 3);
      ++n;
    }
  }
  uint8_t* out = rec + r * 32;
  unsigned long long h = 1469598103934665603ull;   // FNV-1a over the 32-byte record
  for (int s = 0; s < 32; ++s) {
    uint8_t v = 0xFF;
    if (s < S && col[s] >= 0) {
      int rank = 0;
      for (int t = 0; t < S; ++t) rank += (col[t] >= 0 && col[t] < col[s]);
      v = (uint8_t)rank;
    }
    if (s == 31) v = (uint8_t)n;
    out[s] = v;
    h = (h ^ v) * 1099511628211ull;
  }
  if (h == ~0ull) h = 0;
  hash[r] = h;
  if (rowptr[r + 1] - rowptr[r] != n) atomicExch(err, 4);
}

__global__ void k_pat_insert(int64_t n, const unsigned long long* __restrict__ hash, unsigned long long* keys,
                             int32_t* rep, int64_t mask) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const unsigned long long h = hash[r];
  int64_t slot = (int64_t)(h & (unsigned long long)mask);
  for (int64_t probe = 0; probe <= mask; ++probe) {
    unsigned long long prev = atomicCAS(&keys[slot], ~0ull, h);
    if (prev == ~0ull || prev == h) {
      atomicMin(&rep[slot], (int32_t)r);
      return;
    }
    slot = (slot + 1) & mask;
  }
}

__global__ void k_pat_occupied(int64_t cap, const unsigned long long* __restrict__ keys, int32_t* __restrict__ occ) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < cap) occ[i] = keys[i] != ~0ull;
}

__global__ void k_pat_assign(int64_t n, const unsigned long long* __restrict__ hash,
                             const unsigned long long* __restrict__ keys, const int32_t* __restrict__ rep,
                             const int64_t* __restrict__ slot_id, const uint8_t* __restrict__ rec, int64_t mask,
                             uint16_t* __restrict__ row_pat, int32_t* __restrict__ err) {
  int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const unsigned long long h = hash[r];
  int64_t slot = (int64_t)(h & (unsigned long long)mask);
  for (int64_t probe = 0; probe <= mask && keys[slot] != h; ++probe) slot = (slot + 1) & mask;
  if (keys[slot] != h) {
    atomicExch(err, 5);
    return;
  }
  const int64_t id = slot_id[slot];
  const uint8_t* a = rec + (int64_t)r * 32;
  const uint8_t* b = rec + (int64_t)rep[slot] * 32;
  for (int s = 0; s < 32; ++s)
    if (a[s] != b[s]) atomicExch(err, 6);   // hash collision: fall back to the generic kernel
  row_pat[r] = id < 65536 ? (uint16_t)id : 0;
}

__global__ void k_pat_table(int64_t cap, const unsigned long long* __restrict__ keys, const int32_t* __restrict__ rep,
                            const int64_t* __restrict__ slot_id, const uint8_t* __restrict__ rec, int64_t npat,
                            uint8_t* __restrict__ pat) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= cap || keys[i] == ~0ull) return;
  const int64_t id = slot_id[i];
  if (id >= npat) return;
  for (int s = 0; s < 32; ++s) pat[id * 32 + s] = rec[(int64_t)rep[i] * 32 + s];
}

}  // namespace gd

using namespace gd;

// Builds the Q1 pattern table; leaves fast_q1 false (generic kernel) when the
// patterns do not fit 16-bit ids or a hash collision is detected.
static int build_q1_patterns(gd_asm* A, const int32_t* lid_col) {
  gd_space* S = A->test;
  const Geom& g = S->geom;
  cudaStream_t st = S->model->ctx->stream;
  A->fast_q1 = false;
  const int64_t n = A->ngdofs;
  if (g.k != 1 || n == 0) return GD_OK;
  const int T = 256;
  DBuf<uint8_t> rec;
  DBuf<unsigned long long> hash, keys;
  DBuf<int32_t> rep, occ, err;
  DBuf<int64_t> slot_id;
  int64_t cap = 1024;
  while (cap < 2 * n) cap <<= 1;
  GD_TRY(dalloc(rec, n * 32));
  GD_TRY(dalloc(hash, n));
  GD_TRY(dalloc(keys, cap));
  GD_TRY(dalloc(rep, cap));
  GD_TRY(dalloc(occ, cap));
  GD_TRY(dalloc(slot_id, cap + 1));
  GD_TRY(dalloc(err, 1));
  GD_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int32_t), st));
  GD_CUDA_TRY(cudaMemsetAsync(keys.p, 0xFF, sizeof(unsigned long long) * cap, st));
  GD_CUDA_TRY(cudaMemsetAsync(rep.p, 0x7F, sizeof(int32_t) * cap, st));
  if (g.dim == 3)
    k_row_perm_q1<3><<<nblk(n, T), T, 0, st>>>(g, A->d_parts.p, n, A->row_node.p, A->row_part.p, S->node_lid.p,
                                               lid_col, A->rowptr.p, rec.p, hash.p, err.p);
  else
    k_row_perm_q1<2><<<nblk(n, T), T, 0, st>>>(g, A->d_parts.p, n, A->row_node.p, A->row_part.p, S->node_lid.p,
                                               lid_col, A->rowptr.p, rec.p, hash.p, err.p);
  GD_TRY(launch_ok("k_row_perm_q1"));
  k_pat_insert<<<nblk(n, T), T, 0, st>>>(n, hash.p, keys.p, rep.p, cap - 1);
  GD_TRY(launch_ok("k_pat_insert"));
  k_pat_occupied<<<nblk(cap, T), T, 0, st>>>(cap, keys.p, occ.p);
  GD_TRY(launch_ok("k_pat_occupied"));
  GD_TRY(exclusive_scan_i32(occ.p, slot_id.p, cap, st));
  int64_t npat = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&npat, slot_id.p + cap, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  GD_TRY(dalloc(A->row_pat, n));
  k_pat_assign<<<nblk(n, T), T, 0, st>>>(n, hash.p, keys.p, rep.p, slot_id.p, rec.p, cap - 1, A->row_pat.p, err.p);
  GD_TRY(launch_ok("k_pat_assign"));
  GD_TRY(dalloc(A->pat, std::max<int64_t>(npat, 1) * 32));
  k_pat_table<<<nblk(cap, T), T, 0, st>>>(cap, keys.p, rep.p, slot_id.p, rec.p, npat, A->pat.p);
  GD_TRY(launch_ok("k_pat_table"));
  int32_t herr = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&herr, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (herr == 3 || herr == 4) return fail(GD_ERR_STATE, "symbolic: Q1 row pattern disagrees with the CSR pattern");
  if (herr == 0 && npat < 65536) {
    A->fast_q1 = true;
    A->npat = (int)npat;
  } else {
    dfreeb(A->row_pat);
    dfreeb(A->pat);
  }
  return GD_OK;
}

// ---------------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------------
extern "C" int gd_assembler_create(gd_space* trial, gd_space* test, int strategy, gd_asm** out) {
  if (!trial || !test || !out) return fail(GD_ERR_ARG, "gd_assembler_create: null argument");
  if (strategy != GD_SUB_ASSEMBLED_ROWS && strategy != GD_FULLY_ASSEMBLED_ROWS)
    return fail(GD_ERR_ARG, "gd_assembler_create: unknown strategy");
  if (trial->model != test->model || trial->geom.k != test->geom.k)
    return fail(GD_ERR_UNSUPPORTED, "gd_assembler_create: trial and test must share model and order");
  for (int d = 0; d < 2 * kMaxDim; ++d)
    if (trial->geom.dsides[d] != test->geom.dsides[d])
      return fail(GD_ERR_UNSUPPORTED, "gd_assembler_create: trial and test must share Dirichlet sides");
  gd_asm* A = new gd_asm();
  A->trial = trial;
  A->test = test;
  A->strategy = strategy;
  *out = A;
  return GD_OK;
}

extern "C" int gd_assembler_destroy(gd_asm* A) {
  if (!A) return GD_OK;
  dfreeb(A->d_parts);
  dfreeb(A->rowptr);
  dfreeb(A->row_node);
  dfreeb(A->row_part);
  dfreeb(A->colidx);
  dfreeb(A->colgid);
  dfreeb(A->code);
  dfreeb(A->vals);
  dfreeb(A->rhs);
  dfreeb(A->grow_lid);
  dfreeb(A->gcol_lid);
  dfreeb(A->node_col);
  dfreeb(A->Khat);
  dfreeb(A->Mhat);
  dfreeb(A->Fhat);
  dfreeb(A->kappa_dev);
  dfreeb(A->f_dev);
  dfreeb(A->nbad);
  dfreeb(A->w);
  dfreeb(A->dred);
  dfreeb(A->dinv);
  A->sell.release();
  gd::qp_release(A->qp);
  A->qp = nullptr;
  dfreeb(A->gcol_gstart);
  dfreeb(A->gcol_gsize);
  dfreeb(A->row_pat);
  dfreeb(A->pat);
  dfreeb(A->w_cells);
  dfreeb(A->mx.f32);
  dfreeb(A->mx.f64);
  dfreeb(A->mx.red);
  dfreeb(A->mx.node_gid);
  dfreeb(A->mx.wf);
  dfreeb(A->mx.vals32);
  dfreeb(A->mx.zold);
  dfreeb(A->mx.lat);
  dfreeb(A->mx.latred);
  dfreeb(A->mx.plat);
  for (auto& gx : A->mx.fcg_graph) {
    if (gx) cudaGraphExecDestroy(gx);
    gx = nullptr;
  }
  for (int i = 0; i < 4; ++i)
    if (A->ev[i]) cudaEventDestroy(A->ev[i]);
  for (cudaEvent_t e : A->dl_events) cudaEventDestroy(e);
  if (A->dl_stream) cudaStreamDestroy(A->dl_stream);
  delete A;
  return GD_OK;
}

namespace gd {
int gcol_groups(gd_asm* A, const unsigned long long* ckey, const int32_t* rank, int64_t ncand);   // gd_vector.cu
int vector_expand(gd_asm* A);                                                                       // gd_vector.cu
}  // namespace gd

static int symbolic_impl(gd_asm* A) {
  gd_space* S = A->test;
  const Geom& g = S->geom;
  cudaStream_t st = S->model->ctx->stream;
  const int T = 256;
  const int64_t L = S->total_lids;
  const int64_t L1 = std::max<int64_t>(L, 1);
  A->parts = S->parts;
  A->ngdofs = S->ngdofs;
  GD_TRY(dalloc(A->d_parts, g.nparts));
  GD_CUDA_TRY(cudaMemcpyAsync(A->d_parts.p, A->parts.data(), sizeof(DevPart) * g.nparts, cudaMemcpyHostToDevice, st));

  DBuf<int32_t> flag;
  DBuf<int64_t> scan;
  GD_TRY(dalloc(flag, L1));
  GD_TRY(dalloc(scan, L + 1));
  std::vector<int64_t> bnd(g.nparts + 1);
  auto part_bounds = [&](const int64_t* dscan) -> int {
    for (int p = 0; p <= g.nparts; ++p) {
      int64_t at = p < g.nparts ? A->parts[p].lid_off : L;
      GD_CUDA_TRY(cudaMemcpyAsync(&bnd[p], dscan + at, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
    }
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    return GD_OK;
  };

  // 1. ghost rows
  int64_t total_grow = 0;
  if (A->strategy == GD_SUB_ASSEMBLED_ROWS && L > 0) {
    k_ghost_row_flag<<<nblk(L, T), T, 0, st>>>(g, A->d_parts.p, L, S->lid_node.p, S->lid_owner.p, flag.p);
    GD_TRY(launch_ok("k_ghost_row_flag"));
    GD_TRY(exclusive_scan_i32(flag.p, scan.p, L, st));
    GD_TRY(part_bounds(scan.p));
    for (int p = 0; p < g.nparts; ++p) {
      A->parts[p].grow_off = bnd[p];
      A->parts[p].n_grow = bnd[p + 1] - bnd[p];
    }
    total_grow = bnd[g.nparts];
    GD_TRY(dalloc(A->grow_lid, std::max<int64_t>(total_grow, 1)));
    k_ghost_row_fill<<<nblk(L, T), T, 0, st>>>(g, A->d_parts.p, L, flag.p, scan.p, A->grow_lid.p);
    GD_TRY(launch_ok("k_ghost_row_fill"));
  } else {
    for (int p = 0; p < g.nparts; ++p) {
      A->parts[p].grow_off = 0;
      A->parts[p].n_grow = 0;
    }
    GD_TRY(dalloc(A->grow_lid, 1));
  }
  A->nrows_total = A->ngdofs + total_grow;

  // 2. ghost columns
  DBuf<unsigned long long> key, ckey;
  DBuf<int32_t> clid, rank, lex2g;
  GD_TRY(dalloc(key, L1));
  GD_TRY(dalloc(lex2g, S->lex_to_gridap.size()));
  GD_CUDA_TRY(cudaMemcpyAsync(lex2g.p, S->lex_to_gridap.data(), sizeof(int) * S->lex_to_gridap.size(),
                              cudaMemcpyHostToDevice, st));
  if (L > 0) {
    k_ghost_col_key<<<nblk(L, T), T, 0, st>>>(g, A->d_parts.p, L, A->strategy, S->lid_node.p, S->lid_owner.p,
                                              lex2g.p, key.p, flag.p);
    GD_TRY(launch_ok("k_ghost_col_key"));
  }
  GD_TRY(exclusive_scan_i32(flag.p, scan.p, L, st));
  GD_TRY(part_bounds(scan.p));
  int64_t ncand = bnd[g.nparts];
  for (int p = 0; p < g.nparts; ++p) {
    A->parts[p].gcol_off = bnd[p];
    A->parts[p].n_gcol = bnd[p + 1] - bnd[p];
  }
  A->total_gcols = ncand;
  GD_CUDA_TRY(cudaMemcpyAsync(A->d_parts.p, A->parts.data(), sizeof(DevPart) * g.nparts, cudaMemcpyHostToDevice, st));
  GD_TRY(dalloc(ckey, std::max<int64_t>(ncand, 1)));
  GD_TRY(dalloc(clid, std::max<int64_t>(ncand, 1)));
  GD_TRY(dalloc(rank, std::max<int64_t>(ncand, 1)));
  GD_TRY(dalloc(A->gcol_lid, std::max<int64_t>(ncand, 1)));
  DBuf<int32_t> lid_col;
  GD_TRY(dalloc(lid_col, L1));
  if (L > 0) {
    k_compact_candidates<<<nblk(L, T), T, 0, st>>>(L, flag.p, scan.p, key.p, ckey.p, clid.p);
    GD_TRY(launch_ok("k_compact_candidates"));
    for (int p = 0; p < g.nparts; ++p) {
      int64_t n = A->parts[p].n_gcol;
      if (n == 0) continue;
      k_rank_candidates<<<nblk(n, T), T, 0, st>>>(A->parts[p].gcol_off, n, ckey.p, rank.p);
      GD_TRY(launch_ok("k_rank_candidates"));
    }
    k_assign_cols<<<nblk(L, T), T, 0, st>>>(g, A->d_parts.p, L, S->lid_owner.p, S->lid_ownidx.p, lid_col.p);
    GD_TRY(launch_ok("k_assign_cols"));
    if (ncand > 0) {
      k_assign_ghost_cols<<<nblk(ncand, T), T, 0, st>>>(g, A->d_parts.p, ncand, clid.p, rank.p, lid_col.p,
                                                        A->gcol_lid.p);
      GD_TRY(launch_ok("k_assign_ghost_cols"));
    }
  }
  // first-appearance groups of the ghost columns: the vector expansion and the
  // multi-field matrices (SubAssembledRows) order columns group by group
  if (S->ncomp > 1 || A->strategy == GD_SUB_ASSEMBLED_ROWS) GD_TRY(gcol_groups(A, ckey.p, rank.p, ncand));
  dfreeb(key);
  dfreeb(ckey);
  dfreeb(clid);
  dfreeb(rank);

  // 3. rows: owned rows in gid order, then ghost rows per part
  const int64_t R = A->nrows_total;
  DBuf<int32_t> own_lid, len;
  GD_TRY(dalloc(own_lid, std::max<int64_t>(A->ngdofs, 1)));
  GD_TRY(dalloc(len, std::max<int64_t>(R, 1)));
  GD_TRY(dalloc(A->row_node, std::max<int64_t>(R, 1)));
  GD_TRY(dalloc(A->row_part, std::max<int64_t>(R, 1)));
  GD_TRY(dalloc(A->rowptr, R + 1));
  if (L > 0) {
    k_own_lid<<<nblk(L, T), T, 0, st>>>(g, A->d_parts.p, L, S->lid_owner.p, S->lid_ownidx.p, own_lid.p);
    GD_TRY(launch_ok("k_own_lid"));
  }
  if (R > 0) {
    k_row_len<<<nblk(R, T), T, 0, st>>>(g, A->d_parts.p, A->ngdofs, R, own_lid.p, A->grow_lid.p, S->lid_node.p,
                                        len.p, A->row_node.p, A->row_part.p);
    GD_TRY(launch_ok("k_row_len"));
  }
  GD_TRY(exclusive_scan_i32(len.p, A->rowptr.p, R, st));
  int64_t nnz = 0, nnz_own = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&nnz, A->rowptr.p + R, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&nnz_own, A->rowptr.p + A->ngdofs, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  A->nnz_total = nnz;
  A->nnz_own = nnz_own;
  A->code_bytes = (2 * g.k + 1) * (2 * g.k + 1) * (g.dim == 3 ? (2 * g.k + 1) : 1) <= 256 ? 1 : 2;
  GD_TRY(dalloc(A->colidx, std::max<int64_t>(nnz, 1)));
  GD_TRY(dalloc(A->colgid, std::max<int64_t>(nnz, 1)));
  GD_TRY(dalloc(A->code, std::max<int64_t>(nnz, 1) * A->code_bytes));
  GD_TRY(dalloc(A->vals, std::max<int64_t>(nnz, 1)));
  GD_TRY(dalloc(A->rhs, std::max<int64_t>(R, 1)));
  DBuf<int32_t> err;
  GD_TRY(dalloc(err, 1));
  GD_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int32_t), st));
  if (R > 0) {
    if (A->code_bytes == 1)
      k_row_fill<uint8_t><<<nblk(R, 128), 128, 0, st>>>(g, A->d_parts.p, A->ngdofs, R, own_lid.p, A->grow_lid.p,
                                                          S->lid_node.p, S->node_lid.p, lid_col.p, S->lid_gid.p,
                                                          A->rowptr.p, A->colidx.p, A->colgid.p, A->code.p, err.p);
    else
      k_row_fill<uint16_t><<<nblk(R, 128), 128, 0, st>>>(g, A->d_parts.p, A->ngdofs, R, own_lid.p, A->grow_lid.p,
                                                           S->lid_node.p, S->node_lid.p, lid_col.p, S->lid_gid.p,
                                                           A->rowptr.p, A->colidx.p, A->colgid.p,
                                                           (uint16_t*)A->code.p, err.p);
    GD_TRY(launch_ok("k_row_fill"));
  }
  int32_t herr = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&herr, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (!herr) GD_TRY(build_q1_patterns(A, lid_col.p));
  dfreeb(err);
  dfreeb(own_lid);
  dfreeb(len);
  dfreeb(flag);
  dfreeb(scan);
  dfreeb(lid_col);
  dfreeb(lex2g);
  if (herr) return fail(GD_ERR_STATE, "symbolic: a stencil column has no local column id (code " + std::to_string(herr) + ")");
  GD_CUDA_TRY(cudaMemcpyAsync(A->d_parts.p, A->parts.data(), sizeof(DevPart) * g.nparts, cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaMemsetAsync(A->vals.p, 0, sizeof(double) * std::max<int64_t>(nnz, 1), st));
  GD_CUDA_TRY(cudaMemsetAsync(A->rhs.p, 0, sizeof(double) * std::max<int64_t>(R, 1), st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (S->ncomp > 1) GD_TRY(vector_expand(A));
  A->symbolic_done = true;
  return GD_OK;
}

extern "C" int gd_assemble_symbolic(gd_asm* A) {
  if (!A) return fail(GD_ERR_ARG, "gd_assemble_symbolic: null assembler");
  return symbolic_impl(A);
}

// ---- exports ---------------------------------------------------------------------------
extern "C" int gd_matrix_sizes(const gd_asm* A, int part, int64_t* nrows, int64_t* ncols, int64_t* nnz,
                               int64_t* n_ghost_rows, int64_t* n_ghost_cols) {
  if (!A) return fail(GD_ERR_ARG, "gd_matrix_sizes: null assembler");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_matrix_sizes: run gd_assemble_symbolic first");
  if (part < 0 || part >= (int)A->parts.size()) return fail(GD_ERR_ARG, "gd_matrix_sizes: bad part");
  const DevPart& P = A->parts[part];
  cudaStream_t st = A->test->model->ctx->stream;
  int64_t b[4];
  GD_CUDA_TRY(cudaMemcpyAsync(&b[0], A->rowptr.p + P.first_gdof, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[1], A->rowptr.p + P.first_gdof + P.n_own, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[2], A->rowptr.p + A->ngdofs + P.grow_off, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[3], A->rowptr.p + A->ngdofs + P.grow_off + P.n_grow, sizeof(int64_t),
                              cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (nrows) *nrows = P.n_own + P.n_grow;
  if (ncols) *ncols = P.n_own + P.n_gcol;
  if (nnz) *nnz = (b[1] - b[0]) + (b[3] - b[2]);
  if (n_ghost_rows) *n_ghost_rows = P.n_grow;
  if (n_ghost_cols) *n_ghost_cols = P.n_gcol;
  return GD_OK;
}

extern "C" int gd_matrix_export(const gd_asm* A, int part, int64_t* rowptr, int32_t* colidx, double* vals,
                                int64_t* ghost_row_gids, int32_t* ghost_row_owners, int64_t* ghost_col_gids,
                                int32_t* ghost_col_owners) {
  if (!A) return fail(GD_ERR_ARG, "gd_matrix_export: null assembler");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_matrix_export: run gd_assemble_symbolic first");
  if (part < 0 || part >= (int)A->parts.size()) return fail(GD_ERR_ARG, "gd_matrix_export: bad part");
  const DevPart& P = A->parts[part];
  const gd_space* S = A->test;
  cudaStream_t st = S->model->ctx->stream;
  std::vector<int64_t> rp_own(P.n_own + 1), rp_gh(P.n_grow + 1);
  GD_CUDA_TRY(cudaMemcpyAsync(rp_own.data(), A->rowptr.p + P.first_gdof, sizeof(int64_t) * (P.n_own + 1),
                              cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(rp_gh.data(), A->rowptr.p + A->ngdofs + P.grow_off, sizeof(int64_t) * (P.n_grow + 1),
                              cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  int64_t n1 = rp_own[P.n_own] - rp_own[0], n2 = rp_gh[P.n_grow] - rp_gh[0];
  if (rowptr) {
    for (int64_t i = 0; i <= P.n_own; ++i) rowptr[i] = rp_own[i] - rp_own[0];
    for (int64_t i = 1; i <= P.n_grow; ++i) rowptr[P.n_own + i] = n1 + rp_gh[i] - rp_gh[0];
  }
  if (colidx) {
    if (n1) GD_CUDA_TRY(cudaMemcpyAsync(colidx, A->colidx.p + rp_own[0], sizeof(int32_t) * n1, cudaMemcpyDeviceToHost, st));
    if (n2) GD_CUDA_TRY(cudaMemcpyAsync(colidx + n1, A->colidx.p + rp_gh[0], sizeof(int32_t) * n2, cudaMemcpyDeviceToHost, st));
  }
  if (vals) {
    if (n1) GD_CUDA_TRY(cudaMemcpyAsync(vals, A->vals.p + rp_own[0], sizeof(double) * n1, cudaMemcpyDeviceToHost, st));
    if (n2) GD_CUDA_TRY(cudaMemcpyAsync(vals + n1, A->vals.p + rp_gh[0], sizeof(double) * n2, cudaMemcpyDeviceToHost, st));
  }
  if (ghost_row_gids || ghost_row_owners || ghost_col_gids || ghost_col_owners) {
    std::vector<int64_t> gid(P.nfree);
    std::vector<int32_t> own(P.nfree), grl(P.n_grow), gcl(P.n_gcol);
    if (P.nfree) {
      GD_CUDA_TRY(cudaMemcpyAsync(gid.data(), S->lid_gid.p + P.lid_off, sizeof(int64_t) * P.nfree, cudaMemcpyDeviceToHost, st));
      GD_CUDA_TRY(cudaMemcpyAsync(own.data(), S->lid_owner.p + P.lid_off, sizeof(int32_t) * P.nfree, cudaMemcpyDeviceToHost, st));
    }
    if (P.n_grow)
      GD_CUDA_TRY(cudaMemcpyAsync(grl.data(), A->grow_lid.p + P.grow_off, sizeof(int32_t) * P.n_grow, cudaMemcpyDeviceToHost, st));
    if (P.n_gcol)
      GD_CUDA_TRY(cudaMemcpyAsync(gcl.data(), A->gcol_lid.p + P.gcol_off, sizeof(int32_t) * P.n_gcol, cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaStreamSynchronize(st));
    // ghost row / column lids are vector lids (bs * node lid + component) for bs > 1
    const int bs = A->bs;
    for (int64_t i = 0; i < P.n_grow; ++i) {
      if (ghost_row_gids) ghost_row_gids[i] = bs * gid[grl[i] / bs] + grl[i] % bs;
      if (ghost_row_owners) ghost_row_owners[i] = own[grl[i] / bs];
    }
    for (int64_t i = 0; i < P.n_gcol; ++i) {
      if (ghost_col_gids) ghost_col_gids[i] = bs * gid[gcl[i] / bs] + gcl[i] % bs;
      if (ghost_col_owners) ghost_col_owners[i] = own[gcl[i] / bs];
    }
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

extern "C" int gd_vector_export(const gd_asm* A, int part, double* b) {
  if (!A) return fail(GD_ERR_ARG, "gd_vector_export: null assembler");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_vector_export: run gd_assemble_symbolic first");
  if (part < 0 || part >= (int)A->parts.size() || !b) return fail(GD_ERR_ARG, "gd_vector_export: bad argument");
  const DevPart& P = A->parts[part];
  cudaStream_t st = A->test->model->ctx->stream;
  if (P.n_own)
    GD_CUDA_TRY(cudaMemcpyAsync(b, A->rhs.p + P.first_gdof, sizeof(double) * P.n_own, cudaMemcpyDeviceToHost, st));
  if (P.n_grow)
    GD_CUDA_TRY(cudaMemcpyAsync(b + P.n_own, A->rhs.p + A->ngdofs + P.grow_off, sizeof(double) * P.n_grow,
                                cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

extern "C" int gd_system_device_ptrs(const gd_asm* A, const int64_t** rowptr, const int32_t** colidx,
                                     const double** vals, const double** rhs, int64_t* ngdofs) {
  if (!A) return fail(GD_ERR_ARG, "gd_system_device_ptrs: null assembler");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_system_device_ptrs: run gd_assemble_symbolic first");
  if (rowptr) *rowptr = A->rowptr.p;
  if (colidx) *colidx = A->colgid.p;
  if (vals) *vals = A->vals.p;
  if (rhs) *rhs = A->rhs.p;
  if (ngdofs) *ngdofs = A->ngdofs;
  return GD_OK;
}

extern "C" int gd_system_download(const gd_asm* A, double* rhs, double* owned_vals) {
  if (!A) return fail(GD_ERR_ARG, "gd_system_download: null assembler");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_system_download: run gd_assemble_symbolic first");
  cudaStream_t st = A->test->model->ctx->stream;
  if (rhs && A->ngdofs)
    GD_CUDA_TRY(cudaMemcpyAsync(rhs, A->rhs.p, sizeof(double) * A->ngdofs, cudaMemcpyDeviceToHost, st));
  if (owned_vals && A->nnz_own)
    GD_CUDA_TRY(cudaMemcpyAsync(owned_vals, A->vals.p, sizeof(double) * A->nnz_own, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}
