// A1 Cartesian partition, A3 local Q_k numbering, A4 generate_gids -- on the device.
//
// Every part's owned+ghost box is a slab of the concatenated per-node arrays.  The
// Gridap numbering of a part (vertices, edges, faces, cells; higher faces at their
// first appearance in cell order) has a closed form on a Cartesian box, evaluated
// per node; a device scan then splits free and Dirichlet DOFs.  generate_gids
// (FESpaces.jl:139-261) becomes: owner = max owner rank of the cells around the
// node (closed form), a scan of the owned flags in local DOF order, and a gather
// of the owner's owned index.
#include <algorithm>
#include <array>
#include <cstring>
#include <cmath>
#include <string>

#include "gd_internal.h"

namespace gd {

// ------------------------------------------------------------------------------
// Closed-form Gridap DOF position on a local box of m cells (scalar DOFs).
// ------------------------------------------------------------------------------
__host__ __device__ inline int64_t cnt_edges(int dim, int zx, int zy, int zz) {
  if (dim == 2) return (1 + zy) + (1 + zx);
  return (int64_t)(1 + zy) * (1 + zz) + (int64_t)(1 + zx) * (1 + zz) + (int64_t)(1 + zx) * (1 + zy);
}
__host__ __device__ inline int64_t cnt_faces(int zx, int zy, int zz) {
  return (1 + zz) + (1 + zy) + (1 + zx);
}
// Number of faces of the given kind (0 edges, 1 faces) first seen in the cells
// strictly before cell c in lexicographic order.
__host__ __device__ inline int64_t faces_before(int kind, int dim, const int64_t* m, const int64_t* c) {
  auto g = [&](int zx, int zy, int zz) -> int64_t {
    return kind == 0 ? cnt_edges(dim, zx, zy, zz) : cnt_faces(zx, zy, zz);
  };
  auto row = [&](int64_t X, int zy, int zz) -> int64_t {
    return X >= 1 ? g(1, zy, zz) + (X - 1) * g(0, zy, zz) : 0;
  };
  if (dim == 2) {
    int64_t s = c[1] >= 1 ? row(m[0], 1, 0) + (c[1] - 1) * row(m[0], 0, 0) : 0;
    return s + row(c[0], c[1] == 0, 0);
  }
  auto slab = [&](int64_t Y, int zz) -> int64_t {
    return Y >= 1 ? row(m[0], 1, zz) + (Y - 1) * row(m[0], 0, zz) : 0;
  };
  int64_t s = c[2] >= 1 ? slab(m[1], 1) + (c[2] - 1) * slab(m[1], 0) : 0;
  return s + slab(c[1], c[2] == 0) + row(c[0], c[1] == 0, c[2] == 0);
}

__host__ __device__ inline bool edge_is_new(int dim, int l, const int* z) {
  // decode local edge l -> (a, offsets) and test (b_e==1 || z_e) for e != a
  if (dim == 2) {
    int a = l >> 1, b = l & 1;
    int e = 1 - a;
    return b == 1 || z[e];
  }
  int a = l >> 2, b0 = l & 1, b1 = (l >> 1) & 1;
  int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
  return (b0 == 1 || z[o0]) && (b1 == 1 || z[o1]);
}

__host__ __device__ inline int64_t gridap_dof_pos(int dim, int k, const int64_t* m, const int64_t* Y) {
  int64_t q[kMaxDim] = {0, 0, 0}, r[kMaxDim] = {0, 0, 0};
  int nz = 0, a_nz = -1, b_zero = -1;
  for (int d = 0; d < dim; ++d) {
    q[d] = Y[d] / k;
    r[d] = Y[d] % k;
    if (r[d] != 0) {
      ++nz;
      a_nz = d;
    } else {
      b_zero = d;
    }
  }
  int64_t V = 1;
  for (int d = 0; d < dim; ++d) V *= (m[d] + 1);
  if (nz == 0) {
    int64_t v = 0;
    for (int d = dim - 1; d >= 0; --d) v = v * (m[d] + 1) + q[d];
    return v;
  }
  int64_t endc[kMaxDim] = {0, 0, 0};
  endc[dim - 1] = m[dim - 1];
  const int64_t E = faces_before(0, dim, m, endc);
  const int64_t F = dim == 3 ? faces_before(1, dim, m, endc) : 0;
  const int64_t k1 = k - 1;
  if (nz == 1) {  // edge along a_nz starting at vertex q
    int a = a_nz;
    int64_t c[kMaxDim] = {0, 0, 0};
    int b[kMaxDim] = {0, 0, 0};
    for (int e = 0; e < dim; ++e) {
      if (e == a) {
        c[e] = q[e];
      } else {
        c[e] = q[e] - 1 > 0 ? q[e] - 1 : 0;
        b[e] = (int)(q[e] - c[e]);
      }
    }
    int z[kMaxDim] = {0, 0, 0};
    for (int e = 0; e < dim; ++e) z[e] = c[e] == 0;
    int l;
    if (dim == 2) {
      l = a == 0 ? b[1] : 2 + b[0];
    } else {
      int o0 = a == 0 ? 1 : 0, o1 = a == 2 ? 1 : 2;
      l = 4 * a + b[o0] + 2 * b[o1];
    }
    int cnt = 0;
    for (int ll = 0; ll < l; ++ll) cnt += edge_is_new(dim, ll, z);
    int64_t eid = faces_before(0, dim, m, c) + cnt;
    return V + eid * k1 + (r[a] - 1);
  }
  if (dim == 3 && nz == 2) {  // face with normal b_zero
    int bn = b_zero;
    int64_t c[kMaxDim] = {q[0], q[1], q[2]};
    c[bn] = q[bn] - 1 > 0 ? q[bn] - 1 : 0;
    int bb = (int)(q[bn] - c[bn]);
    int z[kMaxDim] = {c[0] == 0, c[1] == 0, c[2] == 0};
    int l = 2 * (2 - bn) + bb;
    int cnt = 0;
    for (int ll = 0; ll < l; ++ll) {
      int nb = 2 - (ll >> 1), o = ll & 1;
      cnt += (o == 1 || z[nb]);
    }
    int64_t fid = faces_before(1, 3, m, c) + cnt;
    int a1 = bn == 0 ? 1 : 0, a2 = bn == 2 ? 1 : 2;
    int64_t own = (r[a1] - 1) + k1 * (r[a2] - 1);
    return V + E * k1 + fid * k1 * k1 + own;
  }
  // cell interior
  int64_t cl = 0, own = 0, kd = 1;
  for (int d = dim - 1; d >= 0; --d) {
    cl = cl * m[d] + q[d];
    own = own * k1 + (r[d] - 1);
    kd *= k1;
  }
  return V + E * k1 + F * k1 * k1 + cl * kd + own;
}

__device__ inline int find_part_by(const DevPart* parts, int nparts, int64_t t, int which) {
  int lo = 0, hi = nparts - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    int64_t off = which == 0 ? parts[mid].node_off : parts[mid].lid_off;
    if (off <= t) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ inline void box_coords(const DevPart& P, int dim, int64_t li, int64_t* Yl) {
  for (int d = 0; d < dim; ++d) {
    Yl[d] = li % P.nb[d];
    li /= P.nb[d];
  }
}

// ---- kernels ------------------------------------------------------------------
__global__ void k_node_pos(Geom g, const DevPart* __restrict__ parts, int64_t total_nodes,
                           int32_t* __restrict__ node_pos, int32_t* __restrict__ posflag) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_nodes) return;
  int p = find_part_by(parts, g.nparts, t, 0);
  const DevPart& P = parts[p];
  int64_t li = t - P.node_off;
  int64_t Yl[kMaxDim] = {0, 0, 0}, X[kMaxDim] = {0, 0, 0}, m[kMaxDim] = {1, 1, 1};
  box_coords(P, g.dim, li, Yl);
  for (int d = 0; d < g.dim; ++d) {
    X[d] = g.k * P.loc_lo[d] + Yl[d];
    m[d] = P.loc_hi[d] - P.loc_lo[d];
  }
  int64_t pos = gridap_dof_pos(g.dim, g.k, m, Yl);
  node_pos[t] = (int32_t)pos;
  posflag[P.node_off + pos] = node_is_dirichlet(g, X) ? 0 : 1;
}

// Gridap's local node order of one Q_k cell (vertices, edges, faces, interior): for
// local dof a, its lattice offsets (pos[3a + d] in [0, k]).
void cell_dof_positions(int dim, int k, std::vector<int>& pos) {
  int nn = 1;
  for (int d = 0; d < dim; ++d) nn *= k + 1;
  pos.assign(3 * nn, 0);
  const int64_t m[kMaxDim] = {1, 1, 1};
  for (int t = 0; t < nn; ++t) {
    int64_t Y[kMaxDim] = {0, 0, 0};
    for (int d = 0, r = t; d < dim; ++d) {
      Y[d] = r % (k + 1);
      r /= k + 1;
    }
    const int64_t a = gridap_dof_pos(dim, k, m, Y);
    for (int d = 0; d < dim; ++d) pos[3 * a + d] = (int)Y[d];
  }
}

__global__ void k_node_lid(Geom g, const DevPart* __restrict__ parts, int64_t total_nodes,
                           const int32_t* __restrict__ node_pos, const int32_t* __restrict__ posflag,
                           const int64_t* __restrict__ pscan, int32_t* __restrict__ node_lid,
                           int32_t* __restrict__ lid_node) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_nodes) return;
  int p = find_part_by(parts, g.nparts, t, 0);
  const DevPart& P = parts[p];
  int64_t pos = node_pos[t];
  int64_t before = pscan[P.node_off + pos] - pscan[P.node_off];
  if (posflag[P.node_off + pos]) {
    node_lid[t] = (int32_t)before;
    lid_node[P.lid_off + before] = (int32_t)(t - P.node_off);
  } else {
    node_lid[t] = (int32_t)(-(pos - before) - 1);
  }
}

__global__ void k_lid_owner(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                            const int32_t* __restrict__ lid_node, int32_t* __restrict__ lid_owner,
                            int32_t* __restrict__ ownflag) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int p = find_part_by(parts, g.nparts, t, 1);
  const DevPart& P = parts[p];
  int64_t Yl[kMaxDim] = {0, 0, 0}, X[kMaxDim] = {0, 0, 0};
  box_coords(P, g.dim, lid_node[t], Yl);
  for (int d = 0; d < g.dim; ++d) X[d] = g.k * P.loc_lo[d] + Yl[d];
  int o = node_owner(g, X);
  lid_owner[t] = o;
  ownflag[t] = o == p;
}

__global__ void k_lid_gid(Geom g, const DevPart* __restrict__ parts, int64_t total_lids,
                          const int32_t* __restrict__ lid_node, const int32_t* __restrict__ lid_owner,
                          const int64_t* __restrict__ oscan, const int32_t* __restrict__ node_lid,
                          int32_t* __restrict__ lid_ownidx, int64_t* __restrict__ lid_gid,
                          int32_t* __restrict__ err) {
  int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total_lids) return;
  int p = find_part_by(parts, g.nparts, t, 1);
  const DevPart& P = parts[p];
  lid_ownidx[t] = (int32_t)(oscan[t] - oscan[P.lid_off]);
  int q = lid_owner[t];
  const DevPart& Q = parts[q];
  int64_t Yl[kMaxDim] = {0, 0, 0}, X[kMaxDim] = {0, 0, 0};
  box_coords(P, g.dim, lid_node[t], Yl);
  int64_t qi = 0;
  bool inside = true;
  for (int d = g.dim - 1; d >= 0; --d) {
    X[d] = g.k * P.loc_lo[d] + Yl[d];
    int64_t y = X[d] - g.k * Q.loc_lo[d];
    if (y < 0 || y >= Q.nb[d]) inside = false;
    qi = qi * Q.nb[d] + y;
  }
  int32_t lq = inside ? node_lid[Q.node_off + qi] : -1;
  if (lq < 0) {
    atomicExch(err, 1);
    lid_gid[t] = -1;
    return;
  }
  int64_t own_q = oscan[Q.lid_off + lq] - oscan[Q.lid_off];
  lid_gid[t] = Q.first_gdof + own_q;
}

// Gridap cell-local node order (vertices, edge interiors, face interiors, cell
// interior) for the lexicographic local node offsets of a Q_k cell.
std::vector<int> lex_to_gridap_table(int dim, int k) {
  std::vector<std::array<int, 3>> nodes;
  int nv = 1 << dim;
  auto vert = [&](int v, int d) { return (v >> d) & 1; };
  for (int v = 0; v < nv; ++v) nodes.push_back({k * vert(v, 0), k * vert(v, 1), dim == 3 ? k * vert(v, 2) : 0});
  static const int qe[4][2] = {{0, 1}, {2, 3}, {0, 2}, {1, 3}};
  static const int he[12][2] = {{0, 1}, {2, 3}, {4, 5}, {6, 7}, {0, 2}, {1, 3},
                                {4, 6}, {5, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
  static const int hf[6][3] = {{0, 1, 2}, {4, 5, 6}, {0, 1, 4}, {2, 3, 6}, {0, 2, 4}, {1, 3, 5}};
  int ne = dim == 2 ? 4 : 12;
  for (int e = 0; e < ne; ++e) {
    int a = dim == 2 ? qe[e][0] : he[e][0], b = dim == 2 ? qe[e][1] : he[e][1];
    for (int t = 1; t < k; ++t) {
      std::array<int, 3> x{0, 0, 0};
      for (int d = 0; d < dim; ++d) x[d] = k * vert(a, d) + t * (vert(b, d) - vert(a, d));
      nodes.push_back(x);
    }
  }
  if (dim == 3) {
    for (int f = 0; f < 6; ++f) {
      int a = hf[f][0], b = hf[f][1], c = hf[f][2];
      for (int t = 1; t < k; ++t)
        for (int s = 1; s < k; ++s) {
          std::array<int, 3> x{0, 0, 0};
          for (int d = 0; d < 3; ++d)
            x[d] = k * vert(a, d) + s * (vert(b, d) - vert(a, d)) + t * (vert(c, d) - vert(a, d));
          nodes.push_back(x);
        }
    }
  }
  if (dim == 2) {
    for (int j = 1; j < k; ++j)
      for (int i = 1; i < k; ++i) nodes.push_back({i, j, 0});
  } else {
    for (int l = 1; l < k; ++l)
      for (int j = 1; j < k; ++j)
        for (int i = 1; i < k; ++i) nodes.push_back({i, j, l});
  }
  int nn = 1;
  for (int d = 0; d < dim; ++d) nn *= (k + 1);
  std::vector<int> table(nn, -1);
  for (int gi = 0; gi < (int)nodes.size(); ++gi) {
    int lex = 0;
    for (int d = dim - 1; d >= 0; --d) lex = lex * (k + 1) + nodes[gi][d];
    table[lex] = gi;
  }
  return table;
}

static int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return GD_OK;
}

static inline unsigned nblocks(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace gd

using namespace gd;

// ---------------------------------------------------------------------------------
// C ABI: model
// ---------------------------------------------------------------------------------
extern "C" int gd_model_cartesian(gd_ctx* ctx, int dim, const int64_t* cells, const int32_t* parts,
                                  const double* domain, gd_model** out) {
  if (!ctx || !cells || !parts || !domain || !out) return fail(GD_ERR_ARG, "gd_model_cartesian: null argument");
  if (dim != 2 && dim != 3) return fail(GD_ERR_ARG, "gd_model_cartesian: dim must be 2 or 3");
  gd_model* M = new gd_model();
  M->ctx = ctx;
  Geom& g = M->geom;
  g.dim = dim;
  g.k = 1;
  g.nparts = 1;
  for (int d = 0; d < kMaxDim; ++d) {
    g.np[d] = 1;
    g.n[d] = 1;
  }
  for (int d = 0; d < dim; ++d) {
    if (parts[d] < 1 || cells[d] < 1 || cells[d] < parts[d]) {
      delete M;
      return fail(GD_ERR_ARG, "gd_model_cartesian: need cells[d] >= parts[d] >= 1 in every direction");
    }
    if (!(domain[2 * d + 1] > domain[2 * d])) {
      delete M;
      return fail(GD_ERR_ARG, "gd_model_cartesian: empty domain interval");
    }
    g.np[d] = parts[d];
    g.n[d] = cells[d];
    g.nparts *= parts[d];
    g.bl[d] = cells[d] / parts[d];
    g.brem[d] = cells[d] % parts[d];
    g.x0[d] = domain[2 * d];
    g.h[d] = (domain[2 * d + 1] - domain[2 * d]) / (double)cells[d];
    g.N[d] = cells[d] + 1;
    M->domain[2 * d] = domain[2 * d];
    M->domain[2 * d + 1] = domain[2 * d + 1];
  }
  if (g.nparts > 65536) {
    delete M;
    return fail(GD_ERR_ARG, "gd_model_cartesian: too many parts");
  }
  M->parts.resize(g.nparts);
  for (int p = 0; p < g.nparts; ++p) {
    DevPart& P = M->parts[p];
    memset(&P, 0, sizeof(P));
    int pc[kMaxDim] = {0, 0, 0};
    int rest = p;
    for (int d = 0; d < dim; ++d) {
      pc[d] = rest % g.np[d];
      rest /= g.np[d];
    }
    for (int d = 0; d < kMaxDim; ++d) {
      P.own_lo[d] = 0; P.own_hi[d] = 1; P.loc_lo[d] = 0; P.loc_hi[d] = 1;
    }
    for (int d = 0; d < dim; ++d) {
      // _local_range (PArraysExtras.jl:72-84), converted to 0-based [lo, hi)
      int64_t l = g.n[d] / g.np[d], rem = g.n[d] % g.np[d];
      int64_t p1 = pc[d] + 1;
      int64_t offset = l * (p1 - 1);
      if (rem >= (g.np[d] - p1 + 1)) {
        l += 1;
        offset += p1 - (g.np[d] - rem) - 1;
      }
      P.own_lo[d] = offset;
      P.own_hi[d] = offset + l;
      P.loc_lo[d] = std::max<int64_t>(0, offset - 1);
      P.loc_hi[d] = std::min<int64_t>(g.n[d], offset + l + 1);
    }
  }
  *out = M;
  return GD_OK;
}

extern "C" int gd_model_destroy(gd_model* m) {
  delete m;
  return GD_OK;
}

extern "C" int gd_model_num_parts(const gd_model* m, int32_t* nparts) {
  if (!m || !nparts) return fail(GD_ERR_ARG, "gd_model_num_parts: null argument");
  *nparts = m->geom.nparts;
  return GD_OK;
}

extern "C" int gd_model_part_boxes(const gd_model* m, int part, int64_t* own_lo, int64_t* own_hi,
                                   int64_t* loc_lo, int64_t* loc_hi) {
  if (!m || part < 0 || part >= m->geom.nparts) return fail(GD_ERR_ARG, "gd_model_part_boxes: bad part");
  const DevPart& P = m->parts[part];
  for (int d = 0; d < m->geom.dim; ++d) {
    if (own_lo) own_lo[d] = P.own_lo[d];
    if (own_hi) own_hi[d] = P.own_hi[d];
    if (loc_lo) loc_lo[d] = P.loc_lo[d];
    if (loc_hi) loc_hi[d] = P.loc_hi[d];
  }
  return GD_OK;
}

// ---------------------------------------------------------------------------------
// C ABI: FE space
// ---------------------------------------------------------------------------------
static int space_build(gd_space* S) {
  Geom& g = S->geom;
  cudaStream_t st = S->model->ctx->stream;
  const int T = 256;
  // part layout of the concatenated node arrays
  int64_t noff = 0, coff = 0;
  for (int p = 0; p < g.nparts; ++p) {
    DevPart& P = S->parts[p];
    P.nnodes = 1;
    P.nlcells = 1;
    for (int d = 0; d < kMaxDim; ++d) P.nb[d] = 1;
    for (int d = 0; d < g.dim; ++d) {
      P.nb[d] = g.k * (P.loc_hi[d] - P.loc_lo[d]) + 1;
      P.nnodes *= P.nb[d];
      P.nlcells *= (P.loc_hi[d] - P.loc_lo[d]);
    }
    P.node_off = noff;
    P.lcell_off = coff;
    noff += P.nnodes;
    coff += P.nlcells;
  }
  S->total_nodes = noff;
  if (noff >= ((int64_t)1 << 31)) return fail(GD_ERR_UNSUPPORTED, "gd_space_create: local node boxes exceed 2^31 nodes");
  GD_TRY(dalloc(S->d_parts, g.nparts));
  GD_CUDA_TRY(cudaMemcpyAsync(S->d_parts.p, S->parts.data(), sizeof(DevPart) * g.nparts, cudaMemcpyHostToDevice, st));

  DBuf<int32_t> node_pos, posflag;
  DBuf<int64_t> pscan;
  GD_TRY(dalloc(node_pos, noff));
  GD_TRY(dalloc(posflag, noff));
  GD_TRY(dalloc(pscan, noff + 1));
  k_node_pos<<<nblocks(noff, T), T, 0, st>>>(g, S->d_parts.p, noff, node_pos.p, posflag.p);
  GD_TRY(launch_check("k_node_pos"));
  GD_TRY(exclusive_scan_i32(posflag.p, pscan.p, noff, st));
  // free dofs per part from the scan at the part boundaries
  std::vector<int64_t> bnd(g.nparts + 1);
  for (int p = 0; p <= g.nparts; ++p) {
    int64_t at = p < g.nparts ? S->parts[p].node_off : noff;
    GD_CUDA_TRY(cudaMemcpyAsync(&bnd[p], pscan.p + at, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  int64_t loff = 0;
  for (int p = 0; p < g.nparts; ++p) {
    S->parts[p].nfree = bnd[p + 1] - bnd[p];
    S->parts[p].lid_off = loff;
    loff += S->parts[p].nfree;
  }
  S->total_lids = loff;
  GD_CUDA_TRY(cudaMemcpyAsync(S->d_parts.p, S->parts.data(), sizeof(DevPart) * g.nparts, cudaMemcpyHostToDevice, st));
  GD_TRY(dalloc(S->node_lid, noff));
  GD_TRY(dalloc(S->lid_node, std::max<int64_t>(loff, 1)));
  k_node_lid<<<nblocks(noff, T), T, 0, st>>>(g, S->d_parts.p, noff, node_pos.p, posflag.p, pscan.p,
                                             S->node_lid.p, S->lid_node.p);
  GD_TRY(launch_check("k_node_lid"));
  dfreeb(node_pos);
  dfreeb(posflag);
  dfreeb(pscan);

  // owners, owned flags and their scan in local DOF order
  DBuf<int32_t> ownflag;
  DBuf<int64_t> oscan;
  GD_TRY(dalloc(S->lid_owner, std::max<int64_t>(loff, 1)));
  GD_TRY(dalloc(S->lid_ownidx, std::max<int64_t>(loff, 1)));
  GD_TRY(dalloc(S->lid_gid, std::max<int64_t>(loff, 1)));
  GD_TRY(dalloc(ownflag, std::max<int64_t>(loff, 1)));
  GD_TRY(dalloc(oscan, loff + 1));
  if (loff > 0) {
    k_lid_owner<<<nblocks(loff, T), T, 0, st>>>(g, S->d_parts.p, loff, S->lid_node.p, S->lid_owner.p, ownflag.p);
    GD_TRY(launch_check("k_lid_owner"));
  }
  GD_TRY(exclusive_scan_i32(ownflag.p, oscan.p, loff, st));
  for (int p = 0; p <= g.nparts; ++p) {
    int64_t at = p < g.nparts ? S->parts[p].lid_off : loff;
    GD_CUDA_TRY(cudaMemcpyAsync(&bnd[p], oscan.p + at, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  int64_t first = 0;   // scan(+, nodofs, type=:exclusive) (FESpaces.jl:186)
  for (int p = 0; p < g.nparts; ++p) {
    S->parts[p].n_own = bnd[p + 1] - bnd[p];
    S->parts[p].first_gdof = first;
    first += S->parts[p].n_own;
  }
  S->ngdofs = first;   // reduction(+, nodofs) (FESpaces.jl:248)
  if (S->ngdofs >= ((int64_t)1 << 31)) return fail(GD_ERR_UNSUPPORTED, "gd_space_create: more than 2^31 global DOFs");
  GD_CUDA_TRY(cudaMemcpyAsync(S->d_parts.p, S->parts.data(), sizeof(DevPart) * g.nparts, cudaMemcpyHostToDevice, st));
  DBuf<int32_t> err;
  GD_TRY(dalloc(err, 1));
  GD_CUDA_TRY(cudaMemsetAsync(err.p, 0, sizeof(int32_t), st));
  if (loff > 0) {
    k_lid_gid<<<nblocks(loff, T), T, 0, st>>>(g, S->d_parts.p, loff, S->lid_node.p, S->lid_owner.p, oscan.p,
                                              S->node_lid.p, S->lid_ownidx.p, S->lid_gid.p, err.p);
    GD_TRY(launch_check("k_lid_gid"));
  }
  int32_t herr = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&herr, err.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  dfreeb(err);
  dfreeb(ownflag);
  dfreeb(oscan);
  if (herr) return fail(GD_ERR_STATE, "generate_gids: a DOF's owner does not hold it as a free DOF");
  S->lex_to_gridap = lex_to_gridap_table(g.dim, g.k);
  return GD_OK;
}

extern "C" int gd_space_create(gd_model* model, int order, int ncomp, const int32_t* dirichlet_sides,
                               gd_space** out) {
  if (!model || !out) return fail(GD_ERR_ARG, "gd_space_create: null argument");
  if (order < 1 || order > kMaxOrder) return fail(GD_ERR_UNSUPPORTED, "gd_space_create: order must be 1..3");
  if (ncomp != 1 && !(ncomp == model->geom.dim && order <= 2))
    return fail(GD_ERR_UNSUPPORTED, "gd_space_create: ncomp must be 1, or the dimension for orders 1 and 2");
  gd_space* S = new gd_space();
  S->model = model;
  S->geom = model->geom;
  S->ncomp = ncomp;
  Geom& g = S->geom;
  g.k = order;
  for (int d = 0; d < 2 * kMaxDim; ++d) g.dsides[d] = 0;
  for (int d = 0; d < g.dim; ++d) {
    g.N[d] = (int64_t)order * g.n[d] + 1;
    g.dsides[2 * d] = dirichlet_sides ? (dirichlet_sides[2 * d] != 0) : 1;
    g.dsides[2 * d + 1] = dirichlet_sides ? (dirichlet_sides[2 * d + 1] != 0) : 1;
  }
  for (int d = g.dim; d < kMaxDim; ++d) g.N[d] = 1;
  S->parts = model->parts;
  int st = space_build(S);
  if (st != GD_OK) {
    std::string msg = gd_last_error();
    gd_space_destroy(S);
    return fail(st, msg);
  }
  *out = S;
  return GD_OK;
}

extern "C" int gd_space_destroy(gd_space* S) {
  if (!S) return GD_OK;
  dfreeb(S->d_parts);
  dfreeb(S->node_lid);
  dfreeb(S->lid_node);
  dfreeb(S->lid_owner);
  dfreeb(S->lid_ownidx);
  dfreeb(S->lid_gid);
  dfreeb(S->u_dir);
  dfreeb(S->lat_gid);
  delete S;
  return GD_OK;
}

// The space keeps node-based arrays; a vector space (ncomp = bs > 1, orders 1 and 2)
// exposes dof = bs * node dof + component for local ids, gids and owners alike.
extern "C" int gd_space_num_free_dofs(const gd_space* S, int64_t* n) {
  if (!S || !n) return fail(GD_ERR_ARG, "gd_space_num_free_dofs: null argument");
  *n = S->ngdofs * S->ncomp;
  return GD_OK;
}

extern "C" int gd_space_local_sizes(const gd_space* S, int part, int64_t* nldofs, int64_t* nown,
                                    int64_t* first_gdof) {
  if (!S || part < 0 || part >= S->geom.nparts) return fail(GD_ERR_ARG, "gd_space_local_sizes: bad part");
  const DevPart& P = S->parts[part];
  if (nldofs) *nldofs = P.nfree * S->ncomp;
  if (nown) *nown = P.n_own * S->ncomp;
  if (first_gdof) *first_gdof = P.first_gdof * S->ncomp;
  return GD_OK;
}

extern "C" int gd_space_get_gids(const gd_space* S, int part, int64_t* ldof_to_gdof, int32_t* ldof_to_owner) {
  if (!S || part < 0 || part >= S->geom.nparts) return fail(GD_ERR_ARG, "gd_space_get_gids: bad part");
  const DevPart& P = S->parts[part];
  cudaStream_t st = S->model->ctx->stream;
  const int bs = S->ncomp;
  std::vector<int64_t> gid(bs > 1 ? P.nfree : 0);
  std::vector<int32_t> own(bs > 1 ? P.nfree : 0);
  int64_t* dg = bs > 1 ? gid.data() : ldof_to_gdof;
  int32_t* dow = bs > 1 ? own.data() : ldof_to_owner;
  if (ldof_to_gdof && P.nfree)
    GD_CUDA_TRY(cudaMemcpyAsync(dg, S->lid_gid.p + P.lid_off, sizeof(int64_t) * P.nfree, cudaMemcpyDeviceToHost, st));
  if (ldof_to_owner && P.nfree)
    GD_CUDA_TRY(cudaMemcpyAsync(dow, S->lid_owner.p + P.lid_off, sizeof(int32_t) * P.nfree, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (bs > 1)
    for (int64_t i = 0; i < P.nfree; ++i)
      for (int c = 0; c < bs; ++c) {
        if (ldof_to_gdof) ldof_to_gdof[bs * i + c] = bs * gid[i] + c;
        if (ldof_to_owner) ldof_to_owner[bs * i + c] = own[i];
      }
  return GD_OK;
}

// lattice node of every local free dof (vector spaces: one entry per component)
extern "C" int gd_space_dof_nodes(const gd_space* S, int part, int64_t* ldof_to_node) {
  if (!S || part < 0 || part >= S->geom.nparts || !ldof_to_node) return fail(GD_ERR_ARG, "gd_space_dof_nodes: bad argument");
  const DevPart& P = S->parts[part];
  cudaStream_t st = S->model->ctx->stream;
  std::vector<int32_t> tmp(P.nfree);
  if (P.nfree)
    GD_CUDA_TRY(cudaMemcpyAsync(tmp.data(), S->lid_node.p + P.lid_off, sizeof(int32_t) * P.nfree, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const Geom& g = S->geom;
  const int bs = S->ncomp;
  for (int64_t i = 0; i < P.nfree; ++i) {
    int64_t li = tmp[i], X[kMaxDim] = {0, 0, 0};
    for (int d = 0; d < g.dim; ++d) {
      X[d] = g.k * P.loc_lo[d] + li % P.nb[d];
      li /= P.nb[d];
    }
    for (int c = 0; c < bs; ++c) ldof_to_node[bs * i + c] = lattice_lin(g, X);
  }
  return GD_OK;
}

extern "C" int gd_space_set_dirichlet(gd_space* S, const double* u, int where) {
  if (!S) return fail(GD_ERR_ARG, "gd_space_set_dirichlet: null space");
  cudaStream_t st = S->model->ctx->stream;
  if (!u) {
    dfreeb(S->u_dir);
    S->has_dirichlet_values = false;
    return GD_OK;
  }
  int64_t n = S->ncomp > 1 ? S->ncomp : 1;   // values per lattice node
  for (int d = 0; d < S->geom.dim; ++d) n *= S->geom.N[d];
  GD_TRY(dalloc(S->u_dir, n));
  GD_CUDA_TRY(cudaMemcpyAsync(S->u_dir.p, u, sizeof(double) * n,
                              where == GD_DEVICE ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  S->has_dirichlet_values = true;
  return GD_OK;
}
