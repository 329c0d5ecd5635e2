// Internal definitions shared by the translation units of libgdgpu.so.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gdgpu.h"

namespace gd {

constexpr int kMaxDim = 3;
constexpr int kMaxOrder = 3;

// ---------------------------------------------------------------------------------
// Error handling: every C entry point returns a status and keeps a message per thread.
// ---------------------------------------------------------------------------------
void set_error(const std::string& msg);
int fail(int code, const std::string& msg);

#define GD_CUDA_TRY(expr)                                                                  \
  do {                                                                                     \
    cudaError_t _e = (expr);                                                               \
    if (_e != cudaSuccess)                                                                 \
      return ::gd::fail(GD_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e));  \
  } while (0)

#define GD_TRY(expr)                 \
  do {                               \
    int _s = (expr);                 \
    if (_s != GD_OK) return _s;      \
  } while (0)

// ---------------------------------------------------------------------------------
// Geometry of the partitioned Cartesian mesh, passed by value to kernels.
// ---------------------------------------------------------------------------------
struct Geom {
  int dim;
  int k;             // polynomial order (1 for a bare model)
  int nparts;
  int np[kMaxDim];   // parts per direction
  int64_t n[kMaxDim];   // cells per direction
  int64_t N[kMaxDim];   // lattice nodes per direction = k*n+1
  int64_t bl[kMaxDim];  // cells of the first (np-rem) parts along d
  int64_t brem[kMaxDim];
  int dsides[2 * kMaxDim];
  double h[kMaxDim];
  double x0[kMaxDim];
};

// One part as seen by the kernels (array in device memory).
struct DevPart {
  int64_t own_lo[kMaxDim], own_hi[kMaxDim];   // owned cells [lo,hi)
  int64_t loc_lo[kMaxDim], loc_hi[kMaxDim];   // owned+ghost cells [lo,hi)
  int64_t nb[kMaxDim];                         // local node box extents
  int64_t nnodes;        // prod(nb)
  int64_t node_off;      // offset in concatenated per-node arrays
  int64_t lid_off;       // offset in concatenated per-free-dof arrays
  int64_t nfree;         // local free dofs
  int64_t n_own;         // owned free dofs
  int64_t first_gdof;    // first owned gid
  int64_t lcell_off;     // offset in concatenated per-local-cell arrays
  int64_t nlcells;
  // assembler data
  int64_t grow_off, n_grow;   // ghost rows of this part in the concatenated row space
  int64_t gcol_off, n_gcol;   // ghost columns (per-part lists concatenated)
};

// Part coordinate along d of global cell index c (_local_range, PArraysExtras.jl:72-84):
// the first np-rem parts hold bl cells, the last rem parts bl+1.
__host__ __device__ inline int cell_part_coord(const Geom& g, int d, int64_t c) {
  int64_t l = g.bl[d];
  int64_t B = (g.np[d] - g.brem[d]) * l;
  if (c < B) return (int)(c / l);
  return (int)((g.np[d] - g.brem[d]) + (c - B) / (l + 1));
}

__host__ __device__ inline int part_of_coords(const Geom& g, const int* pc) {
  int p = 0;
  for (int d = g.dim - 1; d >= 0; --d) p = p * g.np[d] + pc[d];
  return p;
}

// Owner rank of a lattice node: max owner over the cells around it
// (FESpaces.jl:145-183).  Owner part coordinates are monotone in the cell index,
// so the max is reached at the highest cell index touching the node.
__host__ __device__ inline int node_owner(const Geom& g, const int64_t* X) {
  int pc[kMaxDim];
  for (int d = 0; d < g.dim; ++d) {
    int64_t c = X[d] / g.k;
    if (c > g.n[d] - 1) c = g.n[d] - 1;
    pc[d] = cell_part_coord(g, d, c);
  }
  return part_of_coords(g, pc);
}

__host__ __device__ inline int cell_owner(const Geom& g, const int64_t* c) {
  int pc[kMaxDim];
  for (int d = 0; d < g.dim; ++d) pc[d] = cell_part_coord(g, d, c[d]);
  return part_of_coords(g, pc);
}

__host__ __device__ inline bool node_is_dirichlet(const Geom& g, const int64_t* X) {
  for (int d = 0; d < g.dim; ++d) {
    if (g.dsides[2 * d] && X[d] == 0) return true;
    if (g.dsides[2 * d + 1] && X[d] == g.N[d] - 1) return true;
  }
  return false;
}

__host__ __device__ inline int64_t lattice_lin(const Geom& g, const int64_t* X) {
  int64_t r = 0;
  for (int d = g.dim - 1; d >= 0; --d) r = r * g.N[d] + X[d];
  return r;
}

__host__ __device__ inline void lattice_coords(const Geom& g, int64_t lin, int64_t* X) {
  for (int d = 0; d < g.dim; ++d) {
    X[d] = lin % g.N[d];
    lin /= g.N[d];
  }
}

__host__ __device__ inline int64_t cell_lin(const Geom& g, const int64_t* c) {
  int64_t r = 0;
  for (int d = g.dim - 1; d >= 0; --d) r = r * g.n[d] + c[d];
  return r;
}

// ---------------------------------------------------------------------------------
// Device scratch helpers (implemented in gd_util.cu)
// ---------------------------------------------------------------------------------
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
};

int dalloc_bytes(void** p, size_t bytes);
void dfree(void* p);

template <typename T>
int dalloc(DBuf<T>& b, size_t n) {
  if (b.p) dfree(b.p);
  b.p = nullptr;
  b.n = n;
  if (n == 0) return GD_OK;
  return dalloc_bytes((void**)&b.p, n * sizeof(T));
}
template <typename T>
void dfreeb(DBuf<T>& b) {
  if (b.p) dfree(b.p);
  b.p = nullptr;
  b.n = 0;
}

// Exclusive scan of int32 flags/counts into int64 (out has n+1 entries; out[n] = total).
int exclusive_scan_i32(const int32_t* in, int64_t* out, int64_t n, cudaStream_t s);

// Generic Q_k rows with an arbitrary reference table (gd_numeric.cu): values of the owned
// rows, and f_const * (int v) minus the Dirichlet lifting with the table.
int launch_rows_table(gd_asm* A, const double* kappa, const double* table, double* vals, cudaStream_t st);
int launch_rhs_table(gd_asm* A, const double* kappa, const double* table, double f_const, double* rhs, int32_t* bad,
                     cudaStream_t st);
int reference_element(gd_asm* A, int degree);
// Sliced-ELL copy of a CSR's rows for the FP64 solver (gd_solve.cu): slices of 32 rows,
// stored entry k of row r at 32 off[r / 32] + 32 k + r % 32, so the 32 threads of a warp
// (one row each) read their k-th entries from one contiguous 256-byte line.  Exact zeros
// are dropped; the other entries keep their CSR order, so a row's sum is bit-identical to
// the CSR kernel's.  version: the matrix values it was built from (-1: none).
struct SellMat {
  DBuf<int64_t> off;     // per slice, in units of 32 entries (nslices + 1)
  DBuf<int32_t> width;   // per slice: its longest stored row
  DBuf<int32_t> len;     // per row: stored entries
  DBuf<double> val;
  DBuf<int32_t> col;
  int64_t n = -1, version = -1;
  void release() {
    dfreeb(off);
    dfreeb(width);
    dfreeb(len);
    dfreeb(val);
    dfreeb(col);
    n = -1;
    version = -1;
  }
};
// Rows short enough for one thread per row (average below 48 entries) go through the
// sliced-ELL copy; longer ones use lane groups on the CSR itself.
inline bool sell_suits(int64_t n, int64_t nnz) { return n > 0 && nnz / n < 48; }
int sell_build(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, SellMat& S, int64_t version,
               cudaStream_t st);

// FP64 Jacobi-PCG on the owned rows of a CSR with global column ids (gd_solve.cu).  sell:
// the caller's cached sliced-ELL copy for matrix version `version` (null: a temporary one).
int jacobi_pcg_csr(int64_t n, const int64_t* rowptr, const int32_t* colgid, const double* vals, const double* rhs,
                   DBuf<double>& w, DBuf<double>& dinvb, DBuf<double>& dred, cudaStream_t st, double rtol, int maxit,
                   double* x, int where, gd_solve_stats* stats, SellMat* sell = nullptr, int64_t version = -1);
// r = b - A x over the assembler's owned rows with partials of r.r and b.b (the
// sliced-ELL copy where it suits, the CSR otherwise); *nblocks partials each.
int residual_fp64_asm(gd_asm* A, const double* x, const double* b, double* r, double* prr, double* pbb,
                      cudaStream_t st, int* nblocks);

}  // namespace gd

namespace gd {
// Workspace of the quadrature-point assembly (gd_qp.cu).
struct QpState;
void qp_release(QpState* q);
// Workspace of the mixed-precision solver (gd_solve_mixed.cu).
struct MixedState {
  bool ready = false;
  bool matrix_free = false;
  int64_t numeric_epoch = -1;
  float ratio = 0.f;
  int last_outer = 0;
  DBuf<float> f32;        // x r z p q dinv (FP32, 6 n)
  DBuf<double> f64;       // x r (FP64, 2 n)
  DBuf<double> red;       // block partials + scalars
  DBuf<int32_t> node_gid; // lattice node -> gid (-1 Dirichlet)
  DBuf<float> wf;         // prescaled cell coefficients (FP32)
  DBuf<float> vals32;     // FP32 copy of the owned-row values (non-cube spaces)
  int csr_lanes = 1;      // lanes per row of the FP32 CSR operator (1: one thread per row)
  DBuf<float> zold;       // previous preconditioned residual (flexible CG)
  // lattice-order inner iteration (3D cube Q1): x r z0 z1 p0 p1 q dinv, node-lattice sized
  DBuf<float> lat;
  DBuf<double> latred;    // block partials, arrival counter and CG scalars
  // persistent Jacobi-CG on the padded lattice: x r z p q dinv w
  DBuf<float> plat;
  int64_t plat_epoch = -1;
  // captured batches of flexible-CG steps (16, 8, 4 and 2 steps; lattice path, external
  // preconditioner) and the preconditioner key, buffers and sizes they were captured with
  cudaGraphExec_t fcg_graph[4] = {nullptr, nullptr, nullptr, nullptr};
  uint64_t fcg_key[5] = {0, 0, 0, 0, 0};
  int64_t lat_epoch = -1;
};
constexpr int kLatVectors = 8;

// host quadrature helpers (gd_numeric.cu)
void gauss_legendre01(int n, std::vector<double>& x, std::vector<double>& w);
// Gridap's local node order of one Q_k cell: lattice offsets of each local dof (gd_space.cu)
void cell_dof_positions(int dim, int k, std::vector<int>& pos);
void lagrange01(int k, double x, double* v, double* dv);
}  // namespace gd

// ---------------------------------------------------------------------------------
// Opaque objects of the C ABI
// ---------------------------------------------------------------------------------
struct gd_ctx {
  int device = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
};

struct gd_model {
  gd_ctx* ctx = nullptr;
  gd::Geom geom{};   // k = 1
  double domain[2 * gd::kMaxDim] = {0};
  std::vector<gd::DevPart> parts;   // boxes only
};

struct gd_space {
  gd_model* model = nullptr;
  gd::Geom geom{};
  int ncomp = 1;
  std::vector<gd::DevPart> parts;   // host copy
  gd::DBuf<gd::DevPart> d_parts;
  int64_t total_nodes = 0;          // concatenated local node boxes
  int64_t total_lids = 0;           // concatenated local free dofs
  int64_t ngdofs = 0;
  // per concatenated local node: free lid (>=0) or -(dirichlet id + 1)
  gd::DBuf<int32_t> node_lid;
  // per concatenated free dof
  gd::DBuf<int32_t> lid_node;     // local node index in the part's box
  gd::DBuf<int32_t> lid_owner;
  gd::DBuf<int32_t> lid_ownidx;   // index among the part's owned dofs (own: valid)
  gd::DBuf<int64_t> lid_gid;
  // Dirichlet values on the global lattice (dense) or null
  gd::DBuf<double> u_dir;
  bool has_dirichlet_values = false;
  // table: lexicographic cell-local node -> Gridap cell-local node index
  std::vector<int> lex_to_gridap;
  // lattice node -> gid (-1: Dirichlet), built on first use by post-processing
  gd::DBuf<int32_t> lat_gid;
};

struct gd_asm {
  gd_space* trial = nullptr;
  gd_space* test = nullptr;
  int strategy = GD_SUB_ASSEMBLED_ROWS;
  bool symbolic_done = false;
  bool numeric_done = false;
  std::vector<gd::DevPart> parts;   // with ghost row / col data
  gd::DBuf<gd::DevPart> d_parts;
  int64_t ngdofs = 0;
  int64_t nrows_total = 0;          // ngdofs owned rows + all ghost rows
  int64_t nnz_total = 0;
  int64_t nnz_own = 0;              // entries of the owned rows (prefix of the arrays)
  int64_t total_gcols = 0;
  int code_bytes = 1;
  // concatenated row space: [owned rows of all parts in gid order][ghost rows of part 0]...
  gd::DBuf<int64_t> rowptr;       // nrows_total + 1
  gd::DBuf<int32_t> row_node;     // global lattice node of each row
  gd::DBuf<int32_t> row_part;     // part that stores the row
  gd::DBuf<int32_t> colidx;       // local column id (per part numbering)
  gd::DBuf<int32_t> colgid;       // global column id (owned rows only are meaningful)
  gd::DBuf<uint8_t> code;         // stencil offset code of each entry (1 or 2 bytes)
  gd::DBuf<double> vals;
  gd::DBuf<double> rhs;           // nrows_total (ghost rows zero)
  // ghost rows: per concatenated ghost row: lid in its part
  gd::DBuf<int32_t> grow_lid;
  // ghost cols: per concatenated ghost col: lid in its part, gid, owner
  gd::DBuf<int32_t> gcol_lid;
  // per concatenated local node: local column id or -1
  gd::DBuf<int32_t> node_col;
  // Q1 row patterns: per owned row a pattern id; per pattern 32 bytes = the CSR
  // position of each canonical stencil neighbour (0xFF = absent), byte 31 = length
  bool fast_q1 = false;
  int npat = 0;
  gd::DBuf<uint16_t> row_pat;
  gd::DBuf<uint8_t> pat;
  int q1_grid = 0;
  int q1_shape = -1;            // autotuned launch shape (-1: not tuned yet)
  // 2D Q_k rows: the reference tables are reflection-invariant (cached per reference
  // element), and whether the class-sum rows may use it (on by default)
  bool r2d_sym = false;
  int r2d_sym_degree = -1;
  bool r2d_class_sums = true;
  std::vector<double> r2d_F;      // the reference load table, copied with the symmetry check
  int64_t q1_rows[2] = {0, -1};   // owned-row range of the next Q1 launch (hi < 0: all rows)
  // pipelined download (gd_assemble_download): host destinations of the values and the
  // rhs while active, the copy stream, one event per row range, the row ranges and
  // their first CSR entries
  bool dl_active = false;
  double* dl_rhs = nullptr;
  double* dl_vals = nullptr;
  cudaStream_t dl_stream = nullptr;
  std::vector<cudaEvent_t> dl_events;
  std::vector<int64_t> dl_rows, dl_nnz;
  float q1_shape_ms[8] = {0};
  gd::DBuf<double> w_cells;   // prescaled coefficients (cube Q1 path)
  std::string q1c_blob;        // cached Q1 class constants for the current reference element
  double q1c_f0 = 0.0;
  bool q1c_cube = false;
  int q1c_degree = -1;
  // reference element tables (device)
  gd::DBuf<double> Khat, Mhat, Fhat;
  int ref_degree = -1;
  gd::DBuf<double> kappa_dev, f_dev;   // staging for host inputs
  // cell visits whose coefficient failed the check in the numeric kernels since the last
  // synchronous report (zero unless one failed; reset after it is reported)
  gd::DBuf<int32_t> nbad;
  // profiling events: start, after ghost zeroing, after matrix, after rhs
  bool profiling = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // mixed-precision solver
  gd::MixedState mx;
  int64_t numeric_epoch = 0;
  double mf_ratio = 0.0;
  double mf_k2 = 0.0;
  const double* rhs_override = nullptr;   // solve with a caller-given right-hand side
  // vector-valued spaces: bs = components per node; the CSR, row space and per-part
  // counts are expanded to the vector DOFs (dof = bs * node dof + component)
  int bs = 1;
  gd::DBuf<int32_t> gcol_gstart, gcol_gsize;   // scalar ghost-column groups (symbolic only)
  gd::DBuf<double> Kel;                        // elasticity reference matrix (E = 1)
  int el_degree = -1;
  double el_nu = -1.0;
  gd::DBuf<double> E_dev;
  // solver workspace
  gd::DBuf<double> w;              // vectors
  gd::DBuf<double> dred;           // reduction partials
  gd::DBuf<double> dinv;
  gd::SellMat sell;                // sliced-ELL copy of the owned rows (FP64 solves)
  // quadrature-point assembly (gd_qp.cu); qp_values: the current values came from it, so
  // the cell-coefficient shortcuts of the solvers (matrix-free lattice operators) do not apply
  gd::QpState* qp = nullptr;
  bool qp_values = false;
};
