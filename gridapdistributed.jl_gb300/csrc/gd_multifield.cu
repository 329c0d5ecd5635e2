// Multi-field systems over one scalar space: n fields that share the test/trial space of a
// FullyAssembledRows assembler, a bilinear form sum_ij (a_ij grad(u_j).grad(v_i) +
// m_ij u_j v_i) (kappa per cell scaling both) and a linear form sum_i s_i v_i, minus the
// Dirichlet lifting of every field.
//
//   Block (i, j) values: the generic Q_k row kernel over the scalar pattern with the
//   reference table T_ij = a_ij Khat + m_ij Mhat; blocks with a_ij = m_ij = 0 are not
//   touched (no entries), as in Gridap's block assembly.
//   Field i's right-hand side: s_i (int v) minus the lifting with sum_j T_ij.
//
// A matrix over a row group R and a column group C of fields (gd_mfmat) is the block
// (R, C) of BlockMultiFieldStyle, or with R = C = all fields the monolithic matrix of
// ConsecutiveMultiFieldStyle.  Its numbering restates generate_multi_field_gids
// (src/MultiField.jl:356-420): in each part the owned dofs of the group's fields, field
// by field in the fields' own order, numbered part by part; because every field shares
// one part-contiguous scalar numbering, the gid of a field-jj dof with scalar gid g owned
// by part q is |G| first(q) + jj n_own(q) + (g - first(q)).  A part's local columns are
// the group's owned columns (field-major) followed by the ghost columns; a merged row is
// the owned-column prefixes of its touched blocks' scalar rows, then their ghost parts.
//  * FullyAssembledRows: the touched ghost columns of each touched field in field order
//    (each sorted by local id, as the scalar FullyAssembledRows columns are:
//    src/Algebra.jl:1245-1257); owned rows only.
//  * SubAssembledRows (the default of the reference's multi-field assemblers,
//    src/MultiField.jl:473-479): only owned cells are integrated; Gridap walks a cell's
//    block matrix column-major with the block columns outer, so a ghost column (field j,
//    node y) first appears at the scalar column's first-appearance cell, and among the
//    columns first met in one cell field j's come before field j+1's.  The ghost columns
//    are therefore the scalar SubAssembledRows ghost columns grouped by first cell (the
//    groups the vector expansion uses), field-major inside a group.  Rows: the owned
//    rows, then per part the touched ghost rows -- each row field with a touched block
//    times the scalar ghost rows, by local id (field-major) -- holding explicit zeros
//    (their triplets went to the owners, src/Algebra.jl:1048-1131).
#include <algorithm>
#include <string>
#include <vector>

#include "gd_internal.h"

struct gd_mfield {
  gd_asm* A = nullptr;
  int nf = 0;
  bool assembled = false;
  std::vector<int> touched;      // nf * nf
  gd::DBuf<double> bvals;        // nf * nf blocks of nnz_own values (touched blocks written)
  gd::DBuf<double> brhs;         // nf fields of ngdofs values
  gd::DBuf<double> tabs;         // nf * nf + nf reference tables of NN * NN
  gd::DBuf<int32_t> bad;
  int64_t epoch = 0;             // bumped by every assembly
  ~gd_mfield() {
    gd::dfreeb(bvals);
    gd::dfreeb(brhs);
    gd::dfreeb(tabs);
    gd::dfreeb(bad);
  }
};

struct gd_mfmat {
  gd_mfield* M = nullptr;
  std::vector<int> rf, cf;       // row and column fields
  std::vector<int> ctouched;     // per column field: touched by some row field
  std::vector<int> rtouched;     // per row field: touching some column field
  std::vector<int> btouched;     // nr * nc: block touched when the pattern was built
  int64_t nrows = 0, nnz = 0;    // owned rows (group gid order) and all stored entries
  int64_t nrows_total = 0;       // owned rows, then the ghost rows of every part (SubAssembledRows)
  int64_t epoch = -1;            // assembly epoch the values were gathered from
  gd::DBuf<int64_t> rowptr;      // nrows + 1 (rows in group gid order)
  gd::DBuf<int32_t> colidx;      // local column id (per part)
  gd::DBuf<int64_t> colgid;      // global column id (group numbering)
  gd::DBuf<int64_t> src;         // position of each entry in the block value arrays
  gd::DBuf<double> vals;
  gd::DBuf<double> rhs;          // nrows
  ~gd_mfmat() {
    gd::dfreeb(rowptr);
    gd::dfreeb(colidx);
    gd::dfreeb(colgid);
    gd::dfreeb(src);
    gd::dfreeb(vals);
    gd::dfreeb(rhs);
  }
};

namespace gd {
namespace {

constexpr int kMfThreads = 256;

struct MfPartInfo {
  int64_t first;   // first scalar gid of the part
  int64_t n_own;
  int64_t n_gcol;
  int64_t gcol_off;   // scalar ghost columns of the part in the concatenated list
  int64_t grow_off;   // scalar ghost rows of the part (concatenated, after the owned rows)
  int64_t n_grow;
};

// group gid of the field-jj dof with scalar gid g (owner found by bisection over the
// parts' first gids, which increase with the part id)
__device__ __forceinline__ int64_t mf_gid(const MfPartInfo* parts, int np, int ng, int jj, int64_t g) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (parts[mid].first <= g) lo = mid;
    else hi = mid - 1;
  }
  const MfPartInfo& q = parts[lo];
  return (int64_t)ng * q.first + (int64_t)jj * q.n_own + (g - q.first);
}

// merged row m -> (part, row field index, scalar row); rows are in group gid order
__device__ __forceinline__ void mf_row(const MfPartInfo* parts, int np, int nr, int64_t m, int& p, int& ii,
                                       int64_t& r) {
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((int64_t)nr * parts[mid].first <= m) lo = mid;
    else hi = mid - 1;
  }
  p = lo;
  const int64_t off = m - (int64_t)nr * parts[lo].first;
  ii = parts[lo].n_own ? (int)(off / parts[lo].n_own) : 0;
  r = parts[lo].first + (off - (int64_t)ii * parts[lo].n_own);
}

struct MfGroups {
  int nr, nc, nf;
  int rf[8], cf[8];
  int blk[8][8];      // block index rf[ii] * nf + cf[jj], -1 when not touched
  int gofs[8];        // index of column field jj among the touched ones, -1 when untouched
  int ntc;            // touched column fields
  int rt[8];          // row field index of the t-th touched row field
  int nrt;            // touched row fields
  int sub;            // SubAssembledRows
  int64_t nrows_own;  // nr * ngdofs
  int64_t ngdofs;
};

// merged row m -> (part, row field index, scalar row in the scalar row space); ghost rows
// (m >= nrows_own) of part p are nrt * n_grow rows, row field outer
__device__ __forceinline__ void mf_any_row(const MfGroups& G, const MfPartInfo* parts, int np, int64_t m, int& p,
                                           int& ii, int64_t& r, bool& ghost) {
  ghost = m >= G.nrows_own;
  if (!ghost) {
    mf_row(parts, np, G.nr, m, p, ii, r);
    return;
  }
  const int64_t gm = m - G.nrows_own;
  int lo = 0, hi = np - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((int64_t)G.nrt * parts[mid].grow_off <= gm) lo = mid;
    else hi = mid - 1;
  }
  p = lo;
  const int64_t off = gm - (int64_t)G.nrt * parts[lo].grow_off;
  const int t = parts[lo].n_grow ? (int)(off / parts[lo].n_grow) : 0;
  ii = G.rt[t];
  r = G.ngdofs + parts[lo].grow_off + (off - (int64_t)t * parts[lo].n_grow);
}

__global__ void k_mf_rowlen(MfGroups G, const MfPartInfo* __restrict__ parts, int np, int64_t nrows,
                            const int64_t* __restrict__ rowptr, int32_t* __restrict__ len) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nrows; m += (int64_t)gridDim.x * blockDim.x) {
    int p, ii;
    int64_t r;
    bool ghost;
    mf_any_row(G, parts, np, m, p, ii, r, ghost);
    const int64_t l = rowptr[r + 1] - rowptr[r];
    int k = 0;
    for (int jj = 0; jj < G.nc; ++jj) k += G.blk[ii][jj] >= 0;
    len[m] = (int32_t)(l * k);
  }
}

__global__ void k_mf_fill(MfGroups G, const MfPartInfo* __restrict__ parts, int np, int64_t nrows, int64_t nnz_blk,
                          const int64_t* __restrict__ rowptr, const int32_t* __restrict__ colidx,
                          const int32_t* __restrict__ colgid, const int32_t* __restrict__ gstart,
                          const int32_t* __restrict__ gsize, const int64_t* __restrict__ mrowptr,
                          int32_t* __restrict__ mcol, int64_t* __restrict__ mgid, int64_t* __restrict__ msrc) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nrows; m += (int64_t)gridDim.x * blockDim.x) {
    int p, ii;
    int64_t r;
    bool ghost;
    mf_any_row(G, parts, np, m, p, ii, r, ghost);
    const MfPartInfo P = parts[p];
    const int64_t e0 = rowptr[r], e1 = rowptr[r + 1];
    int64_t eo = e0;   // end of the owned-column prefix (columns are sorted: owned first)
    while (eo < e1 && colidx[eo] < P.n_own) ++eo;
    int64_t o = mrowptr[m];
    auto emit = [&](int jj, int b, int64_t e, int32_t col) {
      mcol[o] = col;
      mgid[o] = ghost ? -1 : mf_gid(parts, np, G.nc, jj, (int64_t)colgid[e]);
      msrc[o] = ghost ? -1 : (int64_t)b * nnz_blk + e;   // ghost rows: explicit zeros
      ++o;
    };
    for (int jj = 0; jj < G.nc; ++jj) {   // owned columns, field-major
      const int b = G.blk[ii][jj];
      if (b < 0) continue;
      for (int64_t e = e0; e < eo; ++e) emit(jj, b, e, (int32_t)(jj * P.n_own + colidx[e]));
    }
    if (!G.sub) {   // ghost columns of each touched field in turn
      for (int jj = 0; jj < G.nc; ++jj) {
        const int b = G.blk[ii][jj];
        if (b < 0) continue;
        for (int64_t e = eo; e < e1; ++e)
          emit(jj, b, e, (int32_t)(G.nc * P.n_own + G.gofs[jj] * P.n_gcol + (colidx[e] - P.n_own)));
      }
      continue;
    }
    // SubAssembledRows: first-appearance groups, field-major inside a group
    int64_t e = eo;
    while (e < e1) {
      const int64_t g0 = colidx[e] - P.n_own;
      const int64_t s0 = gstart[P.gcol_off + g0], mg = gsize[P.gcol_off + g0];
      int64_t f = e;
      while (f < e1 && gstart[P.gcol_off + (colidx[f] - P.n_own)] == s0) ++f;
      for (int jj = 0; jj < G.nc; ++jj) {
        const int b = G.blk[ii][jj];
        if (b < 0) continue;
        for (int64_t x = e; x < f; ++x) {
          const int64_t g = colidx[x] - P.n_own;
          emit(jj, b, x, (int32_t)(G.nc * P.n_own + G.ntc * s0 + G.gofs[jj] * mg + (g - s0)));
        }
      }
      e = f;
    }
  }
}

__global__ void k_mf_gather(int64_t n, const int64_t* __restrict__ src, const double* __restrict__ bvals,
                            double* __restrict__ out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t k = src[i];
    out[i] = k >= 0 ? bvals[k] : 0.0;
  }
}

__global__ void k_mf_rhs(MfGroups G, const MfPartInfo* __restrict__ parts, int np, int64_t nrows, int64_t ngdofs,
                         const double* __restrict__ brhs, double* __restrict__ rhs) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nrows; m += (int64_t)gridDim.x * blockDim.x) {
    int p, ii;
    int64_t r;
    mf_row(parts, np, G.nr, m, p, ii, r);
    rhs[m] = brhs[(int64_t)G.rf[ii] * ngdofs + r];
  }
}

// y = A x over group numberings (x indexed by column group gid), one thread per row
__global__ void k_mf_spmv(int64_t nrows, const int64_t* __restrict__ rowptr, const int64_t* __restrict__ colgid,
                          const double* __restrict__ vals, const double* __restrict__ x, double* __restrict__ y) {
  for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nrows; m += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t e = rowptr[m]; e < rowptr[m + 1]; ++e) s = fma(vals[e], x[colgid[e]], s);
    y[m] = s;
  }
}

// T = a Khat + m Mhat for every block, S_i = sum_j T_ij for every field
__global__ void k_mf_tables(int nf, int nn2, const double* __restrict__ coef, const double* __restrict__ Khat,
                            const double* __restrict__ Mhat, double* __restrict__ tabs) {
  const int nb = nf * nf;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < (nb + nf) * nn2; i += gridDim.x * blockDim.x) {
    const int t = i / nn2, e = i - t * nn2;
    if (t < nb) {
      tabs[i] = coef[2 * t] * Khat[e] + coef[2 * t + 1] * Mhat[e];
    } else {
      const int f = t - nb;
      double s = 0.0;
      for (int j = 0; j < nf; ++j) s += coef[2 * (f * nf + j)] * Khat[e] + coef[2 * (f * nf + j) + 1] * Mhat[e];
      tabs[i] = s;
    }
  }
}

unsigned mf_grid(int64_t n) {
  const int64_t b = (n + kMfThreads - 1) / kMfThreads;
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 8));
}

std::vector<MfPartInfo> part_info(const gd_asm* A) {
  std::vector<MfPartInfo> v(A->parts.size());
  for (size_t p = 0; p < A->parts.size(); ++p) {
    const DevPart& P = A->parts[p];
    v[p] = {P.first_gdof, P.n_own, P.n_gcol, P.gcol_off, P.grow_off, P.n_grow};
  }
  return v;
}

int check_fields(const gd_mfield* M, int n, const int* f, const char* who) {
  if (n < 1 || n > 8 || !f) return fail(GD_ERR_ARG, std::string(who) + ": 1 to 8 fields per group");
  for (int i = 0; i < n; ++i)
    if (f[i] < 0 || f[i] >= M->nf) return fail(GD_ERR_ARG, std::string(who) + ": field index out of range");
  return GD_OK;
}

}  // namespace
}  // namespace gd

using namespace gd;

extern "C" int gd_mfield_create(gd_asm* A, int nfields, gd_mfield** out) {
  if (!A || !out) return fail(GD_ERR_ARG, "gd_mfield_create: null argument");
  if (nfields < 1 || nfields > 8) return fail(GD_ERR_ARG, "gd_mfield_create: 1 to 8 fields");
  if (!A->symbolic_done) return fail(GD_ERR_STATE, "gd_mfield_create: run gd_assemble_symbolic first");
  if (A->bs != 1) return fail(GD_ERR_UNSUPPORTED, "gd_mfield_create: fields must be scalar");
  if (A->strategy == GD_SUB_ASSEMBLED_ROWS && A->total_gcols > 0 && !A->gcol_gstart.p)
    return fail(GD_ERR_STATE, "gd_mfield_create: the assembler has no ghost-column groups");
  gd_mfield* M = new gd_mfield();
  M->A = A;
  M->nf = nfields;
  M->touched.assign(nfields * nfields, 0);
  const int64_t nnz = std::max<int64_t>(A->nnz_own, 1);
  int s = dalloc(M->bvals, (size_t)nfields * nfields * nnz);
  if (s == GD_OK) s = dalloc(M->brhs, (size_t)nfields * std::max<int64_t>(A->ngdofs, 1));
  if (s == GD_OK) s = dalloc(M->bad, 1);
  if (s != GD_OK) {
    delete M;
    return s;
  }
  *out = M;
  return GD_OK;
}

extern "C" int gd_mfield_destroy(gd_mfield* M) {
  delete M;
  return GD_OK;
}

// stiff, mass: nf x nf row-major (row = test field i, column = trial field j); src: nf
extern "C" int gd_mfield_assemble(gd_mfield* M, const double* stiff, const double* mass, const double* src,
                                  const gd_coeffs* c) {
  if (!M || !stiff || !mass || !c) return fail(GD_ERR_ARG, "gd_mfield_assemble: null argument");
  gd_asm* A = M->A;
  const Geom& g = A->test->geom;
  cudaStream_t st = A->test->model->ctx->stream;
  const int nf = M->nf;
  GD_TRY(reference_element(A, c->degree));
  int64_t ncells = 1;
  for (int d = 0; d < g.dim; ++d) ncells *= g.n[d];
  const double* kappa = c->kappa;
  if (c->where == GD_HOST || !kappa) {
    if (A->kappa_dev.n != (size_t)ncells) GD_TRY(dalloc(A->kappa_dev, ncells));
    if (kappa) {
      GD_CUDA_TRY(cudaMemcpyAsync(A->kappa_dev.p, kappa, sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
    } else {
      std::vector<double> ones(ncells, 1.0);
      GD_CUDA_TRY(cudaMemcpyAsync(A->kappa_dev.p, ones.data(), sizeof(double) * ncells, cudaMemcpyHostToDevice, st));
      GD_CUDA_TRY(cudaStreamSynchronize(st));
    }
    kappa = A->kappa_dev.p;
  }
  if (c->f_nodal) return fail(GD_ERR_UNSUPPORTED, "gd_mfield_assemble: constant sources per field only");
  int nn = 1;
  for (int d = 0; d < g.dim; ++d) nn *= g.k + 1;
  const int nn2 = nn * nn;
  std::vector<double> coef(2 * nf * nf);
  for (int b = 0; b < nf * nf; ++b) {
    coef[2 * b] = stiff[b];
    coef[2 * b + 1] = mass[b];
    M->touched[b] = stiff[b] != 0.0 || mass[b] != 0.0;
  }
  if (M->tabs.n != (size_t)(nf * nf + nf) * nn2) GD_TRY(dalloc(M->tabs, (size_t)(nf * nf + nf) * nn2));
  DBuf<double> dcoef;
  GD_TRY(dalloc(dcoef, coef.size()));
  GD_CUDA_TRY(cudaMemcpyAsync(dcoef.p, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice, st));
  k_mf_tables<<<mf_grid((int64_t)(nf * nf + nf) * nn2), kMfThreads, 0, st>>>(nf, nn2, dcoef.p, A->Khat.p, A->Mhat.p,
                                                                            M->tabs.p);
  const cudaError_t te = cudaGetLastError();
  const cudaError_t ts = cudaStreamSynchronize(st);
  dfreeb(dcoef);
  if (te != cudaSuccess || ts != cudaSuccess) return fail(GD_ERR_CUDA, "gd_mfield_assemble: reference tables");
  GD_CUDA_TRY(cudaMemsetAsync(M->bad.p, 0, sizeof(int32_t), st));
  const int64_t nnz = std::max<int64_t>(A->nnz_own, 1);
  for (int b = 0; b < nf * nf; ++b)
    if (M->touched[b]) GD_TRY(launch_rows_table(A, kappa, M->tabs.p + (size_t)b * nn2, M->bvals.p + b * nnz, st));
  const int64_t ng = std::max<int64_t>(A->ngdofs, 1);
  for (int i = 0; i < nf; ++i)
    GD_TRY(launch_rhs_table(A, kappa, M->tabs.p + (size_t)(nf * nf + i) * nn2, src ? src[i] : 0.0,
                            M->brhs.p + i * ng, M->bad.p, st));
  int32_t hbad = 0;
  GD_CUDA_TRY(cudaMemcpyAsync(&hbad, M->bad.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (hbad) return fail(GD_ERR_NUMERIC, "gd_mfield_assemble: kappa is not finite and positive");
  M->assembled = true;
  ++M->epoch;
  return GD_OK;
}

// Values of block (i, j) over the owned rows of `part` (the scalar pattern of the part,
// gd_matrix_export order), and field i's right-hand side over the part's owned rows.
extern "C" int gd_mfield_block_export(const gd_mfield* M, int i, int j, int part, double* vals, double* rhs) {
  if (!M) return fail(GD_ERR_ARG, "gd_mfield_block_export: null multi-field system");
  if (!M->assembled) return fail(GD_ERR_STATE, "gd_mfield_block_export: assemble first");
  const gd_asm* A = M->A;
  if (i < 0 || j < 0 || i >= M->nf || j >= M->nf || part < 0 || part >= (int)A->parts.size())
    return fail(GD_ERR_ARG, "gd_mfield_block_export: bad index");
  const DevPart& P = A->parts[part];
  cudaStream_t st = A->test->model->ctx->stream;
  int64_t b[2];
  GD_CUDA_TRY(cudaMemcpyAsync(&b[0], A->rowptr.p + P.first_gdof, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[1], A->rowptr.p + P.first_gdof + P.n_own, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const int64_t nnz = std::max<int64_t>(A->nnz_own, 1);
  if (vals && b[1] > b[0]) {
    if (M->touched[i * M->nf + j])
      GD_CUDA_TRY(cudaMemcpyAsync(vals, M->bvals.p + (int64_t)(i * M->nf + j) * nnz + b[0], sizeof(double) * (b[1] - b[0]),
                                  cudaMemcpyDeviceToHost, st));
    else
      std::fill(vals, vals + (b[1] - b[0]), 0.0);
  }
  if (rhs && P.n_own)
    GD_CUDA_TRY(cudaMemcpyAsync(rhs, M->brhs.p + (int64_t)i * std::max<int64_t>(A->ngdofs, 1) + P.first_gdof,
                                sizeof(double) * P.n_own, cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  return GD_OK;
}

// Group gids of the dofs of `part`: local ids field-major (group position jj times the
// part's free dofs plus the scalar local id), as Gridap's MultiFieldFESpace numbers them.
extern "C" int gd_mfield_gids(const gd_mfield* M, int nfields, const int* fields, int part, int64_t* lid_to_gid,
                              int32_t* lid_to_owner) {
  if (!M) return fail(GD_ERR_ARG, "gd_mfield_gids: null argument");
  GD_TRY(check_fields(M, nfields, fields, "gd_mfield_gids"));
  const gd_asm* A = M->A;
  if (part < 0 || part >= (int)A->parts.size()) return fail(GD_ERR_ARG, "gd_mfield_gids: bad part");
  const DevPart& P = A->parts[part];
  const gd_space* S = A->test;
  cudaStream_t st = S->model->ctx->stream;
  std::vector<int64_t> gid(P.nfree);
  std::vector<int32_t> own(P.nfree);
  if (P.nfree) {
    GD_CUDA_TRY(cudaMemcpyAsync(gid.data(), S->lid_gid.p + P.lid_off, sizeof(int64_t) * P.nfree, cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaMemcpyAsync(own.data(), S->lid_owner.p + P.lid_off, sizeof(int32_t) * P.nfree, cudaMemcpyDeviceToHost, st));
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  for (int jj = 0; jj < nfields; ++jj)
    for (int64_t l = 0; l < P.nfree; ++l) {
      const DevPart& Q = A->parts[own[l]];
      if (lid_to_gid) lid_to_gid[jj * P.nfree + l] = (int64_t)nfields * Q.first_gdof + (int64_t)jj * Q.n_own + (gid[l] - Q.first_gdof);
      if (lid_to_owner) lid_to_owner[jj * P.nfree + l] = own[l];
    }
  return GD_OK;
}

static int mfmat_gather(gd_mfmat* X) {
  gd_mfield* M = X->M;
  const gd_asm* A = M->A;
  cudaStream_t st = A->test->model->ctx->stream;
  if (X->nnz)
    k_mf_gather<<<mf_grid(X->nnz), kMfThreads, 0, st>>>(X->nnz, X->src.p, M->bvals.p, X->vals.p);
  GD_CUDA_TRY(cudaGetLastError());
  X->epoch = M->epoch;
  return GD_OK;
}

static MfGroups make_groups(const gd_mfmat* X) {
  MfGroups G{};
  const gd_mfield* M = X->M;
  G.nr = (int)X->rf.size();
  G.nc = (int)X->cf.size();
  G.nf = M->nf;
  for (int ii = 0; ii < G.nr; ++ii) G.rf[ii] = X->rf[ii];
  for (int jj = 0; jj < G.nc; ++jj) G.cf[jj] = X->cf[jj];
  int k = 0;
  for (int jj = 0; jj < G.nc; ++jj) G.gofs[jj] = X->ctouched[jj] ? k++ : -1;
  G.ntc = k;
  G.nrt = 0;
  for (int ii = 0; ii < G.nr; ++ii)
    if (X->rtouched[ii]) G.rt[G.nrt++] = ii;
  for (int ii = 0; ii < G.nr; ++ii)
    for (int jj = 0; jj < G.nc; ++jj)
      G.blk[ii][jj] = X->btouched[ii * G.nc + jj] ? X->rf[ii] * M->nf + X->cf[jj] : -1;
  G.sub = M->A->strategy == GD_SUB_ASSEMBLED_ROWS;
  G.ngdofs = M->A->ngdofs;
  G.nrows_own = X->nrows;
  return G;
}

// The matrix of row fields rf[0..nr) and column fields cf[0..nc) (block (R, C) of a block
// multi-field system, or the monolithic matrix when both are all fields in order), with
// its right-hand side over the rows.  Values follow later assemblies through
// gd_mfmat_refresh.
extern "C" int gd_mfmat_create(gd_mfield* M, int nr, const int* rf, int nc, const int* cf, gd_mfmat** out) {
  if (!M || !out) return fail(GD_ERR_ARG, "gd_mfmat_create: null argument");
  if (!M->assembled) return fail(GD_ERR_STATE, "gd_mfmat_create: assemble first");
  GD_TRY(check_fields(M, nr, rf, "gd_mfmat_create"));
  GD_TRY(check_fields(M, nc, cf, "gd_mfmat_create"));
  const gd_asm* A = M->A;
  cudaStream_t st = A->test->model->ctx->stream;
  gd_mfmat* X = new gd_mfmat();
  X->M = M;
  X->rf.assign(rf, rf + nr);
  X->cf.assign(cf, cf + nc);
  X->ctouched.assign(nc, 0);
  X->rtouched.assign(nr, 0);
  X->btouched.assign(nr * nc, 0);
  for (int jj = 0; jj < nc; ++jj)
    for (int ii = 0; ii < nr; ++ii) {
      X->btouched[ii * nc + jj] = M->touched[rf[ii] * M->nf + cf[jj]];
      X->ctouched[jj] |= X->btouched[ii * nc + jj];
      X->rtouched[ii] |= X->btouched[ii * nc + jj];
    }
  X->nrows = (int64_t)nr * A->ngdofs;
  int nrt = 0;
  for (int t : X->rtouched) nrt += t;
  int64_t ngrow = 0;
  if (A->strategy == GD_SUB_ASSEMBLED_ROWS)
    for (const DevPart& P : A->parts) ngrow += P.n_grow;
  X->nrows_total = X->nrows + (int64_t)nrt * ngrow;
  const std::vector<MfPartInfo> pi = part_info(A);
  const int np = (int)pi.size();
  DBuf<MfPartInfo> dparts;
  DBuf<int32_t> len;
  auto cleanup = [&](int s) {
    dfreeb(dparts);
    dfreeb(len);
    delete X;
    return s;
  };
  const int64_t NT = X->nrows_total;
  int s = dalloc(dparts, pi.size());
  if (s == GD_OK) s = dalloc(len, std::max<int64_t>(NT, 1));
  if (s == GD_OK) s = dalloc(X->rowptr, NT + 1);
  if (s != GD_OK) return cleanup(s);
  if (cudaMemcpyAsync(dparts.p, pi.data(), sizeof(MfPartInfo) * pi.size(), cudaMemcpyHostToDevice, st) != cudaSuccess)
    return cleanup(fail(GD_ERR_CUDA, "gd_mfmat_create: copy"));
  const MfGroups G = make_groups(X);
  if (NT) k_mf_rowlen<<<mf_grid(NT), kMfThreads, 0, st>>>(G, dparts.p, np, NT, A->rowptr.p, len.p);
  if (cudaGetLastError() != cudaSuccess) return cleanup(fail(GD_ERR_CUDA, "gd_mfmat_create: row lengths"));
  if ((s = exclusive_scan_i32(len.p, X->rowptr.p, NT, st)) != GD_OK) return cleanup(s);
  if (cudaMemcpyAsync(&X->nnz, X->rowptr.p + NT, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return cleanup(fail(GD_ERR_CUDA, "gd_mfmat_create: entry count"));
  const size_t nz = (size_t)std::max<int64_t>(X->nnz, 1);
  if (s == GD_OK) s = dalloc(X->colidx, nz);
  if (s == GD_OK) s = dalloc(X->colgid, nz);
  if (s == GD_OK) s = dalloc(X->src, nz);
  if (s == GD_OK) s = dalloc(X->vals, nz);
  if (s == GD_OK) s = dalloc(X->rhs, std::max<int64_t>(X->nrows, 1));
  if (s != GD_OK) return cleanup(s);
  if (NT) {
    k_mf_fill<<<mf_grid(NT), kMfThreads, 0, st>>>(G, dparts.p, np, NT, std::max<int64_t>(A->nnz_own, 1), A->rowptr.p,
                                                 A->colidx.p, A->colgid.p, A->gcol_gstart.p, A->gcol_gsize.p,
                                                 X->rowptr.p, X->colidx.p, X->colgid.p, X->src.p);
  }
  if (X->nrows) {
    k_mf_rhs<<<mf_grid(X->nrows), kMfThreads, 0, st>>>(G, dparts.p, np, X->nrows, std::max<int64_t>(A->ngdofs, 1),
                                                      M->brhs.p, X->rhs.p);
  }
  if (cudaGetLastError() != cudaSuccess) return cleanup(fail(GD_ERR_CUDA, "gd_mfmat_create: fill"));
  if ((s = mfmat_gather(X)) != GD_OK) return cleanup(s);
  if (cudaStreamSynchronize(st) != cudaSuccess) return cleanup(fail(GD_ERR_CUDA, "gd_mfmat_create: sync"));
  dfreeb(dparts);
  dfreeb(len);
  *out = X;
  return GD_OK;
}

extern "C" int gd_mfmat_destroy(gd_mfmat* X) {
  delete X;
  return GD_OK;
}

// Values and right-hand side from the latest assembly of the fields (the pattern is
// fixed; a block that was not touched when the matrix was created stays empty).
extern "C" int gd_mfmat_refresh(gd_mfmat* X) {
  if (!X) return fail(GD_ERR_ARG, "gd_mfmat_refresh: null argument");
  gd_mfield* M = X->M;
  const int nr = (int)X->rf.size(), nc = (int)X->cf.size();
  for (int ii = 0; ii < nr; ++ii)
    for (int jj = 0; jj < nc; ++jj)
      if ((M->touched[X->rf[ii] * M->nf + X->cf[jj]] != 0) != (X->btouched[ii * nc + jj] != 0))
        return fail(GD_ERR_STATE, "gd_mfmat_refresh: the form touches other blocks than the pattern was built for");
  const gd_asm* A = M->A;
  cudaStream_t st = A->test->model->ctx->stream;
  GD_TRY(mfmat_gather(X));
  const std::vector<MfPartInfo> pi = part_info(A);
  DBuf<MfPartInfo> dparts;
  GD_TRY(dalloc(dparts, pi.size()));
  cudaError_t e = cudaMemcpyAsync(dparts.p, pi.data(), sizeof(MfPartInfo) * pi.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && X->nrows) {
    k_mf_rhs<<<mf_grid(X->nrows), kMfThreads, 0, st>>>(make_groups(X), dparts.p, (int)pi.size(), X->nrows,
                                                      std::max<int64_t>(A->ngdofs, 1), M->brhs.p, X->rhs.p);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dfreeb(dparts);
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, "gd_mfmat_refresh: right-hand side");
  return GD_OK;
}

extern "C" int gd_mfmat_sizes(const gd_mfmat* X, int part, int64_t* nrows, int64_t* ncols, int64_t* nnz,
                              int64_t* n_ghost_rows, int64_t* n_ghost_cols) {
  if (!X) return fail(GD_ERR_ARG, "gd_mfmat_sizes: null argument");
  const gd_asm* A = X->M->A;
  if (part < 0 || part >= (int)A->parts.size()) return fail(GD_ERR_ARG, "gd_mfmat_sizes: bad part");
  const DevPart& P = A->parts[part];
  const int nr = (int)X->rf.size(), nc = (int)X->cf.size();
  int ntc = 0, nrt = 0;
  for (int t : X->ctouched) ntc += t;
  for (int t : X->rtouched) nrt += t;
  const int64_t ngr = A->strategy == GD_SUB_ASSEMBLED_ROWS ? (int64_t)nrt * P.n_grow : 0;
  cudaStream_t st = A->test->model->ctx->stream;
  int64_t b[4];
  const int64_t r0 = (int64_t)nr * P.first_gdof, r1 = r0 + (int64_t)nr * P.n_own;
  const int64_t g0 = X->nrows + (int64_t)nrt * P.grow_off, g1 = g0 + ngr;
  GD_CUDA_TRY(cudaMemcpyAsync(&b[0], X->rowptr.p + r0, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[1], X->rowptr.p + r1, sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[2], X->rowptr.p + (ngr ? g0 : 0), sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaMemcpyAsync(&b[3], X->rowptr.p + (ngr ? g1 : 0), sizeof(int64_t), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (nrows) *nrows = (int64_t)nr * P.n_own + ngr;
  if (ncols) *ncols = (int64_t)nc * P.n_own + (int64_t)ntc * P.n_gcol;
  if (nnz) *nnz = (b[1] - b[0]) + (b[3] - b[2]);
  if (n_ghost_rows) *n_ghost_rows = ngr;
  if (n_ghost_cols) *n_ghost_cols = (int64_t)ntc * P.n_gcol;
  return GD_OK;
}

// The part's rows (owned rows, then its ghost rows): local CSR (columns: the group's owned
// columns, then the ghost columns), ghost row and ghost column gids and owners (group
// numberings) and the right-hand side (ghost rows 0).
extern "C" int gd_mfmat_export(const gd_mfmat* X, int part, int64_t* rowptr, int32_t* colidx, double* vals,
                               int64_t* ghost_row_gids, int32_t* ghost_row_owners, int64_t* ghost_col_gids,
                               int32_t* ghost_col_owners, double* rhs) {
  if (!X) return fail(GD_ERR_ARG, "gd_mfmat_export: null argument");
  const gd_mfield* M = X->M;
  const gd_asm* A = M->A;
  if (part < 0 || part >= (int)A->parts.size()) return fail(GD_ERR_ARG, "gd_mfmat_export: bad part");
  const DevPart& P = A->parts[part];
  const gd_space* S = A->test;
  cudaStream_t st = S->model->ctx->stream;
  const bool sub = A->strategy == GD_SUB_ASSEMBLED_ROWS;
  const int nr = (int)X->rf.size(), nc = (int)X->cf.size();
  int ntc = 0, nrt = 0;
  for (int t : X->ctouched) ntc += t;
  for (int t : X->rtouched) nrt += t;
  const int64_t r0 = (int64_t)nr * P.first_gdof, nrow = (int64_t)nr * P.n_own;
  const int64_t ngr = sub ? (int64_t)nrt * P.n_grow : 0;
  const int64_t g0 = X->nrows + (int64_t)nrt * P.grow_off;
  std::vector<int64_t> rp(nrow + 1), gp(ngr + 1);
  GD_CUDA_TRY(cudaMemcpyAsync(rp.data(), X->rowptr.p + r0, sizeof(int64_t) * (nrow + 1), cudaMemcpyDeviceToHost, st));
  if (ngr) GD_CUDA_TRY(cudaMemcpyAsync(gp.data(), X->rowptr.p + g0, sizeof(int64_t) * (ngr + 1), cudaMemcpyDeviceToHost, st));
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  const int64_t n = rp[nrow] - rp[0], ng = ngr ? gp[ngr] - gp[0] : 0;
  if (rowptr) {
    for (int64_t i = 0; i <= nrow; ++i) rowptr[i] = rp[i] - rp[0];
    for (int64_t i = 1; i <= ngr; ++i) rowptr[nrow + i] = n + gp[i] - gp[0];
  }
  if (colidx && n) GD_CUDA_TRY(cudaMemcpyAsync(colidx, X->colidx.p + rp[0], sizeof(int32_t) * n, cudaMemcpyDeviceToHost, st));
  if (colidx && ng) GD_CUDA_TRY(cudaMemcpyAsync(colidx + n, X->colidx.p + gp[0], sizeof(int32_t) * ng, cudaMemcpyDeviceToHost, st));
  if (vals && n) GD_CUDA_TRY(cudaMemcpyAsync(vals, X->vals.p + rp[0], sizeof(double) * n, cudaMemcpyDeviceToHost, st));
  if (vals && ng) GD_CUDA_TRY(cudaMemcpyAsync(vals + n, X->vals.p + gp[0], sizeof(double) * ng, cudaMemcpyDeviceToHost, st));
  if (rhs && nrow) GD_CUDA_TRY(cudaMemcpyAsync(rhs, X->rhs.p + r0, sizeof(double) * nrow, cudaMemcpyDeviceToHost, st));
  std::vector<int64_t> gid(P.nfree);
  std::vector<int32_t> own(P.nfree), gcl(P.n_gcol), grl(sub ? P.n_grow : 0), gst(sub ? P.n_gcol : 0),
      gsz(sub ? P.n_gcol : 0);
  if (P.nfree) {
    GD_CUDA_TRY(cudaMemcpyAsync(gid.data(), S->lid_gid.p + P.lid_off, sizeof(int64_t) * P.nfree, cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaMemcpyAsync(own.data(), S->lid_owner.p + P.lid_off, sizeof(int32_t) * P.nfree, cudaMemcpyDeviceToHost, st));
  }
  if (P.n_gcol)
    GD_CUDA_TRY(cudaMemcpyAsync(gcl.data(), A->gcol_lid.p + P.gcol_off, sizeof(int32_t) * P.n_gcol, cudaMemcpyDeviceToHost, st));
  if (sub && P.n_grow)
    GD_CUDA_TRY(cudaMemcpyAsync(grl.data(), A->grow_lid.p + P.grow_off, sizeof(int32_t) * P.n_grow, cudaMemcpyDeviceToHost, st));
  if (sub && P.n_gcol) {
    GD_CUDA_TRY(cudaMemcpyAsync(gst.data(), A->gcol_gstart.p + P.gcol_off, sizeof(int32_t) * P.n_gcol, cudaMemcpyDeviceToHost, st));
    GD_CUDA_TRY(cudaMemcpyAsync(gsz.data(), A->gcol_gsize.p + P.gcol_off, sizeof(int32_t) * P.n_gcol, cudaMemcpyDeviceToHost, st));
  }
  GD_CUDA_TRY(cudaStreamSynchronize(st));
  if (rhs)
    for (int64_t i = 0; i < ngr; ++i) rhs[nrow + i] = 0.0;
  auto group_gid = [&](int ng_, int jj, int lid) {
    const DevPart& Q = A->parts[own[lid]];
    return (int64_t)ng_ * Q.first_gdof + (int64_t)jj * Q.n_own + (gid[lid] - Q.first_gdof);
  };
  if (sub) {   // ghost rows: touched row fields in order, each the scalar ghost rows
    int64_t k = 0;
    for (int ii = 0; ii < nr; ++ii) {
      if (!X->rtouched[ii]) continue;
      for (int64_t x = 0; x < P.n_grow; ++x, ++k) {
        if (ghost_row_gids) ghost_row_gids[k] = group_gid(nr, ii, grl[x]);
        if (ghost_row_owners) ghost_row_owners[k] = own[grl[x]];
      }
    }
  }
  int kt = 0;
  for (int jj = 0; jj < nc; ++jj) {
    if (!X->ctouched[jj]) continue;
    for (int64_t g = 0; g < P.n_gcol; ++g) {
      const int64_t pos = sub ? (int64_t)ntc * gst[g] + (int64_t)kt * gsz[g] + (g - gst[g]) : (int64_t)kt * P.n_gcol + g;
      if (ghost_col_gids) ghost_col_gids[pos] = group_gid(nc, jj, gcl[g]);
      if (ghost_col_owners) ghost_col_owners[pos] = own[gcl[g]];
    }
    ++kt;
  }
  return GD_OK;
}

// y = A x: x over the column group's gids (|C| n global values), y over the row group's
extern "C" int gd_mfmat_spmv(const gd_mfmat* X, const double* x, double* y, int where) {
  if (!X || !x || !y) return fail(GD_ERR_ARG, "gd_mfmat_spmv: null argument");
  const gd_asm* A = X->M->A;
  cudaStream_t st = A->test->model->ctx->stream;
  const int64_t nx = (int64_t)X->cf.size() * A->ngdofs, ny = X->nrows;
  const double* dx = x;
  double* dy = y;
  DBuf<double> bx, by;
  if (where == GD_HOST) {
    int s = dalloc(bx, std::max<int64_t>(nx, 1));
    if (s == GD_OK) s = dalloc(by, std::max<int64_t>(ny, 1));
    if (s == GD_OK && nx && cudaMemcpyAsync(bx.p, x, sizeof(double) * nx, cudaMemcpyHostToDevice, st) != cudaSuccess)
      s = fail(GD_ERR_CUDA, "gd_mfmat_spmv: copy");
    if (s != GD_OK) {
      dfreeb(bx);
      dfreeb(by);
      return s;
    }
    dx = bx.p;
    dy = by.p;
  }
  if (ny) k_mf_spmv<<<mf_grid(ny), kMfThreads, 0, st>>>(ny, X->rowptr.p, X->colgid.p, X->vals.p, dx, dy);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && where == GD_HOST && ny) e = cudaMemcpyAsync(y, dy, sizeof(double) * ny, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  dfreeb(bx);
  dfreeb(by);
  if (e != cudaSuccess) return fail(GD_ERR_CUDA, "gd_mfmat_spmv: launch or copy");
  return GD_OK;
}

extern "C" int gd_mfmat_counts(const gd_mfmat* X, int64_t* nrows, int64_t* nnz) {
  if (!X) return fail(GD_ERR_ARG, "gd_mfmat_counts: null argument");
  if (nrows) *nrows = X->nrows;
  if (nnz) *nnz = X->nnz;
  return GD_OK;
}
