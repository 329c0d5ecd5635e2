/*
 * oracle_core.c -- CPU restatement of the reference's assembly hot path for scalar
 * Q1 spaces on a CartesianDiscreteModel.  TEST INFRASTRUCTURE ONLY: it is the
 * timed CPU baseline and a second checker; the shipped library never links it.
 *
 * It follows, part by part, what assemble_matrix_and_vector does on the
 * reference's with_debug path with a DistributedSparseMatrixAssembler:
 *   - partition with a one-cell ghost layer (src/PArraysExtras.jl:21-84);
 *   - local Q1 numbering: free vertices in vertex order, Dirichlet ones negative
 *     (Gridap 0.20 conforming numbering restricted to k = 1);
 *   - generate_gids (src/FESpaces.jl:139-261): owner = max owner rank of the cells
 *     around a DOF, owned DOFs numbered part-contiguously in local order;
 *   - per cell: element matrix and vector by tensor Gauss quadrature
 *     (Gridap integrate; Q1 shape functions on an axis-aligned cell);
 *   - COO numeric loop, columns outer / rows inner (Gridap add_entries!);
 *   - SubAssembledRows create_from_nz (src/Algebra.jl:593-646, 1048-1131): ghost
 *     rows sorted by local id, ghost-row triplets copied to their owner and zeroed
 *     (not removed) locally, received triplets appended in ascending sender order,
 *     ghost columns in first-appearance order, local sparse() compression with
 *     duplicates summed in COO order;
 *   - FullyAssembledRows (src/Algebra.jl:549-579): all local cells, owned rows only,
 *     ghost columns sorted by local id;
 *   - right-hand side with ghost contributions added into their owners
 *     (src/Algebra.jl:720-753, 786-789).
 * Parts run in parallel with OpenMP, one thread per part (the reference's
 * one-rank-per-part layout).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int dim;
  int64_t n[3];
  int32_t np[3];
  double domain[6];
  int32_t dsides[6];
  const double* kappa; /* per global cell, NULL = 1 */
  double f_const;
  int degree;
} orc_problem;

typedef struct {
  int nparts;
  int64_t ngdofs;
  int64_t* nrows;
  int64_t* ncols;
  int64_t* nnz;
  int64_t** rowptr;
  int64_t** colidx;
  double** vals;
  double** b;
  int64_t** row_ghost_gid;
  int64_t** col_ghost_gid;
  int64_t* n_ghost_rows;
  int64_t* n_ghost_cols;
} orc_system;

typedef struct {
  int64_t own_lo[3], own_hi[3], loc_lo[3], loc_hi[3];
  int64_t nb[3];       /* local vertex box */
  int64_t nverts;
  int64_t nfree;
  int32_t* vert_lid;   /* per local vertex: lid or -1 */
  int64_t* lid_vert;   /* lid -> global lattice vertex */
  int32_t* lid_owner;
  int64_t* lid_gid;
  int64_t n_own, first_gdof;
} part_t;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void local_range(int64_t p1, int64_t np, int64_t n, int ghost, int64_t* lo, int64_t* hi) {
  int64_t l = n / np, rem = n % np, offset = l * (p1 - 1);
  if (rem >= (np - p1 + 1)) {
    l += 1;
    offset += p1 - (np - rem) - 1;
  }
  int64_t start = 1 + offset - ghost, stop = l + offset + ghost;
  if (start < 1) start = 1;
  if (stop > n) stop = n;
  *lo = start - 1;
  *hi = stop;
}

static int cell_pc(const orc_problem* pb, int d, int64_t c) {
  for (int p = 0; p < pb->np[d]; ++p) {
    int64_t lo, hi;
    local_range(p + 1, pb->np[d], pb->n[d], 0, &lo, &hi);
    if (c >= lo && c < hi) return p;
  }
  return -1;
}

static int part_id(const orc_problem* pb, const int* pc) {
  int p = 0;
  for (int d = pb->dim - 1; d >= 0; --d) p = p * pb->np[d] + pc[d];
  return p;
}

static int is_dir(const orc_problem* pb, const int64_t* X) {
  for (int d = 0; d < pb->dim; ++d) {
    if (pb->dsides[2 * d] && X[d] == 0) return 1;
    if (pb->dsides[2 * d + 1] && X[d] == pb->n[d]) return 1;
  }
  return 0;
}

/* owner of a vertex: max owner over cells around it */
static int vert_owner(const orc_problem* pb, const int64_t* X) {
  int pc[3] = {0, 0, 0};
  for (int d = 0; d < pb->dim; ++d) {
    int best = -1;
    for (int64_t c = X[d] - 1; c <= X[d]; ++c)
      if (c >= 0 && c < pb->n[d]) {
        int q = cell_pc(pb, d, c);
        if (q > best) best = q;
      }
    pc[d] = best;
  }
  return part_id(pb, pc);
}

static int64_t vlin(const orc_problem* pb, const int64_t* X) {
  int64_t r = 0;
  for (int d = pb->dim - 1; d >= 0; --d) r = r * (pb->n[d] + 1) + X[d];
  return r;
}

/* 1D Gauss-Legendre on [0,1] by Newton iteration on the Legendre recurrence */
static void gauss01(int n, double* x, double* w) {
  for (int i = 0; i < n; ++i) {
    double z = cos(3.14159265358979323846 * (i + 0.75) / (n + 0.5)), pp = 0;
    for (int it = 0; it < 100; ++it) {
      double p1 = 1, p2 = 0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2.0 * j - 1) * z * p2 - (j - 1.0) * p3) / j;
      }
      pp = n * (z * p1 - p2) / (z * z - 1);
      double dz = p1 / pp;
      z -= dz;
      if (fabs(dz) < 1e-16) break;
    }
    x[n - 1 - i] = 0.5 * (z + 1);
    w[n - 1 - i] = 1.0 / ((1 - z * z) * pp * pp);
  }
}

typedef struct {
  int64_t i, j;   /* global ids during routing, local ids after */
  int32_t jo;
  double v;
  int64_t k;      /* COO position (stable duplicate order) */
} trip_t;

typedef struct {
  trip_t* t;
  int64_t n, cap;
} tvec;

static void tpush(tvec* a, trip_t x) {
  if (a->n == a->cap) {
    a->cap = a->cap ? 2 * a->cap : 1024;
    a->t = (trip_t*)realloc(a->t, sizeof(trip_t) * a->cap);
  }
  a->t[a->n++] = x;
}

static int cmp_trip(const void* a, const void* b) {
  const trip_t* x = (const trip_t*)a;
  const trip_t* y = (const trip_t*)b;
  if (x->i != y->i) return x->i < y->i ? -1 : 1;
  if (x->j != y->j) return x->j < y->j ? -1 : 1;
  return x->k < y->k ? -1 : (x->k > y->k);
}

/* simple open-addressing hash gid -> int */
typedef struct {
  int64_t* key;
  int64_t* val;
  int64_t cap;
} hmap;
static void hinit(hmap* h, int64_t n) {
  h->cap = 1;
  while (h->cap < 2 * n + 16) h->cap <<= 1;
  h->key = (int64_t*)malloc(sizeof(int64_t) * h->cap);
  h->val = (int64_t*)malloc(sizeof(int64_t) * h->cap);
  for (int64_t i = 0; i < h->cap; ++i) h->key[i] = -1;
}
static int64_t* hslot(hmap* h, int64_t k) {
  uint64_t x = (uint64_t)k * 0x9E3779B97F4A7C15ull;
  int64_t s = (int64_t)(x >> 17) & (h->cap - 1);
  while (h->key[s] != -1 && h->key[s] != k) s = (s + 1) & (h->cap - 1);
  return &h->key[s];
}
static int hget(hmap* h, int64_t k, int64_t* v) {
  int64_t* ks = hslot(h, k);
  if (*ks == -1) return 0;
  *v = h->val[ks - h->key];
  return 1;
}
static void hput(hmap* h, int64_t k, int64_t v) {
  int64_t* ks = hslot(h, k);
  *ks = k;
  h->val[ks - h->key] = v;
}
static void hfree(hmap* h) {
  free(h->key);
  free(h->val);
}

int orc_assemble(const orc_problem* pb, int strategy, int nthreads, orc_system** out, double* t_setup,
                 double* t_assembly) {
  const int dim = pb->dim;
  int nparts = 1;
  for (int d = 0; d < dim; ++d) nparts *= pb->np[d];
  double t0 = now_s();
  part_t* P = (part_t*)calloc(nparts, sizeof(part_t));
  /* ---- setup: partition, local numbering, gids ---- */
  for (int p = 0; p < nparts; ++p) {
    int pc[3] = {0, 0, 0}, rest = p;
    for (int d = 0; d < dim; ++d) {
      pc[d] = rest % pb->np[d];
      rest /= pb->np[d];
    }
    P[p].nverts = 1;
    for (int d = 0; d < 3; ++d) {
      P[p].own_lo[d] = P[p].loc_lo[d] = 0;
      P[p].own_hi[d] = P[p].loc_hi[d] = 1;
      P[p].nb[d] = 1;
    }
    for (int d = 0; d < dim; ++d) {
      local_range(pc[d] + 1, pb->np[d], pb->n[d], 0, &P[p].own_lo[d], &P[p].own_hi[d]);
      local_range(pc[d] + 1, pb->np[d], pb->n[d], 1, &P[p].loc_lo[d], &P[p].loc_hi[d]);
      P[p].nb[d] = P[p].loc_hi[d] - P[p].loc_lo[d] + 1;
      P[p].nverts *= P[p].nb[d];
    }
    P[p].vert_lid = (int32_t*)malloc(sizeof(int32_t) * P[p].nverts);
    P[p].lid_vert = (int64_t*)malloc(sizeof(int64_t) * P[p].nverts);
    int64_t nf = 0;
    for (int64_t v = 0; v < P[p].nverts; ++v) {
      int64_t X[3] = {0, 0, 0}, r = v;
      for (int d = 0; d < dim; ++d) {
        X[d] = P[p].loc_lo[d] + r % P[p].nb[d];
        r /= P[p].nb[d];
      }
      if (is_dir(pb, X)) {
        P[p].vert_lid[v] = -1;
      } else {
        P[p].vert_lid[v] = (int32_t)nf;
        P[p].lid_vert[nf++] = vlin(pb, X);
      }
    }
    P[p].nfree = nf;
    P[p].lid_owner = (int32_t*)malloc(sizeof(int32_t) * (nf + 1));
    P[p].lid_gid = (int64_t*)malloc(sizeof(int64_t) * (nf + 1));
    P[p].n_own = 0;
    for (int64_t l = 0; l < nf; ++l) {
      int64_t X[3] = {0, 0, 0}, r = P[p].lid_vert[l];
      for (int d = 0; d < dim; ++d) {
        X[d] = r % (pb->n[d] + 1);
        r /= (pb->n[d] + 1);
      }
      P[p].lid_owner[l] = vert_owner(pb, X);
      if (P[p].lid_owner[l] == p) P[p].lid_gid[l] = P[p].n_own++;
    }
  }
  int64_t ng = 0;
  for (int p = 0; p < nparts; ++p) {
    P[p].first_gdof = ng;
    ng += P[p].n_own;
  }
  for (int p = 0; p < nparts; ++p)
    for (int64_t l = 0; l < P[p].nfree; ++l)
      if (P[p].lid_owner[l] == p) P[p].lid_gid[l] += P[p].first_gdof;
  for (int p = 0; p < nparts; ++p)
    for (int64_t l = 0; l < P[p].nfree; ++l) {
      int q = P[p].lid_owner[l];
      if (q == p) continue;
      int64_t X[3] = {0, 0, 0}, r = P[p].lid_vert[l], li = 0;
      for (int d = 0; d < dim; ++d) {
        X[d] = r % (pb->n[d] + 1);
        r /= (pb->n[d] + 1);
      }
      for (int d = dim - 1; d >= 0; --d) li = li * P[q].nb[d] + (X[d] - P[q].loc_lo[d]);
      P[p].lid_gid[l] = P[q].lid_gid[P[q].vert_lid[li]];
    }
  double t1 = now_s();

  /* ---- assembly ---- */
  double h[3] = {1, 1, 1};
  for (int d = 0; d < dim; ++d) h[d] = (pb->domain[2 * d + 1] - pb->domain[2 * d]) / pb->n[d];
  int nq = (pb->degree + 2) / 2;
  double xq[16], wq[16];
  gauss01(nq, xq, wq);
  const int ne = 1 << dim;
  tvec* coo = (tvec*)calloc(nparts, sizeof(tvec));
  double** bl = (double**)calloc(nparts, sizeof(double*));
  char** touched = (char**)calloc(nparts, sizeof(char*));
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
  for (int p = 0; p < nparts; ++p) {
    part_t* Q = &P[p];
    bl[p] = (double*)calloc(Q->nfree + 1, sizeof(double));
    touched[p] = (char*)calloc(Q->nfree + 1, 1);
    int64_t mc[3] = {1, 1, 1}, lo[3] = {0, 0, 0};
    for (int d = 0; d < dim; ++d) {
      if (strategy == 0) {
        lo[d] = Q->own_lo[d];
        mc[d] = Q->own_hi[d] - Q->own_lo[d];
      } else {
        lo[d] = Q->loc_lo[d];
        mc[d] = Q->loc_hi[d] - Q->loc_lo[d];
      }
    }
    int64_t ncell = mc[0] * mc[1] * mc[2];
    int64_t k = 0;
    for (int64_t cl = 0; cl < ncell; ++cl) {
      int64_t c[3] = {0, 0, 0}, r = cl;
      for (int d = 0; d < dim; ++d) {
        c[d] = lo[d] + r % mc[d];
        r /= mc[d];
      }
      int64_t cg = 0;
      for (int d = dim - 1; d >= 0; --d) cg = cg * pb->n[d] + c[d];
      double kap = pb->kappa ? pb->kappa[cg] : 1.0;
      int32_t dofs[8];
      for (int a = 0; a < ne; ++a) {
        int64_t li = 0;
        for (int d = dim - 1; d >= 0; --d) li = li * Q->nb[d] + (c[d] + ((a >> d) & 1) - Q->loc_lo[d]);
        dofs[a] = Q->vert_lid[li];
      }
      /* element matrix / vector by quadrature (per cell, as integrate does) */
      double Ke[64], be[8];
      memset(Ke, 0, sizeof(Ke));
      memset(be, 0, sizeof(be));
      int nqt = 1;
      for (int d = 0; d < dim; ++d) nqt *= nq;
      for (int q = 0; q < nqt; ++q) {
        int qi[3] = {0, 0, 0}, rq = q;
        for (int d = 0; d < dim; ++d) {
          qi[d] = rq % nq;
          rq /= nq;
        }
        double w = 1, phi[8], grad[8][3];
        for (int d = 0; d < dim; ++d) w *= wq[qi[d]] * h[d];
        for (int a = 0; a < ne; ++a) {
          double v = 1;
          for (int d = 0; d < dim; ++d) {
            double x = xq[qi[d]];
            v *= ((a >> d) & 1) ? x : 1 - x;
          }
          phi[a] = v;
          for (int d = 0; d < dim; ++d) {
            double g = (((a >> d) & 1) ? 1.0 : -1.0) / h[d];
            for (int e = 0; e < dim; ++e)
              if (e != d) {
                double x = xq[qi[e]];
                g *= ((a >> e) & 1) ? x : 1 - x;
              }
            grad[a][d] = g;
          }
        }
        for (int i = 0; i < ne; ++i) {
          be[i] += w * pb->f_const * phi[i];
          for (int j = 0; j < ne; ++j) {
            double s = 0;
            for (int d = 0; d < dim; ++d) s += grad[i][d] * grad[j][d];
            Ke[i * ne + j] += w * kap * s;
          }
        }
      }
      for (int j = 0; j < ne; ++j) {
        if (dofs[j] < 0) continue;
        for (int i = 0; i < ne; ++i) {
          if (dofs[i] < 0) continue;
          if (strategy == 1 && Q->lid_owner[dofs[i]] != p) continue;
          trip_t t = {dofs[i], dofs[j], 0, Ke[i * ne + j], k++};
          tpush(&coo[p], t);
        }
      }
      for (int i = 0; i < ne; ++i) {
        if (dofs[i] < 0) continue;
        if (strategy == 1 && Q->lid_owner[dofs[i]] != p) continue;
        bl[p][dofs[i]] += be[i];
        touched[p][dofs[i]] = 1;
      }
    }
    /* to global ids + column owners */
    for (int64_t t = 0; t < coo[p].n; ++t) {
      trip_t* x = &coo[p].t[t];
      x->jo = Q->lid_owner[x->j];
      x->i = Q->lid_gid[x->i];
      x->j = Q->lid_gid[x->j];
    }
  }

  orc_system* S = (orc_system*)calloc(1, sizeof(orc_system));
  S->nparts = nparts;
  S->ngdofs = ng;
  S->nrows = (int64_t*)calloc(nparts, sizeof(int64_t));
  S->ncols = (int64_t*)calloc(nparts, sizeof(int64_t));
  S->nnz = (int64_t*)calloc(nparts, sizeof(int64_t));
  S->rowptr = (int64_t**)calloc(nparts, sizeof(int64_t*));
  S->colidx = (int64_t**)calloc(nparts, sizeof(int64_t*));
  S->vals = (double**)calloc(nparts, sizeof(double*));
  S->b = (double**)calloc(nparts, sizeof(double*));
  S->row_ghost_gid = (int64_t**)calloc(nparts, sizeof(int64_t*));
  S->col_ghost_gid = (int64_t**)calloc(nparts, sizeof(int64_t*));
  S->n_ghost_rows = (int64_t*)calloc(nparts, sizeof(int64_t));
  S->n_ghost_cols = (int64_t*)calloc(nparts, sizeof(int64_t));

  /* gid -> owner and gid -> lid on owner (global tables; the exchange moves data) */
  int32_t* gowner = (int32_t*)malloc(sizeof(int32_t) * (ng + 1));
  for (int p = 0; p < nparts; ++p)
    for (int64_t l = 0; l < P[p].nfree; ++l)
      if (P[p].lid_owner[l] == p) gowner[P[p].lid_gid[l]] = p;

  /* ghost rows (SA): touched non-owned lids in lid order; RHS ghost contributions */
  double* bglob = (double*)calloc(ng + 1, sizeof(double));
  for (int p = 0; p < nparts; ++p)
    for (int64_t l = 0; l < P[p].nfree; ++l)
      if (touched[p][l]) bglob[P[p].lid_gid[l]] += bl[p][l];

  /* triplet routing: send ghost-row triplets (in COO order) to their owners */
  tvec* recv = (tvec*)calloc(nparts * nparts, sizeof(tvec)); /* recv[q*nparts+p]: from p to q */
  if (strategy == 0) {
    for (int p = 0; p < nparts; ++p)
      for (int64_t t = 0; t < coo[p].n; ++t) {
        trip_t* x = &coo[p].t[t];
        int q = gowner[x->i];
        if (q != p) {
          tpush(&recv[q * nparts + p], *x);
          x->v = 0.0;
        }
      }
  }
#pragma omp parallel for schedule(dynamic, 1)
  for (int q = 0; q < nparts; ++q) {
    part_t* Q = &P[q];
    if (strategy == 0)   /* received triplets appended in ascending sender order */
      for (int p = 0; p < nparts; ++p)
        for (int64_t t = 0; t < recv[q * nparts + p].n; ++t) {
          trip_t x = recv[q * nparts + p].t[t];
          x.k = coo[q].n;
          tpush(&coo[q], x);
        }
    /* rows */
    hmap rmap, cmap;
    hinit(&rmap, Q->nfree + 16);
    hinit(&cmap, Q->nfree + coo[q].n / 4 + 16);
    int64_t nown = Q->n_own;
    for (int64_t i = 0; i < nown; ++i) {
      hput(&rmap, Q->first_gdof + i, i);
      hput(&cmap, Q->first_gdof + i, i);
    }
    int64_t ngr = 0;
    int64_t* rg = (int64_t*)malloc(sizeof(int64_t) * (Q->nfree + 1));
    if (strategy == 0) {
      char* tr = (char*)calloc(Q->nfree + 1, 1);
      for (int64_t l = 0; l < Q->nfree; ++l)
        if (touched[q][l] && Q->lid_owner[l] != q) tr[l] = 1;
      for (int64_t l = 0; l < Q->nfree; ++l)
        if (tr[l]) {
          rg[ngr] = Q->lid_gid[l];
          hput(&rmap, rg[ngr], nown + ngr);
          ++ngr;
        }
      free(tr);
    }
    /* columns */
    int64_t ngc = 0, cgcap = 1024;
    int64_t* cg = (int64_t*)malloc(sizeof(int64_t) * cgcap);
    if (strategy == 0) {
      for (int64_t t = 0; t < coo[q].n; ++t) {
        trip_t* x = &coo[q].t[t];
        int64_t dummy;
        if (x->jo != q && !hget(&cmap, x->j, &dummy)) {
          if (ngc == cgcap) cg = (int64_t*)realloc(cg, sizeof(int64_t) * (cgcap *= 2));
          cg[ngc] = x->j;
          hput(&cmap, x->j, nown + ngc);
          ++ngc;
        }
      }
    } else {
      char* tc = (char*)calloc(Q->nfree + 1, 1);
      hmap g2l;
      hinit(&g2l, Q->nfree);
      for (int64_t l = 0; l < Q->nfree; ++l) hput(&g2l, Q->lid_gid[l], l);
      for (int64_t t = 0; t < coo[q].n; ++t) {
        int64_t l;
        if (coo[q].t[t].jo != q && hget(&g2l, coo[q].t[t].j, &l)) tc[l] = 1;
      }
      for (int64_t l = 0; l < Q->nfree; ++l)
        if (tc[l]) {
          if (ngc == cgcap) cg = (int64_t*)realloc(cg, sizeof(int64_t) * (cgcap *= 2));
          cg[ngc] = Q->lid_gid[l];
          hput(&cmap, cg[ngc], nown + ngc);
          ++ngc;
        }
      hfree(&g2l);
      free(tc);
    }
    /* to local ids, compress (sort by row, col, COO order; sum duplicates) */
    for (int64_t t = 0; t < coo[q].n; ++t) {
      trip_t* x = &coo[q].t[t];
      int64_t li = -1, lj = -1;
      hget(&rmap, x->i, &li);
      hget(&cmap, x->j, &lj);
      x->i = li;
      x->j = lj;
    }
    qsort(coo[q].t, coo[q].n, sizeof(trip_t), cmp_trip);
    int64_t nrows = nown + ngr;
    int64_t* rp = (int64_t*)calloc(nrows + 1, sizeof(int64_t));
    int64_t* ci = (int64_t*)malloc(sizeof(int64_t) * (coo[q].n + 1));
    double* vv = (double*)malloc(sizeof(double) * (coo[q].n + 1));
    int64_t nz = 0;
    for (int64_t t = 0; t < coo[q].n; ++t) {
      trip_t* x = &coo[q].t[t];
      if (nz > 0 && t > 0 && x->i == coo[q].t[t - 1].i && x->j == coo[q].t[t - 1].j) {
        vv[nz - 1] += x->v;
      } else {
        ci[nz] = x->j;
        vv[nz] = x->v;
        rp[x->i + 1]++;
        ++nz;
      }
    }
    for (int64_t r = 0; r < nrows; ++r) rp[r + 1] += rp[r];
    double* b = (double*)calloc(nrows + 1, sizeof(double));
    if (strategy == 0) {
      for (int64_t i = 0; i < nown; ++i) b[i] = bglob[Q->first_gdof + i];
    } else {
      int64_t o = 0;
      for (int64_t l = 0; l < Q->nfree; ++l)
        if (Q->lid_owner[l] == q) b[o++] = bl[q][l];
    }
    S->nrows[q] = nrows;
    S->ncols[q] = nown + ngc;
    S->nnz[q] = nz;
    S->rowptr[q] = rp;
    S->colidx[q] = ci;
    S->vals[q] = vv;
    S->b[q] = b;
    S->row_ghost_gid[q] = rg;
    S->col_ghost_gid[q] = cg;
    S->n_ghost_rows[q] = ngr;
    S->n_ghost_cols[q] = ngc;
    hfree(&rmap);
    hfree(&cmap);
  }
  double t2 = now_s();
  for (int i = 0; i < nparts * nparts; ++i) free(recv[i].t);
  free(recv);
  for (int p = 0; p < nparts; ++p) {
    free(coo[p].t);
    free(bl[p]);
    free(touched[p]);
    free(P[p].vert_lid);
    free(P[p].lid_vert);
    free(P[p].lid_owner);
    free(P[p].lid_gid);
  }
  free(coo);
  free(bl);
  free(touched);
  free(P);
  free(gowner);
  free(bglob);
  if (t_setup) *t_setup = t1 - t0;
  if (t_assembly) *t_assembly = t2 - t1;
  *out = S;
  return 0;
}

void orc_free(orc_system* S) {
  if (!S) return;
  for (int p = 0; p < S->nparts; ++p) {
    free(S->rowptr[p]);
    free(S->colidx[p]);
    free(S->vals[p]);
    free(S->b[p]);
    free(S->row_ghost_gid[p]);
    free(S->col_ghost_gid[p]);
  }
  free(S->rowptr);
  free(S->colidx);
  free(S->vals);
  free(S->b);
  free(S->row_ghost_gid);
  free(S->col_ghost_gid);
  free(S->n_ghost_rows);
  free(S->n_ghost_cols);
  free(S->nrows);
  free(S->ncols);
  free(S->nnz);
  free(S);
}

/* Jacobi-PCG in FP64 on the gathered global matrix (owned rows, global columns). */
int orc_pcg(int64_t n, const int64_t* rowptr, const int64_t* col, const double* val, const double* b, double rtol,
            int maxit, int nthreads, double* x, int* iters, double* rel) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  double* r = (double*)malloc(sizeof(double) * n);
  double* z = (double*)malloc(sizeof(double) * n);
  double* p = (double*)malloc(sizeof(double) * n);
  double* q = (double*)malloc(sizeof(double) * n);
  double* dinv = (double*)malloc(sizeof(double) * n);
  double bb = 0, rz = 0, rr = 0;
#pragma omp parallel for reduction(+ : bb, rz, rr)
  for (int64_t i = 0; i < n; ++i) {
    double d = 0;
    for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e)
      if (col[e] == i) d = val[e];
    dinv[i] = 1.0 / d;
    x[i] = 0;
    r[i] = b[i];
    z[i] = dinv[i] * r[i];
    p[i] = z[i];
    bb += b[i] * b[i];
    rz += r[i] * z[i];
    rr += r[i] * r[i];
  }
  double bn = sqrt(bb);
  int it = 0;
  while (sqrt(rr) > rtol * bn && it < maxit) {
    double pq = 0;
#pragma omp parallel for reduction(+ : pq)
    for (int64_t i = 0; i < n; ++i) {
      double s = 0;
      for (int64_t e = rowptr[i]; e < rowptr[i + 1]; ++e) s += val[e] * p[col[e]];
      q[i] = s;
      pq += p[i] * s;
    }
    double alpha = rz / pq, rz2 = 0;
    rr = 0;
#pragma omp parallel for reduction(+ : rz2, rr)
    for (int64_t i = 0; i < n; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dinv[i] * r[i];
      rz2 += r[i] * z[i];
      rr += r[i] * r[i];
    }
    double beta = rz2 / rz;
    rz = rz2;
#pragma omp parallel for
    for (int64_t i = 0; i < n; ++i) p[i] = z[i] + beta * p[i];
    ++it;
  }
  *iters = it;
  *rel = sqrt(rr) / bn;
  free(r);
  free(z);
  free(p);
  free(q);
  free(dinv);
  return 0;
}
