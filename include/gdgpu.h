/*
 * gdgpu.h -- C ABI of the GB300 assembly-and-solve library (libgdgpu.so).
 *
 * The library replaces, for Cartesian meshes, the path
 *   CartesianDiscreteModel(ranks, parts, domain, cells)
 *   -> TestFESpace / TrialFESpace
 *   -> SparseMatrixAssembler(U, V, strategy)
 *   -> assemble_matrix_and_vector (-> PSparseMatrix / PVector)
 *   -> A \ b
 * of GridapDistributed.jl.  Every part of the mesh partition lives on one GPU as a
 * slab of device memory; the PartitionedArrays exchanges become device
 * gather/scatter kernels.
 *
 * Conventions
 *  - Every function returns an int status (GD_OK = 0).  On failure a message is
 *    kept per host thread and returned by gd_last_error().  No exception crosses
 *    the ABI, nothing calls exit/abort.
 *  - Indices are 0-based.  Global DOF ids are int64, part ids and local ids int32.
 *    (The Julia side adds 1 to obtain PartitionedArrays' 1-based ids.)
 *  - Parts are numbered x-fastest (Julia's CartesianIndices(parts) order).
 *    Cells and lattice nodes are numbered lexicographically, x fastest.  The
 *    "node lattice" of an order-k space has k*cells[d]+1 nodes along d.
 *  - Device memory belongs to the object that allocated it and is freed by the
 *    matching *_destroy.  Host buffers are owned by the caller and are only
 *    read or written during the call.  Export functions accept NULL for any
 *    output they should skip; query sizes first with gd_matrix_sizes.
 *  - All device work is ordered on the context's stream.  Calls return after
 *    the stream has been synchronised unless their comment says otherwise.
 */
#ifndef GDGPU_H
#define GDGPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
enum {
  GD_OK = 0,
  GD_ERR_ARG = 1,          /* invalid argument (sizes, pointers, ranges)              */
  GD_ERR_OOM = 2,          /* device or host allocation failed                        */
  GD_ERR_CUDA = 3,         /* a CUDA runtime call failed                              */
  GD_ERR_TIMEOUT = 4,      /* a bounded device wait ran out                           */
  GD_ERR_STALL = 5,        /* iterative solve stalled (the fallback result is kept)   */
  GD_ERR_STATE = 6,        /* call out of order (e.g. numeric before symbolic)        */
  GD_ERR_UNSUPPORTED = 7,  /* configuration not built                                 */
  GD_ERR_NUMERIC = 8,      /* NaN / Inf / non-positive coefficient in the input       */
  GD_ERR_NOTCONVERGED = 9  /* maximum iterations reached before the tolerance         */
};
/* Every function returns one of these (gd_last_error() and gd_version() return text).
 * A null handle or a null required pointer is GD_ERR_ARG; a valid handle used out of
 * order is GD_ERR_STATE; the *_destroy functions accept NULL and do nothing. */

/* Assembly strategies (src/Algebra.jl:397-398). */
enum { GD_SUB_ASSEMBLED_ROWS = 0, GD_FULLY_ASSEMBLED_ROWS = 1 };

/* Solver methods behind `\` (the reference's own is a gathered sparse LU).
 * JACOBI_PCG: FP64 Jacobi-preconditioned CG.
 * MIXED_IR: FP64 iterative refinement (true residual b - Ax with the assembled FP64
 *   matrix) around FP32 Jacobi-PCG with FP64 inner products and step lengths; for Q1 on
 *   cube cells the inner operator is applied matrix-free. */
enum { GD_SOLVE_JACOBI_PCG = 1, GD_SOLVE_MIXED_IR = 2 };

/* Where a coefficient/input pointer lives. */
enum { GD_HOST = 0, GD_DEVICE = 1 };

typedef struct gd_ctx gd_ctx;
typedef struct gd_model gd_model;
typedef struct gd_space gd_space;
typedef struct gd_asm gd_asm;

/* Thread-local message of the last failed call on this host thread ("" if none). */
const char* gd_last_error(void);

/* Library version string. */
const char* gd_version(void);

/* ---- context --------------------------------------------------------------- */
/* A context owns one CUDA device and one stream.  No reference counterpart: it
 * stands in for the `ranks` array handed to every constructor (with_debug's
 * DebugArray), since all parts of the partition live on this device. */
int gd_ctx_create(int device, gd_ctx** out);
int gd_ctx_destroy(gd_ctx* ctx);
/* Order all subsequent work of `ctx` on an externally owned cudaStream_t
 * (NULL restores the context's own stream). */
int gd_ctx_set_stream(gd_ctx* ctx, void* cuda_stream);
int gd_ctx_synchronize(gd_ctx* ctx);

/* ---- A1: CartesianDiscreteModel(ranks, parts, domain, cells) ---------------
 * Replaces Geometry.jl:378-411 and _uniform_partition / _block_with_constant_size
 * / _local_range (PArraysExtras.jl:5-84): block partition of `cells` into
 * `parts` with a one-cell ghost layer.  Non-periodic only.
 * domain = (x0,x1,y0,y1[,z0,z1]); dim = 2 or 3.                                  */
int gd_model_cartesian(gd_ctx* ctx, int dim, const int64_t* cells, const int32_t* parts,
                       const double* domain, gd_model** out);
int gd_model_destroy(gd_model* model);
int gd_model_num_parts(const gd_model* model, int32_t* nparts);
/* Owned and local (owned+ghost) cell boxes of `part`, 0-based half-open
 * [lo, hi) per direction (each array has `dim` entries). */
int gd_model_part_boxes(const gd_model* model, int part, int64_t* own_lo, int64_t* own_hi,
                        int64_t* loc_lo, int64_t* loc_hi);

/* ---- A3-A5: TestFESpace / TrialFESpace ---------------------------------------
 * Replaces FESpaces.jl:570-614 (per-part Lagrangian Q_k space on owned+ghost
 * cells, Gridap's conforming numbering) and generate_gids (FESpaces.jl:139-261).
 * dirichlet_sides[2*d] / [2*d+1] flag the planes x_d = min / max; a node on a
 * flagged plane is a Dirichlet node ("boundary" = all flags set).
 * Scalar spaces (ncomp = 1), order 1..3, or vector spaces (ncomp = dim, the
 * ReferenceFE(lagrangian, VectorValue{dim,Float64}, k) of the reference), order 1..2,
 * all components sharing the Dirichlet sides; their dofs are numbered
 * ncomp * (node dof) + component, which is Gridap's component-major numbering of each
 * face's own DOFs when every face owns one node.                                   */
int gd_space_create(gd_model* model, int order, int ncomp, const int32_t* dirichlet_sides,
                    gd_space** out);
int gd_space_destroy(gd_space* space);
/* num_free_dofs(V) (global). */
int gd_space_num_free_dofs(const gd_space* space, int64_t* n);
/* Local sizes of one part: local free DOFs, owned DOFs, first owned gid. */
int gd_space_local_sizes(const gd_space* space, int part, int64_t* nldofs, int64_t* nown,
                         int64_t* first_gdof);
/* LocalIndices of one part: ldof -> gid and ldof -> owner (FESpaces.jl:248-258). */
int gd_space_get_gids(const gd_space* space, int part, int64_t* ldof_to_gdof,
                      int32_t* ldof_to_owner);
/* Global lattice node index of every local free DOF of one part. */
int gd_space_dof_nodes(const gd_space* space, int part, int64_t* ldof_to_node);
/* TrialFESpace(u, V) (FESpaces.jl:396-401): Dirichlet values as a dense array
 * over the global node lattice (only Dirichlet nodes are read); NULL = zero.  On a
 * vector space, ncomp values per node, the components of a node together
 * (u_lattice[ncomp * node + c]). */
int gd_space_set_dirichlet(gd_space* space, const double* u_lattice, int where);

/* ---- A9-A13: SparseMatrixAssembler + assemble_matrix_and_vector --------------
 * Replaces DistributedSparseMatrixAssembler (FESpaces.jl:746-862) and the
 * PSparseMatrixBuilderCOO / PVectorBuilder protocol with create_from_nz
 * (Algebra.jl:405-907): SubAssembledRows (ghost rows kept with explicit zeros,
 * ghost columns in first-appearance order) or FullyAssembledRows (no ghost rows,
 * ghost columns sorted by local DOF id).                                          */
int gd_assembler_create(gd_space* trial, gd_space* test, int strategy, gd_asm** out);
int gd_assembler_destroy(gd_asm* a);
/* allocate_matrix_and_vector: builds row/col index sets and the local CSR
 * patterns of every part (Algebra.jl:593-646 without the values). */
int gd_assemble_symbolic(gd_asm* a);

/* Coefficients of a(u,v) = int(kappa grad(v).grad(u)) and l(v) = int(v f). */
typedef struct gd_coeffs {
  const double* kappa;   /* per global cell (lexicographic); NULL = 1        */
  const double* f_nodal; /* per global lattice node (load M*f); NULL = const */
  double f_const;        /* constant source when f_nodal is NULL             */
  int degree;            /* quadrature degree (tensor Gauss, (degree+2)/2 pts/dir) */
  int where;             /* GD_HOST or GD_DEVICE for the pointers above      */
} gd_coeffs;

/* assemble_matrix_and_vector! into the symbolic pattern: matrix values and the
 * right-hand side of every part.  Deterministic (no floating-point atomics). */
int gd_assemble_numeric(gd_asm* a, const gd_coeffs* c);
/* Same, without the final stream synchronisation (for timing loops).  A coefficient
 * that fails the check (not finite and positive) is reported by the next synchronous
 * numeric call of the assembler. */
int gd_assemble_numeric_async(gd_asm* a, const gd_coeffs* c);
/* assemble_vector(assem, collect_cell_vector(V, l)) for l(v) = int(v f) (Gridap's
 * assemble_vector, called at test/FESpacesTests.jl:65-69): the load vector without
 * Dirichlet lifting, over the owned rows in global order (length = free DOFs), into b
 * (where_b: GD_HOST or GD_DEVICE).  c->kappa is not used; the assembler's matrix values
 * and right-hand side are not changed.  Scalar spaces. */
int gd_assemble_vector(gd_asm* a, const gd_coeffs* c, double* b, int where_b);

/* Linear elasticity on a vector space (gd_space_create with ncomp = dim, orders 1-2):
 * a(u,v) = int C(E) eps(u):eps(v), isotropic C with Young's modulus E per cell and
 * Poisson ratio nu; l(v) = int v.force (constant body force).  Homogeneous Dirichlet
 * values on the space's Dirichlet sides (all components clamped). */
typedef struct gd_elasticity {
  const double* E;       /* per global cell (lexicographic); NULL = 1 */
  double nu;             /* Poisson ratio, -1 < nu < 0.5 */
  double force[3];       /* body force (components beyond dim ignored) */
  int degree;            /* quadrature degree (tensor Gauss) */
  int where;             /* GD_HOST or GD_DEVICE for E */
} gd_elasticity;
/* assemble_matrix_and_vector! for the elasticity forms into the symbolic pattern of a
 * vector-space assembler (dof = dim * node dof + component). */
int gd_assemble_elasticity(gd_asm* a, const gd_elasticity* c);

/* ---- A7 with coefficients that vary inside a cell --------------------------------------
 * integrate of an integrand built from a CellField known at the quadrature points
 * (src/CellData.jl:234-259, `*(Integrand, Measure)` at :255-259; a CellField from a
 * function of x or from per-point data): a(u,v) = int kappa(x) grad(v).grad(u) with
 * kappa given at the tensor Gauss points of every cell ((degree+2)/2 per direction,
 * at most 64 per cell): kappa_qp[cell * nq^dim + q], cells lexicographic, points x
 * fastest.  l(v) = int v f as in gd_coeffs.  Each element matrix is
 * K_e = sum_q kappa_q H_q; `precision` chooses how it is formed:
 *   GD_QP_FP64:   FP64 on the CUDA cores (matches an FP64 quadrature to rounding);
 *   GD_QP_BF16:   tensor cores (tcgen05, BF16 operands, FP32 accumulation), relative
 *                 error of the element entries about 1e-2 .. 1e-3;
 *   GD_QP_BF16X3: the same with each operand split into two BF16 terms (3 products),
 *                 about 1e-5;
 *   GD_QP_BF16X6: three BF16 terms (6 products), about FP32 rounding (1e-7 .. 1e-6).
 * The element matrices are kept in FP32 (FP64 for GD_QP_FP64) and summed into the
 * symbolic pattern deterministically; the matrix values are stored in FP64 as usual. */
enum { GD_QP_FP64 = 0, GD_QP_BF16 = 1, GD_QP_BF16X3 = 2, GD_QP_BF16X6 = 3 };
typedef struct gd_qp_coeffs {
  const double* kappa_qp; /* per global cell, nq^dim values at the Gauss points          */
  const double* f_nodal;  /* per global lattice node (load M*f); NULL = f_const         */
  double f_const;
  int degree;             /* quadrature degree                                           */
  int precision;          /* GD_QP_*                                                     */
  int where;              /* GD_HOST or GD_DEVICE for kappa_qp and f_nodal               */
} gd_qp_coeffs;
int gd_assemble_qp(gd_asm* a, const gd_qp_coeffs* c);
/* Linear elasticity (vector space, orders 1-2) with Young's modulus at the Gauss points
 * (E_qp in the layout of kappa_qp), constant nu and body force; homogeneous or the trial
 * space's Dirichlet values. */
typedef struct gd_elasticity_qp {
  const double* E_qp;
  double nu;
  double force[3];
  int degree;
  int precision;          /* GD_QP_*                                                     */
  int where;
} gd_elasticity_qp;
int gd_assemble_elasticity_qp(gd_asm* a, const gd_elasticity_qp* c);
/* Sizes of the last quadrature-point assembly: points per cell, element-matrix entries,
 * points padded to the tensor-core K step, 128-entry tiles; with gd_assembler_set_profiling
 * on, the event-timed ms of the element-matrix kernel and of the row kernel. */
int gd_qp_info(const gd_asm* a, int32_t* points, int32_t* entries, int32_t* kpad, int32_t* etiles,
               double* ms_element, double* ms_rows);

/* l(v) += int(v g) dGamma over the boundary sides flagged in `sides` (2*dim flags in the
 * order of dirichlet_sides; the Neumann term of test/PoissonTests.jl:20-41), added to
 * the owned rows of the assembled rhs -- call after gd_assemble_numeric.  g_qp holds g at
 * the face Gauss points ((degree+2)/2 per direction): faces side by side (flagged sides
 * in order x-, x+, y-, y+, z-, z+), on a side lexicographic over the face's cells in the
 * remaining directions (lowest first), points lowest remaining direction fastest.
 * Scalar spaces. */
int gd_add_boundary_source(gd_asm* a, const int32_t* sides, const double* g_qp, int degree, int where);

/* Record CUDA events around the phases of every numeric assembly (off by default). */
int gd_assembler_set_profiling(gd_asm* a, int on);
/* Event-timed durations (ms) of the last profiled numeric assembly: the coefficient
 * pre-scaling (k_prescale on 3D Q1 cube cells, empty otherwise), the matrix-value kernel,
 * the right-hand-side kernel (empty where the matrix kernel computes the rhs too). */
int gd_assembler_phase_times(const gd_asm* a, double* ms_ghost_zero, double* ms_matrix, double* ms_rhs);
/* Counts of the assembled system: global DOFs, stored entries of the owned rows,
 * stored entries of all rows (owned + ghost), and the kernels one numeric
 * assembly launches. */
int gd_assembler_counts(const gd_asm* a, int64_t* ngdofs, int64_t* nnz_owned, int64_t* nnz_total,
                        int32_t* kernels_per_numeric);

/* Launch shape the autotuner chose for the Q1 numeric kernel on the first numeric
 * assembly (-1 before it ran, or when the generic kernel is used): index, rows per
 * chunk, staging buffers, and the measured ms of each of the `nshapes` candidates (the
 * best of 5 timed launches, the candidates timed in turn after one warm-up round). */
int gd_assembler_tuning(const gd_asm* a, int32_t* shape, int32_t* rows, int32_t* nbuf, float* ms_per_shape,
                        int32_t* nshapes);
/* Fix the launch shape of the Q1 numeric kernel (0 .. nshapes-1 of gd_assembler_tuning)
 * for the following numeric assemblies, or -1 to have the next one time every shape
 * again.  Every shape writes the same values; this exists to check that.  GD_ERR_UNSUPPORTED
 * when the assembler does not use the Q1 kernel. */
int gd_assembler_set_shape(gd_asm* a, int shape);
/* 2D Q_k rows (k = 2, 3): on != 0 (the default) forms each entry as one reference value
 * times the sum of the coefficients of the cells that hold both nodes, when the reference
 * tables are invariant under the square's reflections (checked); 0 sums the cells' terms
 * one by one.  The two agree to rounding; this exists to compare them. */
int gd_assembler_set_class_sums(gd_asm* a, int on);

/* Sizes of one part's local matrix: rows (owned + ghost), columns (owned + ghost),
 * stored entries, ghost rows, ghost columns. */
int gd_matrix_sizes(const gd_asm* a, int part, int64_t* nrows, int64_t* ncols, int64_t* nnz,
                    int64_t* n_ghost_rows, int64_t* n_ghost_cols);
/* One part of the PSparseMatrix: local CSR (rowptr[nrows+1], colidx[nnz],
 * vals[nnz], columns sorted within a row) plus the ghost parts of its row and
 * column OwnAndGhostIndices (owned gids are first_gdof .. first_gdof+nown-1). */
int gd_matrix_export(const gd_asm* a, int part, int64_t* rowptr, int32_t* colidx, double* vals,
                     int64_t* ghost_row_gids, int32_t* ghost_row_owners, int64_t* ghost_col_gids,
                     int32_t* ghost_col_owners);
/* One part of the PVector over the matrix rows (ghost entries are zero after
 * assemble!, Algebra.jl:786-789). */
int gd_vector_export(const gd_asm* a, int part, double* b);
/* Device pointers of the assembled system seen as one global CSR over the
 * owned rows (gid order): rowptr (int64, ngdofs+1), global column ids (int32),
 * values (double), rhs (double, ngdofs).  Valid until the assembler is destroyed. */
int gd_system_device_ptrs(const gd_asm* a, const int64_t** rowptr, const int32_t** colidx,
                          const double** vals, const double** rhs, int64_t* ngdofs);
/* Copy the global rhs (ngdofs) and optionally all owned-row values to host. */
int gd_system_download(const gd_asm* a, double* rhs, double* owned_vals);
/* gd_assemble_numeric followed by gd_system_download (either host pointer may be NULL),
 * the download overlapped with the assembly where the Q1 kernel assembles the rows
 * (it runs over 8 ranges of owned rows; each range's values and rhs are copied to the
 * host on a second stream while the next range is assembled).  Same results as the two
 * calls; the copies are complete when it returns.  Host buffers should be pinned. */
int gd_assemble_download(gd_asm* a, const gd_coeffs* coeffs, double* rhs, double* owned_vals);

/* ---- A14-A16: mul!, `\`, FEFunction ------------------------------------------ */
/* y = A*x over global vectors (ngdofs), PSparseMatrix mul! semantics. */
int gd_spmv(gd_asm* a, const double* x, double* y, int where);

typedef struct gd_solve_stats {
  int32_t iterations;
  int32_t converged;
  double rel_residual;   /* ||b - A x|| / ||b|| recomputed in FP64 at exit */
  double seconds;
} gd_solve_stats;
/* x = A \ b for the assembled rhs, Jacobi-preconditioned CG in FP64 to the
 * relative residual rtol.  x: global vector (ngdofs). */
int gd_solve(gd_asm* a, int method, double rtol, int maxit, double* x, int where,
             gd_solve_stats* stats);
/* x = A \ b for a caller-given right-hand side b (ngdofs, gid order); same methods
 * and arguments as gd_solve. */
int gd_solve_rhs(gd_asm* a, int method, double rtol, int maxit, const double* b, double* x, int where,
                 gd_solve_stats* stats);
/* gd_solve without device allocation.  No counterpart in the reference: for callers
 * that cannot allocate device memory while they run (an application whose device
 * memory belongs to its own pool allocator, or a loop where a cudaMalloc -- which can
 * synchronise the device or fail mid-run -- is not acceptable).  The Jacobi-PCG
 * iteration of gd_solve (same steps, restarts and stopping rule; the matrix kernel is
 * the CSR one, where gd_solve uses a sliced-ELL copy for short rows) with the same
 * arguments; all scratch lives in one file-scope device array of fixed size (about
 * 12.6 MB per device that loads the library, held until the process exits).  At most
 * 262,144 global DOFs: larger systems return GD_ERR_ARG.  Each call looks the array's
 * address up with the assembler's device current and restores the caller's current
 * device before it returns.  Every call shares the array and clears what must start at
 * zero; calls that overlap on the GPU race on it. */
int gd_solve_noalloc(gd_asm* a, double rtol, int maxit, double* x, int where, gd_solve_stats* stats);
/* sqrt(sum(int(abs2(u - u_h)) dOmega)) (test/PoissonTests.jl:43-45): u_h = FEFunction(U, x)
 * with x the global free values (dim components interleaved on vector spaces) and the
 * trial space's Dirichlet values; u_qp the exact solution at the tensor Gauss points
 * ((degree+2)/2 per direction, on [0,1] mapped to each cell) of every global cell:
 * index (cell * nq^dim + q) * ncomp + component, cells lexicographic, points x fastest.
 * `where` applies to x and u_qp. */
int gd_l2_error(gd_space* space, const double* x, const double* u_qp, int degree, int where, double* err);
/* FEFunction(U, x) / consistent!: the local (owned+ghost) free values of one part
 * from a global vector (FESpaces.jl:354-371, Algebra.jl:270-293). */
int gd_fe_function_local(const gd_space* space, int part, const double* x_global, int where,
                         double* x_local);

/* ---- batched assembly and solve of many problems ------------------------------
 * No counterpart in the reference (one problem per assemble_matrix_and_vector call).
 * A batch holds assemblers whose symbolic phase is done (any order 1..3, 2D or 3D,
 * one shared context) with their coefficients.  gd_batch_assemble fills every
 * problem's matrix and vector (what gd_assemble_numeric would, same values) in ONE
 * persistent kernel launch with dynamic row-task scheduling; the first call times
 * the candidate launch shapes, keeps the fastest and captures the launch in a CUDA
 * graph that later calls replay.  gd_batch_solve runs Jacobi-PCG in FP64 on every
 * problem at once (one launch per CG step for all unconverged problems, sixteen steps
 * per CUDA graph replay). */
typedef struct gd_batch gd_batch;
int gd_batch_create(gd_asm* const* assemblers, const gd_coeffs* coeffs, int nprobs, gd_batch** out);
int gd_batch_destroy(gd_batch* b);
int gd_batch_assemble(gd_batch* b);
/* Same, without the final stream synchronisation and coefficient check (timing loops). */
int gd_batch_assemble_async(gd_batch* b);
int gd_batch_counts(const gd_batch* b, int32_t* nprobs, int64_t* rows, int64_t* nnz_owned);
/* Chosen launch shape (index, rows per task, CTAs per SM) and the measured ms of each
 * candidate (nshapes of them); -1 before the first assembly. */
int gd_batch_tuning(const gd_batch* b, int32_t* shape, int32_t* rows_per_task, int32_t* ctas_per_sm,
                    float* ms_per_shape, int32_t* nshapes);
/* stats: one entry per problem (may be NULL). */
int gd_batch_solve(gd_batch* b, double rtol, int maxit, gd_solve_stats* stats);
/* Solution of problem p (its ngdofs values, gid order) after gd_batch_solve. */
int gd_batch_solution(const gd_batch* b, int p, double* x, int where);

/* ---- learned preconditioner (3D Q1 on cube cells) ---------------------------------
 * No counterpart in the reference (whose `\` is a gathered LU).  An L-level (1..6,
 * default 3), 8-channel convolutional network on the node lattice, gated by the
 * coefficient field, in the symmetric positive definite form
 * z = D^-1 r + D^-1/2 S^T S D^-1/2 r (S the gated encoder, S^T its adjoint), used as the
 * preconditioner of the mixed-precision flexible CG.
 * Vectors r, e, z are FP32 device arrays over the owned DOFs in gid order. */
typedef struct gd_learned gd_learned;
/* flags: GD_LEARNED_COARSE_START runs the network on the once-restricted lattice,
 * z = D^-1 r + D^-1/2 R^T S^T S R D^-1/2 r (R full-weighting restriction). */
enum { GD_LEARNED_COARSE_START = 1 };
int gd_learned_create(gd_asm* a, int levels, int flags, uint64_t seed, gd_learned** out);
int gd_learned_levels(const gd_learned* net, int32_t* levels);
int gd_learned_flags(const gd_learned* net, int32_t* flags);
int gd_learned_destroy(gd_learned* net);
int gd_learned_num_params(const gd_learned* net, int64_t* n);
int gd_learned_get_params(const gd_learned* net, float* host_params);
int gd_learned_set_params(gd_learned* net, const float* host_params);
/* z = M(r) for the assembler's current coefficients. */
int gd_learned_apply(gd_learned* net, const float* r, float* z);
/* The same map through the training kernels (a check on the tiled application path). */
int gd_learned_apply_reference(gd_learned* net, const float* r, float* z);
/* Mean relative A-norm error ||M(r_b) - e_b||_A^2 / ||e_b||_A^2 over `batch` pairs stored
 * back to back, and (optionally) the summed parameter gradients copied to the host. */
int gd_learned_gradient(gd_learned* net, const float* r, const float* e, int batch, double* loss,
                        float* grads_host);
/* One Adam step on a batch of pairs (mean loss returned). */
int gd_learned_train_step(gd_learned* net, const float* r, const float* e, int batch, float lr, double* loss);
/* x = A \ b with the learned flexible CG inside FP64 refinement; falls back to Jacobi
 * (reported in *fallback_used) if the learned iteration stalls or does not converge. */
int gd_solve_learned(gd_asm* a, gd_learned* net, double rtol, int maxit, double* x, int where,
                     gd_solve_stats* stats, int32_t* fallback_used);

/* ---- Multi-field systems (src/MultiField.jl, test/BlockSparseMatrixAssemblersTests.jl) ----
 * n fields (n <= 8) that share the test/trial spaces of one scalar assembler (after
 * gd_assemble_symbolic); its strategy is the multi-field system's: SubAssembledRows (the
 * default of the reference's multi-field assemblers, MultiField.jl:473-479) or
 * FullyAssembledRows.  The bilinear form is
 *   sum_ij int( stiff[i*n+j] grad(u_j).grad(v_i) + mass[i*n+j] u_j v_i ) kappa dOmega
 * (kappa per cell as in gd_coeffs, NULL = 1; f_nodal must be NULL), the linear form
 * sum_i int( src[i] v_i ) dOmega minus the Dirichlet lifting of every field with the
 * trial space's values.  Blocks with stiff = mass = 0 are not touched (no entries).
 * Replaces the assembly behind MultiFieldFESpace + SparseMatrixAssembler(X, Y, strategy)
 * + AffineFEOperator (MultiField.jl:283-560). */
typedef struct gd_mfield gd_mfield;
typedef struct gd_mfmat gd_mfmat;
int gd_mfield_create(gd_asm* a, int nfields, gd_mfield** out);
int gd_mfield_destroy(gd_mfield* m);
int gd_mfield_assemble(gd_mfield* m, const double* stiff, const double* mass, const double* src,
                       const gd_coeffs* c);
/* Block (i, j) values over the owned rows of `part` in the scalar pattern of
 * gd_matrix_export, and field i's right-hand side over the part's owned rows. */
int gd_mfield_block_export(const gd_mfield* m, int i, int j, int part, double* vals, double* rhs);
/* gids / owners of the multi-field space of `fields` (generate_multi_field_gids,
 * MultiField.jl:356-420) for one part; local ids field-major (position * nfree + lid). */
int gd_mfield_gids(const gd_mfield* m, int nfields, const int* fields, int part, int64_t* lid_to_gid,
                   int32_t* lid_to_owner);
/* The matrix of row fields rf and column fields cf: block (R, C) of a
 * BlockMultiFieldStyle system, or the ConsecutiveMultiFieldStyle matrix for R = C = all
 * fields (MultiField.jl:468-560).  Rows in the row group's gid order; per part the
 * columns are the column group's owned dofs, then the touched ghost columns.  Destroy
 * the matrices before their gd_mfield. */
int gd_mfmat_create(gd_mfield* m, int nr, const int* rf, int nc, const int* cf, gd_mfmat** out);
int gd_mfmat_destroy(gd_mfmat* x);
/* values and right-hand side from the latest gd_mfield_assemble (same touched blocks) */
int gd_mfmat_refresh(gd_mfmat* x);
int gd_mfmat_counts(const gd_mfmat* x, int64_t* nrows, int64_t* nnz);
/* Rows of one part: the owned rows and, under SubAssembledRows, the touched ghost rows
 * (explicit zeros, row field outer, local order); columns: the owned ones, then the ghost
 * ones (FullyAssembledRows: each touched field's in local order, field by field;
 * SubAssembledRows: first-appearance order -- the scalar ghost columns grouped by the cell
 * that first meets them, field by field inside a group). */
int gd_mfmat_sizes(const gd_mfmat* x, int part, int64_t* nrows, int64_t* ncols, int64_t* nnz,
                   int64_t* n_ghost_rows, int64_t* n_ghost_cols);
int gd_mfmat_export(const gd_mfmat* x, int part, int64_t* rowptr, int32_t* colidx, double* vals,
                    int64_t* ghost_row_gids, int32_t* ghost_row_owners, int64_t* ghost_col_gids,
                    int32_t* ghost_col_owners, double* rhs);
/* y = A x (mul!, BlockPartitionedArrays.jl:330-350 per block): x over the column group's
 * global numbering, y over the row group's. */
int gd_mfmat_spmv(const gd_mfmat* x, const double* xin, double* y, int where);

/* ---- Discontinuous Galerkin (test/PoissonTests.jl:47-77) ----
 * FESpace(model, ReferenceFE(lagrangian, Float64, k), conformity=:L2), k <= 3: every
 * cell holds its (k+1)^d dofs (reference node order); a part owns its owned cells' dofs,
 * numbered cell by cell (lexicographic), parts in order. */
typedef struct gd_dgspace gd_dgspace;
int gd_dg_space_create(gd_model* model, int order, gd_dgspace** out);
int gd_dg_space_destroy(gd_dgspace* s);
int gd_dg_num_free_dofs(const gd_dgspace* s, int64_t* n);
int gd_dg_local_sizes(const gd_dgspace* s, int part, int64_t* nlocal, int64_t* nown, int64_t* first);
int gd_dg_get_gids(const gd_dgspace* s, int part, int64_t* gid, int32_t* owner);
/* The assembly strategy of the space's system (SparseMatrixAssembler(V, V, strategy),
 * FESpaces.jl:819-862), before the first gd_dg_assemble; GD_SUB_ASSEMBLED_ROWS (the
 * reference's default and this library's) or GD_FULLY_ASSEMBLED_ROWS. */
int gd_dg_set_strategy(gd_dgspace* s, int strategy);
/* The symmetric interior penalty form of the reference's DG Poisson test:
 *   a(u,v) = int grad(v).grad(u) + sum_Gd int((gamma/h) v u - v dn(u) - dn(v) u)
 *            + sum_Skeleton int((gamma/h) [[v n]].[[u n]] - [[v n]].{grad u} - {grad v}.[[u n]])
 *   l(v)   = int f v + sum_Gn int g v + sum_Gd int((gamma/h) v uD - dn(v) uD)
 * f: f_const, or f_qp at the cells' Gauss points (cells lexicographic, nq^d points x
 * fastest); uD / g at the face Gauss points of the flagged sides (layout of
 * gd_add_boundary_source); nq = (degree + 2) / 2 for cells and faces. */
typedef struct gd_dg_form {
  double gamma;
  double h;
  int degree;
  double f_const;
  const double* f_qp;
  const int32_t* dirichlet_sides;  /* 2*dim flags */
  const double* ud_qp;
  const int32_t* neumann_sides;    /* 2*dim flags */
  const double* g_qp;
  int where;                       /* GD_HOST or GD_DEVICE for f_qp, ud_qp, g_qp */
} gd_dg_form;
/* Matrix and right-hand side (create_from_nz, Algebra.jl:537-646): every owned row summed
 * completely.  FullyAssembledRows: owned rows only; columns: owned dofs, then the touched
 * ghost dofs in local order.  SubAssembledRows: a part integrates the interior faces whose
 * cell with the larger global id it owns (Geometry.jl:864-882); rows: owned dofs, then the
 * touched ghost dofs (local order, explicit zeros); columns: owned dofs, then the ghost dofs
 * in order of first appearance in the local and received triplets. */
int gd_dg_assemble(gd_dgspace* s, const gd_dg_form* form);
int gd_dg_matrix_sizes(const gd_dgspace* s, int part, int64_t* nrows, int64_t* ncols, int64_t* nnz,
                       int64_t* n_ghost_rows, int64_t* n_ghost_cols);
/* One part: local CSR (owned rows, then ghost rows), the ghost parts of its row and column
 * OwnAndGhostIndices, and the right-hand side over the rows (ghost rows 0). */
int gd_dg_matrix_export(const gd_dgspace* s, int part, int64_t* rowptr, int32_t* colidx, double* vals,
                        int64_t* ghost_row_gids, int32_t* ghost_row_owners, int64_t* ghost_col_gids,
                        int32_t* ghost_col_owners, double* rhs);
int gd_dg_spmv(const gd_dgspace* s, const double* x, double* y, int where);
int gd_dg_solve(gd_dgspace* s, double rtol, int maxit, double* x, int where, gd_solve_stats* stats);
/* sqrt(sum(int (u - uh)^2 dOmega)): u at the cells' Gauss points (layout of f_qp) */
int gd_dg_l2_error(const gd_dgspace* s, const double* x, const double* u_qp, int degree, int where, double* err);

/* Diagnostics (no reference counterpart): launches `blocks` blocks of the persistent
 * kernels' grid barrier waiting for `expected` arrivals.  expected > blocks makes the
 * bounded wait run out after timeout_s (<= 5 s): GD_ERR_TIMEOUT, the context stays
 * usable; expected == blocks: GD_OK. */
int gd_debug_barrier_probe(gd_ctx* ctx, int blocks, int expected, double timeout_s);

#ifdef __cplusplus
}
#endif
#endif /* GDGPU_H */
