// Interfaces between the mixed-precision solver and its preconditioners.
#pragma once
#include <cuda_runtime.h>

#include "gd_internal.h"

namespace gd {

// z = M(r) (FP32 vectors), enqueued on `st`: `apply` over the owned rows in gid order,
// `apply_lattice` (may be null) over the node lattice with 0 on Dirichlet nodes.
struct MixedPrecond {
  void* ctx;
  int (*apply)(void* ctx, gd_asm* A, const float* r, float* z, cudaStream_t st);
  int (*apply_lattice)(void* ctx, gd_asm* A, const float* r, float* z, cudaStream_t st);
  // non-zero: apply_lattice launches only stream work on buffers that stay allocated for
  // the preconditioner's lifetime, so a captured graph of it stays valid; unique per object
  uint64_t graph_key;
};

int residual_fp64(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, const double* x,
                  const double* b, double* r, double* prr, double* pbb, cudaStream_t st, int* nblocks);
int mixed_setup(gd_asm* A);
int mixed_apply(gd_asm* A, const float* x, float* y, double* partial, cudaStream_t st);
int mixed_solve(gd_asm* A, double rtol, int maxit, double* x_out, int where, gd_solve_stats* stats,
                const MixedPrecond* precond);
// lattice-order inner iteration (3D Q1 on cube cells; used by mixed_solve when possible)
int lattice_setup(gd_asm* A);
const float* lattice_dinv(const gd_asm* A);   // D^-1 on the lattice (0 on Dirichlet nodes)
int mixed_solve_lattice(gd_asm* A, double rtol, int maxit, double* x_out, int where, gd_solve_stats* stats,
                        const MixedPrecond* precond);

}  // namespace gd
