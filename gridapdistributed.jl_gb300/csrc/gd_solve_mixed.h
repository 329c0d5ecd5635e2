// Interfaces between the mixed-precision solver and its preconditioners.
#pragma once
#include <cuda_runtime.h>

#include "gd_internal.h"

namespace gd {

// z = M(r) on the owned rows (FP32 vectors), enqueued on `st`.
struct MixedPrecond {
  void* ctx;
  int (*apply)(void* ctx, gd_asm* A, const float* r, float* z, cudaStream_t st);
};

int residual_fp64(int64_t n, const int64_t* rowptr, const int32_t* col, const double* val, const double* x,
                  const double* b, double* r, double* prr, double* pbb, cudaStream_t st, int* nblocks);
int mixed_setup(gd_asm* A);
int mixed_apply(gd_asm* A, const float* x, float* y, double* partial, cudaStream_t st);
int mixed_solve(gd_asm* A, double rtol, int maxit, double* x_out, int where, gd_solve_stats* stats,
                const MixedPrecond* precond);

}  // namespace gd
