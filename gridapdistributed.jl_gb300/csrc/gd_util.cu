// Error state, device allocation and a device-wide exclusive scan.
#include <cstdio>
#include <string>

#include "gd_internal.h"

namespace gd {

static thread_local std::string g_last_error;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int dalloc_bytes(void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    cudaGetLastError();
    return fail(GD_ERR_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed: " +
                                cudaGetErrorString(e));
  }
  return GD_OK;
}

void dfree(void* p) { cudaFree(p); }

// ---------------------------------------------------------------------------------
// Exclusive scan int32 -> int64.  Three phases: tile sums, scan of tile sums by one
// block, then each tile scans itself and adds its offset.  Tiles of 2048 entries.
// ---------------------------------------------------------------------------------
constexpr int kScanThreads = 256;
constexpr int kScanPerThread = 8;
constexpr int kScanTile = kScanThreads * kScanPerThread;

__device__ inline int64_t block_exclusive_scan(int64_t v, int64_t* total) {
  __shared__ int64_t warp_sums[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t s = lane < kScanThreads / 32 ? warp_sums[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanThreads / 32) warp_sums[lane] = s;
  }
  __syncthreads();
  int64_t prefix = (wid > 0 ? warp_sums[wid - 1] : 0) + x - v;
  if (total) *total = warp_sums[kScanThreads / 32 - 1];
  __syncthreads();
  return prefix;
}

__global__ void k_tile_sums(const int32_t* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int64_t s = 0;
  for (int i = 0; i < kScanPerThread; ++i) {
    int64_t idx = base + (int64_t)i * kScanThreads + threadIdx.x;
    if (idx < n) s += in[idx];
  }
  int64_t tot;
  block_exclusive_scan(s, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_sums(int64_t* sums, int64_t ntiles) {
  __shared__ int64_t carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int64_t base = 0; base < ntiles; base += kScanThreads) {
    int64_t idx = base + threadIdx.x;
    int64_t v = idx < ntiles ? sums[idx] : 0;
    int64_t tot;
    int64_t ex = block_exclusive_scan(v, &tot);
    if (idx < ntiles) sums[idx] = carry + ex;
    __syncthreads();
    if (threadIdx.x == 0) carry += tot;
    __syncthreads();
  }
  if (threadIdx.x == 0) sums[ntiles] = carry;
}

__global__ void k_tile_scan(const int32_t* __restrict__ in, int64_t n, const int64_t* __restrict__ sums,
                            int64_t* __restrict__ out) {
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanPerThread;
  int32_t v[kScanPerThread];
  int64_t s = 0;
  for (int i = 0; i < kScanPerThread; ++i) {
    int64_t idx = base + i;
    v[i] = idx < n ? in[idx] : 0;
    s += v[i];
  }
  int64_t ex = block_exclusive_scan(s, nullptr) + sums[blockIdx.x];
  for (int i = 0; i < kScanPerThread; ++i) {
    int64_t idx = base + i;
    if (idx < n) out[idx] = ex;
    ex += v[i];
  }
}

int exclusive_scan_i32(const int32_t* in, int64_t* out, int64_t n, cudaStream_t s) {
  int64_t ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles == 0) {
    GD_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(int64_t), s));
    return GD_OK;
  }
  DBuf<int64_t> sums;
  GD_TRY(dalloc(sums, ntiles + 1));
  k_tile_sums<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, sums.p);
  k_scan_sums<<<1, kScanThreads, 0, s>>>(sums.p, ntiles);
  k_tile_scan<<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, sums.p, out);
  // out[n] = total
  cudaError_t e = cudaMemcpyAsync(out + n, sums.p + ntiles, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
  cudaError_t e2 = cudaStreamSynchronize(s);
  dfreeb(sums);
  if (e != cudaSuccess || e2 != cudaSuccess)
    return fail(GD_ERR_CUDA, std::string("scan: ") + cudaGetErrorString(e != cudaSuccess ? e : e2));
  GD_CUDA_TRY(cudaGetLastError());
  return GD_OK;
}

}  // namespace gd

extern "C" const char* gd_last_error(void) { return gd::g_last_error.c_str(); }
