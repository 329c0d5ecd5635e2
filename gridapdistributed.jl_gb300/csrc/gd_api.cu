// Context lifecycle, last-error and version entry points of the C ABI.
#include <string>

#include "gd_internal.h"

extern "C" const char* gd_version(void) { return "gdgpu 0.1.0 (sm_103a)"; }

extern "C" int gd_ctx_create(int device, gd_ctx** out) {
  if (!out) return gd::fail(GD_ERR_ARG, "gd_ctx_create: null output");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return gd::fail(GD_ERR_CUDA, std::string("gd_ctx_create: no CUDA device (") + cudaGetErrorString(e) + ")");
  }
  if (device < 0 || device >= n) return gd::fail(GD_ERR_ARG, "gd_ctx_create: device index out of range");
  GD_CUDA_TRY(cudaSetDevice(device));
  cudaDeviceProp prop;
  GD_CUDA_TRY(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10)
    return gd::fail(GD_ERR_UNSUPPORTED, "gd_ctx_create: this library is built for sm_103a (Blackwell Ultra)");
  gd_ctx* c = new gd_ctx();
  c->device = device;
  cudaError_t es = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  if (es != cudaSuccess) {
    delete c;
    return gd::fail(GD_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(es));
  }
  c->stream = c->own_stream;
  *out = c;
  return GD_OK;
}

extern "C" int gd_ctx_destroy(gd_ctx* c) {
  if (!c) return GD_OK;
  if (c->own_stream) {
    cudaStreamSynchronize(c->own_stream);
    cudaStreamDestroy(c->own_stream);
  }
  delete c;
  return GD_OK;
}

extern "C" int gd_ctx_set_stream(gd_ctx* c, void* s) {
  if (!c) return gd::fail(GD_ERR_ARG, "gd_ctx_set_stream: null context");
  GD_CUDA_TRY(cudaStreamSynchronize(c->stream));
  c->stream = s ? (cudaStream_t)s : c->own_stream;
  return GD_OK;
}

extern "C" int gd_ctx_synchronize(gd_ctx* c) {
  if (!c) return gd::fail(GD_ERR_ARG, "gd_ctx_synchronize: null context");
  GD_CUDA_TRY(cudaStreamSynchronize(c->stream));
  return GD_OK;
}
