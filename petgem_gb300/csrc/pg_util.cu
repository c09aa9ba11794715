// Error reporting and version query of the C ABI.
#include <string.h>
#include <stdio.h>
#include "pg_common.cuh"

namespace {
thread_local char g_last_error[512] = "";
}

void pg_set_error(const char* msg) {
  strncpy(g_last_error, msg, sizeof(g_last_error) - 1);
  g_last_error[sizeof(g_last_error) - 1] = 0;
}

void pg_set_cuda_error(cudaError_t e) {
  snprintf(g_last_error, sizeof(g_last_error), "CUDA error %d: %s", (int)e, cudaGetErrorString(e));
}

extern "C" int pg_abi_version(void) { return 3; }

extern "C" const char* pg_last_error(void) { return g_last_error; }

// FP64 FMA throughput probe: 8 independent FMA chains per thread.  Used by
// the benchmark to measure the FP64 peak that bounds the elemental/assembly
// kernels (no petgem counterpart).
namespace {
__global__ void k_fp64_probe(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

extern "C" int64_t pg_fp64_probe_flops(int blocks, int iters) {
  return (int64_t)blocks * 256 * iters * 8 * 2;
}

extern "C" int pg_fp64_probe(double* out, int blocks, int iters, void* stream) {
  if (!out || blocks < 1 || iters < 1) {
    pg_set_error("pg_fp64_probe: bad argument");
    return PG_ERR_ARG;
  }
  k_fp64_probe<<<blocks, 256, 0, pg_stream(stream)>>>(out, iters, 0.999, 1e-4);
  PG_LAUNCH_CHECK();
  return PG_OK;
}
