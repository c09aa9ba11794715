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

extern "C" int pg_abi_version(void) { return 4; }

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

// Streaming copy by the SMs: 16-byte loads and stores, grid-stride.  Used to
// move results into pinned host memory the GPU maps into its address space
// (on Grace-Blackwell, over NVLink-C2C), where many SMs issuing stores keep
// more bytes in flight than one copy engine.
namespace {
__global__ void __launch_bounds__(512) k_copy16(const int4* __restrict__ src, int4* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __ldcs(src + i);
}
__global__ void k_copy1(const unsigned char* __restrict__ src, unsigned char* __restrict__ dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}
}  // namespace

extern "C" int pg_copy_bytes(const void* src, void* dst, int64_t bytes, int blocks, void* stream) {
  if (!src || !dst || bytes < 0 || blocks < 0) {
    pg_set_error("pg_copy_bytes: bad argument");
    return PG_ERR_ARG;
  }
  if (bytes == 0) return PG_OK;
  if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15) != 0) {
    pg_set_error("pg_copy_bytes: src and dst must be 16-byte aligned");
    return PG_ERR_ARG;
  }
  cudaStream_t s = pg_stream(stream);
  const int g = blocks > 0 ? blocks : 152 * 4;
  const int64_t n16 = bytes / 16;
  if (n16) k_copy16<<<g, 512, 0, s>>>(reinterpret_cast<const int4*>(src), reinterpret_cast<int4*>(dst), n16);
  if (bytes % 16)
    k_copy1<<<1, 32, 0, s>>>(reinterpret_cast<const unsigned char*>(src) + 16 * n16,
                             reinterpret_cast<unsigned char*>(dst) + 16 * n16, bytes % 16);
  PG_LAUNCH_CHECK();
  return PG_OK;
}
