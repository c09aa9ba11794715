// Allocation-free variant of pg_select_equal.
//
// Some callers cannot allocate device memory: host applications whose device
// memory is owned by another allocator (for example a C/Fortran solver that
// reserves all device memory up front and forbids allocation during a time
// step), or services with a fixed device-memory budget that must not
// allocate on their request path.  pg_select_equal_noalloc serves them: its
// scratch is a file-scope static device array, so the call itself allocates
// nothing (no cudaMalloc/cudaFree, no allocating library routine).
//
// Cost of this choice: every GPU that loads the library holds the array
// (PG_NOALLOC_SCRATCH_BYTES, about 2 MB) until the process exits, and all
// calls share it.
#include <mutex>

#include "pg_common.cuh"
#include "pg_sort.cuh"

namespace {

// Sized by the same compile-time formula that pg_select_workspace_bytes
// returns, so the two cannot drift apart.
constexpr int64_t kMaxN = PG_NOALLOC_MAX_N;
constexpr size_t kScratchBytes = pg::select_workspace_bytes_for(kMaxN);
static_assert(kScratchBytes % 256 == 0 && kScratchBytes < ((size_t)4 << 20),
              "the static scratch should stay a modest, 256-byte multiple");

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch, looked up once per device with that
// device current (the host-side symbol is a stand-in, not a device address).
// The cached address belongs to the device's primary context: after
// cudaDeviceReset it is stale, so a process that resets a device must not
// call pg_select_equal_noalloc on that device again.
constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

int scratch_for_current_device(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    pg_set_cuda_error(e);
    return PG_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    pg_set_error("pg_select_equal_noalloc: device ordinal out of range");
    return PG_ERR_UNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      pg_set_cuda_error(e != cudaSuccess ? e : cudaErrorInvalidSymbol);
      return PG_ERR_CUDA;
    }
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return PG_OK;
}

}  // namespace

extern "C" int64_t pg_select_equal_noalloc_max_n(void) { return kMaxN; }

extern "C" int pg_select_equal_noalloc(const int32_t* values, int64_t n, int32_t target, int32_t* out, int64_t* count,
                                       void* stream) {
  if (n > kMaxN) {
    pg_set_error("pg_select_equal_noalloc: n exceeds the static scratch limit (pg_select_equal_noalloc_max_n); "
                 "use pg_select_equal with a caller-provided workspace");
    return PG_ERR_ARG;
  }
  if (n < 1 || !values || !out || !count) {
    pg_set_error("pg_select_equal_noalloc: bad argument");
    return PG_ERR_ARG;
  }
  void* scratch = nullptr;
  const int st = scratch_for_current_device(&scratch);
  if (st) return st;
  // Every scratch byte read by pg_select_equal is written earlier in the same
  // call (flags, scan positions, partial sums, total), so nothing needs to be
  // cleared between calls.
  return pg_select_equal(values, n, target, out, count, scratch, kScratchBytes, stream);
}
