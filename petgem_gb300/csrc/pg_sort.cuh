// Device primitives shared by the topology and pattern builders: a stable
// LSD radix sort of (uint64 key, int32 value) pairs and exclusive scans.
// Both are deterministic (no floating point, no order-dependent atomics).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

// Workspace bytes for sort_pairs on n items (ping-pong buffers included).
size_t sort_workspace_bytes(int64_t n);

// Stable sort of keys[0..n) (uint64) carrying vals (int32); sorts the low
// `key_bits` bits.  Results end in keys/vals (in place).  n < 2^31.
int sort_pairs(uint64_t* keys, int32_t* vals, int64_t n, int key_bits, void* ws, size_t ws_bytes,
               cudaStream_t s);

// Exclusive scans (out may alias in).  `total` (device, may be null)
// receives the sum.  Workspace: scan_workspace_bytes(n), one int64 partial
// per chunk of kScanChunk elements.
constexpr int kScanChunk = 2048;
constexpr size_t align256_bytes(size_t b) { return (b + 255) & ~(size_t)255; }
constexpr size_t scan_workspace_bytes_for(int64_t n) {
  return align256_bytes(sizeof(int64_t) * (size_t)((n + kScanChunk - 1) / kScanChunk > 0
                                                       ? (n + kScanChunk - 1) / kScanChunk
                                                       : 1));
}
size_t scan_workspace_bytes(int64_t n);

// Workspace of pg_select_equal for n entries: flags and positions (int32
// each), the scan partials, and a 512-byte tail for the total.  Compile-time
// so that fixed-size scratch arrays are sized by the same formula.
constexpr size_t select_workspace_bytes_for(int64_t n) {
  return align256_bytes(sizeof(int32_t) * (size_t)n) * 2 + scan_workspace_bytes_for(n) + 512;
}
int scan_exclusive_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* total, void* ws, size_t ws_bytes,
                       cudaStream_t s);
int scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total, void* ws, size_t ws_bytes,
                       cudaStream_t s);

inline int bits_for(uint64_t maxval) {
  int b = 0;
  while (b < 64 && (maxval >> b) != 0) ++b;
  return b < 1 ? 1 : b;
}

}  // namespace pg
