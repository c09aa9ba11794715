// Stable LSD radix sort (8-bit digits) and exclusive scans.
#include "pg_common.cuh"
#include "pg_sort.cuh"

namespace pg {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 16;
constexpr int kTile = kThreads * kItems;  // keys per block per pass
// kScanChunk (elements per block in scans) is declared in pg_sort.cuh

template <typename T>
__global__ void k_reduce_chunks(const T* in, int64_t n, T* partial) {
  __shared__ T red[kThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk;
  T s = 0;
  for (int i = threadIdx.x; i < kScanChunk; i += kThreads) {
    const int64_t g = base + i;
    if (g < n) s += in[g];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int off = kThreads / 2; off > 0; off >>= 1) {
    if (threadIdx.x < off) red[threadIdx.x] += red[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// One block: exclusive scan of nb partial sums in place; total -> *total.
template <typename T>
__global__ void k_scan_single(T* partial, int64_t nb, T* total) {
  __shared__ T sums[1024];
  const int64_t per = (nb + blockDim.x - 1) / blockDim.x;
  const int64_t lo = threadIdx.x * per;
  const int64_t hi = lo + per < nb ? lo + per : nb;
  T s = 0;
  for (int64_t i = lo; i < hi; ++i) s += partial[i];
  sums[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    T run = 0;
    for (int t = 0; t < (int)blockDim.x; ++t) {
      T v = sums[t];
      sums[t] = run;
      run += v;
    }
    if (total) *total = run;
  }
  __syncthreads();
  T run = sums[threadIdx.x];
  for (int64_t i = lo; i < hi; ++i) {
    T v = partial[i];
    partial[i] = run;
    run += v;
  }
}

template <typename T>
__global__ void k_scan_chunks(const T* in, T* out, int64_t n, const T* partial) {
  constexpr int per = kScanChunk / kThreads;
  __shared__ T tsum[kThreads];
  const int64_t base = (int64_t)blockIdx.x * kScanChunk + (int64_t)threadIdx.x * per;
  T v[per];
  T s = 0;
#pragma unroll
  for (int k = 0; k < per; ++k) {
    const int64_t g = base + k;
    v[k] = g < n ? in[g] : (T)0;
    s += v[k];
  }
  tsum[threadIdx.x] = s;
  __syncthreads();
  // Hillis-Steele inclusive scan over the 256 thread sums
  for (int off = 1; off < kThreads; off <<= 1) {
    T add = threadIdx.x >= off ? tsum[threadIdx.x - off] : (T)0;
    __syncthreads();
    tsum[threadIdx.x] += add;
    __syncthreads();
  }
  T run = partial[blockIdx.x] + (threadIdx.x ? tsum[threadIdx.x - 1] : (T)0);
#pragma unroll
  for (int k = 0; k < per; ++k) {
    const int64_t g = base + k;
    if (g < n) out[g] = run;
    run += v[k];
  }
}

template <typename T>
int scan_impl(const T* in, T* out, int64_t n, T* total, void* ws, size_t ws_bytes, cudaStream_t s) {
  if (n <= 0) {
    if (total) PG_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(T), s));
    return PG_OK;
  }
  const int64_t nb = (n + kScanChunk - 1) / kScanChunk;
  if (!ws || ws_bytes < pg_align256(sizeof(int64_t) * nb)) return PG_ERR_WORKSPACE;
  T* partial = reinterpret_cast<T*>(ws);
  k_reduce_chunks<T><<<(unsigned)nb, kThreads, 0, s>>>(in, n, partial);
  k_scan_single<T><<<1, 1024, 0, s>>>(partial, nb, total);
  k_scan_chunks<T><<<(unsigned)nb, kThreads, 0, s>>>(in, out, n, partial);
  PG_LAUNCH_CHECK();
  return PG_OK;
}

__global__ void k_hist(const uint64_t* keys, int64_t n, int shift, int32_t* counts, int nblocks) {
  __shared__ int hist[256];
  hist[threadIdx.x] = 0;
  __syncthreads();
  const int64_t start = (int64_t)blockIdx.x * kTile;
  for (int r = 0; r < kItems; ++r) {
    const int64_t i = start + (int64_t)r * kThreads + threadIdx.x;
    if (i < n) atomicAdd(&hist[(keys[i] >> shift) & 255], 1);
  }
  __syncthreads();
  counts[(int64_t)threadIdx.x * nblocks + blockIdx.x] = hist[threadIdx.x];
}

__global__ void k_scatter(const uint64_t* __restrict__ kin, const int32_t* __restrict__ vin, uint64_t* kout,
                          int32_t* vout, int64_t n, int shift, const int32_t* offs, int nblocks) {
  __shared__ int base[256];
  __shared__ int wcnt[kThreads / 32][256];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  base[tid] = offs[(int64_t)tid * nblocks + blockIdx.x];
  const int64_t start = (int64_t)blockIdx.x * kTile;
  for (int r = 0; r < kItems; ++r) {
    for (int i = tid; i < (kThreads / 32) * 256; i += kThreads) (&wcnt[0][0])[i] = 0;
    __syncthreads();
    const int64_t i = start + (int64_t)r * kThreads + tid;
    const bool valid = i < n;
    const uint64_t k = valid ? kin[i] : 0ull;
    const int32_t v = valid ? vin[i] : 0;
    const unsigned d = valid ? (unsigned)((k >> shift) & 255ull) : 256u + (unsigned)lane;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & ((1u << lane) - 1u));
    const int leader = __ffs(peers) - 1;
    if (valid && lane == leader) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    {
      int run = base[tid];
      for (int w = 0; w < kThreads / 32; ++w) {
        const int c = wcnt[w][tid];
        wcnt[w][tid] = run;
        run += c;
      }
      base[tid] = run;
    }
    __syncthreads();
    if (valid) {
      const int pos = wcnt[warp][d] + rank;
      kout[pos] = k;
      vout[pos] = v;
    }
    __syncthreads();
  }
}

}  // namespace

size_t scan_workspace_bytes(int64_t n) { return scan_workspace_bytes_for(n); }

int scan_exclusive_i32(const int32_t* in, int32_t* out, int64_t n, int32_t* total, void* ws, size_t ws_bytes,
                       cudaStream_t s) {
  return scan_impl<int32_t>(in, out, n, total, ws, ws_bytes, s);
}

int scan_exclusive_i64(const int64_t* in, int64_t* out, int64_t n, int64_t* total, void* ws, size_t ws_bytes,
                       cudaStream_t s) {
  return scan_impl<int64_t>(in, out, n, total, ws, ws_bytes, s);
}

size_t sort_workspace_bytes(int64_t n) {
  const int64_t nblocks = (n + kTile - 1) / kTile;
  return pg_align256(sizeof(uint64_t) * n) + pg_align256(sizeof(int32_t) * n) +
         pg_align256(sizeof(int32_t) * 256 * nblocks) + scan_workspace_bytes(256 * nblocks);
}

int sort_pairs(uint64_t* keys, int32_t* vals, int64_t n, int key_bits, void* ws, size_t ws_bytes,
               cudaStream_t s) {
  if (n <= 1) return PG_OK;
  if (n >= (1ll << 31)) return PG_ERR_ARG;
  if (!ws || ws_bytes < sort_workspace_bytes(n)) return PG_ERR_WORKSPACE;
  const int nblocks = (int)((n + kTile - 1) / kTile);
  PgArena ar(ws, ws_bytes);
  uint64_t* k2 = ar.take<uint64_t>(n);
  int32_t* v2 = ar.take<int32_t>(n);
  int32_t* counts = ar.take<int32_t>((size_t)256 * nblocks);
  const size_t scan_bytes = scan_workspace_bytes(256 * (int64_t)nblocks);
  void* scan_ws = ar.take<char>(scan_bytes);
  if (!k2 || !v2 || !counts || !scan_ws) return PG_ERR_WORKSPACE;
  uint64_t *kin = keys, *kout = k2;
  int32_t *vin = vals, *vout = v2;
  int passes = 0;
  for (int shift = 0; shift < key_bits; shift += 8, ++passes) {
    k_hist<<<nblocks, kThreads, 0, s>>>(kin, n, shift, counts, nblocks);
    int st = scan_exclusive_i32(counts, counts, 256 * (int64_t)nblocks, nullptr, scan_ws, scan_bytes, s);
    if (st) return st;
    k_scatter<<<nblocks, kThreads, 0, s>>>(kin, vin, kout, vout, n, shift, counts, nblocks);
    PG_LAUNCH_CHECK();
    uint64_t* tk = kin; kin = kout; kout = tk;
    int32_t* tv = vin; vin = vout; vout = tv;
  }
  if (passes & 1) {
    PG_CUDA_TRY(cudaMemcpyAsync(keys, kin, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, s));
    PG_CUDA_TRY(cudaMemcpyAsync(vals, vin, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, s));
  }
  return PG_OK;
}

}  // namespace pg
