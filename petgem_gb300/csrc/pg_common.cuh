// Shared helpers for the petgem GB300 kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/petgem_gb300.h"

#define PG_CUDA_TRY(expr)                                   \
  do {                                                      \
    cudaError_t _e = (expr);                                \
    if (_e != cudaSuccess) { pg_set_cuda_error(_e); return PG_ERR_CUDA; } \
  } while (0)

#define PG_LAUNCH_CHECK()                                   \
  do {                                                      \
    cudaError_t _e = cudaGetLastError();                    \
    if (_e != cudaSuccess) { pg_set_cuda_error(_e); return PG_ERR_CUDA; } \
  } while (0)

// Records the last CUDA error string for pg_last_error().
void pg_set_cuda_error(cudaError_t e);
void pg_set_error(const char* msg);

static inline cudaStream_t pg_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

static inline unsigned pg_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > 0x7fffffff) b = 0x7fffffff;
  return (unsigned)b;
}

// Bump allocator over a caller-provided workspace (256-byte aligned slices).
struct PgArena {
  char* base;
  size_t cap;
  size_t off;
  __host__ PgArena(void* b, size_t c) : base((char*)b), cap(c), off(0) {}
  template <typename T>
  __host__ T* take(size_t count) {
    size_t bytes = ((count * sizeof(T)) + 255) & ~(size_t)255;
    if (base == nullptr || off + bytes > cap) return nullptr;
    T* p = reinterpret_cast<T*>(base + off);
    off += bytes;
    return p;
  }
};

static inline size_t pg_align256(size_t b) { return (b + 255) & ~(size_t)255; }

// DOF counts per entity kind (petgem/hvfem.py:45-48).
__host__ __device__ inline int pg_nd_edge(int p) { return p; }
__host__ __device__ inline int pg_nd_face(int p) { return p * (p - 1); }
__host__ __device__ inline int pg_nd_vol(int p) { return p * (p - 1) * (p - 2) / 2; }
__host__ __device__ inline int pg_nd_elem(int p) { return p * (p + 2) * (p + 3) / 2; }
