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

extern "C" int pg_abi_version(void) { return 1; }

extern "C" const char* pg_last_error(void) { return g_last_error; }
