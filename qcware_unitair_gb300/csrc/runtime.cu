// Library bookkeeping: status strings, the per-thread last-error text and
// the process-wide launch counter.
#include <stdarg.h>
#include <stdio.h>

#include <atomic>

#include "common.cuh"

namespace gbsv {

static std::atomic<uint64_t> g_launches{0};
static std::atomic<int> g_c128_arith{GBSV_C128_PAIRS};

int c128_arith() { return g_c128_arith.load(std::memory_order_relaxed); }
static thread_local char g_last_error[512] = "";

int set_error(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

int after_launch(const char* what) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)
    return set_error(GBSV_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return GBSV_OK;
}

}  // namespace gbsv

extern "C" int gbsv_abi_version(void) { return 1; }

extern "C" const char* gbsv_status_string(int status) {
  switch (status) {
    case GBSV_OK: return "ok";
    case GBSV_ERR_INVALID_ARG: return "invalid argument";
    case GBSV_ERR_UNSUPPORTED: return "unsupported";
    case GBSV_ERR_CUDA: return "CUDA error";
    case GBSV_ERR_SCRATCH: return "scratch buffer missing or too small";
    case GBSV_ERR_TIMEOUT: return "device wait timed out";
    default: return "unknown status";
  }
}

extern "C" int gbsv_set_c128_arith(int mode) {
  if (mode != GBSV_C128_PAIRS && mode != GBSV_C128_FP64)
    return gbsv::set_error(GBSV_ERR_INVALID_ARG,
                           "unknown complex128 arithmetic mode %d", mode);
  gbsv::g_c128_arith.store(mode, std::memory_order_relaxed);
  return GBSV_OK;
}

extern "C" int gbsv_get_c128_arith(void) { return gbsv::c128_arith(); }

extern "C" const char* gbsv_last_error(void) { return gbsv::g_last_error; }

extern "C" uint64_t gbsv_launch_count(void) {
  return gbsv::g_launches.load(std::memory_order_relaxed);
}
