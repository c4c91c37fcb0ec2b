// Error state and version of the C ABI.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <string>

#include "si_internal.h"

namespace si {

namespace {
thread_local std::string g_last_error;
}

int set_error(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

void clear_error() { g_last_error.clear(); }

int check_launch(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    return set_error(SI_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  return SI_OK;
}

int sm_count() {
  static std::atomic<int> cached[64];  // 0 until looked up; threads may look it up concurrently
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int n = cached[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    cached[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

}  // namespace si

extern "C" int si_version(void) { return 100; }

extern "C" const char* si_last_error(void) { return si::g_last_error.c_str(); }
