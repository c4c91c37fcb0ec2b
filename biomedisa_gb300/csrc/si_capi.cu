// Error state and version of the C ABI.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <mutex>
#include <string>

#include "si_internal.h"
#include "si_tma.cuh"

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

namespace {
std::atomic<long long> g_wait_limit{-1};  // < 0: kDefaultWaitLimit
}

uint32_t wait_limit() {
  const long long v = g_wait_limit.load(std::memory_order_relaxed);
  return v < 0 ? kDefaultWaitLimit : (uint32_t)(v > 0xFFFFFFFFll ? 0xFFFFFFFFll : v);
}

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

}  // namespace si

extern "C" int si_set_wait_limit(long long spins) {
  si::clear_error();
  si::g_wait_limit.store(spins, std::memory_order_relaxed);
  return SI_OK;
}

extern "C" int si_version(void) { return 100; }

extern "C" const char* si_last_error(void) { return si::g_last_error.c_str(); }
