// Library-wide entry points: version, per-thread error message, device info.
#include <cstdarg>
#include <mutex>

#include "axi_common.cuh"

namespace axi {

static thread_local std::string g_last_error;

void set_error(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
}

void clear_error() { g_last_error.clear(); }

int sm_count() {
  static int cached[64] = {0};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 64) return 152;
  if (cached[dev] == 0) {
    int n = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cached[dev] = n > 0 ? n : 152;
  }
  return cached[dev];
}

}  // namespace axi

extern "C" int axi_version(void) { return 100; }

extern "C" const char* axi_last_error(void) { return axi::g_last_error.c_str(); }
