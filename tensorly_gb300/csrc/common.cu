// Error reporting and device queries shared by every entry point.
#include "common.cuh"

#include <mutex>

namespace tlgb {

namespace {
thread_local std::string g_last_error;
std::mutex g_sm_mutex;
int g_sm_count[64] = {0};
}  // namespace

int set_error(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

void clear_error() { g_last_error.clear(); }

int current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  return dev;
}

int sm_count() {
  const int dev = current_device();
  if (dev < 0 || dev >= 64) return 148;
  std::lock_guard<std::mutex> lock(g_sm_mutex);
  if (g_sm_count[dev] == 0) {
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
      n = 148;
    g_sm_count[dev] = n;
  }
  return g_sm_count[dev];
}

}  // namespace tlgb

extern "C" int tlgb_version(void) { return 100; }

extern "C" const char* tlgb_last_error(void) { return tlgb::g_last_error.c_str(); }
