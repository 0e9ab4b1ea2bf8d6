// MTTKRP entry point that allocates nothing and takes no workspace.
//
// tlgb_mttkrp needs a caller-provided workspace for its per-split partial
// tiles.  Some callers cannot provide one: a plain C, cgo or ctypes host
// binding that owns no device allocator (no torch, no memory pool of its own)
// and must not call cudaMalloc on a latency-critical path.  This variant keeps
// the partial tiles in one file-scope device array of fixed size instead.
//
// Limits and rules:
//  * the scratch holds kNoAllocScratchBytes (16 MiB); a shape whose split plan
//    needs more partial space is rejected with TLGB_EWORKSPACE (nothing runs);
//  * the first call on a device does the set-up for that device (the symbol
//    address lookup and the kernels' shared-memory attributes), so make one
//    call on each device before any stream capture that contains this entry
//    point;
//  * the device address of the scratch is looked up once per device and kept
//    for the life of the process: the entry point assumes one context per
//    device for that time (no cudaDeviceReset, no primary-context teardown
//    and re-creation between calls);
//  * the 16 MiB array is part of the library's device code, so it stays
//    resident on every device where the library's module is loaded, whether
//    or not this entry point is ever called;
//  * nothing in the scratch has to start at zero: every call overwrites all
//    of the partial space it reads;
//  * there is ONE scratch per device and process: two calls that are in
//    flight at the same time (different streams or host threads) race on it.
//    Serialise them on one stream.
// The plan, kernels and reduction order are those of tlgb_mttkrp, so the
// results are bitwise identical to it.
#include <mutex>

#include "mttkrp_simt.cuh"

namespace tlgb {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[64] = {};

// Device address of the scratch on the current device (set up once per device).
int noalloc_scratch(void** ptr) {
  const int dev = current_device();
  if (dev < 0 || dev >= 64) return set_error(TLGB_EUNSUPPORTED, "mttkrp_noalloc: device id >= 64");
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return set_error(TLGB_ECUDA, std::string("mttkrp_noalloc: cudaGetSymbolAddress failed: ") +
                                       cudaGetErrorString(e));
    g_noalloc_ptr[dev] = p;
  }
  *ptr = g_noalloc_ptr[dev];
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_mttkrp_noalloc(int dtype, const void* X, int ndim, const int64_t* shape,
                                   const void* const* factors, const void* weights,
                                   int64_t rank, int mode, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(X && shape && factors && out, "mttkrp_noalloc: null pointer");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "mttkrp_noalloc: ndim must be in [2, 8]");
  Shape sh = make_shape(ndim, shape);
  MttkrpPlan p;
  int rc = mttkrp_make_plan(dtype, sh, rank, mode, &p);
  if (rc) return rc;
  for (int k = 0; k < ndim; ++k)
    TLGB_CHECK_ARG(k == mode || factors[k] != nullptr, "mttkrp_noalloc: missing factor pointer");
  if (p.partial_bytes > kNoAllocScratchBytes)
    return set_error(TLGB_EWORKSPACE,
                     "mttkrp_noalloc: this shape needs " + std::to_string(p.partial_bytes) +
                         " bytes of partial tiles, more than the fixed 16 MiB scratch; "
                         "use tlgb_mttkrp with a workspace");
  void* scratch = nullptr;
  rc = noalloc_scratch(&scratch);
  if (rc) return rc;
  rc = mttkrp_prepare(dtype);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32) {
    rc = mttkrp_launch_partials<float>(p, (const float*)X, (const float* const*)factors,
                                       (const float*)weights, (float*)scratch, nullptr, st);
    if (rc) return rc;
    return mttkrp_launch_reduce<float, float>(p, (const float*)scratch, (float*)out, st);
  }
  rc = mttkrp_launch_partials<double>(p, (const double*)X, (const double* const*)factors,
                                      (const double*)weights, (double*)scratch, nullptr, st);
  if (rc) return rc;
  return mttkrp_launch_reduce<double, double>(p, (const double*)scratch, (double*)out, st);
}
