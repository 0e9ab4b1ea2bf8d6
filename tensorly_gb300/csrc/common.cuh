// Shared definitions for the tensorly_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>
#include <stddef.h>
#include <atomic>
#include <string>

#include "../../include/tensorly_gb300.h"

namespace tlgb {

// Records a message for tlgb_last_error() and returns `code`.
int set_error(int code, const std::string& msg);
void clear_error();

// Tuning keys of the batched CP-ALS kernel variants (batched.cu).
int batched_set_tuning(const std::string& key, int value);

// Programmatic dependent launch.  A kernel launched by launch_maybe_pdl(true,
// ...) may start while the previous kernel of its stream is still running;
// it must call griddep_wait() before it reads anything an earlier kernel
// wrote (or writes anything an earlier kernel reads).  griddep_wait() is a
// no-op in a kernel launched the ordinary way.  griddep_launch_dependents()
// lets the next such kernel of the stream be scheduled early.
// Read-only loads of data read once (a streamed tensor) with an
// evict-first L2 policy, so they do not push data that is read again out of
// L2 (factors, partial tiles, the next product's input).
__device__ __forceinline__ uint64_t l2_evict_first_policy() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float4 ldg_stream(const float4* a, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.nc.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float2 ldg_stream(const float2* a, uint64_t pol) {
  float2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;"
               : "=f"(v.x), "=f"(v.y)
               : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float ldg_stream(const float* a, uint64_t pol) {
  float v;
  asm volatile("ld.global.nc.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ double2 ldg_stream(const double2* a, uint64_t pol) {
  double2 v;
  asm volatile("ld.global.nc.L2::cache_hint.v2.f64 {%0, %1}, [%2], %3;"
               : "=d"(v.x), "=d"(v.y)
               : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ double ldg_stream(const double* a, uint64_t pol) {
  double v;
  asm volatile("ld.global.nc.L2::cache_hint.f64 %0, [%1], %2;" : "=d"(v) : "l"(a), "l"(pol));
  return v;
}

__device__ __forceinline__ void griddep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void griddep_launch_dependents() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
inline cudaError_t launch_maybe_pdl(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                                    size_t smem, cudaStream_t st, Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args&&>(args)...);
}

// Number of SMs of the current device (cached per device).
int sm_count();
int current_device();

#define TLGB_CUDA_TRY(expr)                                                        \
  do {                                                                             \
    cudaError_t _e = (expr);                                                       \
    if (_e != cudaSuccess)                                                         \
      return ::tlgb::set_error(TLGB_ECUDA, std::string(#expr ": ") +               \
                                               cudaGetErrorString(_e));            \
  } while (0)

#define TLGB_CHECK_ARG(cond, msg)                                                  \
  do {                                                                             \
    if (!(cond)) return ::tlgb::set_error(TLGB_EINVAL, msg);                       \
  } while (0)

#define TLGB_LAUNCH_CHECK()                                                        \
  do {                                                                             \
    cudaError_t _e = cudaGetLastError();                                           \
    if (_e != cudaSuccess)                                                         \
      return ::tlgb::set_error(TLGB_ECUDA, std::string("kernel launch: ") +        \
                                               cudaGetErrorString(_e));            \
  } while (0)

constexpr int kMaxModes = TLGB_MAX_MODES;

// Mode geometry of a dense C-order tensor, passed to kernels by value.
struct Shape {
  int ndim;
  int64_t dim[kMaxModes];
  int64_t stride[kMaxModes];  // element strides (C order)
  int64_t numel;
};

inline Shape make_shape(int ndim, const int64_t* dims) {
  Shape s{};
  s.ndim = ndim;
  int64_t st = 1;
  for (int k = ndim - 1; k >= 0; --k) {
    s.dim[k] = dims[k];
    s.stride[k] = st;
    st *= dims[k];
  }
  s.numel = st;
  return s;
}

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Carves aligned sub-buffers out of one caller-provided workspace.
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base(static_cast<char*>(b)) {}
  template <typename T>
  T* take(size_t count) {
    off = align_up(off, 256);
    T* p = base ? reinterpret_cast<T*>(base + off) : nullptr;
    off += count * sizeof(T);
    return p;
  }
  size_t used() const { return align_up(off, 256); }
};

template <typename T> struct TypeCode;
template <> struct TypeCode<float> { static constexpr int value = TLGB_F32; };
template <> struct TypeCode<double> { static constexpr int value = TLGB_F64; };

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

}  // namespace tlgb
