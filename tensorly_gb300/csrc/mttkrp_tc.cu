// BF16 tensor-core MTTKRP (tcgen05 + TMA, sm_103a).
#include "mttkrp_tc.cuh"

namespace tlgb {
namespace {

__global__ void k_to_bf16(const float* __restrict__ X, int64_t n, __nv_bfloat16* __restrict__ Y) {
  const int64_t n4 = n / 4;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = reinterpret_cast<const float4*>(X)[i];
    __nv_bfloat162 a = __floats2bfloat162_rn(v.x, v.y);
    __nv_bfloat162 b = __floats2bfloat162_rn(v.z, v.w);
    reinterpret_cast<__nv_bfloat162*>(Y)[2 * i] = a;
    reinterpret_cast<__nv_bfloat162*>(Y)[2 * i + 1] = b;
  }
  for (int64_t i = n4 * 4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    Y[i] = __float2bfloat16_rn(X[i]);
}

__global__ void k_factor_bf16t(const float* __restrict__ A, int64_t rows, int64_t R,
                               __nv_bfloat16* __restrict__ out) {
  const int64_t n = rows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R, r = e % R;
    out[r * rows + i] = __float2bfloat16_rn(A[e]);
  }
}

}  // namespace

int tc_launch_to_bf16(const float* X, int64_t n, __nv_bfloat16* out, cudaStream_t st) {
  TLGB_CHECK_ARG((reinterpret_cast<uintptr_t>(X) % 16) == 0 &&
                     (reinterpret_cast<uintptr_t>(out) % 8) == 0,
                 "to_bf16: misaligned buffers");
  const int blocks = sm_count() * 8;
  k_to_bf16<<<blocks, 256, 0, st>>>(X, n, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int tc_launch_factor_bf16t(const float* A, int64_t rows, int64_t R, __nv_bfloat16* out,
                           cudaStream_t st) {
  const int64_t n = rows * R;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), sm_count() * 4));
  k_factor_bf16t<<<blocks, 256, 0, st>>>(A, rows, R, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int mttkrp_tc_prepare() { return set_error(TLGB_EUNSUPPORTED, "bf16 tensor-core MTTKRP not built"); }

int mttkrp_tc_make_plan(const Shape& sh, int64_t rank, int mode, TcPlan* plan) {
  (void)sh; (void)rank; (void)mode; (void)plan;
  return set_error(TLGB_EUNSUPPORTED, "bf16 tensor-core MTTKRP not built");
}

int mttkrp_tc_launch(const TcPlan& p, const __nv_bfloat16* Xbf, const float* const* factors,
                     __nv_bfloat16* const* fbt, const float* weights, float* partial,
                     const int* skip_flag, cudaStream_t st) {
  (void)p; (void)Xbf; (void)factors; (void)fbt; (void)weights; (void)partial; (void)skip_flag;
  (void)st;
  return set_error(TLGB_EUNSUPPORTED, "bf16 tensor-core MTTKRP not built");
}

}  // namespace tlgb
