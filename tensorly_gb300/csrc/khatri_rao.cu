// Explicit Khatri-Rao product (tensorly/tenalg/core_tenalg/_khatri_rao.py:9-109).
//
// out[(i_0, ..., i_{n-1}), r] = ((m_0[i_0, r] * w_r) * m_1[i_1, r]) * ... * mask[row]
// The multiplication order is the reference's (weights on the first matrix,
// then one matrix at a time), so results are bit-identical to NumPy's for
// f32 and f64.  Write-bandwidth bound: one output element per thread, rows
// decoded from the flat row index with the first matrix slowest.
#include "common.cuh"

namespace tlgb {
namespace {

struct KrArgs {
  const void* mats[kMaxModes];
  int64_t rows[kMaxModes];
  int n;
  int64_t rank;
  int64_t total_rows;
  const void* weights;
  const void* mask;
  void* out;
};

template <typename T>
__global__ void khatri_rao_kernel(const KrArgs a) {
  const int64_t total = a.total_rows * a.rank;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = e / a.rank;
    const int64_t r = e - row * a.rank;
    int64_t idx[kMaxModes];
    int64_t rr = row;
    for (int k = a.n - 1; k >= 0; --k) {
      idx[k] = rr % a.rows[k];
      rr /= a.rows[k];
    }
    T v = static_cast<const T*>(a.mats[0])[idx[0] * a.rank + r];
    if (a.weights) v = v * static_cast<const T*>(a.weights)[r];
    for (int k = 1; k < a.n; ++k) v = v * static_cast<const T*>(a.mats[k])[idx[k] * a.rank + r];
    if (a.mask) v = v * static_cast<const T*>(a.mask)[row];
    static_cast<T*>(a.out)[e] = v;
  }
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_khatri_rao(int dtype, int n_mats, const void* const* mats,
                               const int64_t* rows, int64_t rank, const void* weights,
                               const void* mask, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "khatri_rao: dtype must be f32 or f64");
  TLGB_CHECK_ARG(n_mats >= 1 && n_mats <= kMaxModes, "khatri_rao: 1..8 matrices supported");
  TLGB_CHECK_ARG(mats && rows && out, "khatri_rao: null pointer");
  TLGB_CHECK_ARG(rank >= 1, "khatri_rao: rank must be >= 1");
  KrArgs a{};
  a.n = n_mats;
  a.rank = rank;
  a.total_rows = 1;
  for (int k = 0; k < n_mats; ++k) {
    TLGB_CHECK_ARG(mats[k] != nullptr && rows[k] >= 0, "khatri_rao: bad matrix");
    a.mats[k] = mats[k];
    a.rows[k] = rows[k];
    a.total_rows *= rows[k];
  }
  a.weights = weights;
  a.mask = mask;
  a.out = out;
  const int64_t total = a.total_rows * rank;
  if (total == 0) return TLGB_OK;
  const int threads = 256;
  const int blocks = (int)std::min<int64_t>(ceil_div(total, threads), (int64_t)sm_count() * 16);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    khatri_rao_kernel<float><<<blocks, threads, 0, st>>>(a);
  else
    khatri_rao_kernel<double><<<blocks, threads, 0, st>>>(a);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
