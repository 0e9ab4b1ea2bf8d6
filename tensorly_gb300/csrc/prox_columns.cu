// Proximal operators of tensorly/tenalg/proximal.py that act per column of a
// factor matrix, or on the ranks of its entries (:270-628):
//   unimodality  (unimodality_prox, :359-441)   monotonicity (:292-356)
//   simplex      (simplex_prox, :558-599)       soft_sparsity (:529-555)
//   smoothness   (smoothness_prox, :270-289)    hard_sparsity (hard_thresholding, :602-628)
//   normalized_sparsity (:496-526)
// Y and P are rows x cols, row-major (a factor matrix); column c is
// Y[i * cols + c].  One CTA per column stages the column in shared memory;
// the sequential parts of the reference (its cumulative sums and the
// backward pass of the monotone fit) run in the reference's order on one
// thread, so the rounding is the reference's.
//   * monotone fit of z: cum = cumsum(z); mon[j] = max over i <= j of the mean
//     z[i..j] (and 0 for j < rows - 1: the reference takes the maximum over
//     a column of a matrix that is zero below the diagonal); then a backward
//     pass replaces mon[i] by mon[i + 1] where it is larger.  Decreasing =
//     the same on the reversed column.
//   * unimodality needs the maximum of the deviation totals over the whole
//     matrix, so it runs as two kernels (per-column fits and totals, then the
//     split point of each column).
//   * smoothness solves (I (1 + 2 r) - r (sub + super diagonal)) x = y by
//     the tridiagonal LU recurrence (the matrix is diagonally dominant, so
//     the reference's partial pivoting never swaps).
//   * simplex sorts the column (bitonic, descending) and applies the
//     reference's threshold rule; soft sparsity is the simplex projection of
//     |y| times sign(y).
//   * hard thresholding keeps the `k` entries of largest magnitude of the
//     whole matrix: an entry's rank is the number of entries of larger
//     magnitude plus the number of equal ones at a lower index (the
//     reference's double argsort breaks such ties in an unspecified order).
#include <algorithm>
#include <cmath>

#include "prox_columns.cuh"

namespace tlgb {
namespace {

constexpr int kPxThreads = 256;
constexpr size_t kPxSmemMax = 200 * 1024;      // dynamic shared memory of one column CTA
constexpr int kHardTile = 2048;                 // magnitudes staged per pass (hard thresholding)

__device__ __forceinline__ bool px_stopped(const int* stop) { return stop && *stop; }

// Monotone non-decreasing fit of z[0..n) into out (block-wide; cum is scratch).
template <typename T>
__device__ void mono_fit(const T* z, T* cum, T* out, int n) {
  if (threadIdx.x == 0) {
    T s = z[0];
    cum[0] = s;
    for (int k = 1; k < n; ++k) {
      s = s + z[k];
      cum[k] = s;
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j < n; j += blockDim.x) {
    T best = cum[j] / T(j + 1);
    if (j < n - 1 && best < T(0)) best = T(0);
    for (int i = 1; i <= j; ++i) {
      const T v = (cum[j] - cum[i - 1]) / T(j - i + 1);
      if (v > best) best = v;
    }
    out[j] = best;
  }
  __syncthreads();
  if (threadIdx.x == 0)
    for (int k = n - 2; k >= 0; --k)
      if (out[k] > out[k + 1]) out[k] = out[k + 1];
  __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(kPxThreads)
k_px_mono(const T* __restrict__ Y, T* __restrict__ P, int rows, int cols, int decreasing,
          const int* stop) {
  if (px_stopped(stop)) return;
  extern __shared__ __align__(16) unsigned char px_smem[];
  T* z = reinterpret_cast<T*>(px_smem);
  T* cum = z + rows;
  T* out = cum + rows;
  const int c = blockIdx.x;
  for (int i = threadIdx.x; i < rows; i += blockDim.x)
    z[i] = Y[(int64_t)(decreasing ? rows - 1 - i : i) * cols + c];
  __syncthreads();
  mono_fit(z, cum, out, rows);
  for (int i = threadIdx.x; i < rows; i += blockDim.x)
    P[(int64_t)(decreasing ? rows - 1 - i : i) * cols + c] = out[i];
}

// Unimodality, first pass: per column the increasing and decreasing fits and
// the deviation totals of every candidate split point; the column's largest
// total in colmax[c].
template <typename T>
__global__ void __launch_bounds__(kPxThreads)
k_px_unimodal_fits(const T* __restrict__ Y, int rows, int cols, T* __restrict__ inc_out,
                   T* __restrict__ dec_out, T* __restrict__ total_out, T* __restrict__ colmax,
                   const int* stop) {
  if (px_stopped(stop)) return;
  extern __shared__ __align__(16) unsigned char px_smem[];
  T* y = reinterpret_cast<T*>(px_smem);
  T* z = y + rows;
  T* cum = z + rows;
  T* inc = cum + rows;
  T* dec = inc + rows;
  const int c = blockIdx.x;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    const T v = Y[(int64_t)i * cols + c];
    y[i] = v;
    z[i] = v;
  }
  __syncthreads();
  mono_fit(z, cum, inc, rows);
  for (int i = threadIdx.x; i < rows; i += blockDim.x) z[i] = y[rows - 1 - i];
  __syncthreads();
  mono_fit(z, cum, dec, rows);            // the decreasing fit, reversed
  for (int i = threadIdx.x; i < rows / 2; i += blockDim.x) {
    const T t = dec[i];
    dec[i] = dec[rows - 1 - i];
    dec[rows - 1 - i] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // sum_inc: exclusive cumulative |y - inc| where both fits lie below y
    T s = T(0), best = T(0);
    for (int i = 0; i < rows; ++i) {
      const T a = fabs(y[i] - inc[i]);
      s = (i == 0) ? a : s + a;
      const bool val = (y[i] - dec[i] >= T(0)) && (y[i] - inc[i] >= T(0));
      cum[i] = val ? s - a : T(0);
    }
    // sum_dec: the same from the bottom, added to sum_inc
    s = T(0);
    for (int k = 0; k < rows; ++k) {
      const int i = rows - 1 - k;
      const T a = fabs(y[i] - dec[i]);
      s = (k == 0) ? a : s + a;
      const bool val = (y[i] - dec[i] >= T(0)) && (y[i] - inc[i] >= T(0));
      const T tot = cum[i] + (val ? s - a : T(0));
      cum[i] = tot;
    }
    for (int i = 0; i < rows; ++i)
      if (i == 0 || cum[i] > best) best = cum[i];
    colmax[c] = best;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    inc_out[(int64_t)i * cols + c] = inc[i];
    dec_out[(int64_t)i * cols + c] = dec[i];
    total_out[(int64_t)i * cols + c] = cum[i];
  }
}

// Unimodality, second pass: the split point k of each column is the first
// minimum of the totals (positions where a fit lies above y count as the
// matrix-wide maximum); increasing fit above k, decreasing fit below, y at k.
template <typename T>
__global__ void __launch_bounds__(kPxThreads)
k_px_unimodal_apply(const T* __restrict__ Y, T* __restrict__ P, int rows, int cols,
                    const T* __restrict__ inc, const T* __restrict__ dec,
                    const T* __restrict__ total, const T* __restrict__ colmax, const int* stop) {
  if (px_stopped(stop)) return;
  __shared__ int s_k;
  const int c = blockIdx.x;
  if (threadIdx.x == 0) {
    T gmax = colmax[0];
    for (int j = 1; j < cols; ++j)
      if (colmax[j] > gmax) gmax = colmax[j];
    int k = 0;
    T bestv = T(0);
    for (int i = 0; i < rows; ++i) {
      const int64_t e = (int64_t)i * cols + c;
      const T y = Y[e];
      const bool val = (y - dec[e] >= T(0)) && (y - inc[e] >= T(0));
      const T d = val ? total[e] : gmax;
      if (i == 0 || d < bestv) { bestv = d; k = i; }
    }
    s_k = k;
  }
  __syncthreads();
  const int k = s_k;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    const int64_t e = (int64_t)i * cols + c;
    P[e] = i < k ? inc[e] : (i > k ? dec[e] : Y[e]);
  }
}

// smoothness_prox: the tridiagonal system with diagonal 2 r + 1 and
// off-diagonals -r, one column per CTA (one thread; the recurrence is serial).
template <typename T>
__global__ void k_px_smooth(const T* __restrict__ Y, T* __restrict__ P, int rows, int cols,
                            double reg, const int* stop) {
  if (px_stopped(stop) || threadIdx.x != 0) return;
  extern __shared__ __align__(16) unsigned char px_smem[];
  T* cp = reinterpret_cast<T*>(px_smem);
  const int c = blockIdx.x;
  const T r = (T)reg;
  const T diag = T(2) * r + T(1), off = -r;
  T m = diag;
  T yp = Y[c] / m;
  cp[0] = off / m;
  P[c] = yp;
  for (int i = 1; i < rows; ++i) {
    m = diag - off * cp[i - 1];
    cp[i] = off / m;
    yp = (Y[(int64_t)i * cols + c] - off * yp) / m;
    P[(int64_t)i * cols + c] = yp;
  }
  T x = P[(int64_t)(rows - 1) * cols + c];
  for (int i = rows - 2; i >= 0; --i) {
    x = P[(int64_t)i * cols + c] - cp[i] * x;
    P[(int64_t)i * cols + c] = x;
  }
}

// simplex_prox (soft = 0) or soft_sparsity_prox (soft = 1) of one column.
template <typename T>
__global__ void __launch_bounds__(kPxThreads)
k_px_simplex(const T* __restrict__ Y, T* __restrict__ P, int rows, int cols, int p2,
             double param, int soft, const int* stop) {
  if (px_stopped(stop)) return;
  extern __shared__ __align__(16) unsigned char px_smem[];
  T* s = reinterpret_cast<T*>(px_smem);   // p2 entries, sorted descending
  T* thr = s + p2;                         // rows entries
  __shared__ T s_diff;
  const int c = blockIdx.x;
  for (int i = threadIdx.x; i < p2; i += blockDim.x) {
    T v = -INFINITY;
    if (i < rows) {
      v = Y[(int64_t)i * cols + c];
      if (soft) v = fabs(v);
    }
    s[i] = v;
  }
  __syncthreads();
  // bitonic sort, descending
  for (int size = 2; size <= p2; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = threadIdx.x; i < p2; i += blockDim.x) {
        const int j = i ^ stride;
        if (j > i) {
          const bool desc = (i & size) == 0;
          const T a = s[i], b = s[j];
          if (desc ? (a < b) : (a > b)) { s[i] = b; s[j] = a; }
        }
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) {
    const T prm = (T)param;
    T cs = T(0);
    int count = 0;
    for (int i = 0; i < rows; ++i) {
      cs = (i == 0) ? s[0] : cs + s[i];
      const T t = (cs - prm) / T(i + 1);
      thr[i] = t;
      if (s[i] > t) ++count;
    }
    const int idx = count - 1 >= 0 ? count - 1 : rows - 1;   // index -1 is the last row
    s_diff = thr[idx];
  }
  __syncthreads();
  const T diff = s_diff;
  for (int i = threadIdx.x; i < rows; i += blockDim.x) {
    const int64_t e = (int64_t)i * cols + c;
    const T y = Y[e];
    if (soft) {
      T v = fabs(y) - diff;
      v = v < T(0) ? T(0) : v;
      const T sg = (y > T(0)) ? T(1) : (y < T(0) ? T(-1) : T(0));
      P[e] = v * sg;
    } else {
      const T v = y - diff;
      P[e] = v < T(0) ? T(0) : v;
    }
  }
}

// hard_thresholding: P = Y where the entry's magnitude rank is below k, else
// 0; per-CTA partial sums of the kept squares in part[] (for the norm).
template <typename T>
__global__ void __launch_bounds__(kPxThreads)
k_px_hard(const T* __restrict__ Y, T* __restrict__ P, int64_t n, double k, double* part,
          const int* stop) {
  if (px_stopped(stop)) return;
  __shared__ T tile[kHardTile];
  __shared__ double red[kPxThreads / 32];
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const T me = e < n ? fabs(Y[e]) : T(0);
  int64_t rank = 0;
  for (int64_t t0 = 0; t0 < n; t0 += kHardTile) {
    const int len = (int)((n - t0) < kHardTile ? (n - t0) : kHardTile);
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += blockDim.x) tile[i] = fabs(Y[t0 + i]);
    __syncthreads();
    if (e < n)
      for (int i = 0; i < len; ++i) {
        const T v = tile[i];
        rank += (v > me) || (v == me && t0 + i < e);
      }
  }
  double sq = 0.0;
  if (e < n) {
    const T y = Y[e];
    const T out = ((double)rank < k) ? y : T(0);
    P[e] = out;
    sq = (double)out * (double)out;
  }
  for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
  __syncthreads();
  if (threadIdx.x == 0 && part) {
    double t = 0.0;
    for (int w = 0; w < kPxThreads / 32; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// normalized_sparsity_prox: P /= ||P|| (the norm from the per-CTA partials,
// summed in a fixed order by every CTA).
template <typename T>
__global__ void k_px_normalise(T* __restrict__ P, int64_t n, const double* part, int nb,
                               const int* stop) {
  if (px_stopped(stop)) return;
  __shared__ double s_norm;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += part[b];
    s_norm = sqrt(t);
  }
  __syncthreads();
  const T nrm = (T)s_norm;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    P[e] = P[e] / nrm;
}

int next_pow2(int n) {
  int p = 1;
  while (p < n) p <<= 1;
  return p;
}

template <typename T>
size_t smem_for_kind(int kind, int64_t rows) {
  const size_t e = sizeof(T);
  switch (kind) {
    case TLGB_CONS_MONOTONICITY: return 3 * (size_t)rows * e;
    case TLGB_CONS_UNIMODALITY: return 5 * (size_t)rows * e;
    case TLGB_CONS_SMOOTHNESS: return (size_t)rows * e;
    case TLGB_CONS_SIMPLEX:
    case TLGB_CONS_SOFT_SPARSITY: return ((size_t)next_pow2((int)rows) + (size_t)rows) * e;
    default: return 0;
  }
}

template <typename T>
int set_smem_attrs() {
  static std::atomic<bool> done[64];   // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && done[dev]) return TLGB_OK;
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_px_mono<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kPxSmemMax));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_px_unimodal_fits<T>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kPxSmemMax));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_px_smooth<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kPxSmemMax));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_px_simplex<T>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kPxSmemMax));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return TLGB_OK;
}

}  // namespace

bool prox_is_matrix_kind(int kind) {
  return kind >= TLGB_CONS_UNIMODALITY && kind <= TLGB_CONS_HARD_SPARSITY;
}

int prox_matrix_check(int dtype, int64_t rows, int64_t cols, int kind) {
  TLGB_CHECK_ARG(rows >= 1 && cols >= 1, "proximal: empty matrix");
  TLGB_CHECK_ARG(cols <= 65535, "proximal: more than 65535 columns");
  if (kind == TLGB_CONS_HARD_SPARSITY || kind == TLGB_CONS_NORM_SPARSITY) {
    if (rows * cols > (int64_t)1 << 22)
      return set_error(TLGB_EUNSUPPORTED,
                       "proximal: hard / normalized sparsity of more than 2^22 entries");
    return TLGB_OK;
  }
  const size_t smem = dtype == TLGB_F64 ? smem_for_kind<double>(kind, rows)
                                        : smem_for_kind<float>(kind, rows);
  if (rows > (1 << 20) || smem > kPxSmemMax)
    return set_error(TLGB_EUNSUPPORTED,
                     "proximal: the column of this operator does not fit one CTA's shared memory");
  return TLGB_OK;
}

size_t prox_matrix_scratch_bytes(int dtype, int64_t rows, int64_t cols, int kind) {
  const size_t e = dtype == TLGB_F64 ? 8 : 4;
  if (kind == TLGB_CONS_UNIMODALITY) return align_up(3 * (size_t)rows * cols * e + cols * e, 256);
  if (kind == TLGB_CONS_HARD_SPARSITY || kind == TLGB_CONS_NORM_SPARSITY)
    return align_up(sizeof(double) * (size_t)ceil_div(rows * cols, (int64_t)kPxThreads), 256);
  return 0;
}

template <typename T>
int prox_matrix_launch(const T* Y, T* P, int64_t rows, int64_t cols, int kind, double param,
                       void* scratch, const int* stop, cudaStream_t st) {
  int rc = set_smem_attrs<T>();
  if (rc) return rc;
  const int I = (int)rows, R = (int)cols;
  const size_t smem = smem_for_kind<T>(kind, rows);
  switch (kind) {
    case TLGB_CONS_MONOTONICITY:   // param != 0: the decreasing fit
      k_px_mono<T><<<R, kPxThreads, smem, st>>>(Y, P, I, R, param != 0.0 ? 1 : 0, stop);
      break;
    case TLGB_CONS_UNIMODALITY: {
      T* inc = static_cast<T*>(scratch);
      T* dec = inc + rows * cols;
      T* tot = dec + rows * cols;
      T* cmax = tot + rows * cols;
      k_px_unimodal_fits<T><<<R, kPxThreads, smem, st>>>(Y, I, R, inc, dec, tot, cmax, stop);
      TLGB_LAUNCH_CHECK();
      k_px_unimodal_apply<T><<<R, kPxThreads, 0, st>>>(Y, P, I, R, inc, dec, tot, cmax, stop);
      break;
    }
    case TLGB_CONS_SMOOTHNESS:
      k_px_smooth<T><<<R, 32, smem, st>>>(Y, P, I, R, param, stop);
      break;
    case TLGB_CONS_SIMPLEX:
    case TLGB_CONS_SOFT_SPARSITY:
      k_px_simplex<T><<<R, kPxThreads, smem, st>>>(Y, P, I, R, next_pow2(I), param,
                                                   kind == TLGB_CONS_SOFT_SPARSITY ? 1 : 0, stop);
      break;
    case TLGB_CONS_HARD_SPARSITY:
    case TLGB_CONS_NORM_SPARSITY: {
      const int64_t n = rows * cols;
      const int nb = (int)ceil_div(n, (int64_t)kPxThreads);
      double* part = static_cast<double*>(scratch);
      k_px_hard<T><<<nb, kPxThreads, 0, st>>>(Y, P, n, param, part, stop);
      if (kind == TLGB_CONS_NORM_SPARSITY) {
        TLGB_LAUNCH_CHECK();
        const unsigned gb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 4);
        k_px_normalise<T><<<gb, 256, 0, st>>>(P, n, part, nb, stop);
      }
      break;
    }
    default:
      return set_error(TLGB_EINVAL, "proximal: not a column-wise operator");
  }
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template int prox_matrix_launch<float>(const float*, float*, int64_t, int64_t, int, double, void*,
                                       const int*, cudaStream_t);
template int prox_matrix_launch<double>(const double*, double*, int64_t, int64_t, int, double,
                                        void*, const int*, cudaStream_t);

}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_proximal_matrix_workspace_size(int dtype, int64_t rows, int64_t cols,
                                                   int kind, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "proximal: dtype must be f32 or f64");
  TLGB_CHECK_ARG(bytes != nullptr, "proximal: null pointer");
  TLGB_CHECK_ARG(kind >= TLGB_CONS_NONE && kind <= TLGB_CONS_HARD_SPARSITY,
                 "proximal: unknown kind");
  if (!prox_is_matrix_kind(kind)) {
    *bytes = tlgb_proximal_workspace_bytes();
    return TLGB_OK;
  }
  int rc = prox_matrix_check(dtype, rows, cols, kind);
  if (rc) return rc;
  *bytes = std::max<size_t>(256, prox_matrix_scratch_bytes(dtype, rows, cols, kind));
  return TLGB_OK;
}

extern "C" int tlgb_proximal_matrix(int dtype, const void* Y, int64_t rows, int64_t cols,
                                    int kind, double param, void* out, void* workspace,
                                    size_t workspace_bytes, void* stream) {
  clear_error();
  size_t need = 0;
  int rc = tlgb_proximal_matrix_workspace_size(dtype, rows, cols, kind, &need);
  if (rc) return rc;
  TLGB_CHECK_ARG(Y && out, "proximal: null pointer");
  if (!prox_is_matrix_kind(kind))
    return tlgb_proximal(dtype, Y, rows * cols, kind, param, out, workspace, workspace_bytes,
                         stream);
  if (!workspace || workspace_bytes < need)
    return set_error(TLGB_EWORKSPACE, "proximal: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return prox_matrix_launch<double>(static_cast<const double*>(Y), static_cast<double*>(out),
                                      rows, cols, kind, param, workspace, nullptr, st);
  return prox_matrix_launch<float>(static_cast<const float*>(Y), static_cast<float*>(out), rows,
                                   cols, kind, param, workspace, nullptr, st);
}
