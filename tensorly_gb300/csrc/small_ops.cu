// Small dense operations the non-negative Tucker update is composed of: a
// strided GEMM for the core-sized products (tensorly's tl.dot on unfolded
// cores and factor Grams), the multiplicative update
// A <- A * clip(num, eps) / clip(den, eps) (tensorly/decomposition/_tucker.py:
// 396-406 and 410-418), and an f64 inner product.
#include "common.cuh"

namespace tlgb {
namespace {

constexpr int kGemmTile = 32;

// C[m, n] = sum_k A[m * sam + k * sak] * B[k * sbk + n * sbn] (C row-major,
// ldc = N); accumulated in T in k order.  32 x 32 output tiles, 16 k a step
// staged in shared memory, 4 outputs a thread.
template <typename T>
__global__ void __launch_bounds__(256)
k_gemm_strided(int64_t M, int64_t N, int64_t K, const T* __restrict__ A, int64_t sam,
               int64_t sak, const T* __restrict__ B, int64_t sbk, int64_t sbn, T* __restrict__ C) {
  constexpr int KS = 16;
  __shared__ T As[KS][kGemmTile + 1];
  __shared__ T Bs[KS][kGemmTile + 1];
  const int tid = threadIdx.x;
  const int tn = tid & 31, tm = tid >> 5;              // 8 row groups of 4
  const int64_t m0 = (int64_t)blockIdx.y * kGemmTile, n0 = (int64_t)blockIdx.x * kGemmTile;
  T acc[4] = {(T)0, (T)0, (T)0, (T)0};
  for (int64_t k0 = 0; k0 < K; k0 += KS) {
    for (int e = tid; e < KS * kGemmTile; e += 256) {
      const int kk = e / kGemmTile, c = e - kk * kGemmTile;
      const int64_t k = k0 + kk;
      As[kk][c] = (k < K && m0 + c < M) ? A[(m0 + c) * sam + k * sak] : (T)0;
      Bs[kk][c] = (k < K && n0 + c < N) ? B[k * sbk + (n0 + c) * sbn] : (T)0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < KS; ++kk) {
      const T b = Bs[kk][tn];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] = fma(As[kk][tm * 4 + i], b, acc[i]);
    }
    __syncthreads();
  }
  const int64_t n = n0 + tn;
  if (n >= N) return;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t m = m0 + tm * 4 + i;
    if (m < M) C[m * N + n] = acc[i];
  }
}

// A <- A * max(num, eps) / max(den, eps)  (the reference's clip(a_min=eps)).
template <typename T>
__global__ void k_mu_apply(T* __restrict__ A, const T* __restrict__ num,
                           const T* __restrict__ den, int64_t n, T eps) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T a = num[e] > eps ? num[e] : eps;
    const T b = den[e] > eps ? den[e] : eps;
    A[e] = A[e] * (a / b);
  }
}

constexpr int kDotBlocks = 128;

template <typename T>
__global__ void k_dot_part(const T* __restrict__ a, const T* __restrict__ b, int64_t n,
                           double* part) {
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    s += (double)a[e] * (double)b[e];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// Missing-entry refill of a masked decomposition:
// x = x * mask + rec * (1 - mask), in place, with the block partials of
// ||x||^2 and ||x - rec||^2 (f64) in part[2 * block + {0, 1}].
template <typename T>
__global__ void k_mask_impute_part(T* __restrict__ x, const T* __restrict__ mask,
                                   const T* __restrict__ rec, int64_t n, double* part) {
  __shared__ double red[2][8];
  double s0 = 0.0, s1 = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T m = mask[e], r = rec[e];
    const T v = x[e] * m + r * (T(1) - m);
    x[e] = v;
    const double dv = (double)v, dr = (double)v - (double)r;
    s0 = fma(dv, dv, s0);
    s1 = fma(dr, dr, s1);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    s1 += __shfl_xor_sync(0xffffffffu, s1, o);
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = s0;
    red[1][threadIdx.x >> 5] = s1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { t0 += red[0][w]; t1 += red[1][w]; }
    part[2 * blockIdx.x] = t0;
    part[2 * blockIdx.x + 1] = t1;
  }
}

__global__ void k_mask_impute_final(const double* part, int nb, double* out) {
  if (threadIdx.x == 0) {
    double t0 = 0.0, t1 = 0.0;
    for (int b = 0; b < nb; ++b) { t0 += part[2 * b]; t1 += part[2 * b + 1]; }
    out[0] = sqrt(t0);
    out[1] = sqrt(t1);
  }
}

// x = where(mask == 0, rec (or fill when rec is null), x), in place
// (tensorly/decomposition/_parafac2.py:21-65, the missing-entry refill).
template <typename T>
__global__ void k_mask_where(T* __restrict__ x, const T* __restrict__ mask,
                             const T* __restrict__ rec, T fill, int64_t n) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    if (mask[e] == T(0)) x[e] = rec ? rec[e] : fill;
}

// Block partials of sum((mask * x - mask * rec)^2) in f64.
template <typename T>
__global__ void k_masked_sq_diff_part(const T* __restrict__ x, const T* __restrict__ mask,
                                      const T* __restrict__ rec, int64_t n, double* part) {
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T m = mask[e];
    const double d = (double)(m * x[e] - m * rec[e]);
    s = fma(d, d, s);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

// x = max(x, lo) in place (NaN stays NaN, as numpy's clip keeps it).
template <typename T>
__global__ void k_clip_min(T* __restrict__ x, int64_t n, T lo) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    if (x[e] < lo) x[e] = lo;
}

// sparsify_tensor (tensorly/decomposition/_cp.py:140-159) on the residual
// R = X - L: the card-th largest |R| by a most-significant-digit radix
// select over the bit patterns of |R| (for non-negative IEEE values the bit
// order is the numeric order), 8 bits a pass, all on the device; then the
// norm of the entries below it (the sparse component keeps the others).
struct SelState {
  unsigned long long prefix;   // the digits of the selected key found so far
  unsigned long long k;        // rank still to find below the fixed digits
};
constexpr int kSelBlocks = 152 * 4;

template <typename T> struct KeyOf;
template <> struct KeyOf<float> {
  using U = unsigned int;
  static constexpr int kBits = 32;
  __device__ static U key(float v) { return __float_as_uint(v) & 0x7fffffffu; }
  __device__ static float from(U k) { return __uint_as_float(k); }
};
template <> struct KeyOf<double> {
  using U = unsigned long long;
  static constexpr int kBits = 64;
  __device__ static U key(double v) {
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
  }
  __device__ static double from(U k) { return __longlong_as_double((long long)k); }
};

template <typename T>
__global__ void __launch_bounds__(256)
k_sel_hist(const T* __restrict__ X, const T* __restrict__ L, int64_t n, int shift,
           const SelState* st, unsigned long long* __restrict__ hist) {
  using K = KeyOf<T>;
  __shared__ unsigned int h[256];
  for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const int hi = shift + 8;
  const unsigned long long hi_mask = hi >= K::kBits ? 0ull : (~0ull << hi);
  const unsigned long long want = st->prefix & hi_mask;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const unsigned long long key = (unsigned long long)K::key(X[e] - L[e]);
    if ((key & hi_mask) == want) atomicAdd(&h[(key >> shift) & 255u], 1u);
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256; b += blockDim.x)
    if (h[b]) atomicAdd(&hist[b], (unsigned long long)h[b]);
}

// Fixes the digit at `shift`: the bin, from the top, where the count of keys
// at or above it first reaches k; clears the histogram for the next pass.
__global__ void k_sel_pick(unsigned long long* hist, int shift, SelState* st) {
  if (threadIdx.x == 0) {
    unsigned long long cum = 0, k = st->k;
    int bin = 0;
    for (int b = 255; b >= 0; --b) {
      if (cum + hist[b] >= k) { bin = b; break; }
      cum += hist[b];
    }
    st->prefix |= (unsigned long long)bin << shift;
    st->k = k - cum;
  }
  __syncthreads();
  for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
}

// sum of R^2 over |R| < bound (f64, per-block partials), and the sparse
// component where(|R| < bound, 0, R) when `sparse` is given.
template <typename T>
__global__ void __launch_bounds__(256)
k_sel_resid(const T* __restrict__ X, const T* __restrict__ L, int64_t n, const SelState* st,
            int keep_all, T* __restrict__ sparse, double* part) {
  using K = KeyOf<T>;
  const T bound = keep_all ? T(0) : K::from((typename K::U)st->prefix);
  __shared__ double red[8];
  double acc = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T r = X[e] - L[e];
    const bool small = !keep_all && fabs(r) < bound;
    if (small) acc += (double)r * (double)r;
    if (sparse) sparse[e] = small ? T(0) : r;
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_sel_init(SelState* st, unsigned long long k, unsigned long long* hist) {
  if (threadIdx.x == 0) {
    st->prefix = 0ull;
    st->k = k;
  }
  for (int b = threadIdx.x; b < 256; b += blockDim.x) hist[b] = 0;
}

__global__ void k_sel_final(const double* part, int nb, double* out) {
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += part[b];
    out[0] = sqrt(t);
  }
}

// Kronecker product of n_mats matrices, left to right (the first matrix
// varies slowest), each entry the product of one entry of every matrix taken
// in that order (tensorly/tenalg/core_tenalg/_kronecker.py).
struct KronArgs {
  const void* m[kMaxModes];
  int64_t rows[kMaxModes], cols[kMaxModes];
  int n;
};
template <typename T>
__global__ void k_kronecker(KronArgs a, int64_t out_rows, int64_t out_cols, T* __restrict__ out) {
  const int64_t total = out_rows * out_cols;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t i = e / out_cols, j = e - (e / out_cols) * out_cols;
    int64_t ri[kMaxModes], ci[kMaxModes];
    for (int k = a.n - 1; k >= 0; --k) {
      ri[k] = i % a.rows[k];
      i /= a.rows[k];
      ci[k] = j % a.cols[k];
      j /= a.cols[k];
    }
    T v = static_cast<const T*>(a.m[0])[ri[0] * a.cols[0] + ci[0]];
    for (int k = 1; k < a.n; ++k) v = v * static_cast<const T*>(a.m[k])[ri[k] * a.cols[k] + ci[k]];
    out[e] = v;
  }
}

// tucker_normalize (tensorly/tucker_tensor.py:78-102): every factor column
// scaled to unit norm, the core multiplied along each mode by the column
// norms of that mode, in mode order; a zero column is left as it is.
struct TnArgs {
  void* f[kMaxModes];
  int64_t rows[kMaxModes], ranks[kMaxModes];
  int64_t foff[kMaxModes + 1];   // cumulative factor entries
  int64_t soff[kMaxModes + 1];   // cumulative columns (offsets into the scales)
  void* core;
  int64_t core_n;
  int n;
};
template <typename T>
__global__ void k_tn_colnorms(TnArgs a, double* __restrict__ scales) {
  const int64_t col = blockIdx.x;
  int m = 0;
  while (col >= a.soff[m + 1]) ++m;
  const int64_t c = col - a.soff[m], R = a.ranks[m];
  const T* f = static_cast<const T*>(a.f[m]);
  double acc = 0.0;
  for (int64_t r = threadIdx.x; r < a.rows[m]; r += blockDim.x) {
    const double v = (double)f[r * R + c];
    acc += v * v;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) scales[col] = (double)(T)sqrt(acc);
  }
}
template <typename T>
__global__ void k_tn_apply(TnArgs a, const double* __restrict__ scales) {
  const int64_t nf = a.foff[a.n], total = nf + a.core_n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    if (e < nf) {
      int m = 0;
      while (e >= a.foff[m + 1]) ++m;
      const int64_t k = e - a.foff[m];
      const T s = (T)scales[a.soff[m] + k % a.ranks[m]];
      T* f = static_cast<T*>(a.f[m]);
      f[k] = f[k] / (s == T(0) ? T(1) : s);
    } else {
      int64_t k = e - nf, rem = k;
      int64_t idx[kMaxModes];
      for (int m = a.n - 1; m >= 0; --m) {
        idx[m] = rem % a.ranks[m];
        rem /= a.ranks[m];
      }
      T* g = static_cast<T*>(a.core);
      T v = g[k];
      for (int m = 0; m < a.n; ++m) v = v * (T)scales[a.soff[m] + idx[m]];
      g[k] = v;
    }
  }
}

// Active-set NNLS of tensorly/solvers/nnls.py:275-406 (Bro and De Jong's
// variant of Lawson-Hanson) for one system of n <= kAsMax unknowns, one CTA:
// x minimises ||Utm - UtU x|| with x >= 0, starting from x.  The passive-set
// systems are solved by LU with partial pivoting (the reference's
// np.linalg.solve); a zero pivot is the reference's singular-matrix
// exception: on the first solve of an iteration it restarts from zero as the
// reference's except branch does, elsewhere it ends the call with
// TLGB_ESINGULAR in *status (the reference raises there).
constexpr int kAsMax = 128;

template <typename T>
__device__ bool as_solve(const T* __restrict__ UtU, const T* __restrict__ Utm, int n,
                         const int* passive, T* A, T* b, int* idx, int* s_m, int* s_sing,
                         int* s_piv, T* support) {
  if (threadIdx.x == 0) {
    int m = 0;
    for (int i = 0; i < n; ++i)
      if (passive[i]) idx[m++] = i;
    *s_m = m;
    *s_sing = 0;
  }
  __syncthreads();
  const int m = *s_m;
  for (int e = threadIdx.x; e < m * m; e += blockDim.x)
    A[e] = UtU[(int64_t)idx[e / m] * n + idx[e % m]];
  for (int e = threadIdx.x; e < m; e += blockDim.x) b[e] = Utm[idx[e]];
  __syncthreads();
  for (int k = 0; k < m; ++k) {
    if (threadIdx.x == 0) {   // partial pivoting (first largest magnitude), row swap
      int p = k;
      T best = fabs(A[k * m + k]);
      for (int i = k + 1; i < m; ++i)
        if (fabs(A[i * m + k]) > best) { best = fabs(A[i * m + k]); p = i; }
      if (best == T(0)) *s_sing = 1;
      *s_piv = p;
    }
    __syncthreads();
    if (*s_sing) break;   // uniform: read after the barrier
    const int p = *s_piv;
    if (p != k) {
      for (int j = threadIdx.x; j < m; j += blockDim.x) {
        const T t = A[k * m + j];
        A[k * m + j] = A[p * m + j];
        A[p * m + j] = t;
      }
      if (threadIdx.x == 0) { const T t = b[k]; b[k] = b[p]; b[p] = t; }
    }
    __syncthreads();
    const T inv = T(1) / A[k * m + k];
    for (int i = k + 1 + threadIdx.x; i < m; i += blockDim.x) A[i * m + k] *= inv;
    __syncthreads();
    const int w = m - k - 1;
    for (int e = threadIdx.x; e < w * w; e += blockDim.x) {
      const int i = k + 1 + e / w, j = k + 1 + e % w;
      A[i * m + j] -= A[i * m + k] * A[k * m + j];
    }
    __syncthreads();
  }
  if (*s_sing) return false;
  if (threadIdx.x == 0) {
    for (int i = 0; i < m; ++i) {            // forward, unit lower
      T v = b[i];
      for (int j = 0; j < i; ++j) v -= A[i * m + j] * b[j];
      b[i] = v;
    }
    for (int i = m - 1; i >= 0; --i) {       // back, upper
      T v = b[i];
      for (int j = i + 1; j < m; ++j) v -= A[i * m + j] * b[j];
      b[i] = v / A[i * m + i];
    }
    for (int i = 0; i < n; ++i) support[i] = T(0);
    for (int j = 0; j < m; ++j) support[idx[j]] = b[j];
  }
  __syncthreads();
  return true;
}

template <typename T>
__global__ void __launch_bounds__(256)
k_active_set_nnls(const T* __restrict__ UtU, const T* __restrict__ Utm, T* __restrict__ xg,
                  int n, int n_iter_max, double tol, int* status) {
  extern __shared__ __align__(16) unsigned char as_smem[];
  T* A = reinterpret_cast<T*>(as_smem);   // n x n
  T* b = A + n * n;
  T* x = b + n;
  T* grad = x + n;
  T* support = grad + n;
  int* passive = reinterpret_cast<int*>(support + n);
  int* idx = passive + n;
  __shared__ int s_m, s_sing, s_piv, s_flag, s_fail;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = xg[i];
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  auto gradient = [&]() {   // grad = Utm - UtU x
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      T v = T(0);
      for (int j = 0; j < n; ++j) v += UtU[(int64_t)i * n + j] * x[j];
      grad[i] = Utm[i] - v;
    }
    __syncthreads();
  };
  auto argmax_grad = [&]() {   // first index of the largest gradient entry
    int best = 0;
    for (int i = 1; i < n; ++i)
      if (grad[i] > grad[best]) best = i;
    return best;
  };
  gradient();
  if (threadIdx.x == 0) {
    for (int i = 0; i < n; ++i) { passive[i] = x[i] > T(0); support[i] = T(0); }
  }
  __syncthreads();
  for (int it = 0; it < n_iter_max; ++it) {
    if (threadIdx.x == 0) {
      bool all0 = true;
      for (int i = 0; i < n; ++i) all0 = all0 && (x[i] == T(0));
      if (it > 0 || all0) passive[argmax_grad()] = 1;
    }
    __syncthreads();
    if (!as_solve(UtU, Utm, n, passive, A, b, idx, &s_m, &s_sing, &s_piv, support)) {
      // the reference's except branch: restart from zero with one passive index
      if (threadIdx.x == 0) {
        for (int i = 0; i < n; ++i) { x[i] = T(0); support[i] = T(0); passive[i] = 0; }
        passive[argmax_grad()] = 1;
      }
      __syncthreads();
      if (!as_solve(UtU, Utm, n, passive, A, b, idx, &s_m, &s_sing, &s_piv, support)) {
        if (threadIdx.x == 0) s_fail = 1;
        __syncthreads();
        break;
      }
    }
    // step back along the segment to x while a passive entry is not positive
    if (threadIdx.x == 0) {
      bool any = false, nonpos = false;
      T mn = T(0);
      for (int i = 0; i < n; ++i)
        if (passive[i]) {
          mn = any ? (support[i] < mn ? support[i] : mn) : support[i];
          any = true;
        }
      nonpos = any && mn <= T(0);
      if (!any) s_fail = 2;                  // the reference's min of an empty selection
      s_flag = nonpos ? 1 : 0;
    }
    __syncthreads();
    if (s_fail) break;
    if (s_flag) {
      for (int rep = 0; rep < n; ++rep) {
        if (threadIdx.x == 0) {
          T alpha = T(0);
          bool first = true;
          for (int i = 0; i < n; ++i)
            if (passive[i] && support[i] <= T(0)) {
              const T r = x[i] / (x[i] - support[i]);
              if (first || r < alpha) alpha = r;
              first = false;
            }
          for (int i = 0; i < n; ++i) {
            x[i] = x[i] + alpha * (support[i] - x[i]);
            passive[i] = x[i] > T(0);
          }
        }
        __syncthreads();
        if (!as_solve(UtU, Utm, n, passive, A, b, idx, &s_m, &s_sing, &s_piv, support)) {
          if (threadIdx.x == 0) s_fail = 1;
          __syncthreads();
          break;
        }
        if (threadIdx.x == 0) {
          bool any = false;
          T mn = T(0);
          for (int i = 0; i < n; ++i)
            if (passive[i]) {
              mn = any ? (support[i] < mn ? support[i] : mn) : support[i];
              any = true;
            }
          s_flag = (!any || mn > T(0)) ? 1 : 0;
        }
        __syncthreads();
        if (s_flag) break;
      }
      if (s_fail) break;
    }
    // x = clip(support, 0, max(support)); the gradient; the stop test
    if (threadIdx.x == 0) {
      T mx = support[0];
      for (int i = 1; i < n; ++i) mx = support[i] > mx ? support[i] : mx;
      for (int i = 0; i < n; ++i) {   // min(max(v, 0), mx), the order of np.clip
        const T v = support[i] < T(0) ? T(0) : support[i];
        x[i] = v > mx ? mx : v;
      }
    }
    __syncthreads();
    gradient();
    if (threadIdx.x == 0) {   // the active set is the complement of the passive set,
      bool any_active = false;  // which the clip above does not recompute
      T gmax = T(0);
      for (int i = 0; i < n; ++i)
        if (!passive[i]) {
          gmax = any_active ? (grad[i] > gmax ? grad[i] : gmax) : grad[i];
          any_active = true;
        }
      s_flag = (!any_active || (double)gmax <= tol) ? 1 : 0;
    }
    __syncthreads();
    if (s_flag) break;
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) xg[i] = x[i];
  if (threadIdx.x == 0 && status) *status = s_fail ? TLGB_ESINGULAR : TLGB_OK;
}

__global__ void k_dot_final(const double* part, int nb, double* out) {
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int b = 0; b < nb; ++b) t += part[b];
    *out = t;
  }
}

// One FISTA iteration on the core (tensorly/solvers/nnls.py:177-272, the
// list-of-Grams branch, non_negative, no ridge):
//   x_new = max-floor(x_upd - lr ((-UtM + g) + sparsity), eps)   (g = x_upd x_k G_k)
//   x_upd = x_new + coef (x_new - x);  x = x_new
// and per-CTA sums of (x - x_new) for the stop test.  Returns at once once
// the stop flag is set.
struct FistaState {
  double norm0;
  int stop;
};

template <typename T>
__global__ void k_fista_step(const T* __restrict__ UtM, const T* __restrict__ g, T* __restrict__ x,
                             T* __restrict__ xu, int64_t n, T lr, T sparsity, T coef, T eps,
                             const FistaState* fs, double* part) {
  if (fs->stop) return;
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T grad = ((-UtM[e] + g[e]) + sparsity);
    T xn = xu[e] - lr * grad;
    xn = xn < eps ? eps : xn;
    const T xo = x[e];
    xu[e] = xn + coef * (xn - xo);
    x[e] = xn;
    s += (double)(xo - xn);
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

__global__ void k_fista_check(const double* part, int nb, int it, double tol, FistaState* fs) {
  if (fs->stop || threadIdx.x != 0) return;
  double t = 0.0;
  for (int b = 0; b < nb; ++b) t += part[b];
  const double nrm = fabs(t);
  if (it == 0) fs->norm0 = nrm;
  if (nrm < tol * fs->norm0) fs->stop = 1;
}

// out = x + (y - x) * s (the line search extrapolation of
// tensorly/decomposition/_parafac2.py:261-264).
template <typename T>
__global__ void k_lerp(const T* __restrict__ x, const T* __restrict__ y, int64_t n, T s,
                       T* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = x[e] + (y[e] - x[e]) * s;
}

// out = 1 / sqrt(x) (inverse square roots of eigenvalues, PARAFAC2 projections).
template <typename T>
__global__ void k_inv_sqrt(const T* __restrict__ x, int64_t n, T* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = (T)1 / sqrt(x[e]);
}

constexpr int kQrThreads = 256;

// Householder QR of an m x n row-major matrix A (m >= n) with LAPACK's
// conventions (dgeqr2 / dlarfg: beta = -sign(alpha) sqrt(alpha^2 + |x|^2),
// tau = (beta - alpha) / beta, v = x / (alpha - beta) with v_0 = 1; a zero
// column below the diagonal gives tau = 0), then the explicit Q (m x n) =
// H_0 H_1 ... H_{n-1} [I; 0] as dorg2r forms it.  One CTA; a warp per column
// for the reflector applications.  W (m x n) and V (m x n) are scratch.
template <typename T>
__global__ void __launch_bounds__(kQrThreads)
k_qr_householder(const T* __restrict__ A, int64_t m, int n, T* W, T* V, T* Q) {
  __shared__ double red[kQrThreads / 32];
  __shared__ double taus[256];
  __shared__ T sh_scale, sh_beta;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = kQrThreads / 32;
  for (int64_t e = tid; e < m * n; e += kQrThreads) W[e] = A[e];
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    double s = 0.0;
    for (int64_t i = k + 1 + tid; i < m; i += kQrThreads) {
      const double w = (double)W[i * n + k];
      s += w * w;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < nw; ++w) t += red[w];
      const double alpha = (double)W[(int64_t)k * n + k];
      const double xnorm = sqrt(t);
      if (xnorm == 0.0) {
        taus[k] = 0.0;
        sh_beta = (T)alpha;
        sh_scale = (T)0;
      } else {
        const double beta = -copysign(sqrt(alpha * alpha + t), alpha);
        taus[k] = (beta - alpha) / beta;
        sh_beta = (T)beta;
        sh_scale = (T)(1.0 / (alpha - beta));
      }
    }
    __syncthreads();
    for (int64_t i = k + 1 + tid; i < m; i += kQrThreads) V[i * n + k] = W[i * n + k] * sh_scale;
    if (tid == 0) {
      V[(int64_t)k * n + k] = (T)1;
      W[(int64_t)k * n + k] = sh_beta;
    }
    __syncthreads();
    const T tau = (T)taus[k];
    if (tau != (T)0) {
      for (int j = k + 1 + warp; j < n; j += nw) {      // W[k:, j] -= tau v (v^T W[k:, j])
        T d = (T)0;
        for (int64_t i = k + lane; i < m; i += 32) d += V[i * n + k] * W[i * n + j];
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        const T f = tau * d;
        for (int64_t i = k + lane; i < m; i += 32) W[i * n + j] -= f * V[i * n + k];
      }
    }
    __syncthreads();
  }
  for (int64_t e = tid; e < m * n; e += kQrThreads) {
    const int64_t i = e / n;
    const int j = (int)(e - i * n);
    Q[e] = (i == j) ? (T)1 : (T)0;
  }
  __syncthreads();
  for (int k = n - 1; k >= 0; --k) {
    const T tau = (T)taus[k];
    if (tau != (T)0) {
      for (int j = k + warp; j < n; j += nw) {          // Q[k:, j] -= tau v (v^T Q[k:, j])
        T d = (T)0;
        for (int64_t i = k + lane; i < m; i += 32) d += V[i * n + k] * Q[i * n + j];
        for (int o = 16; o > 0; o >>= 1) d += __shfl_xor_sync(0xffffffffu, d, o);
        const T f = tau * d;
        for (int64_t i = k + lane; i < m; i += 32) Q[i * n + j] -= f * V[i * n + k];
      }
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_lerp(int dtype, const void* x, const void* y, int64_t n, double s, void* out,
                         void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "lerp: dtype must be f32 or f64");
  TLGB_CHECK_ARG(x && y && out && n >= 0, "lerp: bad argument");
  if (n == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_lerp<double><<<nb, 256, 0, st>>>(static_cast<const double*>(x),
                                       static_cast<const double*>(y), n, s,
                                       static_cast<double*>(out));
  else
    k_lerp<float><<<nb, 256, 0, st>>>(static_cast<const float*>(x), static_cast<const float*>(y),
                                      n, (float)s, static_cast<float*>(out));
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_inv_sqrt(int dtype, const void* x, int64_t n, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "inv_sqrt: dtype must be f32 or f64");
  TLGB_CHECK_ARG(x && out && n >= 0, "inv_sqrt: bad argument");
  if (n == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_inv_sqrt<double><<<nb, 256, 0, st>>>(static_cast<const double*>(x), n,
                                           static_cast<double*>(out));
  else
    k_inv_sqrt<float><<<nb, 256, 0, st>>>(static_cast<const float*>(x), n,
                                          static_cast<float*>(out));
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_qr_workspace_size(int dtype, int64_t m, int64_t n, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "qr: dtype must be f32 or f64");
  TLGB_CHECK_ARG(m >= n && n >= 1 && n <= 256 && bytes, "qr: need m >= n, 1 <= n <= 256");
  *bytes = align_up(2 * (size_t)m * n * (dtype == TLGB_F64 ? 8 : 4), 256);
  return TLGB_OK;
}

extern "C" int tlgb_qr(int dtype, const void* A, int64_t m, int64_t n, void* Q, void* workspace,
                       size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "qr: dtype must be f32 or f64");
  TLGB_CHECK_ARG(A && Q, "qr: null pointer");
  TLGB_CHECK_ARG(m >= n && n >= 1 && n <= 256, "qr: need m >= n, 1 <= n <= 256");
  const size_t esz = dtype == TLGB_F64 ? 8 : 4;
  if (!workspace || workspace_bytes < 2 * (size_t)m * n * esz)
    return set_error(TLGB_EWORKSPACE, "qr: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* w = static_cast<char*>(workspace);
  if (dtype == TLGB_F64)
    k_qr_householder<double><<<1, kQrThreads, 0, st>>>(
        static_cast<const double*>(A), m, (int)n, reinterpret_cast<double*>(w),
        reinterpret_cast<double*>(w + (size_t)m * n * esz), static_cast<double*>(Q));
  else
    k_qr_householder<float><<<1, kQrThreads, 0, st>>>(
        static_cast<const float*>(A), m, (int)n, reinterpret_cast<float*>(w),
        reinterpret_cast<float*>(w + (size_t)m * n * esz), static_cast<float*>(Q));
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_mode_dot(int dtype, const void* X, int ndim, const int64_t* shape,
                             const void* U, int64_t J, int transpose, int mode, void* out,
                             void* stream);

static size_t fista_ws_bytes(int dtype, int64_t n) {
  const size_t esz = dtype == TLGB_F64 ? 8 : 4;
  return align_up(3 * esz * (size_t)n, 256) + align_up(sizeof(double) * kDotBlocks, 256) +
         align_up(sizeof(FistaState), 256);
}

extern "C" int tlgb_fista_tucker_core_workspace_size(int dtype, int ndim, const int64_t* shape,
                                                     size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "fista: dtype must be f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes && shape && bytes, "fista: bad argument");
  int64_t n = 1;
  for (int k = 0; k < ndim; ++k) n *= shape[k];
  *bytes = fista_ws_bytes(dtype, n);
  return TLGB_OK;
}

extern "C" int tlgb_fista_tucker_core(int dtype, const void* UtM, int ndim, const int64_t* shape,
                                      const void* const* grams, void* x, int n_iter_max,
                                      double sparsity, double lr, double tol, double eps,
                                      void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "fista: dtype must be f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes && shape && UtM && grams && x,
                 "fista: bad argument");
  int64_t n = 1;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(shape[k] >= 1 && grams[k] != nullptr, "fista: bad shape or Gram");
    n *= shape[k];
  }
  if (!workspace || workspace_bytes < fista_ws_bytes(dtype, n))
    return set_error(TLGB_EWORKSPACE, "fista: workspace too small");
  const size_t esz = dtype == TLGB_F64 ? 8 : 4;
  char* base = static_cast<char*>(workspace);
  char* xu = base;
  char* b0 = base + esz * n;
  char* b1 = base + 2 * esz * n;
  double* part = reinterpret_cast<double*>(base + align_up(3 * esz * (size_t)n, 256));
  FistaState* fs = reinterpret_cast<FistaState*>(
      base + align_up(3 * esz * (size_t)n, 256) + align_up(sizeof(double) * kDotBlocks, 256));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  TLGB_CUDA_TRY(cudaMemcpyAsync(xu, x, esz * n, cudaMemcpyDeviceToDevice, st));
  TLGB_CUDA_TRY(cudaMemsetAsync(fs, 0, sizeof(FistaState), st));
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, (int64_t)256), kDotBlocks));
  double m_old = 1.0;
  for (int it = 0; it < n_iter_max; ++it) {
    // g = x_upd x_0 G_0 x_1 G_1 ... (ping-pong between b0 and b1)
    const void* src = xu;
    char* dst = b0;
    for (int k = 0; k < ndim; ++k) {
      int rc = tlgb_mode_dot(dtype, src, ndim, shape, grams[k], shape[k], 0, k, dst, stream);
      if (rc) return rc;
      src = dst;
      dst = dst == b0 ? b1 : b0;
    }
    const double m = (1.0 + std::sqrt(1.0 + 4.0 * m_old * m_old)) / 2.0;
    const double coef = (m_old - 1.0) / m;
    m_old = m;
    if (dtype == TLGB_F64)
      k_fista_step<double><<<nb, 256, 0, st>>>(
          static_cast<const double*>(UtM), static_cast<const double*>(src),
          static_cast<double*>(x), reinterpret_cast<double*>(xu), n, lr, sparsity, coef, eps, fs,
          part);
    else
      k_fista_step<float><<<nb, 256, 0, st>>>(
          static_cast<const float*>(UtM), static_cast<const float*>(src), static_cast<float*>(x),
          reinterpret_cast<float*>(xu), n, (float)lr, (float)sparsity, (float)coef, (float)eps, fs,
          part);
    TLGB_LAUNCH_CHECK();
    k_fista_check<<<1, 32, 0, st>>>(part, nb, it, tol, fs);
    TLGB_LAUNCH_CHECK();
  }
  return TLGB_OK;
}

extern "C" int tlgb_gemm(int dtype, int64_t M, int64_t N, int64_t K, const void* A, int64_t sam,
                         int64_t sak, const void* B, int64_t sbk, int64_t sbn, void* C,
                         void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "gemm: dtype must be f32 or f64");
  TLGB_CHECK_ARG(M >= 0 && N >= 0 && K >= 0, "gemm: negative size");
  TLGB_CHECK_ARG(C != nullptr && (K == 0 || (A && B)), "gemm: null pointer");
  if (M == 0 || N == 0) return TLGB_OK;
  const int64_t gx = ceil_div(N, (int64_t)kGemmTile), gy = ceil_div(M, (int64_t)kGemmTile);
  TLGB_CHECK_ARG(gx <= INT32_MAX && gy <= 65535, "gemm: too large");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  dim3 grid((unsigned)gx, (unsigned)gy);
  if (dtype == TLGB_F64)
    k_gemm_strided<double><<<grid, 256, 0, st>>>(M, N, K, static_cast<const double*>(A), sam, sak,
                                                 static_cast<const double*>(B), sbk, sbn,
                                                 static_cast<double*>(C));
  else
    k_gemm_strided<float><<<grid, 256, 0, st>>>(M, N, K, static_cast<const float*>(A), sam, sak,
                                                static_cast<const float*>(B), sbk, sbn,
                                                static_cast<float*>(C));
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_mu_update(int dtype, void* A, const void* num, const void* den, int64_t n,
                              double eps, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "mu_update: dtype must be f32 or f64");
  TLGB_CHECK_ARG(A && num && den && n >= 0, "mu_update: bad argument");
  if (n == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_mu_apply<double><<<nb, 256, 0, st>>>(static_cast<double*>(A),
                                           static_cast<const double*>(num),
                                           static_cast<const double*>(den), n, eps);
  else
    k_mu_apply<float><<<nb, 256, 0, st>>>(static_cast<float*>(A), static_cast<const float*>(num),
                                          static_cast<const float*>(den), n, (float)eps);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" size_t tlgb_dot_workspace_bytes(void) { return sizeof(double) * kDotBlocks; }

extern "C" int tlgb_dot(int dtype, const void* a, const void* b, int64_t n, double* out,
                        void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "dot: dtype must be f32 or f64");
  TLGB_CHECK_ARG(a && b && out && n >= 0, "dot: bad argument");
  if (!workspace || workspace_bytes < sizeof(double) * kDotBlocks)
    return set_error(TLGB_EWORKSPACE, "dot: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, (int64_t)256), kDotBlocks));
  if (dtype == TLGB_F64)
    k_dot_part<double><<<nb, 256, 0, st>>>(static_cast<const double*>(a),
                                           static_cast<const double*>(b), n, part);
  else
    k_dot_part<float><<<nb, 256, 0, st>>>(static_cast<const float*>(a),
                                          static_cast<const float*>(b), n, part);
  TLGB_LAUNCH_CHECK();
  k_dot_final<<<1, 32, 0, st>>>(part, nb, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" size_t tlgb_mask_impute_workspace_bytes(void) { return 2 * sizeof(double) * kDotBlocks; }

extern "C" int tlgb_mask_impute(int dtype, void* x, const void* mask, const void* rec, int64_t n,
                                double* out, void* workspace, size_t workspace_bytes,
                                void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "mask_impute: dtype must be f32 or f64");
  TLGB_CHECK_ARG(x && mask && rec && out && n >= 1, "mask_impute: bad argument");
  if (!workspace || workspace_bytes < 2 * sizeof(double) * kDotBlocks)
    return set_error(TLGB_EWORKSPACE, "mask_impute: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, (int64_t)256), kDotBlocks));
  if (dtype == TLGB_F64)
    k_mask_impute_part<double><<<nb, 256, 0, st>>>(static_cast<double*>(x),
                                                   static_cast<const double*>(mask),
                                                   static_cast<const double*>(rec), n, part);
  else
    k_mask_impute_part<float><<<nb, 256, 0, st>>>(static_cast<float*>(x),
                                                  static_cast<const float*>(mask),
                                                  static_cast<const float*>(rec), n, part);
  TLGB_LAUNCH_CHECK();
  k_mask_impute_final<<<1, 32, 0, st>>>(part, nb, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_mask_where(int dtype, void* x, const void* mask, const void* rec, double fill,
                               int64_t n, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "mask_where: dtype must be f32 or f64");
  TLGB_CHECK_ARG(x && mask && n >= 0, "mask_where: bad argument");
  if (n == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_mask_where<double><<<nb, 256, 0, st>>>(static_cast<double*>(x),
                                             static_cast<const double*>(mask),
                                             static_cast<const double*>(rec), fill, n);
  else
    k_mask_where<float><<<nb, 256, 0, st>>>(static_cast<float*>(x),
                                            static_cast<const float*>(mask),
                                            static_cast<const float*>(rec), (float)fill, n);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_masked_sq_diff(int dtype, const void* x, const void* mask, const void* rec,
                                   int64_t n, double* out, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64,
                 "masked_sq_diff: dtype must be f32 or f64");
  TLGB_CHECK_ARG(x && mask && rec && out && n >= 1, "masked_sq_diff: bad argument");
  if (!workspace || workspace_bytes < sizeof(double) * kDotBlocks)
    return set_error(TLGB_EWORKSPACE, "masked_sq_diff: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, (int64_t)256), kDotBlocks));
  if (dtype == TLGB_F64)
    k_masked_sq_diff_part<double><<<nb, 256, 0, st>>>(static_cast<const double*>(x),
                                                      static_cast<const double*>(mask),
                                                      static_cast<const double*>(rec), n, part);
  else
    k_masked_sq_diff_part<float><<<nb, 256, 0, st>>>(static_cast<const float*>(x),
                                                     static_cast<const float*>(mask),
                                                     static_cast<const float*>(rec), n, part);
  TLGB_LAUNCH_CHECK();
  k_dot_final<<<1, 32, 0, st>>>(part, nb, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_clip_min(int dtype, void* x, int64_t n, double lo, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "clip_min: dtype must be f32 or f64");
  TLGB_CHECK_ARG(x && n >= 0, "clip_min: bad argument");
  if (n == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_clip_min<double><<<nb, 256, 0, st>>>(static_cast<double*>(x), n, lo);
  else
    k_clip_min<float><<<nb, 256, 0, st>>>(static_cast<float*>(x), n, (float)lo);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_kronecker(int dtype, int n_mats, const void* const* mats, const int64_t* rows,
                              const int64_t* cols, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "kronecker: dtype must be f32 or f64");
  TLGB_CHECK_ARG(n_mats >= 1 && n_mats <= kMaxModes && mats && rows && cols && out,
                 "kronecker: bad argument");
  KronArgs a{};
  a.n = n_mats;
  int64_t R = 1, C = 1;
  for (int k = 0; k < n_mats; ++k) {
    TLGB_CHECK_ARG(mats[k] && rows[k] >= 1 && cols[k] >= 1, "kronecker: bad matrix");
    a.m[k] = mats[k];
    a.rows[k] = rows[k];
    a.cols[k] = cols[k];
    R *= rows[k];
    C *= cols[k];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(R * C, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_kronecker<double><<<nb, 256, 0, st>>>(a, R, C, static_cast<double*>(out));
  else
    k_kronecker<float><<<nb, 256, 0, st>>>(a, R, C, static_cast<float*>(out));
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_active_set_nnls(int dtype, const void* UtU, const void* Utm, void* x,
                                    int64_t n, int n_iter_max, double tol, int* status,
                                    void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "active_set_nnls: f32 or f64");
  TLGB_CHECK_ARG(UtU && Utm && x && status && n >= 1 && n_iter_max >= 0,
                 "active_set_nnls: bad argument");
  if (n > kAsMax)
    return set_error(TLGB_EUNSUPPORTED, "active_set_nnls: more than 128 unknowns");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t esz = dtype == TLGB_F64 ? 8 : 4;
  const size_t smem = esz * ((size_t)n * n + 4 * n) + 2 * sizeof(int) * n;
  static std::atomic<bool> attr[64];   // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_active_set_nnls<double>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_active_set_nnls<float>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, 160 * 1024));
    attr[dev] = true;
  }
  if (dtype == TLGB_F64)
    k_active_set_nnls<double><<<1, 256, smem, st>>>(static_cast<const double*>(UtU),
                                                    static_cast<const double*>(Utm),
                                                    static_cast<double*>(x), (int)n, n_iter_max,
                                                    tol, status);
  else
    k_active_set_nnls<float><<<1, 256, smem, st>>>(static_cast<const float*>(UtU),
                                                   static_cast<const float*>(Utm),
                                                   static_cast<float*>(x), (int)n, n_iter_max, tol,
                                                   status);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_tucker_normalize_workspace_size(int ndim, const int64_t* ranks, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes && ranks && bytes,
                 "tucker_normalize: bad argument");
  int64_t cols = 0;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(ranks[k] >= 1, "tucker_normalize: ranks must be >= 1");
    cols += ranks[k];
  }
  *bytes = sizeof(double) * (size_t)cols;
  return TLGB_OK;
}

extern "C" int tlgb_tucker_normalize(int dtype, int ndim, const int64_t* rows, const int64_t* ranks,
                                     void* const* factors, void* core, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "tucker_normalize: f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes && rows && ranks && factors && core,
                 "tucker_normalize: bad argument");
  TnArgs a{};
  a.n = ndim;
  a.core = core;
  a.core_n = 1;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(factors[k] && rows[k] >= 1 && ranks[k] >= 1, "tucker_normalize: bad factor");
    a.f[k] = factors[k];
    a.rows[k] = rows[k];
    a.ranks[k] = ranks[k];
    a.foff[k + 1] = a.foff[k] + rows[k] * ranks[k];
    a.soff[k + 1] = a.soff[k] + ranks[k];
    a.core_n *= ranks[k];
  }
  if (!workspace || workspace_bytes < sizeof(double) * (size_t)a.soff[ndim])
    return set_error(TLGB_EWORKSPACE, "tucker_normalize: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* scales = static_cast<double*>(workspace);
  const unsigned nb =
      (unsigned)std::min<int64_t>(ceil_div(a.foff[ndim] + a.core_n, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64) {
    k_tn_colnorms<double><<<(unsigned)a.soff[ndim], 256, 0, st>>>(a, scales);
    TLGB_LAUNCH_CHECK();
    k_tn_apply<double><<<nb, 256, 0, st>>>(a, scales);
  } else {
    k_tn_colnorms<float><<<(unsigned)a.soff[ndim], 256, 0, st>>>(a, scales);
    TLGB_LAUNCH_CHECK();
    k_tn_apply<float><<<nb, 256, 0, st>>>(a, scales);
  }
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" size_t tlgb_sparse_residual_workspace_bytes(void) {
  return align_up(sizeof(SelState), 256) + align_up(sizeof(unsigned long long) * 256, 256) +
         align_up(sizeof(double) * kSelBlocks, 256);
}

extern "C" int tlgb_sparse_residual(int dtype, const void* X, const void* L, int64_t n,
                                    int64_t k, double* out, void* sparse, void* workspace,
                                    size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "sparse_residual: f32 or f64");
  TLGB_CHECK_ARG(X && L && out && n >= 1 && k >= 1, "sparse_residual: bad argument");
  if (!workspace || workspace_bytes < tlgb_sparse_residual_workspace_bytes())
    return set_error(TLGB_EWORKSPACE, "sparse_residual: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  char* base = static_cast<char*>(workspace);
  SelState* ss = reinterpret_cast<SelState*>(base);
  unsigned long long* hist =
      reinterpret_cast<unsigned long long*>(base + align_up(sizeof(SelState), 256));
  double* part = reinterpret_cast<double*>(base + align_up(sizeof(SelState), 256) +
                                           align_up(sizeof(unsigned long long) * 256, 256));
  const int keep_all = k > n ? 1 : 0;   // the reference returns the residual itself
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, (int64_t)256), kSelBlocks));
  if (!keep_all) {
    k_sel_init<<<1, 256, 0, st>>>(ss, (unsigned long long)k, hist);
    TLGB_LAUNCH_CHECK();
    const int bits = dtype == TLGB_F64 ? 64 : 32;
    for (int shift = bits - 8; shift >= 0; shift -= 8) {
      if (dtype == TLGB_F64)
        k_sel_hist<double><<<nb, 256, 0, st>>>(static_cast<const double*>(X),
                                               static_cast<const double*>(L), n, shift, ss, hist);
      else
        k_sel_hist<float><<<nb, 256, 0, st>>>(static_cast<const float*>(X),
                                              static_cast<const float*>(L), n, shift, ss, hist);
      TLGB_LAUNCH_CHECK();
      k_sel_pick<<<1, 256, 0, st>>>(hist, shift, ss);
      TLGB_LAUNCH_CHECK();
    }
  }
  if (dtype == TLGB_F64)
    k_sel_resid<double><<<nb, 256, 0, st>>>(static_cast<const double*>(X),
                                            static_cast<const double*>(L), n, ss, keep_all,
                                            static_cast<double*>(sparse), part);
  else
    k_sel_resid<float><<<nb, 256, 0, st>>>(static_cast<const float*>(X),
                                           static_cast<const float*>(L), n, ss, keep_all,
                                           static_cast<float*>(sparse), part);
  TLGB_LAUNCH_CHECK();
  k_sel_final<<<1, 32, 0, st>>>(part, nb, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
