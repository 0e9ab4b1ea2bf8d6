// Non-negative CP by multiplicative updates on the GPU: the loop of
// tensorly/decomposition/_nn_cp.py:26-183 (non_negative_parafac, weights all
// one, normalize_factors=False, no mask).  Per iteration and free mode:
//   accum = Hadamard product of the other factors' Grams        (:116-125)
//   M     = MTTKRP of the mode                                   (:129)
//   A    <- A * clip(M, eps) / clip(A accum, eps)                (:131-134)
// and, when tol > 0, the relative error from the last mode's MTTKRP and the
// Grams with the reference's stop test (:140-170).  The MTTKRP is the SIMT
// split kernel of CP-ALS; the Grams are kept in f64 and refreshed after every
// update; the stop flag lives on the device, so kernels after convergence
// return at once and the host reads the flag every few iterations.
//
// The NNDSVD helpers of the non-negative SVD initialisation
// (tensorly/tenalg/svd.py:68-134) are here too: the norms of the positive and
// negative parts of rows, and the column update that follows.
#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

#include "als_kernels.cuh"
#include "mttkrp_simt.cuh"
#include "mttkrp_tc.cuh"

namespace tlgb {
namespace {

constexpr int kMuThreads = 256;
constexpr int kMuSumsqBlocks = 256;
constexpr int kMuCheckEvery = 8;

// V = Hadamard product of the Grams of every mode but `mode`.
__global__ void k_mu_accum(const double* __restrict__ G, int ndim, int mode, int R, double* V,
                           const int* done) {
  if (*done) return;
  const int RR = R * R;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < RR; e += gridDim.x * blockDim.x) {
    double v = 0.0;
    bool first = true;
    for (int k = 0; k < ndim; ++k) {
      if (k == mode) continue;
      v = first ? G[(int64_t)k * RR + e] : v * G[(int64_t)k * RR + e];
      first = false;
    }
    V[e] = first ? 1.0 : v;
  }
}

// A <- A * max(M, eps) / max(A V, eps) for a block of rows; M is the sum of
// the MTTKRP's split partials.  The block's rows are staged in shared memory
// before any is overwritten.  With ipart, the block's sum of M * A_new (the
// <X, [[A]]> term of the error, from the MTTKRP taken before the update as
// in the reference).
template <typename T>
__global__ void __launch_bounds__(kMuThreads)
k_mu_update(const T* __restrict__ partial, int splits, int64_t I, int R,
            const double* __restrict__ V, T eps, T* A, double* ipart, const int* done,
            int64_t rpb) {
  if (*done) return;
  extern __shared__ double smu[];   // [rows of the block][R]
  __shared__ double red[kMuThreads / 32];
  const int tid = threadIdx.x;
  const int64_t row0 = blockIdx.x * rpb;
  const int64_t row1 = min(row0 + rpb, I);
  const int n = (int)(row1 - row0) * R;
  const int64_t IR = I * R;
  for (int e = tid; e < n; e += kMuThreads) smu[e] = (double)A[row0 * R + e];
  __syncthreads();
  double ip = 0.0;
  for (int e = tid; e < n; e += kMuThreads) {
    const int i = e / R, c = e - (e / R) * R;
    const int64_t off = (row0 + i) * R + c;
    double m0 = 0.0, m1 = 0.0;
    int p = 0;
    for (; p + 1 < splits; p += 2) {
      m0 += (double)partial[(int64_t)p * IR + off];
      m1 += (double)partial[(int64_t)(p + 1) * IR + off];
    }
    if (p < splits) m0 += (double)partial[(int64_t)p * IR + off];
    const double m = m0 + m1;
    double den = 0.0;
    for (int s = 0; s < R; ++s) den = fma(smu[i * R + s], V[(int64_t)s * R + c], den);
    const T mt = (T)m;
    const T num = mt > eps ? mt : eps;
    const T dt = (T)den;
    const T dn = dt > eps ? dt : eps;
    const T a = (T)smu[i * R + c] * num / dn;
    A[off] = a;
    if (ipart) ip += (double)mt * (double)a;
  }
  if (ipart) {
    for (int o = 16; o > 0; o >>= 1) ip += __shfl_xor_sync(0xffffffffu, ip, o);
    if ((tid & 31) == 0) red[tid >> 5] = ip;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < kMuThreads / 32; ++w) t += red[w];
      ipart[blockIdx.x] = t;
    }
  }
}

// Norms of the positive and the negative part of each mode-n slice of Y, a
// tensor viewed as (L, k, T): out[2 j] = ||max(Y[:, j, :], 0)||,
// out[2 j + 1] = ||min(Y[:, j, :], 0)||.  One block per slice.
template <typename T>
__global__ void k_posneg_norms(const T* __restrict__ Y, int64_t L, int k, int64_t Tt, T* out) {
  __shared__ double rp[32], rn[32];
  const int j = blockIdx.x;
  double sp = 0.0, sn = 0.0;
  for (int64_t x = threadIdx.x; x < L * Tt; x += blockDim.x) {
    const int64_t l = x / Tt, t = x - (x / Tt) * Tt;
    const double v = (double)Y[(l * k + j) * Tt + t];
    if (v > 0.0) sp += v * v; else sn += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sp += __shfl_xor_sync(0xffffffffu, sp, o);
    sn += __shfl_xor_sync(0xffffffffu, sn, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { rp[warp] = sp; rn[warp] = sn; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += rp[w]; b += rn[w]; }
    out[2 * blockIdx.x] = (T)sqrt(a);
    out[2 * blockIdx.x + 1] = (T)sqrt(b);
  }
}

// NNDSVD columns of W (I x k, row-major) from U (I x k), S (k) and the norms
// of the row parts of U^T M (2 k; V = S^-1 U^T M).  Column 0 = sqrt(S_0) |U_0|;
// column j >= 1 takes U_j's positive or negative part, whichever side has the
// larger product of norms, divided by its norm and scaled by
// sqrt(S_j * that product); with `fill`, entries below eps become `avg`
// ('nndsvda'), else they are soft-thresholded by eps ('nndsvd').
template <typename T>
__global__ void k_nndsvd_columns(const T* __restrict__ U, const T* __restrict__ S,
                                 const T* __restrict__ vnorms, int64_t I, int k, T eps, int fill,
                                 T avg, T* W) {
  // one block per column; the column's positive / negative norms first
  __shared__ double rp[32], rn[32];
  const int j = blockIdx.x;
  double sp = 0.0, sn = 0.0;
  for (int64_t i = threadIdx.x; i < I; i += blockDim.x) {
    const double v = (double)U[i * k + j];
    if (v > 0.0) sp += v * v; else sn += v * v;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sp += __shfl_xor_sync(0xffffffffu, sp, o);
    sn += __shfl_xor_sync(0xffffffffu, sn, o);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) { rp[warp] = sp; rn[warp] = sn; }
  __syncthreads();
  double xp = 0.0, xn = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { xp += rp[w]; xn += rn[w]; }
  const T x_p = (T)sqrt(xp), x_n = (T)sqrt(xn);
  // the rows of V are those of U^T M divided by the singular values
  const T y_p = vnorms[2 * j] / S[j], y_n = vnorms[2 * j + 1] / S[j];
  const T m_p = x_p * y_p, m_n = x_n * y_n;
  const bool pos = m_p > m_n;
  const T nrm = pos ? x_p : x_n;
  const T lbd = (j == 0) ? (T)0 : (T)sqrt((double)S[j] * (double)(pos ? m_p : m_n));
  const T s0 = (T)sqrt((double)S[0]);
  for (int64_t i = threadIdx.x; i < I; i += blockDim.x) {
    const T x = U[i * k + j];
    T w;
    if (j == 0) w = s0 * (x < (T)0 ? -x : x);
    else {
      const T part = pos ? (x > (T)0 ? x : (T)0) : (x < (T)0 ? -x : (T)0);
      w = lbd * (part / nrm);
    }
    if (fill) w = (w < eps) ? avg : w;
    else w = (w > eps) ? w - eps : ((w < -eps) ? w + eps : (T)0);
    W[i * k + j] = w;
  }
}

// Sum of a tensor in f64 (block partials, then one block), for the mean
// that 'nndsvda' fills with.
template <typename T>
__global__ void k_sum_part(const T* __restrict__ X, int64_t n, double* part) {
  __shared__ double red[32];
  double s0 = 0.0, s1 = 0.0;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + step < n; i += 2 * step) { s0 += (double)X[i]; s1 += (double)X[i + step]; }
  if (i < n) s0 += (double)X[i];
  double s = s0 + s1;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}
__global__ void k_sum_final(const double* part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < n; ++i) t += part[i];
    *out = t;
  }
}

// ---------------------------------------------------------------- HALS
// HALS (tensorly/decomposition/_nn_cp.py:186-377 with the inner solver
// tensorly/solvers/nnls.py:5-150): per free mode, M = MTTKRP is summed once,
// then up to n_inner iterations of row-wise (Gauss-Seidel over k) updates of
// V = A^T.  Every column of V (row of A) is an independent problem, so one
// warp owns one row of A in registers and runs all iterations of a chunk in
// one launch; the rows are coupled only by the inner stop test, whose per-row
// terms k_hals_scan sums after the launch.  A test that stops before the end
// of the chunk reruns the rows from their saved start for exactly the
// iterations the reference runs.

// M (I x R, in the factor type) = the sum of the MTTKRP's split partials.
template <typename T>
__global__ void k_sum_splits_to(const T* __restrict__ partial, int splits, int64_t IR, T* M) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < IR;
       e += (int64_t)gridDim.x * blockDim.x) {
    double m0 = 0.0, m1 = 0.0;
    int p = 0;
    for (; p + 1 < splits; p += 2) {
      m0 += (double)partial[(int64_t)p * IR + e];
      m1 += (double)partial[(int64_t)(p + 1) * IR + e];
    }
    if (p < splits) m0 += (double)partial[(int64_t)p * IR + e];
    M[e] = (T)(m0 + m1);
  }
}

constexpr int kHalsWarps = 4;       // rows (one per warp) per block
constexpr int kHalsChunk = 100;     // speculative inner iterations per launch
constexpr int64_t kHalsPartCap = int64_t(8) << 20;   // doubles of per-row stop partials

// Inner iterations per speculative launch: kHalsChunk, fewer when the per-row
// partials of that many iterations would pass kHalsPartCap doubles.
int hals_chunk(int64_t rows) {
  return (int)std::max<int64_t>(
      1, std::min<int64_t>(kHalsChunk, kHalsPartCap / std::max<int64_t>(rows, 1)));
}

// Products and sums of the row update with one rounding each, so that a
// rerun of the same rows repeats the speculative launch bit for bit.
__device__ __forceinline__ float rn_mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rn_mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rn_add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double rn_add(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rn_sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rn_sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rn_div(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rn_div(double a, double b) { return __ddiv_rn(a, b); }

// n HALS iterations of row i = block * kHalsWarps + warp of A (a column of the
// reference's V = A^T), k = 0..R-1 in order (rows k with P[k, k] == 0 kept):
//   num = (M[i, k] - sum_s P[k, s] A[i, s]) + P[k, k] A[i, k]   (- sparsity)
//   A[i, k] <- max(num / P[k, k], 0)
// computed in the factor type T, as the reference computes (without a
// sparsity coefficient sp is 0, and num - 0 is num).  Lane l holds elements
// s = l + 32 j (j < NJ) of the row, of M's row and of P's diagonal in
// registers, with w = P A[i, :]^T: w is formed afresh at the start of each
// iteration and, after step k, moved by P[:, k] (A_new[i, k] - A_old[i, k]),
// so a step costs the owner lane's arithmetic, one broadcast and one FMA per
// element instead of two warp reductions; steps run in unrolled groups of 8.  The reference's stop term
// ||V - newV||^2 (newV broadcast against every row of V) is, for this column,
// sum_s (A[i, s] - newV)^2 before the update; each lane sums its elements'
// share and the warp's total for iteration t goes to part[t * rows + row].
// The rows are independent: the launch runs all n iterations, and the stop
// test over all rows is applied afterwards by k_hals_scan, which asks for a
// rerun of the first t + 1 iterations from the rows saved in `save` when the
// test stopped early.  Rows are read from src and written to dst (the same
// buffer in place).  PS: P staged in shared memory (else read from global).
template <typename T, int NJ, bool PS>
__global__ void __launch_bounds__(32 * kHalsWarps)
k_hals_rows(const T* __restrict__ M, const T* __restrict__ Pg, int64_t I, int R, const T* src,
            T* dst, T* save, int n_iter, const int* n_dev, double sparsity, double* part,
            const int* done) {
  if (*done) return;
  const int n = n_dev ? *n_dev : n_iter;
  if (n <= 0) return;
  extern __shared__ __align__(16) unsigned char hsm[];
  T* Ps = reinterpret_cast<T*>(hsm);                       // R x R (PS)
  T* vbuf = Ps + (PS ? R * R : 0);                         // [kHalsWarps][R]
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if constexpr (PS) {
    for (int e = threadIdx.x; e < R * R; e += 32 * kHalsWarps) Ps[e] = Pg[e];
    __syncthreads();
  }
  const T* P = PS ? Ps : Pg;
  T* vw = vbuf + warp * R;
  const int64_t row = (int64_t)blockIdx.x * kHalsWarps + warp;
  const int64_t rows = (int64_t)gridDim.x * kHalsWarps;
  const bool live = row < I;
  const T sp = (T)sparsity;
  T v[NJ], w[NJ], m[NJ], pd[NJ];
  int sx[NJ];                                               // in-range element index for P reads
  unsigned zero[NJ];                                        // steps with P[k, k] == 0 (uniform)
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int s = 32 * j + lane;
    sx[j] = s < R ? s : 0;
    v[j] = (T)0;
    m[j] = (T)0;
    pd[j] = P[sx[j] * R + sx[j]];
    zero[j] = __ballot_sync(0xffffffffu, s < R && pd[j] == (T)0);
    if (live && s < R) {
      v[j] = src[row * R + s];
      m[j] = M[row * R + s];
      if (save) save[row * R + s] = v[j];
    }
  }
  for (int t = 0; t < n; ++t) {
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (32 * j + lane < R) vw[32 * j + lane] = v[j];
    __syncwarp();
#pragma unroll
    for (int j = 0; j < NJ; ++j) {
      T a0 = (T)0, a1 = (T)0;
      int q = 0;
      for (; q + 1 < R; q += 2) {
        a0 = fma(P[q * R + sx[j]], vw[q], a0);
        a1 = fma(P[(q + 1) * R + sx[j]], vw[q + 1], a1);
      }
      if (q < R) a0 = fma(P[q * R + sx[j]], vw[q], a0);
      w[j] = rn_add(a0, a1);
    }
    __syncwarp();
    T sq = (T)0;
#pragma unroll
    for (int J = 0; J < NJ; ++J) {
      const int kn = (J == NJ - 1) ? R - 32 * J : 32;      // steps of slot J
#pragma unroll 1
      for (int kb = 0; kb < kn; kb += 8) {
        const unsigned zb = zero[J] >> kb;
        const T* prow = P + (32 * J + kb) * R;             // row k of P
#pragma unroll
        for (int u = 0; u < 8; ++u, prow += R) {
          const int kk = kb + u;
          if (J == NJ - 1 && kk >= kn) break;
          if ((zb >> u) & 1u) continue;
          // lane kk's w[J], v[J], m[J], pd[J] are element k = 32 J + kk's
          const T num = rn_sub(rn_add(rn_sub(m[J], w[J]), rn_mul(pd[J], v[J])), sp);
          T nv = rn_div(num, pd[J]);
          nv = nv > (T)0 ? nv : (T)0;
          nv = __shfl_sync(0xffffffffu, nv, kk);
          const T delta = rn_sub(nv, __shfl_sync(0xffffffffu, v[J], kk));
#pragma unroll
          for (int j = 0; j < NJ; ++j) {
            if (j < NJ - 1 || 32 * j + lane < R) {
              const T d = rn_sub(v[j], nv);
              sq = fma(d, d, sq);
            }
            w[j] = fma(prow[sx[j]], delta, w[j]);
          }
          if (lane == kk) v[J] = nv;
        }
      }
    }
    if (part) {
      double e = live ? (double)sq : 0.0;
      for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
      if (lane == 0) part[(int64_t)t * rows + row] = e;
    }
  }
  if (live) {
#pragma unroll
    for (int j = 0; j < NJ; ++j)
      if (32 * j + lane < R) dst[row * R + 32 * j + lane] = v[j];
  }
}

// P in the factor type, symmetric (the upper triangle mirrored, as the
// reference's Gram products are), for the HALS kernel.
template <typename T>
__global__ void k_to_type(const double* __restrict__ V, int R, T* out, const int* done) {
  if (*done) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < R * R; e += gridDim.x * blockDim.x) {
    const int r = e / R, c = e - r * R;
    out[e] = (T)(r <= c ? V[e] : V[c * R + r]);
  }
}

// After a speculative launch of n iterations (global iterations t0..t0+n-1):
// tot[t] = the sum of the row partials of iteration t (fixed order, lane 0's
// butterfly); iteration 0's total is the reference e0, and the first t with
// tot[t] < tol * e0 ends the inner loop (tensorly/solvers/nnls.py:169-172).
// rerun = t + 1 iterations from the saved rows when that t is not the last
// of the launch, else 0 (the speculative rows stand).
__global__ void k_hals_scan(const double* __restrict__ part, int64_t rows, int t0, int n,
                            double tol, double* e0, int* stop, int* rerun, const int* done) {
  if (*done) return;
  extern __shared__ double tot[];                          // n
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int t = warp; t < n; t += nw) {
    double s = 0.0;
    for (int64_t r = lane; r < rows; r += 32) s += part[(int64_t)t * rows + r];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) tot[t] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int st = 0, rr = 0;
    for (int t = 0; t < n; ++t) {
      if (t0 + t == 0) *e0 = tot[t];
      if (tot[t] < tol * *e0) {
        st = 1;
        rr = (t + 1 < n) ? t + 1 : 0;
        break;
      }
    }
    *stop = st;
    *rerun = rr;
  }
}

constexpr size_t kHalsPSmemMax = 112 * 1024;   // P staged in shared memory up to this size

template <typename T, int NJ, bool PS>
int hals_launch_nj(int R, int nb, size_t smem, cudaStream_t st, const T* M, const T* P,
                   int64_t I, const T* src, T* dst, T* save, int n, const int* n_dev, double sp,
                   double* part, const int* done) {
  if (smem > 48 * 1024)
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_hals_rows<T, NJ, PS>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  k_hals_rows<T, NJ, PS><<<nb, 32 * kHalsWarps, smem, st>>>(M, P, I, R, src, dst, save, n, n_dev,
                                                            sp, part, done);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

// k_hals_rows with NJ = ceil(R / 32) register slots per lane (R <= 160), P in
// shared memory when it fits kHalsPSmemMax (every f32 rank: 160^2 * 4 bytes
// fit; f64 up to rank 119).
template <typename T>
int hals_launch_rows(int R, int nb, size_t smem, int ps, cudaStream_t st, const T* M,
                     const T* P, int64_t I, const T* src, T* dst, T* save, int n,
                     const int* n_dev, double sp, double* part, const int* done) {
#define TLGB_HALS_NJ(NJ)                                                                      \
  if constexpr (sizeof(T) == 4)                                                                \
    return hals_launch_nj<T, NJ, true>(R, nb, smem, st, M, P, I, src, dst, save, n, n_dev, sp, \
                                       part, done);                                            \
  else                                                                                         \
    return ps ? hals_launch_nj<T, NJ, true>(R, nb, smem, st, M, P, I, src, dst, save, n,       \
                                            n_dev, sp, part, done)                             \
              : hals_launch_nj<T, NJ, false>(R, nb, smem, st, M, P, I, src, dst, save, n,      \
                                             n_dev, sp, part, done)
  switch ((R + 31) / 32) {
    case 1: TLGB_HALS_NJ(1);
    case 2: TLGB_HALS_NJ(2);
    case 3: TLGB_HALS_NJ(3);
    case 4: TLGB_HALS_NJ(4);
    case 5: TLGB_HALS_NJ(5);
    default: return set_error(TLGB_EINVAL, "cp_nn_hals: rank above 160 is not supported");
  }
#undef TLGB_HALS_NJ
}

// <M, A> partial sums per block of rows (the error's inner product).
template <typename T>
__global__ void k_inner_part(const T* __restrict__ M, const T* __restrict__ A, int64_t n,
                             double* part, const int* done) {
  if (*done) return;
  __shared__ double red[32];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    s += (double)M[e] * (double)A[e];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    part[blockIdx.x] = t;
  }
}

constexpr int kInnerBlocks = 128;

struct MuLayout {
  size_t ctrl, errors, G, V, partial, gpart, ipart, sumsq, bytes;
  size_t M, hpart, hstate, Pt, save;   // HALS: summed MTTKRP, stop partials, e0 + stop +
                                       // rerun, typed P, rows at the start of a chunk
  size_t fac, perm, vmat, w32;         // HALS modes outside nn_modes: the CP-ALS solve
  size_t tcs;                          // f32 tensors: the split tensor-core MTTKRP's buffers
};

int64_t mu_rows_per_block(int64_t I, int R, int nparts);

template <typename T>
int mu_layout(const Shape& sh, int64_t R, int n_iter_max, std::vector<MttkrpPlan>* plans,
              int* nparts, MuLayout* L) {
  const int dtype = TypeCode<T>::value;
  plans->resize(sh.ndim);
  size_t pmax = 0;
  int64_t imax = 0;
  for (int k = 0; k < sh.ndim; ++k) {
    int rc = mttkrp_make_plan(dtype, sh, R, k, &(*plans)[k]);
    if (rc) return rc;
    pmax = std::max(pmax, (*plans)[k].partial_bytes);
    imax = std::max(imax, sh.dim[k]);
  }
  *nparts = solve_blocks_for(imax);
  int64_t nb_max = 1;
  for (int k = 0; k < sh.ndim; ++k)
    nb_max = std::max<int64_t>(nb_max, ceil_div(sh.dim[k], mu_rows_per_block(sh.dim[k], (int)R,
                                                                              *nparts)));
  size_t off = 0;
  auto take = [&](size_t b) { off = align_up(off, 256); const size_t o = off; off += b; return o; };
  const size_t RR = (size_t)R * R;
  L->ctrl = take(sizeof(AlsCtrl));
  L->errors = take(sizeof(double) * (size_t)std::max(1, n_iter_max));
  L->G = take(sizeof(double) * RR * sh.ndim);
  L->V = take(sizeof(double) * RR);
  L->partial = take(pmax);
  L->gpart = take(sizeof(double) * RR * (size_t)*nparts);
  L->ipart = take(sizeof(double) * (size_t)std::max<int64_t>(nb_max, kInnerBlocks));
  L->sumsq = take(sizeof(double) * kMuSumsqBlocks);
  L->M = take(sizeof(T) * (size_t)imax * R);
  const int64_t hrows = ceil_div(imax, (int64_t)kHalsWarps) * kHalsWarps;
  L->hpart = take(sizeof(double) * (size_t)(hrows * hals_chunk(hrows)));
  L->hstate = take(sizeof(double) * 2);
  L->Pt = take(sizeof(T) * RR);
  L->save = take(sizeof(T) * (size_t)imax * R);
  L->fac = take(sizeof(double) * (RR + R));
  L->perm = take(sizeof(int) * R);
  L->vmat = take(sizeof(double) * RR);
  L->w32 = take(sizeof(float) * 3 * RR);
  size_t tcs_bytes = 0;
  if (dtype == TLGB_F32) {
    SplitMttkrp stc;
    int rc = split_mttkrp_plan(sh, R, &stc);
    if (rc) return rc;
    tcs_bytes = split_mttkrp_bytes(stc);
  }
  L->tcs = take(tcs_bytes);
  L->bytes = align_up(off, 256);
  return TLGB_OK;
}

// Rows per update block: about `nparts` blocks, the block's rows (f64) within
// 48 KiB of shared memory.
int64_t mu_rows_per_block(int64_t I, int R, int nparts) {
  const int64_t cap = std::max<int64_t>(1, (48 * 1024 / 8) / R);
  return std::max<int64_t>(1, std::min<int64_t>(ceil_div(I, (int64_t)nparts), cap));
}

template <typename T>
int mu_run(const T* X, const Shape& sh, T* const* factors, int64_t R, const int* free_modes,
           int n_free, int n_iter_max, double tol, int crit, double* errors, int* n_errors,
           void* ws, size_t ws_bytes, cudaStream_t st) {
  std::vector<MttkrpPlan> plans;
  int nparts = 0;
  MuLayout L;
  int rc = mu_layout<T>(sh, R, n_iter_max, &plans, &nparts, &L);
  if (rc) return rc;
  if (!ws || ws_bytes < L.bytes) return set_error(TLGB_EWORKSPACE, "cp_nn_mu: workspace too small");
  rc = als_prepare(TypeCode<T>::value);
  if (rc) return rc;
  char* base = static_cast<char*>(ws);
  AlsCtrl* ctrl = reinterpret_cast<AlsCtrl*>(base + L.ctrl);
  double* derr = reinterpret_cast<double*>(base + L.errors);
  double* G = reinterpret_cast<double*>(base + L.G);
  double* V = reinterpret_cast<double*>(base + L.V);
  T* partial = reinterpret_cast<T*>(base + L.partial);
  double* gpart = reinterpret_cast<double*>(base + L.gpart);
  double* ipart = reinterpret_cast<double*>(base + L.ipart);
  double* sumsq = reinterpret_cast<double*>(base + L.sumsq);
  const int N = sh.ndim;
  const int RR = (int)(R * R);
  const int* done = &ctrl->done;
  const T eps = std::numeric_limits<T>::epsilon();

  TLGB_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(AlsCtrl), st));
  rc = als_launch_sumsq(TypeCode<T>::value, X, sh.numel, sumsq, kMuSumsqBlocks, ctrl, st);
  if (rc) return rc;
  for (int k = 0; k < N; ++k) {
    rc = als_launch_gram<T>(factors[k], sh.dim[k], (int)R, gpart, nparts, G + (size_t)k * RR,
                            done, st);
    if (rc) return rc;
  }
  LoopMttkrp<T> mk;
  rc = mk.setup(X, sh, R, factors, &plans, partial, base + L.tcs, &ctrl->tc_err, st);
  if (rc) return rc;
  const T* cf[kMaxModes];
  for (int k = 0; k < N; ++k) cf[k] = factors[k];
  const int last = free_modes[n_free - 1];
  int it = 0;
  AlsCtrl hc{};
  for (; it < n_iter_max; ++it) {
    int last_nb = 0;
    for (int q = 0; q < n_free; ++q) {
      const int mode = free_modes[q];
      k_mu_accum<<<(RR + 255) / 256, 256, 0, st>>>(G, N, mode, (int)R, V, done);
      TLGB_LAUNCH_CHECK();
      rc = mk.launch(mode, cf, nullptr, done, st);
      if (rc) return rc;
      const int64_t I = sh.dim[mode];
      const int64_t rpb = mu_rows_per_block(I, (int)R, nparts);
      const int nb = (int)ceil_div(I, rpb);
      k_mu_update<T><<<nb, kMuThreads, (size_t)rpb * R * sizeof(double), st>>>(
          mk.partial(), mk.splits(mode), I, (int)R, V, eps, factors[mode],
          mode == last ? ipart : nullptr, done, rpb);
      TLGB_LAUNCH_CHECK();
      rc = mk.refresh(mode, factors[mode], st);
      if (rc) return rc;
      if (mode == last) last_nb = nb;
      rc = als_launch_gram<T>(factors[mode], I, (int)R, gpart, nparts, G + (size_t)mode * RR,
                              done, st);
      if (rc) return rc;
    }
    if (tol > 0.0) {
      rc = als_launch_fit<T>(G, N, (int)R, nullptr, ipart, last_nb, ctrl, derr, n_iter_max, tol,
                             crit, st);
      if (rc) return rc;
      if (((it + 1) % kMuCheckEvery) == 0 || it + 1 == n_iter_max) {
        TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
        TLGB_CUDA_TRY(cudaStreamSynchronize(st));
        if (hc.done) break;
      }
    }
  }
  TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (hc.tc_err != 0)
    return set_error(TLGB_ETIMEOUT, "cp_nn_mu: a tensor-core MTTKRP wait timed out");
  const int ne = (tol > 0.0) ? std::min(hc.iter, n_iter_max) : 0;
  if (n_errors) *n_errors = ne;
  if (errors && ne > 0)
    TLGB_CUDA_TRY(cudaMemcpy(errors, derr, sizeof(double) * ne, cudaMemcpyDeviceToHost));
  return TLGB_OK;
}

// One hals_nnls call (tensorly/solvers/nnls.py:5-175) on the rows of A
// (I x R, the reference's V transposed), given M (I x R, the reference's
// UtM transposed) and the typed symmetric P (R x R, its UtU): chunks of
// speculative iterations with the stop test applied afterwards and an exact
// rerun when it stopped inside a chunk; a host read of the stop flag between
// chunks.  state: e0 (double), then the stop and rerun ints.
template <typename T>
int hals_solve(const T* M, const T* Pt, T* A, int64_t I, int R, int n_inner, double tol_inner,
               double sp, T* save, double* hpart, double* state, int chunk, size_t hals_smem,
               int p_in_smem, const int* done, cudaStream_t st) {
  int* stop = reinterpret_cast<int*>(state + 1);
  int* rerun = stop + 1;
  TLGB_CUDA_TRY(cudaMemsetAsync(state, 0, 2 * sizeof(double), st));
  const int nb = (int)ceil_div(I, (int64_t)kHalsWarps);
  const int64_t hrows = (int64_t)nb * kHalsWarps;
  for (int t0 = 0; t0 < n_inner; t0 += chunk) {
    const int n = std::min(chunk, n_inner - t0);
    int rc = hals_launch_rows<T>(R, nb, hals_smem, p_in_smem, st, M, Pt, I, A, A, save, n,
                                 nullptr, sp, hpart, done);
    if (rc) return rc;
    k_hals_scan<<<1, 1024, sizeof(double) * n, st>>>(hpart, hrows, t0, n, tol_inner, state, stop,
                                                     rerun, done);
    TLGB_LAUNCH_CHECK();
    rc = hals_launch_rows<T>(R, nb, hals_smem, p_in_smem, st, M, Pt, I, save, A, nullptr, 0,
                             rerun, sp, nullptr, done);
    if (rc) return rc;
    if (t0 + n < n_inner) {
      int hs = 0;
      TLGB_CUDA_TRY(cudaMemcpyAsync(&hs, stop, sizeof(int), cudaMemcpyDeviceToHost, st));
      TLGB_CUDA_TRY(cudaStreamSynchronize(st));
      if (hs) break;
    }
  }
  return TLGB_OK;
}

// P symmetric in the factor type: the upper triangle of the input mirrored.
template <typename T>
__global__ void k_sym_typed(const T* __restrict__ in, int R, T* out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < R * R; e += gridDim.x * blockDim.x) {
    const int r = e / R, c = e - r * R;
    out[e] = r <= c ? in[e] : in[c * R + r];
  }
}

// P = (w_r * P) * w_s, the weights of tensorly/decomposition/_nn_cp.py:316-320.
template <typename T>
__global__ void k_weight_outer(double* __restrict__ P, const T* __restrict__ w, int R,
                               const int* done) {
  if (*done) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < R * R; e += gridDim.x * blockDim.x) {
    const int r = e / R, c = e - r * R;
    P[e] = ((double)w[r] * P[e]) * (double)w[c];
  }
}

// nn_mask: bit k set = mode k is updated by HALS, else by the least-squares
// solve (tensorly/decomposition/_nn_cp.py:324-341).  weights: device, rank
// entries, in/out, or null (all ones).  normalize: cp_normalize after every
// updated mode but the last and after every iteration (:342-343, :373-374).
template <typename T>
int hals_run(const T* X, const Shape& sh, T* const* factors, T* weights, int64_t R,
             const int* free_modes, int n_free, unsigned nn_mask, int normalize, int n_iter_max,
             double tol, int crit, const double* sparsity, int exact, double* errors,
             int* n_errors, void* ws, size_t ws_bytes, cudaStream_t st) {
  std::vector<MttkrpPlan> plans;
  int nparts = 0;
  MuLayout L;
  int rc = mu_layout<T>(sh, R, n_iter_max, &plans, &nparts, &L);
  if (rc) return rc;
  if (!ws || ws_bytes < L.bytes) return set_error(TLGB_EWORKSPACE, "cp_nn_hals: workspace too small");
  rc = als_prepare(TypeCode<T>::value);
  if (rc) return rc;
  char* base = static_cast<char*>(ws);
  AlsCtrl* ctrl = reinterpret_cast<AlsCtrl*>(base + L.ctrl);
  double* derr = reinterpret_cast<double*>(base + L.errors);
  double* G = reinterpret_cast<double*>(base + L.G);
  double* P = reinterpret_cast<double*>(base + L.V);
  T* partial = reinterpret_cast<T*>(base + L.partial);
  double* gpart = reinterpret_cast<double*>(base + L.gpart);
  double* ipart = reinterpret_cast<double*>(base + L.ipart);
  double* sumsq = reinterpret_cast<double*>(base + L.sumsq);
  T* M = reinterpret_cast<T*>(base + L.M);
  double* hpart = reinterpret_cast<double*>(base + L.hpart);
  double* e0 = reinterpret_cast<double*>(base + L.hstate);
  T* Pt = reinterpret_cast<T*>(base + L.Pt);
  T* save = reinterpret_cast<T*>(base + L.save);
  double* fac = reinterpret_cast<double*>(base + L.fac);
  int* perm = reinterpret_cast<int*>(base + L.perm);
  double* vmat = reinterpret_cast<double*>(base + L.vmat);
  float* w32 = reinterpret_cast<float*>(base + L.w32);
  const int p_in_smem = ((size_t)R * R * sizeof(T) <= kHalsPSmemMax) ? 1 : 0;
  const size_t hals_smem = (p_in_smem ? (size_t)R * R * sizeof(T) : 0) +
                           (size_t)kHalsWarps * R * sizeof(T);
  int64_t imax = 0;
  for (int k = 0; k < sh.ndim; ++k) imax = std::max(imax, sh.dim[k]);
  const int chunk = hals_chunk(ceil_div(imax, (int64_t)kHalsWarps) * kHalsWarps);
  const int N = sh.ndim;
  const int RR = (int)(R * R);
  const int* done = &ctrl->done;
  // tensorly/decomposition/_nn_cp.py:329-336: hals_nnls(..., n_iter_max=100), or exact
  const int n_inner = exact ? 50000 : 100;
  const double tol_inner = exact ? 1e-16 : 1e-8;

  TLGB_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(AlsCtrl), st));
  rc = als_launch_sumsq(TypeCode<T>::value, X, sh.numel, sumsq, kMuSumsqBlocks, ctrl, st);
  if (rc) return rc;
  for (int k = 0; k < N; ++k) {
    rc = als_launch_gram<T>(factors[k], sh.dim[k], (int)R, gpart, nparts, G + (size_t)k * RR,
                            done, st);
    if (rc) return rc;
  }
  LoopMttkrp<T> mk;
  rc = mk.setup(X, sh, R, factors, &plans, partial, base + L.tcs, &ctrl->tc_err, st);
  if (rc) return rc;
  const T* cf[kMaxModes];
  for (int k = 0; k < N; ++k) cf[k] = factors[k];
  const int last = free_modes[n_free - 1];
  // cp_normalize of the model, then the Grams (and planes) of every rescaled factor
  auto normalize_all = [&]() -> int {
    int r2 = als_launch_normalize<T>(factors, sh.dim, N, (int)R, weights, done, st);
    for (int k = 0; k < N && !r2; ++k) {
      r2 = als_launch_gram<T>(factors[k], sh.dim[k], (int)R, gpart, nparts, G + (size_t)k * RR,
                              done, st);
      if (!r2) r2 = mk.refresh(k, factors[k], st);
    }
    return r2;
  };
  AlsCtrl hc{};
  for (int it = 0; it < n_iter_max; ++it) {
    for (int q = 0; q < n_free; ++q) {
      const int mode = free_modes[q];
      const int64_t I = sh.dim[mode];
      const int64_t IR = I * R;
      const bool nn = (nn_mask >> mode) & 1u;
      if (nn) {
        k_mu_accum<<<(RR + 255) / 256, 256, 0, st>>>(G, N, mode, (int)R, P, done);
        TLGB_LAUNCH_CHECK();
        if (weights) {
          k_weight_outer<T><<<(RR + 255) / 256, 256, 0, st>>>(P, weights, (int)R, done);
          TLGB_LAUNCH_CHECK();
        }
        k_to_type<T><<<(RR + 255) / 256, 256, 0, st>>>(P, (int)R, Pt, done);
        TLGB_LAUNCH_CHECK();
      } else {
        // factorisation of V = (prod G) * w w^T for the least-squares update
        rc = als_launch_factorize<T>(G, N, mode, (int)R, weights, 0.0, fac, perm, vmat, w32,
                                     ctrl, st);
        if (rc) return rc;
      }
      rc = mk.launch(mode, cf, weights, done, st);
      if (rc) return rc;
      k_sum_splits_to<T><<<(unsigned)std::min<int64_t>(ceil_div(IR, 256), 4096), 256, 0, st>>>(
          mk.partial(), mk.splits(mode), IR, M);
      TLGB_LAUNCH_CHECK();
      if (nn) {
        // no sparsity coefficient (NaN): subtract 0, which leaves num unchanged
        const double sp = (sparsity && !std::isnan(sparsity[mode])) ? sparsity[mode] : 0.0;
        rc = hals_solve<T>(M, Pt, factors[mode], I, (int)R, n_inner, tol_inner, sp, save, hpart,
                           e0, chunk, hals_smem, p_in_smem, done, st);
      } else {
        int nb = 0;
        rc = als_launch_solve<T>(mk.partial(), mk.splits(mode), I, (int)R, fac, perm, vmat, w32,
                                 factors[mode], nullptr, gpart, nullptr, ctrl, kIrMaxPasses, &nb,
                                 st);
      }
      if (rc) return rc;
      rc = mk.refresh(mode, factors[mode], st);
      if (rc) return rc;
      if (mode == last) {
        k_inner_part<T><<<kInnerBlocks, 256, 0, st>>>(M, factors[mode], IR, ipart, done);
        TLGB_LAUNCH_CHECK();
      }
      rc = als_launch_gram<T>(factors[mode], I, (int)R, gpart, nparts, G + (size_t)mode * RR,
                              done, st);
      if (rc) return rc;
      if (normalize && q + 1 < n_free) {
        rc = normalize_all();
        if (rc) return rc;
      }
    }
    if (tol > 0.0) {
      rc = als_launch_fit<T>(G, N, (int)R, weights, ipart, kInnerBlocks, ctrl, derr, n_iter_max,
                             tol, crit, st);
      if (rc) return rc;
      TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
      TLGB_CUDA_TRY(cudaStreamSynchronize(st));
      if (hc.status == TLGB_ESINGULAR)
        return set_error(TLGB_ESINGULAR, "cp_nn_hals: normal equations singular");
      if (hc.done) break;
    }
    if (normalize) {
      rc = normalize_all();
      if (rc) return rc;
    }
  }
  TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (hc.tc_err != 0)
    return set_error(TLGB_ETIMEOUT, "cp_nn_hals: a tensor-core MTTKRP wait timed out");
  const int ne = (tol > 0.0) ? std::min(hc.iter, n_iter_max) : 0;
  if (n_errors) *n_errors = ne;
  if (errors && ne > 0)
    TLGB_CUDA_TRY(cudaMemcpy(errors, derr, sizeof(double) * ne, cudaMemcpyDeviceToHost));
  return TLGB_OK;
}

int check_nn_args(int dtype, const int64_t* shape, int ndim, int64_t rank) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "cp_nn_mu: dtype must be f32 or f64");
  TLGB_CHECK_ARG(shape != nullptr, "cp_nn_mu: null shape");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "cp_nn_mu: ndim must be in [2, 8]");
  TLGB_CHECK_ARG(rank >= 1, "cp_nn_mu: rank must be >= 1");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(shape[k] >= 1, "cp_nn_mu: empty mode");
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_cp_nn_mu_workspace_size(int dtype, int ndim, const int64_t* shape,
                                            int64_t rank, int n_iter_max, size_t* bytes) {
  clear_error();
  int rc = check_nn_args(dtype, shape, ndim, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(bytes != nullptr && n_iter_max >= 0, "cp_nn_mu_workspace_size: bad argument");
  Shape sh = make_shape(ndim, shape);
  std::vector<MttkrpPlan> plans;
  int nparts = 0;
  MuLayout L;
  rc = (dtype == TLGB_F64) ? mu_layout<double>(sh, rank, n_iter_max, &plans, &nparts, &L)
                           : mu_layout<float>(sh, rank, n_iter_max, &plans, &nparts, &L);
  if (rc) return rc;
  *bytes = L.bytes;
  return TLGB_OK;
}

extern "C" int tlgb_cp_nn_mu(int dtype, const void* X, int ndim, const int64_t* shape,
                             void* const* factors, int64_t rank, const int* free_modes,
                             int n_free, int n_iter_max, double tol, int cvg_criterion,
                             double* errors, int* n_errors, void* workspace,
                             size_t workspace_bytes, void* stream) {
  clear_error();
  int rc = check_nn_args(dtype, shape, ndim, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(X && factors && free_modes, "cp_nn_mu: null pointer");
  TLGB_CHECK_ARG(n_free >= 1 && n_free <= ndim, "cp_nn_mu: bad number of free modes");
  TLGB_CHECK_ARG(free_modes[n_free - 1] == ndim - 1, "cp_nn_mu: the last mode must be free");
  for (int q = 0; q < n_free; ++q)
    TLGB_CHECK_ARG(free_modes[q] >= 0 && free_modes[q] < ndim &&
                       (q == 0 || free_modes[q] > free_modes[q - 1]),
                   "cp_nn_mu: free modes must be ascending and in range");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(factors[k] != nullptr, "cp_nn_mu: null factor");
  TLGB_CHECK_ARG(n_iter_max >= 0 && tol >= 0.0, "cp_nn_mu: bad n_iter_max or tol");
  TLGB_CHECK_ARG(cvg_criterion == 0 || cvg_criterion == 1, "cp_nn_mu: bad cvg_criterion");
  Shape sh = make_shape(ndim, shape);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return mu_run<double>((const double*)X, sh, (double* const*)factors, rank, free_modes, n_free,
                          n_iter_max, tol, cvg_criterion, errors, n_errors, workspace,
                          workspace_bytes, st);
  return mu_run<float>((const float*)X, sh, (float* const*)factors, rank, free_modes, n_free,
                       n_iter_max, tol, cvg_criterion, errors, n_errors, workspace,
                       workspace_bytes, st);
}

extern "C" int tlgb_cp_nn_hals(int dtype, const void* X, int ndim, const int64_t* shape,
                               void* const* factors, void* weights, int64_t rank,
                               const int* free_modes, int n_free, unsigned nn_modes_mask,
                               int normalize_factors, int n_iter_max, double tol,
                               int cvg_criterion, const double* sparsity, int exact,
                               double* errors, int* n_errors, void* workspace,
                               size_t workspace_bytes, void* stream) {
  clear_error();
  int rc = check_nn_args(dtype, shape, ndim, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(X && factors && free_modes, "cp_nn_hals: null pointer");
  TLGB_CHECK_ARG(n_free >= 1 && n_free <= ndim, "cp_nn_hals: bad number of free modes");
  TLGB_CHECK_ARG(free_modes[n_free - 1] == ndim - 1, "cp_nn_hals: the last mode must be free");
  for (int q = 0; q < n_free; ++q)
    TLGB_CHECK_ARG(free_modes[q] >= 0 && free_modes[q] < ndim &&
                       (q == 0 || free_modes[q] > free_modes[q - 1]),
                   "cp_nn_hals: free modes must be ascending and in range");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(factors[k] != nullptr, "cp_nn_hals: null factor");
  TLGB_CHECK_ARG(n_iter_max >= 0 && tol >= 0.0, "cp_nn_hals: bad n_iter_max or tol");
  TLGB_CHECK_ARG(cvg_criterion == 0 || cvg_criterion == 1, "cp_nn_hals: bad cvg_criterion");
  TLGB_CHECK_ARG(rank <= kMaxAlsRank, "cp_nn_hals: rank above 160 is not supported");
  TLGB_CHECK_ARG(!normalize_factors || weights != nullptr,
                 "cp_nn_hals: normalize_factors needs a weights buffer");
  Shape sh = make_shape(ndim, shape);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return hals_run<double>((const double*)X, sh, (double* const*)factors, (double*)weights, rank,
                            free_modes, n_free, nn_modes_mask, normalize_factors, n_iter_max, tol,
                            cvg_criterion, sparsity, exact, errors, n_errors, workspace,
                            workspace_bytes, st);
  return hals_run<float>((const float*)X, sh, (float* const*)factors, (float*)weights, rank,
                         free_modes, n_free, nn_modes_mask, normalize_factors, n_iter_max, tol,
                         cvg_criterion, sparsity, exact, errors, n_errors, workspace,
                         workspace_bytes, st);
}

extern "C" int tlgb_sum(int dtype, const void* X, int64_t n, double* out, void* workspace,
                        size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "sum: dtype must be f32 or f64");
  TLGB_CHECK_ARG(X && out && n >= 1, "sum: bad argument");
  constexpr int kBlocks = 256;
  TLGB_CHECK_ARG(workspace && workspace_bytes >= kBlocks * sizeof(double),
                 "sum: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  double* part = static_cast<double*>(workspace);
  if (dtype == TLGB_F64)
    k_sum_part<double><<<kBlocks, 256, 0, st>>>((const double*)X, n, part);
  else
    k_sum_part<float><<<kBlocks, 256, 0, st>>>((const float*)X, n, part);
  TLGB_LAUNCH_CHECK();
  k_sum_final<<<1, 32, 0, st>>>(part, kBlocks, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_nndsvd_columns(int dtype, const void* U, const void* S, const void* Y,
                                   int64_t I, int64_t k, int64_t L, int64_t Tt, int fill,
                                   double avg, void* W, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "nndsvd: dtype must be f32 or f64");
  TLGB_CHECK_ARG(U && S && Y && W && I >= 1 && k >= 1 && L >= 1 && Tt >= 1,
                 "nndsvd: bad argument");
  const size_t es = dtype == TLGB_F64 ? 8 : 4;
  TLGB_CHECK_ARG(workspace && workspace_bytes >= 2 * (size_t)k * es, "nndsvd: workspace too small");
  TLGB_CHECK_ARG(k <= 65535, "nndsvd: too many columns");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64) {
    k_posneg_norms<double><<<(unsigned)k, 256, 0, st>>>((const double*)Y, L, (int)k, Tt,
                                                        (double*)workspace);
    TLGB_LAUNCH_CHECK();
    k_nndsvd_columns<double><<<(unsigned)k, 256, 0, st>>>(
        (const double*)U, (const double*)S, (const double*)workspace, I, (int)k,
        std::numeric_limits<double>::epsilon(), fill, avg, (double*)W);
  } else {
    k_posneg_norms<float><<<(unsigned)k, 256, 0, st>>>((const float*)Y, L, (int)k, Tt,
                                                       (float*)workspace);
    TLGB_LAUNCH_CHECK();
    k_nndsvd_columns<float><<<(unsigned)k, 256, 0, st>>>(
        (const float*)U, (const float*)S, (const float*)workspace, I, (int)k,
        std::numeric_limits<float>::epsilon(), fill, (float)avg, (float*)W);
  }
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

// ---- standalone hals_nnls ----------------------------------------------------

namespace {

struct HalsLayout {
  size_t done, state, Pt, save, hpart, bytes;
};

HalsLayout hals_layout(int dtype, int64_t I, int64_t R) {
  HalsLayout L{};
  const size_t esz = dtype == TLGB_F64 ? 8 : 4;
  const int64_t hrows = ceil_div(I, (int64_t)kHalsWarps) * kHalsWarps;
  size_t off = 0;
  auto take = [&](size_t b) { off = align_up(off, 256); const size_t o = off; off += b; return o; };
  L.done = take(sizeof(int));
  L.state = take(2 * sizeof(double));
  L.Pt = take(esz * (size_t)R * R);
  L.save = take(esz * (size_t)I * R);
  L.hpart = take(sizeof(double) * (size_t)(hrows * hals_chunk(hrows)));
  L.bytes = align_up(off, 256);
  return L;
}

template <typename T>
int hals_nnls_run(const T* MtU, const T* UtU, T* V, int64_t I, int64_t R, int n_iter_max,
                  double tol, double sparsity, void* ws, cudaStream_t st) {
  const HalsLayout L = hals_layout(TypeCode<T>::value, I, R);
  char* base = static_cast<char*>(ws);
  int* done = reinterpret_cast<int*>(base + L.done);
  double* state = reinterpret_cast<double*>(base + L.state);
  T* Pt = reinterpret_cast<T*>(base + L.Pt);
  T* save = reinterpret_cast<T*>(base + L.save);
  double* hpart = reinterpret_cast<double*>(base + L.hpart);
  TLGB_CUDA_TRY(cudaMemsetAsync(done, 0, sizeof(int), st));
  const int RR = (int)(R * R);
  k_sym_typed<T><<<(RR + 255) / 256, 256, 0, st>>>(UtU, (int)R, Pt);
  TLGB_LAUNCH_CHECK();
  const int p_in_smem = ((size_t)R * R * sizeof(T) <= kHalsPSmemMax) ? 1 : 0;
  const size_t hals_smem = (p_in_smem ? (size_t)R * R * sizeof(T) : 0) +
                           (size_t)kHalsWarps * R * sizeof(T);
  const int chunk = hals_chunk(ceil_div(I, (int64_t)kHalsWarps) * kHalsWarps);
  const double sp = std::isnan(sparsity) ? 0.0 : sparsity;
  return hals_solve<T>(MtU, Pt, V, I, (int)R, n_iter_max, tol, sp, save, hpart, state, chunk,
                       hals_smem, p_in_smem, done, st);
}

}  // namespace

extern "C" int tlgb_hals_nnls_workspace_size(int dtype, int64_t I, int64_t R, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "hals_nnls: dtype must be f32 or f64");
  TLGB_CHECK_ARG(I >= 1 && R >= 1 && R <= kMaxAlsRank && bytes, "hals_nnls: bad argument");
  *bytes = hals_layout(dtype, I, R).bytes;
  return TLGB_OK;
}

extern "C" int tlgb_hals_nnls(int dtype, const void* MtU, const void* UtU, void* V, int64_t I,
                              int64_t R, int n_iter_max, double tol, double sparsity,
                              void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "hals_nnls: dtype must be f32 or f64");
  TLGB_CHECK_ARG(MtU && UtU && V, "hals_nnls: null pointer");
  TLGB_CHECK_ARG(I >= 1 && R >= 1 && R <= kMaxAlsRank, "hals_nnls: rank must be in [1, 160]");
  TLGB_CHECK_ARG(n_iter_max >= 0 && tol >= 0.0, "hals_nnls: bad n_iter_max or tol");
  if (!workspace || workspace_bytes < hals_layout(dtype, I, R).bytes)
    return set_error(TLGB_EWORKSPACE, "hals_nnls: workspace too small");
  int rc = als_prepare(dtype);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return hals_nnls_run<double>(static_cast<const double*>(MtU), static_cast<const double*>(UtU),
                                 static_cast<double*>(V), I, R, n_iter_max, tol, sparsity,
                                 workspace, st);
  return hals_nnls_run<float>(static_cast<const float*>(MtU), static_cast<const float*>(UtU),
                              static_cast<float*>(V), I, R, n_iter_max, tol, sparsity, workspace,
                              st);
}
