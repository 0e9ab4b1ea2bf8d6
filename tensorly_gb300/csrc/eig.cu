// Symmetric eigensolver for the partial SVDs of Tucker-HOOI and the SVD
// initialisations (tensorly/tenalg/svd.py:211-235 truncated_svd,
// :366-447 svd_interface, :13-65 svd_flip).
//
// The left singular vectors of an unfolding M are the eigenvectors of the
// Gram matrix G = M M^T, so the SVD of a wide unfolding reduces to the top-k
// eigenpairs of a small symmetric matrix (S = sqrt(lambda)).  One CTA solves
// it in the element type T (f64 for f64 tensors, f32 for f32 tensors, which
// is the precision the reference's LAPACK call works in):
//   1. Householder tridiagonalisation Q^T G Q = tridiag(d, e), G held in
//      shared memory (reflectors kept below the diagonal);
//   2. the k largest eigenvalues of the tridiagonal matrix by multisection on
//      Sturm counts (each eigenvalue's interval is cut into many pieces per
//      round by a group of threads, so ~log_33 instead of log_2 rounds);
//   3. eigenvectors of the tridiagonal matrix by inverse iteration (one
//      thread per eigenvalue, LU with partial pivoting), re-orthogonalised
//      within clusters of close eigenvalues, in shared memory when they fit;
//   4. back-transformation by the reflectors, then the sign convention of
//      svd_flip (the largest-magnitude entry of every column is positive).
// The eigenvalues come out in descending order, as LAPACK's singular values.
#include "linalg.cuh"

namespace tlgb {
namespace {

constexpr int kEigThreads = 512;
constexpr int kEigWarps = kEigThreads / 32;

template <typename T> struct EigLimits;
template <> struct EigLimits<double> {
  static constexpr int max_n = 160;
  static constexpr double eps = 1.1102230246251565e-16;
  static constexpr double tiny = 1e-290;
};
template <> struct EigLimits<float> {
  static constexpr int max_n = 224;
  static constexpr float eps = 5.9604645e-08f;
  static constexpr float tiny = 1e-35f;
};

template <typename T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum; every thread gets the result.
template <typename T>
__device__ T block_sum_t(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_t(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T t = (threadIdx.x < kEigWarps) ? red[threadIdx.x] : T(0);
  if (warp == 0) {
#pragma unroll
    for (int o = kEigWarps / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[0] = t;
  }
  __syncthreads();
  const T r = red[0];
  __syncthreads();
  return r;
}

// Block-wide sum with a single barrier: warp partials go to `red` (kEigWarps
// slots) and every thread adds them up.  `red` must not be written again
// before a later barrier, so consecutive calls alternate between two buffers.
template <typename T>
__device__ __forceinline__ T block_sum_1(T v, T* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_t(v);
  if (lane == 0) red[warp] = v;
  __syncthreads();
  T t = T(0);
#pragma unroll
  for (int w = 0; w < kEigWarps; ++w) t += red[w];
  return t;
}

// Number of eigenvalues of tridiag(d, e) below x (Sturm count); e2 = e^2.
template <typename T>
__device__ int sturm_count(const T* d, const T* e2, int n, T x) {
  int cnt = 0;
  T q = d[0] - x;
  if (q < T(0)) ++cnt;
  for (int i = 1; i < n; ++i) {
    if (q == T(0)) q = EigLimits<T>::tiny;
    q = (d[i] - x) - e2[i - 1] / q;
    if (q < T(0)) ++cnt;
  }
  return cnt;
}

// A: n x n symmetric (row-major, both triangles).  Outputs: U (n x k,
// row-major), lam (k), descending.  Zg: global workspace of 6 k n elements per
// matrix; with zsm the k eigenvectors and the three diagonals of their
// triangular factors live in shared memory instead (4 k n elements).
template <typename T>
__global__ void __launch_bounds__(kEigThreads)
k_sym_eig(const T* __restrict__ A, int n, int k, T* U, T* lam, int flip, T* Zg, int zsm) {
  // batched launches: CTA b solves matrix b (every operand advanced by its size)
  A += (int64_t)blockIdx.x * n * n;
  U += (int64_t)blockIdx.x * n * k;
  lam += (int64_t)blockIdx.x * k;
  Zg += (int64_t)blockIdx.x * 6 * k * n;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int ld = n | 1;                      // odd: rows and columns are both conflict-free
  T* As = reinterpret_cast<T*>(smem_raw);   // n * ld
  T* d = As + (size_t)n * ld;                // n
  T* e = d + n;                              // n
  T* e2 = e + n;                             // n
  T* tau = e2 + n;                           // n
  T* vv = tau + n;                           // n (the current reflector, contiguous)
  T* red = vv + n;                           // 32 (two halves for block_sum_1)
  T* bnd = red + 32;                         // 2 * kEigThreads (multisection bounds, scratch)
  T* Zb = zsm ? bnd + 2 * kEigThreads : Zg;  // k * n eigenvectors, then 3 * k * n
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

  for (int i = tid; i < n * n; i += kEigThreads) {
    const int r = i / n, c = i - (i / n) * n;
    As[r * ld + c] = A[i];
  }
  for (int i = tid; i < n; i += kEigThreads) { e[i] = T(0); tau[i] = T(0); }
  __syncthreads();

  // ---- 1. tridiagonalisation on the lower triangle.  Reflector j zeroes
  // column j below the subdiagonal and is stored there (v[0] = 1); a
  // contiguous copy serves the step.  Only the lower triangle (diagonal
  // included) of the trailing block is updated; the matrix-vector product
  // reads each element from whichever triangle holds it.
  for (int j = 0; j + 2 < n; ++j) {
    const int m = n - j - 1;               // length of the reflected part
    T* x = As + (j + 1) * ld + j;          // x[i] at x[i * ld]
    T s2 = T(0);
    for (int i = 1 + tid; i < m; i += kEigThreads) s2 += x[i * ld] * x[i * ld];
    s2 = block_sum_1(s2, red);
    const T alpha = x[0];
    T t = T(0), beta = alpha, scale = T(0);
    if (s2 > T(0)) {
      const T mu = sqrt(alpha * alpha + s2);
      beta = (alpha >= T(0)) ? -mu : mu;
      t = (beta - alpha) / beta;
      scale = T(1) / (alpha - beta);
    }
    __syncthreads();   // all threads have read x[0] before it is overwritten
    if (tid == 0) { e[j] = beta; tau[j] = t; d[j] = As[j * ld + j]; x[0] = T(1); vv[0] = T(1); }
    if (t != T(0))
      for (int i = 1 + tid; i < m; i += kEigThreads) {
        const T v = x[i * ld] * scale;
        x[i * ld] = v;
        vv[i] = v;
      }
    __syncthreads();
    if (t == T(0)) continue;
    // p = t * A22 v, thread r summing over c (H groups split the sum)
    T* A22 = As + (j + 1) * ld + (j + 1);
    const int H = kEigThreads / m;         // >= 2 (m < n <= 224)
    {
      const int r = tid % m, h = tid / m;
      if (h < H) {
        T acc = T(0);
        for (int c = h; c < m; c += H)
          acc += ((c <= r) ? A22[r * ld + c] : A22[c * ld + r]) * vv[c];
        bnd[h * m + r] = acc;
      }
    }
    __syncthreads();
    T pv = T(0);
    for (int r = tid; r < m; r += kEigThreads) {
      T acc = T(0);
      for (int h = 0; h < H; ++h) acc += bnd[h * m + r];
      e2[r] = t * acc;                     // e2 holds p, then w, until the loop ends
      pv += e2[r] * vv[r];
    }
    pv = block_sum_1(pv, red + kEigWarps);
    const T K = T(0.5) * t * pv;
    for (int r = tid; r < m; r += kEigThreads) e2[r] -= K * vv[r];   // w
    __syncthreads();
    // lower triangle of A22 -= v w^T + w v^T (warp per row, lanes along it)
    for (int r = warp; r < m; r += kEigWarps) {
      const T vr = vv[r], wr = e2[r];
      T* row = A22 + r * ld;
      for (int c = lane; c <= r; c += 32) row[c] -= vr * e2[c] + wr * vv[c];
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (n >= 2) {
      d[n - 2] = As[(n - 2) * ld + (n - 2)];
      e[n - 2] = As[(n - 1) * ld + (n - 2)];
    }
    d[n - 1] = As[(n - 1) * ld + (n - 1)];
  }
  __syncthreads();
  for (int i = tid; i < n; i += kEigThreads) e2[i] = (i + 1 < n) ? e[i] * e[i] : T(0);
  __syncthreads();

  // ---- 2. the k largest eigenvalues by multisection
  T glo = T(0), ghi = T(0);
  {
    T lo = T(0), hi = T(0);
    bool first = true;
    for (int i = 0; i < n; ++i) {   // Gerschgorin bounds (every thread, n <= 224)
      const T rad = ((i > 0) ? fabs(e[i - 1]) : T(0)) + ((i + 1 < n) ? fabs(e[i]) : T(0));
      const T a = d[i] - rad, b = d[i] + rad;
      if (first || a < lo) lo = a;
      if (first || b > hi) hi = b;
      first = false;
    }
    const T pad = T(2) * EigLimits<T>::eps * fmax(fabs(lo), fabs(hi)) * T(n) + EigLimits<T>::tiny;
    glo = lo - pad;
    ghi = hi + pad;
  }
  const T tnorm = fmax(fabs(glo), fabs(ghi));
  for (int k0 = 0; k0 < k; k0 += kEigThreads) {
    const int kb = min(k - k0, kEigThreads);
    const int G = max(1, kEigThreads / kb);   // threads per eigenvalue
    const int g = tid / G, gi = tid - (tid / G) * G;
    const bool act = g < kb;
    const int target = n - 1 - (k0 + g);     // ascending index of this eigenvalue
    T lo = glo, hi = ghi;
    for (int it = 0; it < 200; ++it) {
      const T width = hi - lo;
      const bool conv = !act || width <= T(4) * EigLimits<T>::eps * fmax(fabs(lo), fabs(hi)) +
                                             T(4) * EigLimits<T>::eps * tnorm * T(1e-3);
      if (__syncthreads_and(conv ? 1 : 0)) break;
      T x = lo, xnew_lo = lo, xnew_hi = hi;
      int cnt = 0;
      if (act && !conv) {
        x = lo + width * (T)(gi + 1) / (T)(G + 1);
        cnt = sturm_count(d, e2, n, x);
      }
      // group reduction of the new bounds through shared memory
      bnd[2 * tid] = (act && !conv && cnt <= target) ? x : lo;
      bnd[2 * tid + 1] = (act && !conv && cnt > target) ? x : hi;
      __syncthreads();
      if (act && !conv) {
        for (int q = 0; q < G; ++q) {
          xnew_lo = fmax(xnew_lo, bnd[2 * (g * G + q)]);
          xnew_hi = fmin(xnew_hi, bnd[2 * (g * G + q) + 1]);
        }
      }
      __syncthreads();
      if (act && !conv) { lo = xnew_lo; hi = xnew_hi; }
    }
    if (act && gi == 0) lam[k0 + g] = T(0.5) * (lo + hi);
  }
  __syncthreads();

  // ---- 3. eigenvectors of the tridiagonal matrix by inverse iteration
  const T pert = T(10) * EigLimits<T>::eps * tnorm + EigLimits<T>::tiny;
  for (int c = tid; c < k; c += kEigThreads) {
    T* z = Zb + (int64_t)c * n;
    T* ua = Zb + (int64_t)k * n + (int64_t)c * 3 * n;   // U of the LU of (T - mu I):
    T* ub = ua + n;                                      // diagonal and two superdiagonals
    T* uc = ub + n;
    // nudge mu off the eigenvalue (alternating direction per index) so the
    // LU is non-singular; the shift is far below the eigenvalue's accuracy
    const T mu = lam[c] + ((c & 1) ? pert : -pert);
    // start vector: deterministic, no special alignment with any eigenvector
    for (int i = 0; i < n; ++i) z[i] = T(1) + T(0.01) * (T)((i * 7 + c * 3) % 11);
    for (int iter = 0; iter < 3; ++iter) {
      // LU with partial pivoting (tridiagonal, fill in one super), its row
      // swaps and multipliers applied to z on the way (only U is kept)
      T a_i = d[0] - mu, b_i = (n > 1) ? e[0] : T(0);
      T zi = z[0];
      for (int i = 0; i + 1 < n; ++i) {
        const T sub = e[i];
        const T a_n = d[i + 1] - mu;
        const T b_n = (i + 2 < n) ? e[i + 1] : T(0);
        const T zn = z[i + 1];
        if (fabs(sub) > fabs(a_i)) {   // swap rows i and i+1
          const T mult = a_i / sub;
          ua[i] = sub; ub[i] = a_n; uc[i] = b_n;
          a_i = b_i - mult * a_n;
          b_i = -mult * b_n;
          z[i] = zn;
          zi = zi - mult * zn;
        } else {
          const T div = (a_i == T(0)) ? pert : a_i;
          const T mult = sub / div;
          ua[i] = div; ub[i] = b_i; uc[i] = T(0);
          a_i = a_n - mult * b_i;
          b_i = b_n;
          z[i] = zi;
          zi = zn - mult * zi;
        }
      }
      ua[n - 1] = (a_i == T(0)) ? pert : a_i;
      z[n - 1] = zi;
      z[n - 1] = z[n - 1] / ua[n - 1];   // back substitution with U (diag, two supers)
      if (n >= 2) z[n - 2] = (z[n - 2] - ub[n - 2] * z[n - 1]) / ua[n - 2];
      for (int i = n - 3; i >= 0; --i)
        z[i] = (z[i] - ub[i] * z[i + 1] - uc[i] * z[i + 2]) / ua[i];
      T nrm = T(0);
      for (int i = 0; i < n; ++i) nrm += z[i] * z[i];
      nrm = T(1) / sqrt(nrm);
      for (int i = 0; i < n; ++i) z[i] *= nrm;
    }
  }
  __syncthreads();
  // re-orthogonalise within clusters of close eigenvalues (descending order)
  const T clus = T(1e-3) * tnorm;
  for (int c = 1; c < k; ++c) {
    if (fabs(lam[c - 1] - lam[c]) > clus) continue;
    int c0 = c - 1;
    while (c0 > 0 && fabs(lam[c0 - 1] - lam[c0]) <= clus) --c0;
    T* zc = Zb + (int64_t)c * n;
    for (int q = c0; q < c; ++q) {
      const T* zq = Zb + (int64_t)q * n;
      T dot = T(0);
      for (int i = tid; i < n; i += kEigThreads) dot += zq[i] * zc[i];
      dot = block_sum_t(dot, red);
      for (int i = tid; i < n; i += kEigThreads) zc[i] -= dot * zq[i];
      __syncthreads();
    }
    T nrm = T(0);
    for (int i = tid; i < n; i += kEigThreads) nrm += zc[i] * zc[i];
    nrm = block_sum_t(nrm, red);
    const T inv = T(1) / sqrt(nrm);
    for (int i = tid; i < n; i += kEigThreads) zc[i] *= inv;
    __syncthreads();
  }

  // ---- 4. back-transformation (one warp per vector) and svd_flip signs
  for (int c = warp; c < k; c += kEigWarps) {
    T* z = Zb + (int64_t)c * n;
    for (int j = n - 3; j >= 0; --j) {
      const T tj = tau[j];
      if (tj == T(0)) continue;
      const int m = n - j - 1;
      const T* v = As + (j + 1) * ld + j;   // column j, v[0] = 1 stored explicitly
      T s = T(0);
      for (int i = lane; i < m; i += 32) s += v[i * ld] * z[j + 1 + i];
      s = tj * warp_sum_t(s);
      for (int i = lane; i < m; i += 32) z[j + 1 + i] -= s * v[i * ld];
      __syncwarp();
    }
    // first index of the largest |z| (ties resolved to the lowest index)
    T best = T(-1);
    int bi = n;
    for (int i = lane; i < n; i += 32) {
      const T a = fabs(z[i]);
      if (a > best) { best = a; bi = i; }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const T ob = __shfl_xor_sync(0xffffffffu, best, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
    }
    const T sgn = (flip && z[bi] < T(0)) ? T(-1) : T(1);
    for (int i = lane; i < n; i += 32) U[(int64_t)i * k + c] = sgn * z[i];
  }
}

constexpr size_t kEigSmemLimit = 227 * 1024;

template <typename T>
size_t eig_smem(int n) {
  return ((size_t)n * (n | 1) + 5 * (size_t)n + 32 + 2 * kEigThreads) * sizeof(T);
}
// with the eigenvectors and triangular factors in shared memory as well
template <typename T>
size_t eig_smem_z(int n, int k) {
  return eig_smem<T>(n) + 4 * (size_t)k * n * sizeof(T);
}

}  // namespace

int sym_eig_max_n(int dtype) {
  return dtype == TLGB_F64 ? EigLimits<double>::max_n : EigLimits<float>::max_n;
}

size_t sym_eig_workspace(int dtype, int64_t n, int64_t k) {
  const size_t es = dtype == TLGB_F64 ? 8 : 4;
  return align_up((size_t)k * 6 * n * es, 256);
}

template <typename T>
int sym_eig_launch(const T* A, int n, int k, T* U, T* lam, int flip, void* ws, cudaStream_t st) {
  return sym_eig_batched_launch<T>(A, n, k, 1, U, lam, flip, ws, st);
}

template <typename T>
int sym_eig_batched_launch(const T* A, int n, int k, int batch, T* U, T* lam, int flip, void* ws,
                           cudaStream_t st) {
  TLGB_CHECK_ARG(batch >= 1 && batch <= 2147483647, "sym_eig: bad batch");
  TLGB_CHECK_ARG(n >= 1 && k >= 1 && k <= n, "sym_eig: need 1 <= k <= n");
  if (n > EigLimits<T>::max_n)
    return set_error(TLGB_EUNSUPPORTED, "sym_eig: matrix order above " +
                                            std::to_string(EigLimits<T>::max_n) +
                                            " is not supported");
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_sym_eig<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kEigSmemLimit));
    attr[dev] = true;
  }
  T* Z = static_cast<T*>(ws);
  const int zsm = eig_smem_z<T>(n, k) <= kEigSmemLimit ? 1 : 0;
  k_sym_eig<T><<<batch, kEigThreads, zsm ? eig_smem_z<T>(n, k) : eig_smem<T>(n), st>>>(
      A, n, k, U, lam, flip, Z, zsm);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template int sym_eig_launch<float>(const float*, int, int, float*, float*, int, void*,
                                   cudaStream_t);
template int sym_eig_batched_launch<float>(const float*, int, int, int, float*, float*, int,
                                           void*, cudaStream_t);
template int sym_eig_batched_launch<double>(const double*, int, int, int, double*, double*, int,
                                            void*, cudaStream_t);
template int sym_eig_launch<double>(const double*, int, int, double*, double*, int, void*,
                                    cudaStream_t);

}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_sym_eig_workspace_size(int dtype, int64_t n, int64_t k, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(bytes != nullptr, "sym_eig_workspace_size: null pointer");
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "sym_eig: dtype must be f32 or f64");
  TLGB_CHECK_ARG(n >= 1 && k >= 1 && k <= n, "sym_eig: need 1 <= k <= n");
  *bytes = sym_eig_workspace(dtype, n, k);
  return TLGB_OK;
}

extern "C" int tlgb_sym_eig(int dtype, const void* A, int64_t n, int64_t k, void* U, void* evals,
                            int flip_sign, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "sym_eig: dtype must be f32 or f64");
  TLGB_CHECK_ARG(A && U && evals, "sym_eig: null pointer");
  TLGB_CHECK_ARG(n >= 1 && k >= 1 && k <= n, "sym_eig: need 1 <= k <= n");
  if (!workspace || workspace_bytes < sym_eig_workspace(dtype, n, k))
    return set_error(TLGB_EWORKSPACE, "sym_eig: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return sym_eig_launch<double>((const double*)A, (int)n, (int)k, (double*)U, (double*)evals,
                                  flip_sign, workspace, st);
  return sym_eig_launch<float>((const float*)A, (int)n, (int)k, (float*)U, (float*)evals,
                               flip_sign, workspace, st);
}
