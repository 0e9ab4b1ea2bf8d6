// f64 kernels of the CP-ALS sweep: tensor norm, factor Grams, the normal-
// equation factorisation and solve, the fit, and column normalisation.
//
// Reference steps (tensorly/decomposition/_cp.py):
//   :411-422  V = (prod_{i != mode} A_i^H A_i + l2_reg I) scaled by w w^T
//   :425-428  A_mode = solve(V^H, M^T)^T            (LAPACK gesv there)
//   :217-225  ||X - [[w; A]]||^2 = ||X||^2 + cp_norm^2 - 2 sum(M_last * A_last)
//   :529-530  cp_normalize (tensorly/cp_tensor.py:278-321)
// V is symmetric positive (semi)definite, so it is factorised by Cholesky;
// if a pivot is not positive the kernel falls back to LU with partial
// pivoting (what gesv does), and an exactly zero LU pivot reports
// TLGB_ESINGULAR.  All of this runs in f64 regardless of the tensor dtype.
#include "als_kernels.cuh"

namespace tlgb {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum for blockDim.x a multiple of 32 (<= 1024); result valid in all threads.
__device__ double block_sum(double v, double* scratch /* >= 32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double t = (threadIdx.x < nw) ? scratch[threadIdx.x] : 0.0;
  if (warp == 0) t = warp_sum(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  const double r = scratch[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- sum of squares
template <typename T>
__global__ void k_sumsq(const T* __restrict__ X, int64_t n, double* part) {
  __shared__ double scratch[32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double x = (double)X[i];
    s = fma(x, x, s);
  }
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_sumsq_final(const double* part, int n, AlsCtrl* ctrl) {
  __shared__ double scratch[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) ctrl->norm_x2 = s;
}

// ---------------------------------------------------------------- Gram partials
constexpr int kGramRows = 8;  // rows staged per pass (keeps R = 160 under 227 KB)

// CTA b owns rows [b*rpb, (b+1)*rpb); writes sum_rows a a^T (full square) to gpart[b].
template <typename T>
__global__ void k_gram_partial(const T* __restrict__ A, int64_t I, int R, int64_t rpb,
                               double* gpart, const int* done) {
  if (done && *done) return;
  extern __shared__ double sm[];
  const int RR = R * R;
  double* gacc = sm;        // [R][R]
  double* rows = sm + RR;   // [kGramRows][R]
  const int64_t r0 = blockIdx.x * rpb;
  const int64_t r1 = min(r0 + rpb, I);
  for (int e = threadIdx.x; e < RR; e += blockDim.x) gacc[e] = 0.0;
  for (int64_t base = r0; base < r1; base += kGramRows) {
    const int nrow = (int)((r1 - base) < kGramRows ? (r1 - base) : kGramRows);
    __syncthreads();
    for (int e = threadIdx.x; e < kGramRows * R; e += blockDim.x) {
      const int i = e / R, r = e % R;
      rows[e] = (i < nrow) ? (double)A[(base + i) * R + r] : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < RR; e += blockDim.x) {
      const int r = e / R, s = e % R;
      if (s > r) continue;
      double g = gacc[e];
      for (int i = 0; i < nrow; ++i) g = fma(rows[i * R + r], rows[i * R + s], g);
      gacc[e] = g;
    }
  }
  __syncthreads();
  double* out = gpart + (int64_t)blockIdx.x * RR;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    out[e] = (s <= r) ? gacc[r * R + s] : gacc[s * R + r];
  }
}

__global__ void k_gram_reduce(const double* __restrict__ gpart, int nparts, int RR, double* G,
                              const int* done) {
  if (done && *done) return;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < RR; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int p = 0; p < nparts; ++p) s += gpart[(int64_t)p * RR + e];
    G[e] = s;
  }
}

// ---------------------------------------------------------------- factorisation
template <typename T>
__device__ void build_v(double* V, const double* G, int ndim, int mode, int R, const T* w,
                        double l2) {
  const int RR = R * R;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k)
      if (k != mode) v = v * G[(int64_t)k * RR + e];
    if (r == s) v = v + l2;
    if (w) v = ((double)w[r] * v) * (double)w[s];
    V[e] = v;
  }
}

// fac layout: [R*R] factor(s), then [R] reciprocal diagonal.
template <typename T>
__global__ void k_factorize(const double* G, int ndim, int mode, int R, const T* w, double l2,
                            double* fac, int* perm, AlsCtrl* ctrl) {
  if (ctrl->done) return;
  extern __shared__ double V[];  // R*R
  __shared__ int s_fail;
  __shared__ int s_piv;
  const int RR = R * R;
  build_v<T>(V, G, ndim, mode, R, w, l2);
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  // right-looking Cholesky on the lower triangle with unscaled columns:
  // after step k, V[i][k] = sqrt(d_k) * L[i][k] and V[k][k] = d_k.
  for (int k = 0; k < R; ++k) {
    const double d = V[k * R + k];
    if (!(d > 0.0)) {
      if (threadIdx.x == 0) s_fail = 1;
      break;  // uniform: every thread read the same d
    }
    const double inv = 1.0 / d;
    const int n = R - k - 1;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = k + 1 + e / n, j = k + 1 + e % n;
      if (j <= i) V[i * R + j] -= V[i * R + k] * V[j * R + k] * inv;
    }
    __syncthreads();
  }
  __syncthreads();
  if (!s_fail) {
    for (int e = threadIdx.x; e < RR; e += blockDim.x) {
      const int i = e / R, k = e % R;
      fac[e] = (k <= i) ? V[e] / sqrt(V[k * R + k]) : 0.0;
    }
    for (int k = threadIdx.x; k < R; k += blockDim.x) {
      fac[RR + k] = 1.0 / sqrt(V[k * R + k]);
      perm[k] = k;
    }
    if (threadIdx.x == 0) ctrl->fac_kind = 0;
    return;
  }
  // LU with partial pivoting (row interchanges tracked in perm).
  __syncthreads();
  build_v<T>(V, G, ndim, mode, R, w, l2);
  for (int k = threadIdx.x; k < R; k += blockDim.x) perm[k] = k;
  __syncthreads();
  for (int k = 0; k < R; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(V[k * R + k]);
      for (int i = k + 1; i < R; ++i) {
        const double a = fabs(V[i * R + k]);
        if (a > best) { best = a; p = i; }
      }
      s_piv = p;
      if (best == 0.0 && s_fail != 2) s_fail = 2;
      if (p != k) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k)
      for (int j = threadIdx.x; j < R; j += blockDim.x) {
        const double t = V[k * R + j];
        V[k * R + j] = V[p * R + j];
        V[p * R + j] = t;
      }
    __syncthreads();
    const double piv = V[k * R + k];
    if (piv != 0.0) {
      const double inv = 1.0 / piv;
      for (int i = k + 1 + threadIdx.x; i < R; i += blockDim.x) V[i * R + k] *= inv;
      __syncthreads();
      const int n = R - k - 1;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = k + 1 + e / n, j = k + 1 + e % n;
        V[i * R + j] -= V[i * R + k] * V[k * R + j];
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < RR; e += blockDim.x) fac[e] = V[e];
  for (int k = threadIdx.x; k < R; k += blockDim.x) {
    const double u = V[k * R + k];
    fac[RR + k] = (u != 0.0) ? 1.0 / u : 0.0;
  }
  if (threadIdx.x == 0) {
    ctrl->fac_kind = 1;
    if (s_fail == 2) ctrl->status = TLGB_ESINGULAR;
  }
}

// ---------------------------------------------------------------- solve
constexpr int kRQ = kMaxAlsRank / 32;  // register slots per lane

__device__ __forceinline__ double pick(const double (&v)[kRQ], int q) {
  double t = v[0];
#pragma unroll
  for (int i = 1; i < kRQ; ++i)
    if (q == i) t = v[i];
  return t;
}
__device__ __forceinline__ void put(double (&v)[kRQ], int q, double x) {
#pragma unroll
  for (int i = 0; i < kRQ; ++i)
    if (q == i) v[i] = x;
}

template <typename T>
__global__ void __launch_bounds__(32 * kSolveWarps)
k_solve(const T* __restrict__ partial, int splits, int64_t I, int R,
        const double* __restrict__ fac, const int* __restrict__ perm, T* A,
        __nv_bfloat16* A_bt, double* gpart, double* ipart, AlsCtrl* ctrl, int64_t rpb,
        int fac_in_smem) {
  if (ctrl->done) return;
  extern __shared__ double sm[];
  const int RR = R * R;
  double* gacc = sm;                      // RR
  double* rowbuf = gacc + RR;             // kSolveWarps * R
  double* sfac = rowbuf + kSolveWarps * R;  // RR + R (optional)
  __shared__ double s_ip[kSolveWarps];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kind = ctrl->fac_kind;
  for (int e = tid; e < RR; e += blockDim.x) gacc[e] = 0.0;
  if (fac_in_smem)
    for (int e = tid; e < RR + R; e += blockDim.x) sfac[e] = fac[e];
  __syncthreads();
  const double* F = fac_in_smem ? sfac : fac;
  const double* invd = F + RR;
  const int64_t row0 = blockIdx.x * rpb;
  const int64_t row1 = min(row0 + rpb, I);
  double ip = 0.0;
  const int64_t IR = I * R;
  for (int64_t base = row0; base < row1; base += kSolveWarps) {
    const int64_t row = base + warp;
    double* rb = rowbuf + warp * R;
    if (row < row1) {
      double v[kRQ], mv[kRQ];
#pragma unroll
      for (int q = 0; q < kRQ; ++q) {
        const int r = lane + 32 * q;
        double s = 0.0;
        if (r < R)
          for (int p = 0; p < splits; ++p) s += (double)partial[(int64_t)p * IR + row * R + r];
        mv[q] = s;
        v[q] = s;
      }
      if (kind == 1) {  // b = P m
#pragma unroll
        for (int q = 0; q < kRQ; ++q) {
          const int r = lane + 32 * q;
          if (r < R) rb[r] = v[q];
        }
        __syncwarp();
#pragma unroll
        for (int q = 0; q < kRQ; ++q) {
          const int r = lane + 32 * q;
          if (r < R) v[q] = rb[perm[r]];
        }
        __syncwarp();
      }
      // forward substitution with the lower factor
      for (int j = 0; j < R; ++j) {
        const int qj = j >> 5;
        double yj = __shfl_sync(0xffffffffu, pick(v, qj), j & 31);
        if (kind == 0) yj *= invd[j];
        if (lane == (j & 31)) put(v, qj, yj);
#pragma unroll
        for (int q = 0; q < kRQ; ++q) {
          const int i = lane + 32 * q;
          if (i > j && i < R) v[q] = fma(-F[i * R + j], yj, v[q]);
        }
      }
      // back substitution with the upper factor (L^T for Cholesky)
      for (int j = R - 1; j >= 0; --j) {
        const int qj = j >> 5;
        const double xj = __shfl_sync(0xffffffffu, pick(v, qj), j & 31) * invd[j];
        if (lane == (j & 31)) put(v, qj, xj);
#pragma unroll
        for (int q = 0; q < kRQ; ++q) {
          const int i = lane + 32 * q;
          if (i < j) {
            const double u = (kind == 0) ? F[j * R + i] : F[i * R + j];
            v[q] = fma(-u, xj, v[q]);
          }
        }
      }
#pragma unroll
      for (int q = 0; q < kRQ; ++q) {
        const int r = lane + 32 * q;
        if (r < R) {
          const T x = (T)v[q];
          A[row * R + r] = x;
          const double xd = (double)x;
          rb[r] = xd;
          if (A_bt) A_bt[(int64_t)r * I + row] = __float2bfloat16_rn((float)x);
          ip = fma(mv[q], xd, ip);
        }
      }
    } else {
      for (int r = lane; r < R; r += 32) rb[r] = 0.0;
    }
    __syncthreads();
    for (int e = tid; e < RR; e += blockDim.x) {
      const int r = e / R, s = e % R;
      if (s > r) continue;
      double g = gacc[e];
#pragma unroll
      for (int w = 0; w < kSolveWarps; ++w) g = fma(rowbuf[w * R + r], rowbuf[w * R + s], g);
      gacc[e] = g;
    }
    __syncthreads();
  }
  ip = warp_sum(ip);
  if (lane == 0) s_ip[warp] = ip;
  double* out = gpart + (int64_t)blockIdx.x * RR;
  for (int e = tid; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    out[e] = (s <= r) ? gacc[r * R + s] : gacc[s * R + r];
  }
  __syncthreads();
  if (ipart && tid == 0) {
    double t = 0.0;
    for (int w = 0; w < kSolveWarps; ++w) t += s_ip[w];
    ipart[blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------- fit
template <typename T>
__global__ void k_fit(const double* G, int ndim, int R, const T* w, const double* ipart, int nip,
                      AlsCtrl* ctrl, double* errors, int n_iter_max, double tol, int crit) {
  if (ctrl->done) return;
  __shared__ double scratch[32];
  const int RR = R * R;
  double c = 0.0;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k) v = v * G[(int64_t)k * RR + e];
    if (w) v = v * ((double)w[r] * (double)w[s]);
    c += v;
  }
  c = block_sum(c, scratch);
  double ip = 0.0;
  for (int i = threadIdx.x; i < nip; i += blockDim.x) ip += ipart[i];
  ip = block_sum(ip, scratch);
  if (threadIdx.x == 0) {
    const double nx2 = ctrl->norm_x2;
    const double err = sqrt(fabs(nx2 + c - 2.0 * ip)) / sqrt(nx2);
    const int it = ctrl->iter;
    if (it < n_iter_max) errors[it] = err;
    if (tol > 0.0 && it >= 1) {
      const double dec = errors[it - 1] - err;
      const bool stop = (crit == 0) ? (fabs(dec) < tol) : (dec < tol);
      if (stop) ctrl->done = 1;
    }
    ctrl->iter = it + 1;
  }
}

// <X, [[w; A]]> partials: sum over rows of (sum of MTTKRP split partials) * A.
template <typename T>
__global__ void k_inner_partial(const T* __restrict__ partial, int splits, int64_t n,
                                const T* __restrict__ A, double* ipart) {
  __shared__ double scratch[32];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double m = 0.0;
    for (int p = 0; p < splits; ++p) m += (double)partial[(int64_t)p * n + e];
    s = fma(m, (double)A[e], s);
  }
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) ipart[blockIdx.x] = s;
}

// Relative error of the current model without updating anything:
// sqrt(|nx2 + cp_norm^2 - 2 <X, rec>|) / sqrt(nx2) -> *out.
template <typename T>
__global__ void k_probe_error(const double* G, int ndim, int R, const T* w, const double* ipart,
                              int nip, const AlsCtrl* ctrl, double* out) {
  __shared__ double scratch[32];
  const int RR = R * R;
  double c = 0.0;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k) v = v * G[(int64_t)k * RR + e];
    if (w) v = v * ((double)w[r] * (double)w[s]);
    c += v;
  }
  c = block_sum(c, scratch);
  double ip = 0.0;
  for (int i = threadIdx.x; i < nip; i += blockDim.x) ip += ipart[i];
  ip = block_sum(ip, scratch);
  if (threadIdx.x == 0) {
    const double nx2 = ctrl->norm_x2;
    *out = sqrt(fabs(nx2 + c - 2.0 * ip)) / sqrt(nx2);
  }
}

// cp_norm (tensorly/cp_tensor.py:614-644): sqrt(sum(prod_k G_k * w w^T)).
template <typename T>
__global__ void k_cp_norm(const double* G, int ndim, int R, const T* w, double* out) {
  __shared__ double scratch[32];
  const int RR = R * R;
  double c = 0.0;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k) v = v * G[(int64_t)k * RR + e];
    if (w) v = v * ((double)w[r] * (double)w[s]);
    c += v;
  }
  c = block_sum(c, scratch);
  if (threadIdx.x == 0) *out = sqrt(c);
}

// ---------------------------------------------------------------- normalisation
template <typename T>
struct FactorPtrs {
  T* f[kMaxModes];
  int64_t rows[kMaxModes];
};

template <typename T>
__global__ void k_normalize(FactorPtrs<T> fp, int ndim, int R, T* weights, const int* done) {
  if (done && *done) return;
  __shared__ double scratch[32];
  const int r = blockIdx.x;
  T wacc = weights ? weights[r] : T(1);
  for (int k = 0; k < ndim; ++k) {
    T* f = fp.f[k];
    const int64_t I = fp.rows[k];
    if (k == 0) {
      for (int64_t i = threadIdx.x; i < I; i += blockDim.x) f[i * R + r] = f[i * R + r] * wacc;
      wacc = T(1);
      __syncthreads();
    }
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < I; i += blockDim.x) {
      const double x = (double)f[i * R + r];
      s = fma(x, x, s);
    }
    s = block_sum(s, scratch);
    const T scale = (T)sqrt(s);
    wacc = wacc * scale;
    const T div = (scale == T(0)) ? T(1) : scale;
    for (int64_t i = threadIdx.x; i < I; i += blockDim.x) f[i * R + r] = f[i * R + r] / div;
    __syncthreads();
  }
  if (threadIdx.x == 0 && weights) weights[r] = wacc;
}

}  // namespace

// ====================================================================== launchers
int solve_blocks_for(int64_t I) {
  const int64_t want = ceil_div(I, kSolveWarps);
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 2));
}

int als_launch_sumsq(int dtype, const void* X, int64_t n, double* part, int nblocks,
                     AlsCtrl* ctrl, cudaStream_t st) {
  if (dtype == TLGB_F32)
    k_sumsq<float><<<nblocks, 256, 0, st>>>((const float*)X, n, part);
  else
    k_sumsq<double><<<nblocks, 256, 0, st>>>((const double*)X, n, part);
  TLGB_LAUNCH_CHECK();
  k_sumsq_final<<<1, 256, 0, st>>>(part, nblocks, ctrl);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_gram(const T* A, int64_t I, int R, double* gpart, int nparts_max, double* G,
                    const int* done, cudaStream_t st) {
  int nparts = (int)std::min<int64_t>(nparts_max, std::max<int64_t>(1, ceil_div(I, 4)));
  const int64_t rpb = ceil_div(I, nparts);
  nparts = (int)ceil_div(I, rpb);
  const int threads = 256;
  const size_t smem = ((size_t)R * R + (size_t)kGramRows * R) * sizeof(double);
  static bool attr[64] = {};
  const int dev = current_device();
  if (dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(
        k_gram_partial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)(((size_t)kMaxAlsRank * kMaxAlsRank + kGramRows * kMaxAlsRank) * sizeof(double))));
    attr[dev] = true;
  }
  k_gram_partial<T><<<nparts, threads, smem, st>>>(A, I, R, rpb, gpart, done);
  TLGB_LAUNCH_CHECK();
  return als_launch_gram_reduce(gpart, nparts, R, G, done, st);
}

int als_launch_gram_reduce(const double* gpart, int nparts, int R, double* G, const int* done,
                           cudaStream_t st) {
  const int RR = R * R;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(RR, 128), sm_count()));
  k_gram_reduce<<<blocks, 128, 0, st>>>(gpart, nparts, RR, G, done);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_factorize(const double* G, int ndim, int mode, int R, const T* weights,
                         double l2_reg, double* fac, int* perm, AlsCtrl* ctrl, cudaStream_t st) {
  const size_t smem = (size_t)R * R * sizeof(double);
  static bool attr[64] = {};
  const int dev = current_device();
  if (dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_factorize<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)((size_t)kMaxAlsRank * kMaxAlsRank * sizeof(double))));
    attr[dev] = true;
  }
  k_factorize<T><<<1, 256, smem, st>>>(G, ndim, mode, R, weights, l2_reg, fac, perm, ctrl);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_solve(const T* partial, int splits, int64_t I, int R, const double* fac,
                     const int* perm, T* A, __nv_bfloat16* A_bt, double* gpart, double* ipart,
                     AlsCtrl* ctrl, int* nblocks, cudaStream_t st) {
  const int nb = solve_blocks_for(I);
  const int64_t rpb = ceil_div(I, nb);
  const int nbe = (int)ceil_div(I, rpb);
  const int fac_in_smem = R <= 96 ? 1 : 0;
  const size_t smem = ((size_t)R * R + (size_t)kSolveWarps * R +
                       (fac_in_smem ? (size_t)R * R + R : 0)) * sizeof(double);
  static bool attr[64] = {};
  const int dev = current_device();
  if (dev < 64 && !attr[dev]) {
    // the larger of the two layouts: R <= 96 with the factor in shared memory,
    // or R up to kMaxAlsRank without it
    const size_t with_fac = ((size_t)2 * 96 * 96 + (size_t)kSolveWarps * 96 + 96) * sizeof(double);
    const size_t without = ((size_t)kMaxAlsRank * kMaxAlsRank + (size_t)kSolveWarps * kMaxAlsRank) *
                           sizeof(double);
    const size_t maxs = with_fac > without ? with_fac : without;
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)maxs));
    attr[dev] = true;
  }
  k_solve<T><<<nbe, 32 * kSolveWarps, smem, st>>>(partial, splits, I, R, fac, perm, A, A_bt,
                                                  gpart, ipart, ctrl, rpb, fac_in_smem);
  TLGB_LAUNCH_CHECK();
  *nblocks = nbe;
  return TLGB_OK;
}

template <typename T>
int als_launch_fit(const double* G, int ndim, int R, const T* weights, const double* ipart,
                   int nip, AlsCtrl* ctrl, double* errors, int n_iter_max, double tol,
                   int cvg_criterion, cudaStream_t st) {
  k_fit<T><<<1, 256, 0, st>>>(G, ndim, R, weights, ipart, nip, ctrl, errors, n_iter_max, tol,
                              cvg_criterion);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_normalize(T* const* factors, const int64_t* rows, int ndim, int R, T* weights,
                         const int* done, cudaStream_t st) {
  FactorPtrs<T> fp{};
  for (int k = 0; k < ndim; ++k) { fp.f[k] = factors[k]; fp.rows[k] = rows[k]; }
  k_normalize<T><<<R, 256, 0, st>>>(fp, ndim, R, weights, done);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_cp_norm(const double* G, int ndim, int R, const T* weights, double* out,
                       cudaStream_t st) {
  k_cp_norm<T><<<1, 256, 0, st>>>(G, ndim, R, weights, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
template int als_launch_cp_norm<float>(const double*, int, int, const float*, double*, cudaStream_t);
template int als_launch_cp_norm<double>(const double*, int, int, const double*, double*,
                                        cudaStream_t);

template <typename T>
int als_launch_probe_error(const T* partial, int splits, int64_t I, int R, const T* A,
                           const double* G, int ndim, const T* weights, double* ipart,
                           int nip_max, const AlsCtrl* ctrl, double* out, cudaStream_t st) {
  const int64_t n = I * R;
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(nip_max, ceil_div(n, 256)));
  k_inner_partial<T><<<nb, 256, 0, st>>>(partial, splits, n, A, ipart);
  TLGB_LAUNCH_CHECK();
  k_probe_error<T><<<1, 256, 0, st>>>(G, ndim, R, weights, ipart, nb, ctrl, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
template int als_launch_probe_error<float>(const float*, int, int64_t, int, const float*,
                                           const double*, int, const float*, double*, int,
                                           const AlsCtrl*, double*, cudaStream_t);
template int als_launch_probe_error<double>(const double*, int, int64_t, int, const double*,
                                            const double*, int, const double*, double*, int,
                                            const AlsCtrl*, double*, cudaStream_t);

template <typename T>
static int als_prepare_typed() {
  static bool done[64] = {};
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && done[dev]) return TLGB_OK;
  TLGB_CUDA_TRY(cudaFuncSetAttribute(
      k_factorize<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)((size_t)kMaxAlsRank * kMaxAlsRank * sizeof(double))));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(
      k_gram_partial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)(((size_t)kMaxAlsRank * kMaxAlsRank + kGramRows * kMaxAlsRank) * sizeof(double))));
  const size_t with_fac = ((size_t)2 * 96 * 96 + (size_t)kSolveWarps * 96 + 96) * sizeof(double);
  const size_t without =
      ((size_t)kMaxAlsRank * kMaxAlsRank + (size_t)kSolveWarps * kMaxAlsRank) * sizeof(double);
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_solve<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(with_fac > without ? with_fac : without)));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return TLGB_OK;
}

int als_prepare(int dtype) {
  return dtype == TLGB_F64 ? als_prepare_typed<double>() : als_prepare_typed<float>();
}

#define TLGB_INST(T)                                                                          \
  template int als_launch_gram<T>(const T*, int64_t, int, double*, int, double*, const int*,  \
                                  cudaStream_t);                                             \
  template int als_launch_factorize<T>(const double*, int, int, int, const T*, double,       \
                                       double*, int*, AlsCtrl*, cudaStream_t);               \
  template int als_launch_solve<T>(const T*, int, int64_t, int, const double*, const int*,   \
                                   T*, __nv_bfloat16*, double*, double*, AlsCtrl*, int*,     \
                                   cudaStream_t);                                            \
  template int als_launch_fit<T>(const double*, int, int, const T*, const double*, int,      \
                                 AlsCtrl*, double*, int, double, int, cudaStream_t);         \
  template int als_launch_normalize<T>(T* const*, const int64_t*, int, int, T*, const int*,  \
                                       cudaStream_t);
TLGB_INST(float)
TLGB_INST(double)
#undef TLGB_INST

}  // namespace tlgb
