// Gram matrices of tensor unfoldings and the truncated SVD built on them
// (tensorly/tenalg/svd.py:366-447 svd_interface with method 'truncated_svd',
// :211-235 truncated_svd, :13-65 svd_flip).
//
// For M = unfold(X, mode) (I x J, never materialised):
//   I <= J: G = M M^T (I x I); U = top-k eigenvectors of G, S = sqrt(lambda);
//   I >  J: G = M^T M (J x J); V = top-k eigenvectors, S = sqrt(lambda),
//           U = M V S^-1.
// Then U's columns get the svd_flip signs (largest |entry| positive).  The
// reference's LAPACK SVD returns the same singular triplets (up to that sign)
// wherever the k-th singular value is separated from the (k+1)-th.
//
// Gram kernel: C = A A^T for a virtual matrix A whose element (a, k) sits at
// offset row(a) + col(k) of the tensor, each offset of the form
// (x / D) * S1 + (x % D) * S0.  64 x 64 output tiles (only tiles on or above
// the diagonal), the contraction split across CTAs; f32 tensors sum each
// 32-long chunk in f32 and the chunk sums with Neumaier compensation, f64
// tensors use f64 FMAs; the split partials (f64) are summed in a fixed order,
// so the result is deterministic.
#include "linalg.cuh"

namespace tlgb {
namespace {

constexpr int kGT = 64;        // Gram tile
constexpr int kGK = 32;        // contraction chunk
constexpr int kGThreads = 256;
constexpr int kGPad = kGT + 1;

struct GramArgs {
  int64_t Na, Nk;
  int64_t aD, aS1, aS0, kD, kS1, kS0;
  int nt, npairs;
  int64_t chunks, cps;
  double* partial;
};

__device__ __forceinline__ int64_t off2(int64_t x, int64_t D, int64_t S1, int64_t S0) {
  const int64_t q = x / D;
  return q * S1 + (x - q * D) * S0;
}

template <typename T>
__global__ void __launch_bounds__(kGThreads) k_gram_tiles(const T* __restrict__ X, const GramArgs g) {
  __shared__ T As[kGK * kGPad];
  __shared__ T Bs[kGK * kGPad];
  __shared__ int64_t offa[kGT], offb[kGT], offk[kGK];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  // pair index -> (ta, tb), ta <= tb, row-wise enumeration
  int p = blockIdx.x, ta = 0;
  while (p >= g.nt - ta) { p -= g.nt - ta; ++ta; }
  const int tb = ta + p;
  const bool diag = ta == tb;
  const int64_t a0 = (int64_t)ta * kGT, b0 = (int64_t)tb * kGT;
  if (tid < kGT) {
    const int64_t a = a0 + tid, b = b0 + tid;
    offa[tid] = (a < g.Na) ? off2(a, g.aD, g.aS1, g.aS0) : -1;
    offb[tid] = (b < g.Na) ? off2(b, g.aD, g.aS1, g.aS0) : -1;
  }
  const int64_t c_begin = (int64_t)blockIdx.y * g.cps;
  const int64_t c_end = min(c_begin + g.cps, g.chunks);
  double hi[4][4];             // f64 path: running totals
  float fh[4][4], fc[4][4];    // f32 path: Neumaier sum of the chunk sums (hi, compensation)
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { hi[i][j] = 0.0; fh[i][j] = 0.f; fc[i][j] = 0.f; }
  const int kk = tid & 31, rr = tid >> 5;   // loader: k fastest, 8 rows per pass
  for (int64_t c = c_begin; c < c_end; ++c) {
    const int64_t k0 = c * kGK;
    __syncthreads();
    if (tid < kGK) offk[tid] = (k0 + tid < g.Nk) ? off2(k0 + tid, g.kD, g.kS1, g.kS0) : -1;
    __syncthreads();
    const int64_t ok = offk[kk];
#pragma unroll
    for (int q = 0; q < kGT / 8; ++q) {
      const int r = rr + 8 * q;
      const int64_t oa = offa[r];
      As[kk * kGPad + r] = (oa >= 0 && ok >= 0) ? X[oa + ok] : T(0);
      if (!diag) {
        const int64_t ob = offb[r];
        Bs[kk * kGPad + r] = (ob >= 0 && ok >= 0) ? X[ob + ok] : T(0);
      }
    }
    __syncthreads();
    const T* Bsrc = diag ? As : Bs;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = T(0);
#pragma unroll 8
    for (int k = 0; k < kGK; ++k) {
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[k * kGPad + ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bsrc[k * kGPad + tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    if constexpr (sizeof(T) == 4) {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float v = (float)acc[i][j];
          const float t = fh[i][j] + v;
          fc[i][j] += (fabsf(fh[i][j]) >= fabsf(v)) ? ((fh[i][j] - t) + v) : ((v - t) + fh[i][j]);
          fh[i][j] = t;
        }
    } else {
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) hi[i][j] += (double)acc[i][j];
    }
  }
  double* out = g.partial + ((int64_t)blockIdx.y * g.npairs + blockIdx.x) * (kGT * kGT);
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const double v = (sizeof(T) == 4) ? (double)fh[i][j] + (double)fc[i][j] : hi[i][j];
      out[(ty + 16 * i) * kGT + tx + 16 * j] = v;
    }
}

// f32 Gram tiles, tuned: 128 threads, each owning an 8 x 4 block of the
// 64 x 64 tile (rows 8 ty.., columns 4 tx..), read from shared memory as
// 16-byte vectors (three loads per 32 FMAs); the next chunk's tensor elements
// are fetched into registers while the current chunk is multiplied.  Same
// chunking and Neumaier compensation as k_gram_tiles, so the same accuracy.
constexpr int kGT2Threads = 128;
constexpr int kGPad4 = kGT + 4;   // 16-byte aligned rows of the k-major tiles
constexpr int kGLoads = kGK * kGT / kGT2Threads;   // 16 elements per thread per operand

__global__ void __launch_bounds__(kGT2Threads)
k_gram_tiles_f32(const float* __restrict__ X, const GramArgs g) {
  __shared__ __align__(16) float As[kGK * kGPad4];
  __shared__ __align__(16) float Bs[kGK * kGPad4];
  __shared__ int64_t offa[kGT], offb[kGT];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;   // ty 0..7, tx 0..15
  int p = blockIdx.x, ta = 0;
  while (p >= g.nt - ta) { p -= g.nt - ta; ++ta; }
  const int tb = ta + p;
  const bool diag = ta == tb;
  const int64_t a0 = (int64_t)ta * kGT, b0 = (int64_t)tb * kGT;
  if (tid < kGT) {
    const int64_t a = a0 + tid, b = b0 + tid;
    offa[tid] = (a < g.Na) ? off2(a, g.aD, g.aS1, g.aS0) : -1;
    offb[tid] = (b < g.Na) ? off2(b, g.aD, g.aS1, g.aS0) : -1;
  }
  __syncthreads();
  const int64_t c_begin = (int64_t)blockIdx.y * g.cps;
  const int64_t c_end = min(c_begin + g.cps, g.chunks);
  // loader: k = tid & 31 (fastest, coalesced), rows (tid >> 5) + 4 q
  const int kk = tid & 31, rr = tid >> 5;
  float ra[kGLoads], rb[kGLoads];
  auto fetch = [&](int64_t c) {
    const int64_t k = c * kGK + kk;
    const int64_t ok = (k < g.Nk) ? off2(k, g.kD, g.kS1, g.kS0) : -1;
#pragma unroll
    for (int q = 0; q < kGLoads; ++q) {
      const int r = rr + 4 * q;
      const int64_t oa = offa[r];
      ra[q] = (oa >= 0 && ok >= 0) ? __ldg(X + oa + ok) : 0.f;
      if (!diag) {
        const int64_t ob = offb[r];
        rb[q] = (ob >= 0 && ok >= 0) ? __ldg(X + ob + ok) : 0.f;
      }
    }
  };
  float fh[8][4], fc[8][4];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) { fh[i][j] = 0.f; fc[i][j] = 0.f; }
  if (c_begin < c_end) fetch(c_begin);
  for (int64_t c = c_begin; c < c_end; ++c) {
    __syncthreads();   // the previous chunk's tiles have been read
#pragma unroll
    for (int q = 0; q < kGLoads; ++q) {
      As[kk * kGPad4 + rr + 4 * q] = ra[q];
      if (!diag) Bs[kk * kGPad4 + rr + 4 * q] = rb[q];
    }
    __syncthreads();
    if (c + 1 < c_end) fetch(c + 1);
    const float* Bsrc = diag ? As : Bs;
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
#pragma unroll 4
    for (int k = 0; k < kGK; ++k) {
      const float4 a_lo = *reinterpret_cast<const float4*>(As + k * kGPad4 + 8 * ty);
      const float4 a_hi = *reinterpret_cast<const float4*>(As + k * kGPad4 + 8 * ty + 4);
      const float4 bq = *reinterpret_cast<const float4*>(Bsrc + k * kGPad4 + 4 * tx);
      const float av[8] = {a_lo.x, a_lo.y, a_lo.z, a_lo.w, a_hi.x, a_hi.y, a_hi.z, a_hi.w};
      const float bv[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float v = acc[i][j];
        const float t = fh[i][j] + v;
        fc[i][j] += (fabsf(fh[i][j]) >= fabsf(v)) ? ((fh[i][j] - t) + v) : ((v - t) + fh[i][j]);
        fh[i][j] = t;
      }
  }
  double* out = g.partial + ((int64_t)blockIdx.y * g.npairs + blockIdx.x) * (kGT * kGT);
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
      out[(8 * ty + i) * kGT + 4 * tx + j] = (double)fh[i][j] + (double)fc[i][j];
}

// G[a][b] = G[b][a] = sum over splits of the partial tiles, in split order.
template <typename T>
__global__ void k_gram_finish(const double* __restrict__ partial, int64_t Na, int nt, int npairs,
                              int splits, T* G) {
  // one thread per tile element: grid (elements / blockDim, tile pairs)
  const int p0 = blockIdx.y;
  int p = p0, ta = 0;
  while (p >= nt - ta) { p -= nt - ta; ++ta; }
  const int tb = ta + p;
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= kGT * kGT) return;
  const int i = e / kGT, j = e % kGT;
  const int64_t a = (int64_t)ta * kGT + i, b = (int64_t)tb * kGT + j;
  if (a >= Na || b >= Na) return;
  // the split order of the sum is fixed, so the result is deterministic
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int q = 0;
  for (; q + 3 < splits; q += 4) {
    s0 += partial[((int64_t)q * npairs + p0) * (kGT * kGT) + e];
    s1 += partial[((int64_t)(q + 1) * npairs + p0) * (kGT * kGT) + e];
    s2 += partial[((int64_t)(q + 2) * npairs + p0) * (kGT * kGT) + e];
    s3 += partial[((int64_t)(q + 3) * npairs + p0) * (kGT * kGT) + e];
  }
  for (; q < splits; ++q) s0 += partial[((int64_t)q * npairs + p0) * (kGT * kGT) + e];
  const double s = (s0 + s1) + (s2 + s3);
  G[a * Na + b] = (T)s;
  G[b * Na + a] = (T)s;
}

// U[i][c] = (sum_j M[i][j] V[j][c]) / S[c]  (M = unfold(X, mode), tall case)
template <typename T>
__global__ void k_unfold_times(const T* __restrict__ X, int64_t I, int64_t J, int64_t L,
                               int64_t Tt, const T* __restrict__ V, const T* __restrict__ S,
                               int k, T* U) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= I * k) return;
  const int64_t i = idx / k;
  const int c = (int)(idx - i * k);
  double acc = 0.0;
  for (int64_t j = 0; j < J; ++j) {
    const int64_t l = j / Tt, t = j - (j / Tt) * Tt;
    acc += (double)X[(l * I + i) * Tt + t] * (double)V[j * k + c];
  }
  const double s = (double)S[c];
  U[i * k + c] = (s > 0.0) ? (T)(acc / s) : T(0);
}

// svd_flip signs on the columns of U (I x k): one warp per column.
template <typename T>
__global__ void k_flip_columns(T* U, int64_t I, int k) {
  const int lane = threadIdx.x & 31;
  const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (c >= k) return;
  T best = T(-1);
  int64_t bi = I;
  for (int64_t i = lane; i < I; i += 32) {
    const T a = fabs(U[i * k + c]);
    if (a > best) { best = a; bi = i; }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T ob = __shfl_xor_sync(0xffffffffu, best, o);
    const int64_t oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
  }
  if (U[bi * k + c] < T(0))
    for (int64_t i = lane; i < I; i += 32) U[i * k + c] = -U[i * k + c];
}

template <typename T>
__global__ void k_sqrt_clamp(T* v, int k) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < k) v[i] = v[i] > T(0) ? sqrt(v[i]) : T(0);
}

}  // namespace

int gram_make_plan(const Shape& sh, int mode, int side, GramPlan* out) {
  TLGB_CHECK_ARG(mode >= 0 && mode < sh.ndim, "gram: mode out of range");
  GramPlan p{};
  int64_t L = 1, Tt = 1;
  for (int k = 0; k < mode; ++k) L *= sh.dim[k];
  for (int k = mode + 1; k < sh.ndim; ++k) Tt *= sh.dim[k];
  const int64_t I = sh.dim[mode];
  if (side == 0) {   // rows = i, columns = (l, t)
    p.Na = I;          p.aD = I;  p.aS1 = 0;      p.aS0 = Tt;
    p.Nk = L * Tt;     p.kD = Tt; p.kS1 = I * Tt; p.kS0 = 1;
  } else {           // rows = (l, t), columns = i
    p.Na = L * Tt;     p.aD = Tt; p.aS1 = I * Tt; p.aS0 = 1;
    p.Nk = I;          p.kD = I;  p.kS1 = 0;      p.kS0 = Tt;
  }
  p.nt = (int)ceil_div(p.Na, kGT);
  p.npairs = p.nt * (p.nt + 1) / 2;
  p.chunks = ceil_div(p.Nk, kGK);
  int64_t splits = std::max<int64_t>(1, ceil_div(2 * (int64_t)sm_count(), p.npairs));
  splits = std::min<int64_t>(splits, std::max<int64_t>(1, p.chunks / 2));
  splits = std::min<int64_t>(splits, 65535);
  p.cps = ceil_div(p.chunks, splits);
  p.splits = (int)ceil_div(p.chunks, p.cps);
  p.partial_bytes = (size_t)p.splits * p.npairs * kGT * kGT * sizeof(double);
  *out = p;
  return TLGB_OK;
}

template <typename T>
int gram_launch(const GramPlan& p, const T* X, T* G, double* partial, cudaStream_t st) {
  GramArgs g{};
  g.Na = p.Na; g.Nk = p.Nk;
  g.aD = p.aD; g.aS1 = p.aS1; g.aS0 = p.aS0;
  g.kD = p.kD; g.kS1 = p.kS1; g.kS0 = p.kS0;
  g.nt = p.nt; g.npairs = p.npairs; g.chunks = p.chunks; g.cps = p.cps;
  g.partial = partial;
  TLGB_CHECK_ARG(p.npairs <= 2147483647, "gram: too many tiles");
  if constexpr (sizeof(T) == 4)
    k_gram_tiles_f32<<<dim3((unsigned)p.npairs, (unsigned)p.splits), kGT2Threads, 0, st>>>(
        reinterpret_cast<const float*>(X), g);
  else
    k_gram_tiles<T><<<dim3((unsigned)p.npairs, (unsigned)p.splits), kGThreads, 0, st>>>(X, g);
  TLGB_LAUNCH_CHECK();
  TLGB_CHECK_ARG(p.npairs <= 65535, "gram: too many tile pairs for the finish grid");
  k_gram_finish<T><<<dim3((kGT * kGT + 255) / 256, (unsigned)p.npairs), 256, 0, st>>>(
      partial, p.Na, p.nt, p.npairs, p.splits, G);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template int gram_launch<float>(const GramPlan&, const float*, float*, double*, cudaStream_t);
template int gram_launch<double>(const GramPlan&, const double*, double*, double*, cudaStream_t);

namespace {
struct SvdLayout {
  GramPlan gp;
  int64_t I, J, n;     // unfolding rows / columns, Gram order
  bool tall;
  size_t g_off, part_off, eig_off, v_off, lam_off, bytes;
};

int svd_layout(int dtype, const Shape& sh, int mode, int64_t k, SvdLayout* L) {
  const size_t es = dtype == TLGB_F64 ? 8 : 4;
  L->I = sh.dim[mode];
  L->J = sh.numel / std::max<int64_t>(1, L->I);
  L->tall = L->I > L->J;
  L->n = L->tall ? L->J : L->I;
  TLGB_CHECK_ARG(k >= 1, "svd: n_eigenvecs must be >= 1");
  if (k > L->n)
    return set_error(TLGB_EUNSUPPORTED,
                     "svd: n_eigenvecs above min(unfolding shape) (full_matrices SVD) is not "
                     "supported");
  if (L->n > sym_eig_max_n(dtype))
    return set_error(TLGB_EUNSUPPORTED, "svd: the Gram matrix of this unfolding has order " +
                                            std::to_string(L->n) + ", above the eigensolver's " +
                                            std::to_string(sym_eig_max_n(dtype)));
  int rc = gram_make_plan(sh, mode, L->tall ? 1 : 0, &L->gp);
  if (rc) return rc;
  size_t off = 0;
  auto take = [&](size_t bytes) { off = align_up(off, 256); const size_t o = off; off += bytes; return o; };
  L->g_off = take((size_t)L->n * L->n * es);
  L->part_off = take(L->gp.partial_bytes);
  L->eig_off = take(sym_eig_workspace(dtype, L->n, k));
  L->v_off = take((size_t)L->n * k * es);
  L->lam_off = take((size_t)k * es);
  L->bytes = align_up(off, 256);
  return TLGB_OK;
}
}  // namespace

size_t svd_unfolding_workspace(int dtype, const Shape& sh, int mode, int64_t k) {
  SvdLayout L;
  if (svd_layout(dtype, sh, mode, k, &L)) return 0;
  return L.bytes;
}

template <typename T>
int svd_unfolding_launch(const T* X, const Shape& sh, int mode, int k, T* U, T* S, int flip,
                         void* ws, size_t ws_bytes, cudaStream_t st, cudaEvent_t input_done) {
  SvdLayout L;
  int rc = svd_layout(TypeCode<T>::value, sh, mode, k, &L);
  if (rc) return rc;
  if (!ws || ws_bytes < L.bytes) return set_error(TLGB_EWORKSPACE, "svd: workspace too small");
  char* base = static_cast<char*>(ws);
  T* G = reinterpret_cast<T*>(base + L.g_off);
  double* part = reinterpret_cast<double*>(base + L.part_off);
  void* eigws = base + L.eig_off;
  T* V = reinterpret_cast<T*>(base + L.v_off);
  rc = gram_launch<T>(L.gp, X, G, part, st);
  if (rc) return rc;
  if (!L.tall) {
    if (input_done) TLGB_CUDA_TRY(cudaEventRecord(input_done, st));   // X is not read again
    rc = sym_eig_launch<T>(G, (int)L.n, k, U, S, flip, eigws, st);
    if (rc) return rc;
    k_sqrt_clamp<T><<<(k + 255) / 256, 256, 0, st>>>(S, k);
    TLGB_LAUNCH_CHECK();
    return TLGB_OK;
  }
  rc = sym_eig_launch<T>(G, (int)L.n, k, V, S, 0, eigws, st);
  if (rc) return rc;
  k_sqrt_clamp<T><<<(k + 255) / 256, 256, 0, st>>>(S, k);
  TLGB_LAUNCH_CHECK();
  int64_t Lb = 1, Tt = 1;
  for (int q = 0; q < mode; ++q) Lb *= sh.dim[q];
  for (int q = mode + 1; q < sh.ndim; ++q) Tt *= sh.dim[q];
  const int64_t tot = L.I * k;
  k_unfold_times<T><<<(unsigned)ceil_div(tot, 256), 256, 0, st>>>(X, L.I, L.J, Lb, Tt, V, S, k, U);
  TLGB_LAUNCH_CHECK();
  if (input_done) TLGB_CUDA_TRY(cudaEventRecord(input_done, st));
  if (flip) {
    k_flip_columns<T><<<(unsigned)ceil_div(k, 8), 256, 0, st>>>(U, L.I, k);
    TLGB_LAUNCH_CHECK();
  }
  return TLGB_OK;
}

template int svd_unfolding_launch<float>(const float*, const Shape&, int, int, float*, float*, int,
                                         void*, size_t, cudaStream_t, cudaEvent_t);
template int svd_unfolding_launch<double>(const double*, const Shape&, int, int, double*, double*,
                                          int, void*, size_t, cudaStream_t, cudaEvent_t);

}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_gram_unfolding_workspace_size(int ndim, const int64_t* shape, int mode,
                                                  int side, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(shape && bytes, "gram_unfolding_workspace_size: null pointer");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "gram: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(side == 0 || side == 1, "gram: side must be 0 or 1");
  GramPlan p;
  int rc = gram_make_plan(make_shape(ndim, shape), mode, side, &p);
  if (rc) return rc;
  *bytes = align_up(p.partial_bytes, 256);
  return TLGB_OK;
}

extern "C" int tlgb_gram_unfolding(int dtype, const void* X, int ndim, const int64_t* shape,
                                   int mode, int side, void* G, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "gram: dtype must be f32 or f64");
  TLGB_CHECK_ARG(X && shape && G, "gram: null pointer");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "gram: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(side == 0 || side == 1, "gram: side must be 0 or 1");
  Shape sh = make_shape(ndim, shape);
  GramPlan p;
  int rc = gram_make_plan(sh, mode, side, &p);
  if (rc) return rc;
  if (!workspace || workspace_bytes < p.partial_bytes)
    return set_error(TLGB_EWORKSPACE, "gram: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    return gram_launch<float>(p, (const float*)X, (float*)G, (double*)workspace, st);
  return gram_launch<double>(p, (const double*)X, (double*)G, (double*)workspace, st);
}

extern "C" int tlgb_svd_unfolding_workspace_size(int dtype, int ndim, const int64_t* shape,
                                                 int mode, int64_t k, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(shape && bytes, "svd_unfolding_workspace_size: null pointer");
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "svd: dtype must be f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "svd: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(mode >= 0 && mode < ndim, "svd: mode out of range");
  SvdLayout L;
  int rc = svd_layout(dtype, make_shape(ndim, shape), mode, k, &L);
  if (rc) return rc;
  *bytes = L.bytes;
  return TLGB_OK;
}

extern "C" int tlgb_svd_unfolding(int dtype, const void* X, int ndim, const int64_t* shape,
                                  int mode, int64_t k, void* U, void* S, int flip_sign,
                                  void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "svd: dtype must be f32 or f64");
  TLGB_CHECK_ARG(X && shape && U && S, "svd: null pointer");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "svd: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(mode >= 0 && mode < ndim, "svd: mode out of range");
  Shape sh = make_shape(ndim, shape);
  TLGB_CHECK_ARG(sh.numel >= 1, "svd: empty tensor");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    return svd_unfolding_launch<float>((const float*)X, sh, mode, (int)k, (float*)U, (float*)S,
                                       flip_sign, workspace, workspace_bytes, st);
  return svd_unfolding_launch<double>((const double*)X, sh, mode, (int)k, (double*)U, (double*)S,
                                      flip_sign, workspace, workspace_bytes, st);
}
