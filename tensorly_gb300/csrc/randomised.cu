// Randomised CP-ALS (tensorly/decomposition/_cp.py:546-762): per mode, the
// least-squares update from n_samples sampled rows of the Khatri-Rao product,
//   KR_s[s, r] = prod_{k != mode} A_k[idx_k[s], r]       (sample_khatri_rao)
//   X_s[s, i]  = X[idx_0[s], .., i (at mode), .., idx_{N-1}[s]]
//   A_mode     = solve(KR_s^T KR_s, KR_s^T X_s)^T = (X_s^T KR_s) (KR_s^T KR_s)^-1
// and after each iteration ||X - [[A]]|| by the fused reconstruction kernel
// in its residual form (the full tensor is never written).  The sample
// indices come from the caller: the reference draws them with NumPy's
// RandomState on the host, mode by mode, and the host mirror does the same.
// The normal equations go through the CP-ALS factorisation and solve
// kernels with the sampled Gram in place of the Hadamard of Grams.
#include "als_kernels.cuh"
#include "reconstruct.cuh"

namespace tlgb {
namespace {

struct SampleArgs {
  const void* mats[kMaxModes];   // the factors sampled (the others than `mode`), in order
  const int64_t* idx[kMaxModes]; // their n_samples row indices (device)
  int64_t rows[kMaxModes];
  int64_t stride[kMaxModes];     // X strides of those modes (unfolding gather)
  int n;
};

// kr[s, r]: the reference starts from ones and multiplies one sampled matrix
// at a time (1 * a = a exactly).  Out-of-range indices read row 0 and set
// *bad (when given).
template <typename T>
__global__ void k_sample_kr(const SampleArgs a, int64_t ns, int R, T* __restrict__ kr, int* bad) {
  const int64_t total = ns * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / R;
    const int r = (int)(e - s * R);
    T v = (T)1;
    for (int k = 0; k < a.n; ++k) {
      int64_t i = a.idx[k][s];
      if (i < 0 || i >= a.rows[k]) {
        if (bad) *bad = 1;
        i = 0;
      }
      v = v * static_cast<const T*>(a.mats[k])[i * R + r];
    }
    kr[e] = v;
  }
}

// xs[s, i] = X at the sampled position of the other modes and i at `mode`.
template <typename T>
__global__ void k_sample_unfolding(const T* __restrict__ X, const SampleArgs a, int64_t ns,
                                   int64_t I, int64_t stride_mode, T* __restrict__ xs, int* bad) {
  const int64_t total = ns * I;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = e / I;
    const int64_t i = e - s * I;
    int64_t off = i * stride_mode;
    for (int k = 0; k < a.n; ++k) {
      int64_t j = a.idx[k][s];
      if (j < 0 || j >= a.rows[k]) {
        *bad = 1;
        j = 0;
      }
      off += j * a.stride[k];
    }
    xs[e] = X[off];
  }
}

// C_p[m, n] = sum over the samples s of split p of A[s, m] B[s, n]
// (A: ns x M, B: ns x N, row-major), in the factor type, one partial plane
// per split: 64 x 64 output tiles, 16 samples a step staged in shared
// memory, 4 x 4 outputs a thread.  With A = X_s, B = KR_s the planes are
// the split partials of M = X_s^T KR_s that the solve sums; with A = B = KR_s
// they are those of the sampled Gram.
constexpr int kAtbTile = 64, kAtbStep = 16;

template <typename T>
__global__ void __launch_bounds__(256)
k_atb_split(const T* __restrict__ A, int64_t M, const T* __restrict__ B, int64_t N, int64_t ns,
            int64_t per_split, T* __restrict__ C) {
  __shared__ T As[kAtbStep][kAtbTile];
  __shared__ T Bs[kAtbStep][kAtbTile];
  const int tid = threadIdx.x, tm = tid >> 4, tn = tid & 15;
  const int64_t m0 = (int64_t)blockIdx.x * kAtbTile, n0 = (int64_t)blockIdx.y * kAtbTile;
  const int64_t s_begin = (int64_t)blockIdx.z * per_split;
  const int64_t s_end = s_begin + per_split < ns ? s_begin + per_split : ns;
  T acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = (T)0;
  for (int64_t s0 = s_begin; s0 < s_end; s0 += kAtbStep) {
    for (int e = tid; e < kAtbStep * kAtbTile; e += 256) {
      const int ss = e / kAtbTile, c = e - ss * kAtbTile;
      const int64_t s = s0 + ss;
      As[ss][c] = (s < s_end && m0 + c < M) ? A[s * M + m0 + c] : (T)0;
      Bs[ss][c] = (s < s_end && n0 + c < N) ? B[s * N + n0 + c] : (T)0;
    }
    __syncthreads();
#pragma unroll
    for (int ss = 0; ss < kAtbStep; ++ss) {
      T av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[ss][tm + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[ss][tn + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
  T* Cp = C + (int64_t)blockIdx.z * M * N;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t m = m0 + tm + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t n = n0 + tn + 16 * j;
      if (n < N) Cp[m * N + n] = acc[i][j];
    }
  }
}

// G[e] = sum_p parts[p][e] in split order, as f64 for the factorisation.
template <typename T>
__global__ void k_sum_parts(const T* __restrict__ parts, int splits, int n, double* G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double s = 0.0;
  for (int p = 0; p < splits; ++p) s += (double)parts[(int64_t)p * n + e];
  G[e] = s;
}

// Sample splits: about 2 waves of 256-thread CTAs over the larger product.
int atb_splits(int64_t ns, int64_t M, int64_t N) {
  const int64_t tiles = ceil_div(M, (int64_t)kAtbTile) * ceil_div(N, (int64_t)kAtbTile);
  const int64_t want = std::max<int64_t>(1, ceil_div((int64_t)152 * 6, tiles));
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, ceil_div(ns, (int64_t)(4 * kAtbStep))));
}

struct RandLayout {
  size_t ctrl, G, fac, perm, vmat, w32, gpart, kr, xs, M, Vp, resid, bad, rec, bytes;
};

RandLayout rand_layout(int dtype, int ndim, const int64_t* shape, int64_t R, int64_t ns) {
  RandLayout L{};
  const size_t esz = dtype == TLGB_F64 ? 8 : 4;
  int64_t imax = 0;
  for (int k = 0; k < ndim; ++k) imax = std::max(imax, shape[k]);
  size_t off = 0;
  auto take = [&](size_t b) { off = align_up(off, 256); const size_t o = off; off += b; return o; };
  const size_t RR = (size_t)R * R;
  L.ctrl = take(sizeof(AlsCtrl));
  L.G = take(sizeof(double) * 2 * RR);
  L.fac = take(sizeof(double) * (RR + R));
  L.perm = take(sizeof(int) * R);
  L.vmat = take(sizeof(double) * RR);
  L.w32 = take(sizeof(float) * 3 * RR);
  L.gpart = take(sizeof(double) * RR * (size_t)solve_blocks_for(imax));
  L.kr = take(esz * (size_t)ns * R);
  L.xs = take(esz * (size_t)ns * imax);
  size_t mparts = 0;                     // the largest split-partial set over the modes
  for (int k = 0; k < ndim; ++k)
    mparts = std::max(mparts, (size_t)shape[k] * R * atb_splits(ns, shape[k], R));
  L.M = take(esz * mparts);
  L.Vp = take(esz * (size_t)R * R * atb_splits(ns, R, R));
  L.resid = take(sizeof(double));
  L.bad = take(sizeof(int));
  L.rec = take(cp_full_ws_bytes(dtype, ndim, shape, R));
  L.bytes = align_up(off, 256);
  return L;
}

int rand_check(int dtype, int ndim, const int64_t* shape, int64_t rank, int64_t ns) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "randomised_parafac: dtype f32 or f64");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "randomised_parafac: ndim must be in [2, 8]");
  TLGB_CHECK_ARG(shape != nullptr, "randomised_parafac: null shape");
  TLGB_CHECK_ARG(rank >= 1 && rank <= kMaxAlsRank, "randomised_parafac: rank must be in [1, 160]");
  TLGB_CHECK_ARG(ns >= 1, "randomised_parafac: n_samples must be >= 1");
  for (int k = 0; k < ndim; ++k)
    TLGB_CHECK_ARG(shape[k] >= 1 && shape[k] <= INT32_MAX, "randomised_parafac: bad mode size");
  return TLGB_OK;
}

template <typename T>
int rand_enqueue(const T* X, int ndim, const int64_t* shape, int64_t R, T* const* factors,
                 int64_t ns, const int64_t* indices, void* ws, cudaStream_t st) {
  const int dtype = TypeCode<T>::value;
  const RandLayout L = rand_layout(dtype, ndim, shape, R, ns);
  char* base = static_cast<char*>(ws);
  AlsCtrl* ctrl = reinterpret_cast<AlsCtrl*>(base + L.ctrl);
  double* G = reinterpret_cast<double*>(base + L.G);
  double* fac = reinterpret_cast<double*>(base + L.fac);
  int* perm = reinterpret_cast<int*>(base + L.perm);
  double* vmat = reinterpret_cast<double*>(base + L.vmat);
  float* w32 = reinterpret_cast<float*>(base + L.w32);
  double* gpart = reinterpret_cast<double*>(base + L.gpart);
  T* kr = reinterpret_cast<T*>(base + L.kr);
  T* xs = reinterpret_cast<T*>(base + L.xs);
  T* M = reinterpret_cast<T*>(base + L.M);
  double* resid = reinterpret_cast<double*>(base + L.resid);
  int* bad = reinterpret_cast<int*>(base + L.bad);
  int64_t stride[kMaxModes];
  stride[ndim - 1] = 1;
  for (int k = ndim - 2; k >= 0; --k) stride[k] = stride[k + 1] * shape[k + 1];
  TLGB_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(AlsCtrl), st));
  TLGB_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), st));
  const int RR = (int)(R * R);
  for (int mode = 0; mode < ndim; ++mode) {
    SampleArgs a{};
    a.n = ndim - 1;
    for (int k = 0, q = 0; k < ndim; ++k) {
      if (k == mode) continue;
      a.mats[q] = factors[k];
      a.idx[q] = indices + ((int64_t)mode * (ndim - 1) + q) * ns;
      a.rows[q] = shape[k];
      a.stride[q] = stride[k];
      ++q;
    }
    const int64_t I = shape[mode];
    const unsigned bk = (unsigned)std::min<int64_t>(ceil_div(ns * R, (int64_t)256), 152 * 8);
    k_sample_kr<T><<<bk, 256, 0, st>>>(a, ns, (int)R, kr, bad);
    TLGB_LAUNCH_CHECK();
    const unsigned bx = (unsigned)std::min<int64_t>(ceil_div(ns * I, (int64_t)256), 152 * 8);
    k_sample_unfolding<T><<<bx, 256, 0, st>>>(X, a, ns, I, stride[mode], xs, bad);
    TLGB_LAUNCH_CHECK();
    // G slot 1 holds the sampled Gram: the factorisation of mode 0 of a
    // 2-mode problem uses exactly that matrix
    T* Vp = reinterpret_cast<T*>(base + L.Vp);
    const int sv = atb_splits(ns, R, R);
    {
      dim3 g((unsigned)ceil_div(R, (int64_t)kAtbTile), (unsigned)ceil_div(R, (int64_t)kAtbTile),
             (unsigned)sv);
      k_atb_split<T><<<g, 256, 0, st>>>(kr, R, kr, R, ns, ceil_div(ns, (int64_t)sv), Vp);
      TLGB_LAUNCH_CHECK();
      k_sum_parts<T><<<(RR + 255) / 256, 256, 0, st>>>(Vp, sv, RR, G + RR);
      TLGB_LAUNCH_CHECK();
    }
    const int sm = atb_splits(ns, I, R);
    {
      dim3 g((unsigned)ceil_div(I, (int64_t)kAtbTile), (unsigned)ceil_div(R, (int64_t)kAtbTile),
             (unsigned)sm);
      k_atb_split<T><<<g, 256, 0, st>>>(xs, I, kr, R, ns, ceil_div(ns, (int64_t)sm), M);
      TLGB_LAUNCH_CHECK();
    }
    int rc = als_launch_factorize<T>(G, 2, 0, (int)R, nullptr, 0.0, fac, perm, vmat, w32, ctrl,
                                     st);
    if (rc) return rc;
    int nb = 0;
    rc = als_launch_solve<T>(M, sm, I, (int)R, fac, perm, vmat, w32, factors[mode], nullptr, gpart,
                             nullptr, ctrl, kIrMaxPasses, &nb, st);
    if (rc) return rc;
  }
  const void* fp[kMaxModes];
  for (int k = 0; k < ndim; ++k) fp[k] = factors[k];
  return cp_full_run(dtype, ndim, shape, R, fp, nullptr, nullptr, nullptr, X, resid,
                     base + L.rec, cp_full_ws_bytes(dtype, ndim, shape, R), st);
}

// Waits for an enqueued iteration; its checks and the residual norm.
int rand_finish(int dtype, int ndim, const int64_t* shape, int64_t R, int64_t ns,
                double* rec_error, void* ws, cudaStream_t st) {
  const RandLayout L = rand_layout(dtype, ndim, shape, R, ns);
  char* base = static_cast<char*>(ws);
  const AlsCtrl* ctrl = reinterpret_cast<const AlsCtrl*>(base + L.ctrl);
  const double* resid = reinterpret_cast<const double*>(base + L.resid);
  const int* bad = reinterpret_cast<const int*>(base + L.bad);
  struct { double resid; int bad; AlsCtrl ctrl; } h{};
  TLGB_CUDA_TRY(cudaMemcpyAsync(&h.resid, resid, sizeof(double), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaMemcpyAsync(&h.bad, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaMemcpyAsync(&h.ctrl, ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (h.bad) return set_error(TLGB_EINVAL, "randomised_parafac: sample index out of range");
  if (h.ctrl.status == TLGB_ESINGULAR)
    return set_error(TLGB_ESINGULAR, "randomised_parafac: sampled normal equations singular");
  if (rec_error) *rec_error = h.resid;
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_cp_randomised_workspace_size(int dtype, int ndim, const int64_t* shape,
                                                 int64_t rank, int64_t n_samples,
                                                 size_t* bytes) {
  clear_error();
  int rc = rand_check(dtype, ndim, shape, rank, n_samples);
  if (rc) return rc;
  TLGB_CHECK_ARG(bytes != nullptr, "randomised_parafac: null bytes");
  *bytes = rand_layout(dtype, ndim, shape, rank, n_samples).bytes;
  return TLGB_OK;
}

extern "C" int tlgb_cp_randomised_launch(int dtype, const void* X, int ndim,
                                         const int64_t* shape, int64_t rank,
                                         void* const* factors, int64_t n_samples,
                                         const int64_t* indices, void* workspace,
                                         size_t workspace_bytes, void* stream) {
  clear_error();
  int rc = rand_check(dtype, ndim, shape, rank, n_samples);
  if (rc) return rc;
  TLGB_CHECK_ARG(X && factors && indices, "randomised_parafac: null pointer");
  for (int k = 0; k < ndim; ++k)
    TLGB_CHECK_ARG(factors[k] != nullptr, "randomised_parafac: null factor");
  if (!workspace || workspace_bytes < rand_layout(dtype, ndim, shape, rank, n_samples).bytes)
    return set_error(TLGB_EWORKSPACE, "randomised_parafac: workspace too small");
  rc = als_prepare(dtype);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return rand_enqueue<double>(static_cast<const double*>(X), ndim, shape, rank,
                                reinterpret_cast<double* const*>(factors), n_samples, indices,
                                workspace, st);
  return rand_enqueue<float>(static_cast<const float*>(X), ndim, shape, rank,
                             reinterpret_cast<float* const*>(factors), n_samples, indices,
                             workspace, st);
}

extern "C" int tlgb_cp_randomised_iteration(int dtype, const void* X, int ndim,
                                            const int64_t* shape, int64_t rank,
                                            void* const* factors, int64_t n_samples,
                                            const int64_t* indices, double* rec_error,
                                            void* workspace, size_t workspace_bytes,
                                            void* stream) {
  int rc = tlgb_cp_randomised_launch(dtype, X, ndim, shape, rank, factors, n_samples, indices,
                                     workspace, workspace_bytes, stream);
  if (rc) return rc;
  return rand_finish(dtype, ndim, shape, rank, n_samples, rec_error, workspace,
                     static_cast<cudaStream_t>(stream));
}

extern "C" int tlgb_cp_randomised_finish(int dtype, int ndim, const int64_t* shape,
                                         int64_t rank, int64_t n_samples, void* workspace,
                                         size_t workspace_bytes, double* rec_error,
                                         void* stream) {
  clear_error();
  int rc = rand_check(dtype, ndim, shape, rank, n_samples);
  if (rc) return rc;
  if (!workspace || workspace_bytes < rand_layout(dtype, ndim, shape, rank, n_samples).bytes)
    return set_error(TLGB_EWORKSPACE, "randomised_parafac: workspace too small");
  return rand_finish(dtype, ndim, shape, rank, n_samples, rec_error, workspace,
                     static_cast<cudaStream_t>(stream));
}

extern "C" int tlgb_sample_khatri_rao(int dtype, int n_mats, const void* const* mats,
                                      const int64_t* rows, int64_t rank, int64_t n_samples,
                                      const int64_t* indices, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "sample_khatri_rao: dtype f32 or f64");
  TLGB_CHECK_ARG(n_mats >= 1 && n_mats <= kMaxModes, "sample_khatri_rao: 1..8 matrices");
  TLGB_CHECK_ARG(mats && rows && indices && out, "sample_khatri_rao: null pointer");
  TLGB_CHECK_ARG(rank >= 1 && n_samples >= 0, "sample_khatri_rao: bad rank or n_samples");
  if (n_samples == 0) return TLGB_OK;
  SampleArgs a{};
  a.n = n_mats;
  for (int k = 0; k < n_mats; ++k) {
    TLGB_CHECK_ARG(mats[k] != nullptr && rows[k] >= 1, "sample_khatri_rao: bad matrix");
    a.mats[k] = mats[k];
    a.idx[k] = indices + (int64_t)k * n_samples;
    a.rows[k] = rows[k];
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned bk = (unsigned)std::min<int64_t>(ceil_div(n_samples * rank, (int64_t)256), 152 * 8);
  if (dtype == TLGB_F64)
    k_sample_kr<double><<<bk, 256, 0, st>>>(a, n_samples, (int)rank, static_cast<double*>(out),
                                            nullptr);
  else
    k_sample_kr<float><<<bk, 256, 0, st>>>(a, n_samples, (int)rank, static_cast<float*>(out),
                                           nullptr);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
