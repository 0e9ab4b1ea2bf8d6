// Tensor-times-matrix (mode_dot), tensorly/tenalg/core_tenalg/n_mode_product.py:5-76.
//
// The reference unfolds (a copy for middle modes), multiplies and refolds.
// Here the tensor is viewed in place as (L, I, T) with I the contracted mode:
//   Y[l, j, t] = sum_i W(i, j) X[l, i, t],   W = U^T (or U when transpose)
// as a strided batched GEMM.  When T > 1 the GEMM's M dimension is t (the
// contiguous one) and l is the batch; when T == 1 (last mode) M is l and the
// contraction runs along the contiguous dimension.  SIMT f32 / f64 tiles,
// 16-byte vector loads along whichever dimension is contiguous.
#include <type_traits>
#include "mttkrp_tc.cuh"   // tc_tuning

#include "linalg.cuh"

namespace tlgb {
namespace {

constexpr int kThreads = 128;

template <typename T> struct TVec;
template <> struct TVec<float> { using type = float4; static constexpr int n = 4; };
template <> struct TVec<double> { using type = double2; static constexpr int n = 2; };
template <typename T> struct TCfg;
template <> struct TCfg<float> { static constexpr int BM = 128, TM = 8, BK = 32; };
template <> struct TCfg<double> { static constexpr int BM = 64, TM = 4, BK = 16; };

template <typename T>
struct TtmArgs {
  const T* X;
  const T* U;
  T* Y;
  int64_t M, N, K, B;            // GEMM sizes and batch count
  int64_t sam, sak, sab;         // A (= X) strides for m, k, batch
  int64_t swk, swn;              // W strides
  int64_t sym, syn, syb;         // Y strides
  int a_m_contig;                // 1: m has stride 1 in X; 0: k has stride 1
  int vec_a;
  int64_t b_off;                 // first batch index of this launch
};

template <typename T, int BN>
__global__ void __launch_bounds__(kThreads) ttm_kernel(const TtmArgs<T> a) {
  constexpr int BM = TCfg<T>::BM, TM = TCfg<T>::TM, BK = TCfg<T>::BK;
  constexpr int TN = BN / 8;
  constexpr int VEC = TVec<T>::n;
  constexpr int PADM = BM + VEC, PADN = BN + VEC;
  constexpr int XV = BM * BK / VEC / kThreads;
  constexpr int WN = (BK * BN + kThreads - 1) / kThreads;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);
  T* Bs = As + 2 * BK * PADM;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int lm = lane >> 3, ln = lane & 7;
  const int64_t m0 = (int64_t)blockIdx.x * BM;
  const int64_t n0 = (int64_t)blockIdx.y * BN;
  const int64_t b = a.b_off + blockIdx.z;
  const T* Xb = a.X + b * a.sab;

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);
  T xr[XV][VEC];
  T wr[WN];
  const int64_t KC = ceil_div(a.K, BK);

  auto load = [&](int64_t kc) {
    const int64_t k0 = kc * BK;
#pragma unroll
    for (int v = 0; v < XV; ++v) {
      const int e = v * kThreads + tid;
      int64_t m, k;
      if (!a.a_m_contig) { m = m0 + e / (BK / VEC); k = k0 + (e % (BK / VEC)) * VEC; }
      else { k = k0 + e / (BM / VEC); m = m0 + (e % (BM / VEC)) * VEC; }
      if (a.vec_a) {
        if (m < a.M && k < a.K) {
          using V = typename TVec<T>::type;
          V x = __ldg(reinterpret_cast<const V*>(Xb + m * a.sam + k * a.sak));
          if constexpr (VEC == 4) { xr[v][0] = x.x; xr[v][1] = x.y; xr[v][2] = x.z; xr[v][3] = x.w; }
          else { xr[v][0] = x.x; xr[v][1] = x.y; }
        } else {
#pragma unroll
          for (int j = 0; j < VEC; ++j) xr[v][j] = T(0);
        }
      } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
          const int64_t mm = a.a_m_contig ? m + j : m;
          const int64_t kk = a.a_m_contig ? k : k + j;
          xr[v][j] = (mm < a.M && kk < a.K) ? __ldg(Xb + mm * a.sam + kk * a.sak) : T(0);
        }
      }
    }
#pragma unroll
    for (int v = 0; v < WN; ++v) {
      const int e = v * kThreads + tid;
      if (e < BK * BN) {
        const int64_t k = k0 + e / BN, n = n0 + e % BN;
        wr[v] = (k < a.K && n < a.N) ? __ldg(a.U + k * a.swk + n * a.swn) : T(0);
      }
    }
  };
  auto store = [&](int buf) {
    T* A = As + buf * BK * PADM;
    T* B = Bs + buf * BK * PADN;
#pragma unroll
    for (int v = 0; v < XV; ++v) {
      const int e = v * kThreads + tid;
      if (!a.a_m_contig) {
        const int m = e / (BK / VEC), k = (e % (BK / VEC)) * VEC;
#pragma unroll
        for (int j = 0; j < VEC; ++j) A[(k + j) * PADM + m] = xr[v][j];
      } else {
        const int k = e / (BM / VEC), m = (e % (BM / VEC)) * VEC;
#pragma unroll
        for (int j = 0; j < VEC; ++j) A[k * PADM + m + j] = xr[v][j];
      }
    }
#pragma unroll
    for (int v = 0; v < WN; ++v) {
      const int e = v * kThreads + tid;
      if (e < BK * BN) B[(e / BN) * PADN + e % BN] = wr[v];
    }
  };

  int mrow[TM];
#pragma unroll
  for (int g = 0; g < TM / 4; ++g)
#pragma unroll
    for (int i = 0; i < 4; ++i) mrow[g * 4 + i] = warp * (4 * TM) + g * 16 + lm * 4 + i;
  int ncol[TN];
  if constexpr (TN >= 4) {
#pragma unroll
    for (int g = 0; g < TN / 4; ++g)
#pragma unroll
      for (int j = 0; j < 4; ++j) ncol[g * 4 + j] = g * 32 + ln * 4 + j;
  } else {
#pragma unroll
    for (int j = 0; j < TN; ++j) ncol[j] = ln * TN + j;
  }

  load(0);
  store(0);
  __syncthreads();
  int buf = 0;
  for (int64_t kc = 0; kc < KC; ++kc) {
    const bool has_next = kc + 1 < KC;
    if (has_next) load(kc + 1);
    const T* A = As + buf * BK * PADM;
    const T* B = Bs + buf * BK * PADN;
#pragma unroll
    for (int k = 0; k < BK; ++k) {
      T av[TM], bv[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) av[i] = A[k * PADM + mrow[i]];
#pragma unroll
      for (int j = 0; j < TN; ++j) bv[j] = B[k * PADN + ncol[j]];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    if (has_next) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
  }
  T* Yb = a.Y + b * a.syb;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t m = m0 + mrow[i];
    if (m >= a.M) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t n = n0 + ncol[j];
      if (n < a.N) Yb[m * a.sym + n * a.syn] = acc[i][j];
    }
  }
}

// Small J (<= 32), contracted mode not the last: Y[l, j, t] = sum_i W(i, j)
// X[l, i, t] streamed once.  A thread owns V consecutive t for one l and keeps
// all JP (J padded) outputs for them in registers; X rows come straight from
// global memory as V-wide vectors, kRowBatch rows in flight; W sits in shared
// memory, padded to JP columns, and is read as broadcast vectors.  Per row a
// thread issues one X load, JP/4 (f32) or JP/2 (f64) shared loads and JP * V
// FMAs, so the kernel streams at the HBM rate instead of being issue-bound.
constexpr int kStreamThreads = 128;
constexpr int kRowBatch = 8;
constexpr size_t kStreamSmemMax = 96 * 1024;   // W in shared memory: I * JP elements

template <typename T, int JP, int V>
__global__ void __launch_bounds__(kStreamThreads)
ttm_stream_kernel(const T* __restrict__ X, const T* __restrict__ U, T* __restrict__ Y, int64_t L,
                  int I, int64_t Tt, int J, int transpose, int l2_stream) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* Ws = reinterpret_cast<T*>(smem_raw);   // [I][JP]
  const int tid = threadIdx.x;
  for (int e = tid; e < I * JP; e += kStreamThreads) {
    const int i = e / JP, j = e - (e / JP) * JP;
    Ws[e] = (j < J) ? (transpose ? U[(int64_t)i * J + j] : U[(int64_t)j * I + i]) : T(0);
  }
  __syncthreads();
  using Vec = typename std::conditional<sizeof(T) == 4,
      typename std::conditional<V == 4, float4, typename std::conditional<V == 2, float2, float>::type>::type,
      typename std::conditional<V == 2, double2, double>::type>::type;
  // threads over (l, t / V) jointly, so a short t range does not idle lanes
  const int64_t tv = Tt / V;
  const int64_t total = L * tv;
  const uint64_t xpol = l2_evict_first_policy();   // X is streamed once
  for (int64_t g = (int64_t)blockIdx.x * kStreamThreads + tid; g < total;
       g += (int64_t)gridDim.x * kStreamThreads) {
    const int64_t l = g / tv;
    const int64_t t0 = (g - l * tv) * V;
    const T* xp = X + (l * I) * Tt + t0;
    T acc[JP][V];
#pragma unroll
    for (int j = 0; j < JP; ++j)
#pragma unroll
      for (int v = 0; v < V; ++v) acc[j][v] = T(0);
    for (int i0 = 0; i0 < I; i0 += kRowBatch) {
      T xs[kRowBatch][V];
#pragma unroll
      for (int u = 0; u < kRowBatch; ++u) {
        if (i0 + u < I) {
          const Vec* xa = reinterpret_cast<const Vec*>(xp + (int64_t)(i0 + u) * Tt);
          const Vec x = l2_stream ? ldg_stream(xa, xpol) : __ldg(xa);
          const T* xv = reinterpret_cast<const T*>(&x);
#pragma unroll
          for (int v = 0; v < V; ++v) xs[u][v] = xv[v];
        } else {
#pragma unroll
          for (int v = 0; v < V; ++v) xs[u][v] = T(0);
        }
      }
#pragma unroll
      for (int u = 0; u < kRowBatch; ++u) {
        if (i0 + u < I) {
          const T* w = Ws + (i0 + u) * JP;
#pragma unroll
          for (int j = 0; j < JP; ++j) {
            const T wj = w[j];
#pragma unroll
            for (int v = 0; v < V; ++v) acc[j][v] = fma(wj, xs[u][v], acc[j][v]);
          }
        }
      }
    }
    T* yp = Y + (l * J) * Tt + t0;
#pragma unroll
    for (int j = 0; j < JP; ++j) {
      if (j < J) {
        Vec o;
        T* ov = reinterpret_cast<T*>(&o);
#pragma unroll
        for (int v = 0; v < V; ++v) ov[v] = acc[j][v];
        *reinterpret_cast<Vec*>(yp + (int64_t)j * Tt) = o;
      }
    }
  }
}

template <typename T, int JP, int V>
int launch_stream(const T* X, const T* U, T* Y, int64_t L, int I, int64_t Tt, int J,
                  int transpose, cudaStream_t st) {
  const size_t smem = (size_t)I * JP * sizeof(T);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(ttm_stream_kernel<T, JP, V>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kStreamSmemMax));
    attr[dev] = true;
  }
  const int64_t tb = std::min<int64_t>(ceil_div(L * (Tt / V), kStreamThreads), 1ll << 30);
  dim3 grid((unsigned)tb);
  ttm_stream_kernel<T, JP, V><<<grid, kStreamThreads, smem, st>>>(X, U, Y, L, I, Tt, J, transpose,
                                                                  tc_tuning().l2_keep ? 0 : 1);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T, int BN>
int launch(const TtmArgs<T>& a, cudaStream_t st) {
  constexpr int VEC = TVec<T>::n;
  const size_t smem = (size_t)2 * TCfg<T>::BK * (TCfg<T>::BM + VEC) * sizeof(T) +
                      (size_t)2 * TCfg<T>::BK * (BN + VEC) * sizeof(T);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(ttm_kernel<T, BN>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    attr[dev] = true;
  }
  const int64_t mt = ceil_div(a.M, TCfg<T>::BM), nt = ceil_div(a.N, BN);
  TLGB_CHECK_ARG(mt < (1ll << 31) && nt <= 65535, "mode_dot: tensor too large for the grid");
  for (int64_t b0 = 0; b0 < a.B; b0 += 65535) {
    TtmArgs<T> c = a;
    c.b_off = b0;
    dim3 grid((unsigned)mt, (unsigned)nt, (unsigned)std::min<int64_t>(65535, a.B - b0));
    ttm_kernel<T, BN><<<grid, kThreads, smem, st>>>(c);
    TLGB_LAUNCH_CHECK();
  }
  return TLGB_OK;
}

template <typename T>
int ttm_typed(const T* X, const Shape& sh, const T* U, int64_t J, int transpose, int mode, T* Y,
              cudaStream_t st) {
  TtmArgs<T> a{};
  int64_t L = 1, Tt = 1;
  for (int k = 0; k < mode; ++k) L *= sh.dim[k];
  for (int k = mode + 1; k < sh.ndim; ++k) Tt *= sh.dim[k];
  const int64_t I = sh.dim[mode];
  a.X = X; a.U = U; a.Y = Y;
  a.N = J; a.K = I;
  if (transpose) { a.swk = J; a.swn = 1; } else { a.swk = 1; a.swn = I; }
  constexpr int VEC = TVec<T>::n;
  const bool al = (reinterpret_cast<uintptr_t>(X) % 16) == 0;
  if (Tt > 1) {
    a.M = Tt; a.B = L;
    a.sam = 1; a.sak = Tt; a.sab = I * Tt;
    a.sym = 1; a.syn = Tt; a.syb = J * Tt;
    a.a_m_contig = 1;
    a.vec_a = al && (Tt % VEC == 0);
  } else {
    a.M = L; a.B = 1;
    a.sam = I; a.sak = 1; a.sab = 0;
    a.sym = J; a.syn = 1; a.syb = 0;
    a.a_m_contig = 0;
    a.vec_a = al && (I % VEC == 0);
  }
  if (a.M == 0 || a.N == 0 || a.B == 0) return TLGB_OK;
  // streaming kernel: small J, contracted mode not last, vector-aligned rows
  const bool yal = (reinterpret_cast<uintptr_t>(Y) % 16) == 0;
  const int jp = J <= 4 ? 4 : J <= 8 ? 8 : J <= 16 ? 16 : 32;
  if (Tt > 1 && J <= 32 && (size_t)I * jp * sizeof(T) <= kStreamSmemMax && al && yal) {
    if constexpr (sizeof(T) == 4) {
      if (Tt % 4 == 0) {
        if (J <= 4) return launch_stream<T, 4, 4>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
        if (J <= 8) return launch_stream<T, 8, 4>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
        if (J <= 16) return launch_stream<T, 16, 4>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
        return launch_stream<T, 32, 2>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
      }
    } else {
      if (Tt % 2 == 0) {
        if (J <= 4) return launch_stream<T, 4, 2>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
        if (J <= 8) return launch_stream<T, 8, 2>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
        if (J <= 16) return launch_stream<T, 16, 2>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
        return launch_stream<T, 32, 1>(X, U, Y, L, (int)I, Tt, (int)J, transpose, st);
      }
    }
  }
  if (J <= 16) return launch<T, 16>(a, st);
  if (J <= 32) return launch<T, 32>(a, st);
  return launch<T, 64>(a, st);
}

}  // namespace

template <typename T>
int ttm_launch(const T* X, const Shape& sh, const T* U, int64_t J, int transpose, int mode, T* Y,
               cudaStream_t st) {
  if (sh.numel == 0) return TLGB_OK;
  return ttm_typed<T>(X, sh, U, J, transpose, mode, Y, st);
}
template int ttm_launch<float>(const float*, const Shape&, const float*, int64_t, int, int, float*,
                               cudaStream_t);
template int ttm_launch<double>(const double*, const Shape&, const double*, int64_t, int, int,
                                double*, cudaStream_t);

}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_mode_dot(int dtype, const void* X, int ndim, const int64_t* shape,
                             const void* U, int64_t J, int transpose, int mode, void* out,
                             void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "mode_dot: dtype must be f32 or f64");
  TLGB_CHECK_ARG(X && shape && U && out, "mode_dot: null pointer");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "mode_dot: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(mode >= 0 && mode < ndim, "mode_dot: mode out of range");
  TLGB_CHECK_ARG(J >= 1, "mode_dot: J must be >= 1");
  Shape sh = make_shape(ndim, shape);
  if (sh.numel == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    return ttm_typed<float>((const float*)X, sh, (const float*)U, J, transpose, mode,
                            (float*)out, st);
  return ttm_typed<double>((const double*)X, sh, (const double*)U, J, transpose, mode,
                           (double*)out, st);
}
