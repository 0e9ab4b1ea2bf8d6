// SIMT MTTKRP kernels (f32 / f64).  See mttkrp_simt.cuh for the formulation.
#include "mttkrp_simt.cuh"
#include "mttkrp_tc.cuh"   // tc_tuning

namespace tlgb {

namespace {

constexpr int kThreads = 128;  // 4 warps

template <typename T> struct Vec;
template <> struct Vec<float> { using type = float4; static constexpr int n = 4; };
template <> struct Vec<double> { using type = double2; static constexpr int n = 2; };

template <typename T, int N>
__device__ __forceinline__ void ld_smem(const T* p, T (&v)[N]) {
  // N consecutive elements from a 16-byte aligned shared address
  if constexpr (sizeof(T) * N == 16) {
    using V = typename Vec<T>::type;
    V x = *reinterpret_cast<const V*>(p);
    if constexpr (Vec<T>::n == 4) { v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w; }
    else { v[0] = x.x; v[1] = x.y; }
  } else {
#pragma unroll
    for (int i = 0; i < N; ++i) v[i] = p[i];
  }
}

// Tile shape per element type: BM output rows x BN rank columns, BK inner chunk.
//   f32: BM=128 (8 rows per thread), f64: BM=64 (4 rows per thread).
template <typename T> struct TileCfg;
template <> struct TileCfg<float> { static constexpr int BM = 128, TM = 8, BK = 32; };
template <> struct TileCfg<double> { static constexpr int BM = 64, TM = 4, BK = 16; };

template <typename T, int BN>
__global__ void __launch_bounds__(kThreads, 3)
mttkrp_split_kernel(const MttkrpArgs<T> a) {
  if (a.skip_flag && *a.skip_flag) return;
  constexpr int BM = TileCfg<T>::BM, TM = TileCfg<T>::TM, BK = TileCfg<T>::BK;
  constexpr int TN = BN / 8;            // columns per thread (8 lanes along n)
  constexpr int VEC = Vec<T>::n;
  constexpr int PADM = BM + VEC;        // row pitch of As (keeps 16-byte alignment)
  constexpr int PADN = BN + VEC;
  constexpr int XV = BM * BK / VEC / kThreads;   // vector loads of X per thread per step
  constexpr int FV = (BK * BN / VEC + kThreads - 1) / kThreads;

  extern __shared__ __align__(16) unsigned char smem_raw[];
  T* As = reinterpret_cast<T*>(smem_raw);           // [2][BK][PADM]
  T* Bs = As + 2 * BK * PADM;                        // [2][BK][PADN]

  const int tid = threadIdx.x;
  const int warp = tid >> 5, lane = tid & 31;
  const int lm = lane >> 3, ln = lane & 7;
  const int64_t r0 = (int64_t)blockIdx.x * BN;
  const int split = blockIdx.y;
  const int64_t m0 = (int64_t)blockIdx.z * BM;

  const int64_t t_begin = (int64_t)split * a.steps_per_split;
  const int64_t t_end = min(t_begin + a.steps_per_split, a.total_steps);

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = T(0);

  // register staging for the next step's tiles
  T xr[XV][VEC];
  T fr[FV][VEC];
  // The factor tile is staged as F_inner[c, r] * s(o, r), s(o, r) = w_r *
  // prod_k A_k(i_k(o), r) (the Khatri-Rao row of the outer modes), so one
  // accumulator set carries the whole contraction.  This thread stages the
  // columns r0 + (tid % (BN / VEC)) * VEC + j of every B row; sv holds their
  // scales for the staged step's o (recomputed when o changes).
  static_assert(kThreads % (BN / VEC) == 0, "staging columns must be fixed per thread");
  const int64_t rcol = r0 + (tid % (BN / VEC)) * VEC;
  T sv[VEC];
  int64_t s_o = -1;

  auto outer_offset = [&](int64_t o) -> int64_t {
    int64_t off = 0;
    for (int k = a.n_outer - 1; k >= 0; --k) {
      int64_t d = a.outer_dim[k];
      int64_t ik = o % d;
      o /= d;
      off += ik * a.outer_stride[k];
    }
    return off;
  };

  auto load_scales = [&](int64_t o) {
    int64_t idx[kMaxModes];
    int64_t oo = o;
    for (int k = a.n_outer - 1; k >= 0; --k) {
      idx[k] = oo % a.outer_dim[k];
      oo /= a.outer_dim[k];
    }
#pragma unroll
    for (int j = 0; j < VEC; ++j) {
      const int64_t r = rcol + j;
      T v = T(0);
      if (r < a.R) {
        v = a.weights ? a.weights[r] : T(1);
        for (int k = 0; k < a.n_outer; ++k) v *= a.outer_f[k][idx[k] * a.R + r];
      }
      sv[j] = v;
    }
    s_o = o;
  };

  const uint64_t xpol = l2_evict_first_policy();
  // (outer slice, chunk) of the next step to load, advanced incrementally:
  // the 64-bit divisions of the slice index run once per slice, not per step
  int64_t ld_o = t_begin / a.KC;
  int64_t ld_kc = t_begin - ld_o * a.KC;
  int64_t ld_xoff = outer_offset(ld_o);
  auto load_step = [&]() {
    const int64_t o = ld_o;
    const int64_t c0 = ld_kc * BK;
    const T* Xo = a.X + ld_xoff;
    if (o != s_o) load_scales(o);
    if (++ld_kc == a.KC) {
      ld_kc = 0;
      ++ld_o;
      if (ld_o * a.KC < a.total_steps) ld_xoff = outer_offset(ld_o);
    }
#pragma unroll
    for (int v = 0; v < XV; ++v) {
      const int e = v * kThreads + tid;
      int64_t m, c;
      if (!a.out_contig) {            // rows m, contiguous c
        m = m0 + e / (BK / VEC);
        c = c0 + (e % (BK / VEC)) * VEC;
      } else {                        // rows c, contiguous m
        c = c0 + e / (BM / VEC);
        m = m0 + (e % (BM / VEC)) * VEC;
      }
      if (a.vec_x) {
        const bool inb = (m < a.I_out) && (c < a.C);
        if (inb) {
          using V = typename Vec<T>::type;
          const V* xp = reinterpret_cast<const V*>(Xo + m * a.s_out + c * a.s_c);
          V x = a.l2_stream ? ldg_stream(xp, xpol) : __ldg(xp);
          if constexpr (VEC == 4) { xr[v][0] = x.x; xr[v][1] = x.y; xr[v][2] = x.z; xr[v][3] = x.w; }
          else { xr[v][0] = x.x; xr[v][1] = x.y; }
        } else {
#pragma unroll
          for (int j = 0; j < VEC; ++j) xr[v][j] = T(0);
        }
      } else {
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
          const int64_t mm = a.out_contig ? m + j : m;
          const int64_t cc = a.out_contig ? c : c + j;
          xr[v][j] = (mm < a.I_out && cc < a.C) ? __ldg(Xo + mm * a.s_out + cc * a.s_c) : T(0);
        }
      }
    }
#pragma unroll
    for (int v = 0; v < FV; ++v) {
      const int e = v * kThreads + tid;
      if (e < BK * BN / VEC) {
        const int64_t c = c0 + e / (BN / VEC);
        const int64_t r = r0 + (e % (BN / VEC)) * VEC;
        if (a.vec_f && c < a.C && r + VEC <= a.R) {
          using V = typename Vec<T>::type;
          V x = __ldg(reinterpret_cast<const V*>(a.F + c * a.R + r));
          if constexpr (VEC == 4) { fr[v][0] = x.x; fr[v][1] = x.y; fr[v][2] = x.z; fr[v][3] = x.w; }
          else { fr[v][0] = x.x; fr[v][1] = x.y; }
        } else {
#pragma unroll
          for (int j = 0; j < VEC; ++j)
            fr[v][j] = (c < a.C && r + j < a.R) ? __ldg(a.F + c * a.R + r + j) : T(0);
        }
      }
    }
  };

  auto store_step = [&](int buf) {
    T* A = As + buf * BK * PADM;
    T* B = Bs + buf * BK * PADN;
#pragma unroll
    for (int v = 0; v < XV; ++v) {
      const int e = v * kThreads + tid;
      if (!a.out_contig) {
        const int m = e / (BK / VEC);
        const int c = (e % (BK / VEC)) * VEC;
#pragma unroll
        for (int j = 0; j < VEC; ++j) A[(c + j) * PADM + m] = xr[v][j];
      } else {
        const int c = e / (BM / VEC);
        const int m = (e % (BM / VEC)) * VEC;
#pragma unroll
        for (int j = 0; j < VEC; ++j) A[c * PADM + m + j] = xr[v][j];
      }
    }
#pragma unroll
    for (int v = 0; v < FV; ++v) {
      const int e = v * kThreads + tid;
      if (e < BK * BN / VEC) {
        const int c = e / (BN / VEC);
        const int r = (e % (BN / VEC)) * VEC;
#pragma unroll
        for (int j = 0; j < VEC; ++j) B[c * PADN + r + j] = fr[v][j] * sv[j];
      }
    }
  };

  // thread-owned output coordinates inside the tile
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

  if (t_begin < t_end) {
    load_step();
    store_step(0);
    __syncthreads();
    int buf = 0;
    for (int64_t t = t_begin; t < t_end; ++t) {
      const bool has_next = (t + 1 < t_end);
      if (has_next) load_step();
      const T* A = As + buf * BK * PADM;
      const T* B = Bs + buf * BK * PADN;
      // unrolled by 8: the fully unrolled step (BK x TM x TN FMAs) outgrows
      // the instruction cache
#pragma unroll 8
      for (int k = 0; k < BK; ++k) {
        T av[TM], bv[TN];
#pragma unroll
        for (int g = 0; g < TM / 4; ++g) {
          T tmp[4];
          ld_smem<T, 4>(A + k * PADM + mrow[g * 4], tmp);
#pragma unroll
          for (int i = 0; i < 4; ++i) av[g * 4 + i] = tmp[i];
        }
        if constexpr (TN >= 4) {
#pragma unroll
          for (int g = 0; g < TN / 4; ++g) {
            T tmp[4];
            ld_smem<T, 4>(B + k * PADN + ncol[g * 4], tmp);
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[g * 4 + j] = tmp[j];
          }
        } else {
#pragma unroll
          for (int j = 0; j < TN; ++j) bv[j] = B[k * PADN + ncol[j]];
        }
#pragma unroll
        for (int i = 0; i < TM; ++i)
#pragma unroll
          for (int j = 0; j < TN; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
      }
      if (has_next) store_step(buf ^ 1);
      __syncthreads();
      buf ^= 1;
    }
  }

  // write this split's partial tile
  T* out = a.partial + (int64_t)split * a.I_out * a.R;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int64_t m = m0 + mrow[i];
    if (m >= a.I_out) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int64_t r = r0 + ncol[j];
      if (r < a.R) out[m * a.R + r] = acc[i][j];
    }
  }
}

template <typename T, typename TO>
__global__ void mttkrp_reduce_kernel(const T* __restrict__ partial, int splits, int64_t n,
                                     TO* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < splits; ++k) s += (double)partial[(int64_t)k * n + e];
    out[e] = (TO)s;
  }
}

template <typename T, int BN>
size_t smem_bytes() {
  constexpr int VEC = Vec<T>::n;
  return (size_t)2 * TileCfg<T>::BK * (TileCfg<T>::BM + VEC) * sizeof(T) +
         (size_t)2 * TileCfg<T>::BK * (BN + VEC) * sizeof(T);
}

template <typename T, int BN>
int set_attr() {
  TLGB_CUDA_TRY(cudaFuncSetAttribute(mttkrp_split_kernel<T, BN>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem_bytes<T, BN>()));
  return TLGB_OK;
}

template <typename T>
int prepare_typed() {
  static std::atomic<bool> done[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && done[dev]) return TLGB_OK;
  int rc = set_attr<T, 16>();
  if (!rc) rc = set_attr<T, 32>();
  if (!rc) rc = set_attr<T, 64>();
  if (!rc && dev >= 0 && dev < 64) done[dev] = true;
  return rc;
}

template <typename T, int BN>
int launch_bn(const MttkrpArgs<T>& a, const MttkrpPlan& p, cudaStream_t stream) {
  const size_t smem = smem_bytes<T, BN>();
  int rc = prepare_typed<T>();
  if (rc) return rc;
  dim3 grid(p.r_tiles, p.splits, p.m_tiles);
  mttkrp_split_kernel<T, BN><<<grid, kThreads, smem, stream>>>(a);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

}  // namespace

int mttkrp_prepare(int dtype) {
  return dtype == TLGB_F64 ? prepare_typed<double>() : prepare_typed<float>();
}

int mttkrp_make_plan(int dtype, const Shape& sh, int64_t rank, int mode, MttkrpPlan* plan) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "mttkrp: dtype must be f32 or f64");
  TLGB_CHECK_ARG(sh.ndim >= 2 && sh.ndim <= kMaxModes, "mttkrp: ndim must be in [2, 8]");
  TLGB_CHECK_ARG(mode >= 0 && mode < sh.ndim, "mttkrp: mode out of range");
  TLGB_CHECK_ARG(rank >= 1, "mttkrp: rank must be >= 1");
  for (int k = 0; k < sh.ndim; ++k) TLGB_CHECK_ARG(sh.dim[k] >= 1, "mttkrp: empty mode");
  MttkrpPlan p{};
  const int N = sh.ndim;
  p.R = rank;
  p.I_out = sh.dim[mode];
  p.s_out = sh.stride[mode];
  p.inner_mode = (mode == N - 1) ? N - 2 : N - 1;
  p.C = sh.dim[p.inner_mode];
  p.s_c = sh.stride[p.inner_mode];
  p.out_contig = (mode == N - 1) ? 1 : 0;
  p.n_outer = 0;
  p.O = 1;
  for (int k = 0; k < N; ++k) {
    if (k == mode || k == p.inner_mode) continue;
    p.outer_mode[p.n_outer] = k;
    p.outer_dim[p.n_outer] = sh.dim[k];
    p.outer_stride[p.n_outer] = sh.stride[k];
    p.n_outer++;
    p.O *= sh.dim[k];
  }
  const bool f64 = dtype == TLGB_F64;
  p.bm = f64 ? 64 : 128;
  p.bk = f64 ? 16 : 32;
  p.bn = rank <= 16 ? 16 : (rank <= 32 ? 32 : 64);
  p.r_tiles = (int)ceil_div(rank, p.bn);
  p.m_tiles = (int)ceil_div(p.I_out, p.bm);
  p.KC = ceil_div(p.C, p.bk);
  p.total_steps = p.O * p.KC;
  const int64_t tiles = (int64_t)p.r_tiles * p.m_tiles;
  const int64_t target = (int64_t)sm_count() * 3;
  int64_t splits = ceil_div(target, tiles);
  // keep at least 4 steps per split so the partial buffer stays small
  splits = std::min<int64_t>(splits, std::max<int64_t>(1, p.total_steps / 4));
  splits = std::max<int64_t>(1, std::min<int64_t>(splits, 65535));
  p.steps_per_split = ceil_div(p.total_steps, splits);
  p.splits = (int)ceil_div(p.total_steps, p.steps_per_split);
  p.partial_bytes = (size_t)p.splits * p.I_out * p.R * (f64 ? 8 : 4);
  *plan = p;
  return TLGB_OK;
}

template <typename T>
int mttkrp_launch_partials(const MttkrpPlan& p, const T* X, const T* const* factors,
                           const T* weights, T* partial, const int* skip_flag,
                           cudaStream_t stream) {
  MttkrpArgs<T> a{};
  a.X = X;
  a.F = factors[p.inner_mode];
  for (int k = 0; k < p.n_outer; ++k) {
    a.outer_f[k] = factors[p.outer_mode[k]];
    a.outer_dim[k] = p.outer_dim[k];
    a.outer_stride[k] = p.outer_stride[k];
  }
  a.weights = weights;
  a.I_out = p.I_out; a.C = p.C; a.O = p.O; a.R = p.R;
  a.s_out = p.s_out; a.s_c = p.s_c;
  a.n_outer = p.n_outer;
  a.KC = p.KC; a.steps_per_split = p.steps_per_split; a.total_steps = p.total_steps;
  a.splits = p.splits;
  a.out_contig = p.out_contig;
  constexpr int VEC = Vec<T>::n;
  const bool x_al = (reinterpret_cast<uintptr_t>(X) % 16) == 0;
  a.vec_x = x_al && (p.out_contig ? (p.I_out % VEC == 0) : (p.C % VEC == 0));
  a.vec_f = ((reinterpret_cast<uintptr_t>(a.F) % 16) == 0) && (p.R % VEC == 0);
  a.partial = partial;
  a.skip_flag = skip_flag;
  a.l2_stream = tc_tuning().l2_keep ? 0 : 1;
  switch (p.bn) {
    case 16: return launch_bn<T, 16>(a, p, stream);
    case 32: return launch_bn<T, 32>(a, p, stream);
    default: return launch_bn<T, 64>(a, p, stream);
  }
}

template <typename T, typename TO>
int mttkrp_launch_reduce(const MttkrpPlan& p, const T* partial, TO* out, cudaStream_t stream) {
  const int64_t n = p.I_out * p.R;
  const int threads = 256;
  const int blocks = (int)std::min<int64_t>(ceil_div(n, threads), (int64_t)sm_count() * 8);
  mttkrp_reduce_kernel<T, TO><<<blocks, threads, 0, stream>>>(partial, p.splits, n, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T, typename TO>
int mttkrp_launch_reduce_n(const T* partial, int splits, int64_t n, TO* out, cudaStream_t stream) {
  const int threads = 256;
  const int blocks = (int)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(n, (int64_t)threads), (int64_t)sm_count() * 8));
  mttkrp_reduce_kernel<T, TO><<<blocks, threads, 0, stream>>>(partial, splits, n, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
template int mttkrp_launch_reduce_n<float, float>(const float*, int, int64_t, float*, cudaStream_t);
template int mttkrp_launch_reduce_n<double, double>(const double*, int, int64_t, double*,
                                                    cudaStream_t);

template int mttkrp_launch_partials<float>(const MttkrpPlan&, const float*, const float* const*,
                                           const float*, float*, const int*, cudaStream_t);
template int mttkrp_launch_partials<double>(const MttkrpPlan&, const double*,
                                            const double* const*, const double*, double*,
                                            const int*, cudaStream_t);
template int mttkrp_launch_reduce<float, float>(const MttkrpPlan&, const float*, float*, cudaStream_t);
template int mttkrp_launch_reduce<double, double>(const MttkrpPlan&, const double*, double*, cudaStream_t);

}  // namespace tlgb

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
using namespace tlgb;

extern "C" int tlgb_mttkrp_workspace_size(int dtype, int ndim, const int64_t* shape,
                                          int64_t rank, int mode, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(shape && bytes, "mttkrp_workspace_size: null pointer");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "mttkrp: ndim must be in [2, 8]");
  Shape sh = make_shape(ndim, shape);
  MttkrpPlan p;
  int rc = mttkrp_make_plan(dtype, sh, rank, mode, &p);
  if (rc) return rc;
  *bytes = align_up(p.partial_bytes, 256);
  return TLGB_OK;
}

extern "C" int tlgb_mttkrp(int dtype, const void* X, int ndim, const int64_t* shape,
                           const void* const* factors, const void* weights, int64_t rank,
                           int mode, void* out, void* workspace, size_t workspace_bytes,
                           void* stream) {
  clear_error();
  TLGB_CHECK_ARG(X && shape && factors && out, "mttkrp: null pointer");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "mttkrp: ndim must be in [2, 8]");
  Shape sh = make_shape(ndim, shape);
  MttkrpPlan p;
  int rc = mttkrp_make_plan(dtype, sh, rank, mode, &p);
  if (rc) return rc;
  for (int k = 0; k < ndim; ++k)
    TLGB_CHECK_ARG(k == mode || factors[k] != nullptr, "mttkrp: missing factor pointer");
  if (workspace_bytes < p.partial_bytes || !workspace)
    return set_error(TLGB_EWORKSPACE, "mttkrp: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32) {
    rc = mttkrp_launch_partials<float>(p, (const float*)X, (const float* const*)factors,
                                       (const float*)weights, (float*)workspace, nullptr, st);
    if (rc) return rc;
    return mttkrp_launch_reduce<float, float>(p, (const float*)workspace, (float*)out, st);
  }
  rc = mttkrp_launch_partials<double>(p, (const double*)X, (const double* const*)factors,
                                      (const double*)weights, (double*)workspace, nullptr, st);
  if (rc) return rc;
  return mttkrp_launch_reduce<double, double>(p, (const double*)workspace, (double*)out, st);
}
