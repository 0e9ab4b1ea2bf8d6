// Full tensor of a CP model (tensorly/cp_tensor.py:433-485) and the mode-n
// unfolding / folding of a dense tensor (tensorly/base.py:39-79).
//
// cp_to_tensor computes the mode-0 unfolding
//   out[i_0, c] = sum_r (A_0[i_0, r] * w_r) * KR[c, r],
//   KR[c, r] = ((A_1[i_1, r] * A_2[i_2, r]) * ...) * A_{N-1}[i_{N-1}, r]
// with c the C-order flat index of (i_1, ..., i_{N-1}), which is the C-order
// full tensor.  The products are formed in the reference's order (weights on
// the first factor, the Khatri-Rao product one factor at a time); the sum over
// r runs in r order with FMAs.  The Khatri-Rao matrix is never written to
// HBM: each CTA forms its columns' KR entries for a chunk of r in shared
// memory and multiplies them with its rows' (A_0 w) entries, 8 x 8 outputs
// per thread in registers (a SIMT GEMM whose B operand is generated).  A
// pre-pass writes the factors transposed (R x I_k, A_0 times the weights) to
// the workspace, so the tile fills read contiguous runs along i and store to
// shared memory without bank conflicts.  A mask (the full tensor's shape)
// multiplies the result.
#include "reconstruct.cuh"

namespace tlgb {
namespace {

constexpr int kFullThreads = 256;
constexpr int kFullTM = 64;    // rows (i_0) per CTA: 8 row groups of 8
constexpr int kFullTN = 256;   // flat columns per CTA: 32 lanes x 8
template <typename T> struct FullChunk { static constexpr int value = 32; };
template <> struct FullChunk<double> { static constexpr int value = 16; };

struct FullArgs {
  const void* ft[kMaxModes];   // transposed factors R x I_k (ft[0] = (A_0 w)^T, padded)
  int64_t dim[kMaxModes];
  int64_t ld0;                 // row stride of ft[0]: I_0 rounded up to kFullTM
  int n;
};

// ft_k[r * I_k + i] = A_k[i * R + r] for k >= 1, and ft_0[r * ld0 + i] =
// A_0[i * R + r] * w_r (the reference's factors[0] * weights) over a padded
// RP x ld0 block (RP = R rounded up to 8, ld0 = I_0 rounded up to kFullTM)
// whose pad is zero; all factors in one launch.
struct TransArgs {
  const void* f[kMaxModes];
  void* ft[kMaxModes];
  int64_t dim[kMaxModes];
  int64_t start[kMaxModes + 1];  // prefix sums: RP * ld0, then I_k * R
  int64_t ld0;
  int rp;
  int n;
};

template <typename T>
__global__ void k_transpose_factors(const TransArgs a, const T* __restrict__ w, int R) {
  const int64_t total = a.start[a.n];
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int k = 0;
    while (e >= a.start[k + 1]) ++k;
    const int64_t l = e - a.start[k];
    if (k == 0) {
      const int64_t r = l / a.ld0, i = l - r * a.ld0;
      T v = (T)0;
      if (r < R && i < a.dim[0]) {
        v = static_cast<const T*>(a.f[0])[i * R + r];
        if (w) v = v * w[r];
      }
      static_cast<T*>(a.ft[0])[l] = v;
    } else {
      const int64_t i = l / R;
      const int r = (int)(l - i * R);
      static_cast<T*>(a.ft[k])[(int64_t)r * a.dim[k] + i] = static_cast<const T*>(a.f[k])[l];
    }
  }
}

template <typename T, int V> struct VecOf;
template <> struct VecOf<float, 4> { using type = float4; };
template <> struct VecOf<double, 2> { using type = double2; };

// Fixed-order CTA sum of one double per thread (warp butterfly, then warp 0).
__device__ __forceinline__ void block_sum_to(double v, double* dst) {
  __shared__ double red[kFullThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kFullThreads / 32; ++w) t += red[w];
    *dst = t;
  }
}

// One CTA: rows row0..row0+63 x flat columns col0..col0+255; thread (ty, tx)
// owns rows ty*8..ty*8+7 and columns {tx*4..tx*4+3, 128+tx*4..128+tx*4+3}, so
// its shared-memory reads and its global stores are contiguous float4 runs
// across the warp.  Fill: thread c forms KR[col0 + c, r] for the chunk's r
// (NF Khatri-Rao factors, a compile-time count so the loads of the unrolled
// loop are in flight together); rows of (A_0 w)^T are copied contiguously.
// RESID: instead of storing, read X at the same positions and add
// (X - value)^2 to a double per thread; the CTA's sum goes to part[cta].

template <typename T, int NF, bool RESID>
__global__ void __launch_bounds__(kFullThreads, sizeof(T) == 4 ? 2 : 1)
k_cp_full(const FullArgs a, int R, int64_t rows, int64_t cols, const T* __restrict__ mask,
          T* __restrict__ out, int vec_ok, const T* __restrict__ X, double* part) {
  constexpr int RC = FullChunk<T>::value;
  constexpr int NFA = NF > 0 ? NF : 1;
  __shared__ __align__(16) T As[RC][kFullTM];          // (A_0 w)[row, r], r-major
  __shared__ __align__(16) T Bs[RC][kFullTN];          // KR[col, r], r-major
  const int tid = threadIdx.x;
  const int ty = tid >> 5, tx = tid & 31;
  const int64_t row0 = (int64_t)blockIdx.y * kFullTM;
  const int64_t col0 = (int64_t)blockIdx.x * kFullTN;
  const T* A0t = static_cast<const T*>(a.ft[0]);
  // this thread's fill column: indices into the Khatri-Rao factors
  const T* fcol[NFA];
  int64_t fstride[NFA];
  {
    int64_t col = col0 + tid;
    if (col >= cols) col = cols - 1;                     // in range; not stored
#pragma unroll
    for (int k = NF; k >= 1; --k) {
      const int64_t i = col % a.dim[k];
      col /= a.dim[k];
      fcol[k - 1] = static_cast<const T*>(a.ft[k]) + i;
      fstride[k - 1] = a.dim[k];
    }
    if (NF == 0) { fcol[0] = nullptr; fstride[0] = 0; }
  }
  const int am = tid & (kFullTM - 1), aq = tid / kFullTM;   // As fill: row am, r = aq + 4j
  const int64_t arow = row0 + am;
  T acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = (T)0;
  for (int r0 = 0; r0 < R; r0 += RC) {
#pragma unroll
    for (int rr = aq; rr < RC; rr += kFullThreads / kFullTM) {
      const int r = r0 + rr;
      As[rr][am] = (r < R && arow < rows) ? A0t[(int64_t)r * a.ld0 + arow] : (T)0;
    }
#pragma unroll 8
    for (int rr = 0; rr < RC; ++rr) {
      const int r = r0 + rr;
      T v = (T)0;
      if (r < R) {
        if (NF == 0) {
          v = (T)1;
        } else {
          v = fcol[0][(int64_t)r * fstride[0]];
#pragma unroll
          for (int k = 1; k < NF; ++k) v = v * fcol[k][(int64_t)r * fstride[k]];
        }
      }
      Bs[rr][tid] = v;
    }
    __syncthreads();
#pragma unroll 4
    for (int rr = 0; rr < RC; ++rr) {
      T av[8], bv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) av[i] = As[rr][ty * 8 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        bv[j] = Bs[rr][tx * 4 + j];
        bv[4 + j] = Bs[rr][kFullTN / 2 + tx * 4 + j];
      }
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fma(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
  double rsum = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t row = row0 + ty * 8 + i;
    if (row >= rows) break;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int64_t cb = col0 + h * (kFullTN / 2) + tx * 4;
      if constexpr (RESID) {
        const T* xr = X + row * cols;
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int64_t col = cb + q;
          if (col < cols) {
            const T d = xr[col] - acc[i][h * 4 + q];
            rsum += (double)d * (double)d;
          }
        }
        continue;
      }
      T* o = out + row * cols;
      const T* mk = mask ? mask + row * cols : nullptr;
      if (vec_ok && cb + 4 <= cols) {
        constexpr int V = 16 / sizeof(T);
        using VT = typename VecOf<T, V>::type;
#pragma unroll
        for (int q = 0; q < 4; q += V) {
          T v[V];
#pragma unroll
          for (int u = 0; u < V; ++u) v[u] = acc[i][h * 4 + q + u];
          if (mk) {
            VT m = *reinterpret_cast<const VT*>(mk + cb + q);
            const T* mp = reinterpret_cast<const T*>(&m);
#pragma unroll
            for (int u = 0; u < V; ++u) v[u] = v[u] * mp[u];
          }
          *reinterpret_cast<VT*>(o + cb + q) = *reinterpret_cast<const VT*>(v);
        }
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int64_t col = cb + q;
          if (col < cols) o[col] = mk ? acc[i][h * 4 + q] * mk[col] : acc[i][h * 4 + q];
        }
      }
    }
  }
  if constexpr (RESID) block_sum_to(rsum, part + (int64_t)blockIdx.y * gridDim.x + blockIdx.x);
}

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}

constexpr int kFastRank = 64;   // f32 fast path: the whole (padded) rank in one pass

// f32, R <= 64: the CTA forms the Khatri-Rao tile of its 256 columns for the
// whole (padded) rank once, in shared memory (RP x 256), then walks
// `tiles_per_cta` row tiles of 64, each tile's (A_0 w)^T block (RP x 64, a
// contiguous copy of the padded transposed factor) arriving by cp.async into
// one of two buffers while the previous tile computes.  Same arithmetic per
// output as k_cp_full: products in the reference's order, FMAs in r order.
template <int NF, bool RESID>
__global__ void __launch_bounds__(kFullThreads, 2)
k_cp_full_r64(const FullArgs a, int R, int RP, int64_t rows, int64_t cols, int tiles_per_cta,
              const float* __restrict__ mask, float* __restrict__ out, int vec_ok,
              const float* __restrict__ X, double* part) {
  extern __shared__ __align__(16) float fsm[];
  float* Bs = fsm;                                     // [RP][256]
  float* As = fsm + RP * kFullTN;                      // [2][RP][64]
  const int tid = threadIdx.x;
  const int ty = tid >> 5, tx = tid & 31;
  const int64_t col0 = (int64_t)blockIdx.x * kFullTN;
  const int64_t tiles = a.ld0 / kFullTM;
  const int64_t t0 = (int64_t)blockIdx.y * tiles_per_cta;
  const int64_t t1 = t0 + tiles_per_cta < tiles ? t0 + tiles_per_cta : tiles;
  const float* A0t = static_cast<const float*>(a.ft[0]);
  const int chunks = RP * (kFullTM / 4);               // 16-byte pieces of one (A_0 w) tile
  auto fetch = [&](int64_t t, int buf) {
    float* dst = As + buf * RP * kFullTM;
    for (int q = tid; q < chunks; q += kFullThreads) {
      const int rr = q / (kFullTM / 4), m4 = (q - rr * (kFullTM / 4)) * 4;
      cp_async16(dst + rr * kFullTM + m4, A0t + (int64_t)rr * a.ld0 + t * kFullTM + m4);
    }
    cp_async_commit();
  };
  if (t0 < t1) fetch(t0, 0);
  {
    int64_t col = col0 + tid;
    if (col >= cols) col = cols - 1;                   // in range; not stored
    const float* fcol[NF > 0 ? NF : 1];
    int64_t fstride[NF > 0 ? NF : 1];
#pragma unroll
    for (int k = NF; k >= 1; --k) {
      const int64_t i = col % a.dim[k];
      col /= a.dim[k];
      fcol[k - 1] = static_cast<const float*>(a.ft[k]) + i;
      fstride[k - 1] = a.dim[k];
    }
#pragma unroll 16
    for (int r = 0; r < RP; ++r) {
      float v = 0.f;
      if (r < R) {
        if (NF == 0) {
          v = 1.f;
        } else {
          v = fcol[0][(int64_t)r * fstride[0]];
#pragma unroll
          for (int k = 1; k < NF; ++k) v = v * fcol[k][(int64_t)r * fstride[k]];
        }
      }
      Bs[r * kFullTN + tid] = v;
    }
  }
  double rsum = 0.0;
  for (int64_t t = t0; t < t1; ++t) {
    const int buf = (int)((t - t0) & 1);
    if (t + 1 < t1) {
      fetch(t + 1, buf ^ 1);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
    const float* Ab = As + buf * RP * kFullTM;
    float acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc[i][j] = 0.f;
#pragma unroll 8
    for (int rr = 0; rr < RP; ++rr) {
      const float4 a0 = *reinterpret_cast<const float4*>(Ab + rr * kFullTM + ty * 8);
      const float4 a1 = *reinterpret_cast<const float4*>(Ab + rr * kFullTM + ty * 8 + 4);
      const float4 b0 = *reinterpret_cast<const float4*>(Bs + rr * kFullTN + tx * 4);
      const float4 b1 = *reinterpret_cast<const float4*>(Bs + rr * kFullTN + kFullTN / 2 + tx * 4);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    const int64_t row0 = t * kFullTM;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int64_t row = row0 + ty * 8 + i;
      if (row >= rows) break;
      float* o = out + row * cols;
      const float* mk = mask ? mask + row * cols : nullptr;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int64_t cb = col0 + h * (kFullTN / 2) + tx * 4;
        if constexpr (RESID) {
          const float* xr = X + row * cols;
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            if (cb + q < cols) {
              const float d = xr[cb + q] - acc[i][h * 4 + q];
              rsum += (double)d * (double)d;
            }
          }
          continue;
        }
        if (vec_ok && cb + 4 <= cols) {
          float4 v = make_float4(acc[i][h * 4], acc[i][h * 4 + 1], acc[i][h * 4 + 2],
                                 acc[i][h * 4 + 3]);
          if (mk) {
            const float4 m = *reinterpret_cast<const float4*>(mk + cb);
            v.x *= m.x; v.y *= m.y; v.z *= m.z; v.w *= m.w;
          }
          *reinterpret_cast<float4*>(o + cb) = v;
        } else {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int64_t col = cb + q;
            if (col < cols) o[col] = mk ? acc[i][h * 4 + q] * mk[col] : acc[i][h * 4 + q];
          }
        }
      }
    }
    __syncthreads();                                   // buffer `buf` is refilled next
  }
  if constexpr (RESID) block_sum_to(rsum, part + (int64_t)blockIdx.y * gridDim.x + blockIdx.x);
}

// Grid of the rank <= 64 path: about 2400 CTAs (8 waves of 2 CTAs on 152
// SMs); the Khatri-Rao tile is formed once per CTA and reused by its row tiles.
void r64_grid(int64_t rows_padded, int64_t cols, int64_t* gx, int64_t* gy, int* tpc) {
  *gx = ceil_div(cols, (int64_t)kFullTN);
  const int64_t tiles = rows_padded / kFullTM;
  const int64_t gy0 = std::min<int64_t>(tiles, std::max<int64_t>(1, ceil_div((int64_t)2400, *gx)));
  *tpc = (int)ceil_div(tiles, gy0);
  *gy = ceil_div(tiles, (int64_t)*tpc);
}

template <int NF>
int launch_cp_full_r64(const FullArgs& a, int R, int64_t rows, int64_t cols, const float* mask,
                       float* out, int vec_ok, const float* X, double* part, cudaStream_t st) {
  const int RP = (int)(ceil_div((int64_t)R, (int64_t)8) * 8);
  const size_t smem = (size_t)RP * (kFullTN + 2 * kFullTM) * sizeof(float);
  int64_t gx, gy;
  int tpc;
  r64_grid(a.ld0, cols, &gx, &gy, &tpc);
  dim3 grid((unsigned)gx, (unsigned)gy);
  if (X) {
    if (smem > 48 * 1024)
      TLGB_CUDA_TRY(cudaFuncSetAttribute(k_cp_full_r64<NF, true>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_cp_full_r64<NF, true><<<grid, kFullThreads, smem, st>>>(a, R, RP, rows, cols, tpc, mask,
                                                              out, vec_ok, X, part);
  } else {
    if (smem > 48 * 1024)
      TLGB_CUDA_TRY(cudaFuncSetAttribute(k_cp_full_r64<NF, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_cp_full_r64<NF, false><<<grid, kFullThreads, smem, st>>>(a, R, RP, rows, cols, tpc, mask,
                                                               out, vec_ok, X, part);
  }
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int dispatch_cp_full_r64(const FullArgs& a, int R, int64_t rows, int64_t cols, const float* mask,
                         float* out, int vec_ok, cudaStream_t st, const float* X = nullptr,
                         double* part = nullptr) {
  switch (a.n - 1) {
    case 0: return launch_cp_full_r64<0>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    case 1: return launch_cp_full_r64<1>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    case 2: return launch_cp_full_r64<2>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    case 3: return launch_cp_full_r64<3>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    case 4: return launch_cp_full_r64<4>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    case 5: return launch_cp_full_r64<5>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    case 6: return launch_cp_full_r64<6>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
    default: return launch_cp_full_r64<7>(a, R, rows, cols, mask, out, vec_ok, X, part, st);
  }
}

template <typename T, int NF>
void launch_cp_full(dim3 grid, cudaStream_t st, const FullArgs& a, int R, int64_t rows,
                    int64_t cols, const T* mask, T* out, int vec_ok, const T* X, double* part) {
  if (X)
    k_cp_full<T, NF, true><<<grid, kFullThreads, 0, st>>>(a, R, rows, cols, mask, out, vec_ok, X,
                                                          part);
  else
    k_cp_full<T, NF, false><<<grid, kFullThreads, 0, st>>>(a, R, rows, cols, mask, out, vec_ok,
                                                           X, part);
}

template <typename T>
void dispatch_cp_full(dim3 grid, cudaStream_t st, const FullArgs& a, int R, int64_t rows,
                      int64_t cols, const T* mask, T* out, int vec_ok, const T* X = nullptr,
                      double* part = nullptr) {
  switch (a.n - 1) {
    case 0: launch_cp_full<T, 0>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    case 1: launch_cp_full<T, 1>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    case 2: launch_cp_full<T, 2>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    case 3: launch_cp_full<T, 3>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    case 4: launch_cp_full<T, 4>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    case 5: launch_cp_full<T, 5>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    case 6: launch_cp_full<T, 6>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
    default: launch_cp_full<T, 7>(grid, st, a, R, rows, cols, mask, out, vec_ok, X, part); break;
  }
}

// Mode-n unfolding (dir 0) and folding (dir 1) of a C-order tensor:
// unfold(X, n)[i_n, j] = X[..., i_n, ...], j the C-order flat index of the
// other modes in their order (moveaxis(X, n, 0).reshape(I_n, -1)).  Element e
// of the tensor in C order is (pre, i_n, post); its unfolded position is
// i_n * (pre_size * post_size) + pre * post_size + post.  The tensor side is
// walked in C order, so runs of post_size elements are contiguous on both
// sides.
template <typename T>
__global__ void k_unfold(const T* __restrict__ src, T* __restrict__ dst, int64_t pre_size,
                         int64_t n_size, int64_t post_size, int dir) {
  const int64_t total = pre_size * n_size * post_size;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t post = e % post_size;
    const int64_t t = e / post_size;
    const int64_t in = t % n_size;
    const int64_t pre = t / n_size;
    const int64_t u = (in * pre_size + pre) * post_size + post;
    if (dir == 0) dst[u] = src[e];
    else dst[e] = src[u];
  }
}

// ||X - [[w; A]]|| from the CTA partial sums, in a fixed order.
__global__ void k_resid_final(const double* __restrict__ part, int64_t n, double* out) {
  double v = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += kFullThreads) v += part[i];
  __shared__ double tot;
  block_sum_to(v, &tot);
  __syncthreads();
  if (threadIdx.x == 0) out[0] = sqrt(tot);
}

}  // namespace

int cp_full_check(int dtype, int ndim, const int64_t* shape, int64_t rank) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "cp_to_tensor: dtype must be f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "cp_to_tensor: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(shape != nullptr, "cp_to_tensor: null shape");
  TLGB_CHECK_ARG(rank >= 1 && rank <= (int64_t)1 << 30, "cp_to_tensor: bad rank");
  for (int k = 0; k < ndim; ++k)
    TLGB_CHECK_ARG(shape[k] >= 0 && shape[k] <= INT32_MAX, "cp_to_tensor: bad mode size");
  return TLGB_OK;
}

static int64_t cp_full_rp(int64_t rank) { return ceil_div(rank, (int64_t)8) * 8; }
static int64_t cp_full_ld0(int64_t rows) { return ceil_div(rows, (int64_t)kFullTM) * kFullTM; }

// Transposed factors, then one double per CTA for the residual sums.
size_t cp_full_ws_bytes(int dtype, int ndim, const int64_t* shape, int64_t rank) {
  const size_t elem = dtype == TLGB_F64 ? 8 : 4;
  size_t b = align_up((size_t)cp_full_rp(rank) * (size_t)cp_full_ld0(shape[0]) * elem, 256);
  int64_t cols = 1;
  for (int k = 1; k < ndim; ++k) {
    b += align_up((size_t)shape[k] * (size_t)rank * elem, 256);
    cols *= shape[k];
  }
  b += align_up(sizeof(double) * (size_t)(ceil_div(cols, (int64_t)kFullTN) *
                                          ceil_div(shape[0], (int64_t)kFullTM)), 256);
  return std::max<size_t>(b, 256);
}

int cp_full_run(int dtype, int ndim, const int64_t* shape, int64_t rank,
                const void* const* factors, const void* weights, const void* mask, void* out,
                const void* X, double* resid, void* workspace, size_t workspace_bytes,
                cudaStream_t st) {
  int rc = cp_full_check(dtype, ndim, shape, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(factors && (out || (X && resid)), "cp_to_tensor: null pointer");
  int64_t cols = 1;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(factors[k] != nullptr || shape[k] == 0, "cp_to_tensor: null factor");
    if (k > 0) cols *= shape[k];
  }
  const int64_t rows = shape[0];
  if (rows == 0 || cols == 0) {
    if (resid) TLGB_CUDA_TRY(cudaMemsetAsync(resid, 0, sizeof(double), st));
    return TLGB_OK;
  }
  if (!workspace || workspace_bytes < cp_full_ws_bytes(dtype, ndim, shape, rank))
    return set_error(TLGB_EWORKSPACE, "cp_to_tensor: workspace too small");
  const int64_t gx = ceil_div(cols, (int64_t)kFullTN), gy = ceil_div(rows, (int64_t)kFullTM);
  TLGB_CHECK_ARG(gx <= INT32_MAX && gy <= 65535, "cp_to_tensor: tensor too large");
  const size_t elem = dtype == TLGB_F64 ? 8 : 4;
  TransArgs t{};
  FullArgs a{};
  t.n = a.n = ndim;
  t.ld0 = a.ld0 = cp_full_ld0(rows);
  t.rp = (int)cp_full_rp(rank);
  char* ws = static_cast<char*>(workspace);
  size_t off = 0;
  t.start[0] = 0;
  for (int k = 0; k < ndim; ++k) {
    t.f[k] = factors[k];
    t.ft[k] = ws + off;
    a.ft[k] = ws + off;
    t.dim[k] = a.dim[k] = shape[k];
    const int64_t n_el = k == 0 ? (int64_t)t.rp * t.ld0 : shape[k] * rank;
    t.start[k + 1] = t.start[k] + n_el;
    off += align_up((size_t)n_el * elem, 256);
  }
  double* part = reinterpret_cast<double*>(ws + off);
  const bool res = X != nullptr;
  const int vec_ok = !res && (cols % 4 == 0) && ((reinterpret_cast<uintptr_t>(out) & 15) == 0) &&
                     (!mask || (reinterpret_cast<uintptr_t>(mask) & 15) == 0);
  const unsigned tb = (unsigned)std::min<int64_t>(ceil_div(t.start[ndim], (int64_t)256), 152 * 8);
  dim3 grid((unsigned)gx, (unsigned)gy);
  int64_t nparts = gx * gy;
  if (dtype == TLGB_F32) {
    k_transpose_factors<float><<<tb, 256, 0, st>>>(t, static_cast<const float*>(weights),
                                                   (int)rank);
    TLGB_LAUNCH_CHECK();
    const float* xf = static_cast<const float*>(X);
    if (rank <= kFastRank) {
      int64_t rgx, rgy;
      int tpc;
      r64_grid(a.ld0, cols, &rgx, &rgy, &tpc);
      nparts = rgx * rgy;
      rc = dispatch_cp_full_r64(a, (int)rank, rows, cols, static_cast<const float*>(mask),
                                static_cast<float*>(out), vec_ok, st, xf, res ? part : nullptr);
      if (rc) return rc;
    } else {
      dispatch_cp_full<float>(grid, st, a, (int)rank, rows, cols,
                              static_cast<const float*>(mask), static_cast<float*>(out), vec_ok,
                              xf, res ? part : nullptr);
    }
  } else {
    k_transpose_factors<double><<<tb, 256, 0, st>>>(t, static_cast<const double*>(weights),
                                                    (int)rank);
    TLGB_LAUNCH_CHECK();
    dispatch_cp_full<double>(grid, st, a, (int)rank, rows, cols,
                             static_cast<const double*>(mask), static_cast<double*>(out), vec_ok,
                             static_cast<const double*>(X), res ? part : nullptr);
  }
  TLGB_LAUNCH_CHECK();
  if (res) {
    k_resid_final<<<1, kFullThreads, 0, st>>>(part, nparts, resid);
    TLGB_LAUNCH_CHECK();
  }
  return TLGB_OK;
}

}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_cp_to_tensor_workspace_size(int dtype, int ndim, const int64_t* shape,
                                                int64_t rank, size_t* bytes) {
  clear_error();
  int rc = cp_full_check(dtype, ndim, shape, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(bytes != nullptr, "cp_to_tensor_workspace_size: null bytes");
  *bytes = cp_full_ws_bytes(dtype, ndim, shape, rank);
  return TLGB_OK;
}

extern "C" int tlgb_cp_to_tensor(int dtype, int ndim, const int64_t* shape, int64_t rank,
                                 const void* const* factors, const void* weights,
                                 const void* mask, void* out, void* workspace,
                                 size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(out != nullptr, "cp_to_tensor: null output");
  return cp_full_run(dtype, ndim, shape, rank, factors, weights, mask, out, nullptr, nullptr,
                     workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

extern "C" int tlgb_cp_residual_norm(int dtype, const void* X, int ndim, const int64_t* shape,
                                     int64_t rank, const void* const* factors,
                                     const void* weights, double* out, void* workspace,
                                     size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(X && out, "cp_residual_norm: null pointer");
  return cp_full_run(dtype, ndim, shape, rank, factors, weights, nullptr, nullptr, X, out,
                     workspace, workspace_bytes, static_cast<cudaStream_t>(stream));
}

static int unfold_common(int dtype, const void* src, int ndim, const int64_t* shape, int mode,
                         void* dst, void* stream, int dir) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "unfold: dtype must be f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "unfold: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(shape && src && dst, "unfold: null pointer");
  TLGB_CHECK_ARG(mode >= 0 && mode < ndim, "unfold: mode out of range");
  int64_t pre = 1, post = 1;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(shape[k] >= 0, "unfold: negative mode size");
    if (k < mode) pre *= shape[k];
    if (k > mode) post *= shape[k];
  }
  const int64_t total = pre * shape[mode] * post;
  if (total == 0) return TLGB_OK;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned blocks = (unsigned)std::min<int64_t>(ceil_div(total, (int64_t)256), 152 * 16);
  if (dtype == TLGB_F32)
    k_unfold<float><<<blocks, 256, 0, st>>>(static_cast<const float*>(src),
                                            static_cast<float*>(dst), pre, shape[mode], post, dir);
  else
    k_unfold<double><<<blocks, 256, 0, st>>>(static_cast<const double*>(src),
                                             static_cast<double*>(dst), pre, shape[mode], post,
                                             dir);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_unfold(int dtype, const void* X, int ndim, const int64_t* shape, int mode,
                           void* out, void* stream) {
  clear_error();
  return unfold_common(dtype, X, ndim, shape, mode, out, stream, 0);
}

extern "C" int tlgb_fold(int dtype, const void* unfolded, int ndim, const int64_t* shape,
                         int mode, void* out, void* stream) {
  clear_error();
  return unfold_common(dtype, unfolded, ndim, shape, mode, out, stream, 1);
}
