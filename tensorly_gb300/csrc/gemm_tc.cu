// Dense f32 GEMM on the tensor cores (tcgen05 + TMA, sm_103a) for the
// learned warm start's network (forward, backward and inference products):
//   C(m, n) = epi(sum_k A(m, k) B(k, n)),  A(m, k) = A[m sam + k sak],
//   B(k, n) = B[k sbk + n sbn] (any strides), epilogue + bias[n], ReLU,
//   times (mask(m, n) > 0).
// Both operands are split exactly into three bf16 planes, v = v0 + v1 + v2
// (v0 = bf16(v), v1 = bf16(v - v0), v2 = bf16(v - v0 - v1)), stored K-major by
// a split kernel that also transposes (so the MMA reads both operands K-major
// whatever the caller's strides), and each 128 x 128 output tile accumulates
// every product a_i b_j with i + j <= 2 in TMEM with f32 accumulation; the
// dropped terms are below 2^-26 of |a||b|, so the product is f32-faithful.
//
// One CTA per output tile and K split (split-K when the tiles alone would
// leave SMs idle; the splits' raw tiles are then summed in a fixed order by
// k_gemm_reduce, which applies the epilogue), 192 threads:
//   warp 0      TMA producer: per 64-wide K step the six 128 x 64 bf16 tiles
//               (three planes of A and of B; 96 KiB) into a ring of two stages
//   warp 1      TMEM allocation (128 columns) and the single-thread MMA issue
//               (M = 128, N = 128, K = 16; twenty-four per step)
//   warps 2-5   epilogue: tcgen05.ld of the finished tile (one row per
//               thread), bias / ReLU / mask, stores
// Every mbarrier wait is bounded: on expiry the kernel records TLGB_ETIMEOUT
// in the workspace status word, stops waiting, frees its TMEM and returns.
#include <cuda_bf16.h>

#include <atomic>

#include "common.cuh"
#include "tc_ptx.cuh"

namespace tlgb {
namespace {

constexpr int kGM = 128;                       // output rows per tile (MMA M)
constexpr int kGN = 128;                       // output columns per tile (MMA N)
constexpr int kGK = 64;                        // K per step (128-byte swizzle rows)
constexpr int kGStages = 2;
constexpr int kGPlanes = 3;
constexpr int kGThreads = 192;
constexpr int kGTile = kGM * kGK * 2;          // one bf16 plane tile: 16 KiB (A and B alike)
constexpr int kGStageBytes = 2 * kGPlanes * kGTile;   // A planes, then B planes
constexpr size_t kGSmem = 1024 + (size_t)kGStages * kGStageBytes + 256;

struct GemmArgs {
  int M, N;
  int ksteps;                 // 64-wide K steps (K padded to a multiple of 8 in the planes)
  int kps;                    // K steps per split (blockIdx.z selects the split)
  float* partial;             // splits > 1: raw tiles [split][M][N], reduced by k_gemm_reduce
  float* C;
  int64_t ldc;
  const float* bias;
  int relu;
  const float* mask;
  int* err;
};

// kind::f16 instruction descriptor: f32 accumulation, bf16 A and B, both
// K-major, M = 128, N = 128.
constexpr uint32_t kGemmIdesc = (1u << 4) | (1u << 7) | (1u << 10) |
                                ((uint32_t)(kGN >> 3) << 17) | ((uint32_t)(kGM >> 4) << 24);

__global__ void __launch_bounds__(kGThreads, 1)
k_gemm_tc(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
          const GemmArgs a) {
  extern __shared__ __align__(1024) unsigned char gsm_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(gsm_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + kGStages * kGStageBytes);   // [S]
  uint64_t* empty = full + kGStages;                                               // [S]
  uint64_t* done = empty + kGStages;                                               // [1]
  uint64_t* mdrain = done + 1;                                                     // [1]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdrain + 1);
  int* ok_flag = reinterpret_cast<int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int n0 = blockIdx.x * kGN, m0 = blockIdx.y * kGM;
  const int t0 = blockIdx.z * a.kps;
  const int t1 = min(t0 + a.kps, a.ksteps);

  if (threadIdx.x == 32) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmA)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmB)) : "memory");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < kGStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(done, 1);
    mbar_init(mdrain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(kGN)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool failed = false;

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      int issued = 0;
      for (int t = t0; t < t1; ++t) {
        if (!mbar_wait(&empty[stage], phase ^ 1u, a.err, failed)) break;
        mbar_expect_tx(&full[stage], (uint32_t)kGStageBytes);
        unsigned char* dst = base + stage * kGStageBytes;
        const int k0 = t * kGK;
#pragma unroll
        for (int pl = 0; pl < kGPlanes; ++pl) {
          tma_load_3d(dst + pl * kGTile, &tmA, &full[stage], k0, m0, pl);
          tma_load_3d(dst + (kGPlanes + pl) * kGTile, &tmB, &full[stage], k0, n0, pl);
        }
        ++issued;
        if (++stage == kGStages) { stage = 0; phase ^= 1u; }
      }
      // every issued copy has landed before the CTA may exit
      const int n = issued < kGStages ? issued : kGStages;
      int st_j = stage, ph_j = (int)phase;
      for (int j = 0; j < n; ++j) {
        if (--st_j < 0) { st_j = kGStages - 1; ph_j ^= 1; }
        mbar_drain(&full[st_j], (uint32_t)ph_j);
      }
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issue
    if (lane == 0) {
      int stage = 0;
      uint32_t phase = 0;
      for (int t = t0; t < t1 && !failed; ++t) {
        if (!mbar_wait(&full[stage], phase, a.err, failed)) break;
        tc_fence_after();
        const uint32_t sb = smem_u32(base + stage * kGStageBytes);
#pragma unroll
        for (int k = 0; k < kGK / 16; ++k) {
          const uint32_t ko = (uint32_t)k * 32;
          // a_i b_j for i + j <= 2, the smallest terms first
#pragma unroll
          for (int q = 0; q < 6; ++q) {
            const int i = q < 3 ? q : (q == 3 ? 0 : (q == 4 ? 1 : 0));
            const int j = q < 3 ? 2 - q : (q == 3 ? 1 : (q == 4 ? 0 : 0));
            const uint32_t ad = sb + (uint32_t)(i * kGTile) + ko;
            const uint32_t bd = sb + (uint32_t)((kGPlanes + j) * kGTile) + ko;
            umma_bf16(tmem, smem_desc(ad, 16, 1024), smem_desc(bd, 16, 1024), kGemmIdesc,
                      (t == t0 && k == 0 && q == 0) ? 0u : 1u);
          }
        }
        umma_commit(&empty[stage]);
        if (++stage == kGStages) { stage = 0; phase ^= 1u; }
      }
      if (!failed) umma_commit(done);
      // all issued MMAs have completed before TMEM is freed
      umma_commit(mdrain);
      mbar_drain(mdrain, 0);
    }
  } else {
    // ------------------------------------------------------------ epilogue
    const int e = threadIdx.x - 64;   // 0..127
    if (e == 0) *ok_flag = mbar_wait(done, 0, a.err, failed) ? 1 : 0;
    asm volatile("bar.sync 1, 128;" ::: "memory");
    if (*ok_flag) {
      __syncwarp();
      tc_fence_after();
      const int q = warp & 3;   // TMEM lane quarter of this warp
      const int m = m0 + 32 * q + lane;
      const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16);
#pragma unroll
      for (int c = 0; c < kGN / 32; ++c) {
        uint32_t v[32];
        tmem_ld32_nowait(lane_addr + (uint32_t)(c * 32), v);
        tmem_wait_ld();
        if (m < a.M && a.partial) {   // a split's raw tile; k_gemm_reduce finishes it
          float* prow = a.partial + ((int64_t)blockIdx.z * a.M + m) * a.N;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c * 32 + j;
            if (n < a.N) prow[n] = __uint_as_float(v[j]);
          }
        } else if (m < a.M) {
          float* crow = a.C + (int64_t)m * a.ldc;
          const float* mrow = a.mask ? a.mask + (int64_t)m * a.ldc : nullptr;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            const int n = n0 + c * 32 + j;
            if (n < a.N) {
              float x = __uint_as_float(v[j]);
              if (a.bias) x += a.bias[n];
              if (a.relu) x = fmaxf(x, 0.f);
              if (mrow && !(mrow[n] > 0.f)) x = 0.f;
              crow[n] = x;
            }
          }
        }
      }
    }
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kGN)
                 : "memory");
  }
}

// C(m, n) = epi(sum over splits of partial[split][m][n]), in split order.
__global__ void k_gemm_reduce(const float* __restrict__ partial, int splits, int M, int N,
                              float* __restrict__ C, int64_t ldc, const float* __restrict__ bias,
                              int relu, const float* __restrict__ mask) {
  const int64_t n_el = (int64_t)M * N;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n_el;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int m = (int)(e / N), n = (int)(e - (e / N) * N);
    float x = 0.f;
    for (int s = 0; s < splits; ++s) x += partial[(int64_t)s * n_el + e];
    if (bias) x += bias[n];
    if (relu) x = fmaxf(x, 0.f);
    if (mask && !(mask[(int64_t)m * ldc + n] > 0.f)) x = 0.f;
    C[(int64_t)m * ldc + n] = x;
  }
}

// out[p][r][k] (the three exact bf16 planes; K-major, row length kp) from
// src(r, k) = src[r * s_r + k * s_k] for r < rows, k < K; zero for K <= k < kp.
__global__ void k_gemm_split(const float* __restrict__ src, int rows, int K, int kp,
                             int64_t s_r, int64_t s_k, __nv_bfloat16* __restrict__ out) {
  const int64_t n = (int64_t)rows * kp, plane = n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int r = (int)(e / kp), k = (int)(e - (e / kp) * kp);
    const float v = k < K ? src[r * s_r + k * s_k] : 0.f;
    const __nv_bfloat16 p0 = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(p0);
    const __nv_bfloat16 p1 = __float2bfloat16_rn(r1);
    out[e] = p0;
    out[plane + e] = p1;
    out[2 * plane + e] = __float2bfloat16_rn(r1 - __bfloat162float(p1));
  }
}

int64_t kpad(int K) { return ((int64_t)K + 7) / 8 * 8; }

struct GemmLayout {
  size_t a_off, b_off, p_off, bytes;
  int ksteps, splits, kps;
};
// Split-K when the output has fewer tiles than SMs: splits of the K steps
// over blockIdx.z bring the grid to about one CTA per SM (small products).
GemmLayout gemm_layout(int M, int N, int K) {
  GemmLayout L{};
  const int64_t kp = kpad(K);
  L.ksteps = (int)ceil_div(kp, (int64_t)kGK);
  const int64_t tiles = ceil_div((int64_t)M, (int64_t)kGM) * ceil_div((int64_t)N, (int64_t)kGN);
  const int want = (int)std::max<int64_t>(1, std::min<int64_t>(L.ksteps, sm_count() / tiles));
  L.kps = (int)ceil_div((int64_t)L.ksteps, (int64_t)want);
  L.splits = (int)ceil_div((int64_t)L.ksteps, (int64_t)L.kps);
  L.a_off = 256;   // the status word first
  L.b_off = L.a_off + align_up(sizeof(__nv_bfloat16) * kGPlanes * (size_t)M * kp, 256);
  L.p_off = L.b_off + align_up(sizeof(__nv_bfloat16) * kGPlanes * (size_t)N * kp, 256);
  L.bytes = L.p_off + (L.splits > 1 ? align_up(sizeof(float) * L.splits * (size_t)M * N, 256) : 0);
  return L;
}

int encode_planes(CUtensorMap* map, const __nv_bfloat16* planes, int rows, int64_t kp) {
  auto enc = tma_encode_fn();
  if (!enc) return set_error(TLGB_EUNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  const cuuint64_t dim[3] = {(cuuint64_t)kp, (cuuint64_t)rows, (cuuint64_t)kGPlanes};
  const cuuint64_t stride[2] = {(cuuint64_t)kp * 2, (cuuint64_t)kp * 2 * rows};
  const cuuint32_t box[3] = {(cuuint32_t)kGK, (cuuint32_t)kGM, 1};
  const cuuint32_t estride[3] = {1, 1, 1};
  CUresult cr = enc(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3,
                    const_cast<__nv_bfloat16*>(planes), dim, stride, box, estride,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(TLGB_ECUDA, "gemm_tc: tensor map encoding failed");
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_ws_gemm_tc_workspace_size(int M, int N, int K, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(M >= 1 && N >= 1 && K >= 1 && bytes, "ws_gemm_tc: bad argument");
  *bytes = gemm_layout(M, N, K).bytes;
  return TLGB_OK;
}

extern "C" int tlgb_ws_gemm_tc(int M, int N, int K, const void* A, int64_t sam, int64_t sak,
                               const void* B, int64_t sbk, int64_t sbn, void* C, int64_t ldc,
                               const void* bias, int relu, const void* mask, void* workspace,
                               size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(A && B && C && M >= 1 && N >= 1 && K >= 1 && ldc >= N,
                 "ws_gemm_tc: bad argument");
  TLGB_CHECK_ARG(ceil_div((int64_t)M, (int64_t)kGM) <= 65535 && N <= (1 << 30),
                 "ws_gemm_tc: too many rows");
  const GemmLayout L = gemm_layout(M, N, K);
  if (!workspace || workspace_bytes < L.bytes ||
      (reinterpret_cast<uintptr_t>(workspace) & 255) != 0)
    return set_error(TLGB_EWORKSPACE, "ws_gemm_tc: workspace too small or misaligned");
  static std::atomic<bool> attr[64];   // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_gemm_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kGSmem));
    attr[dev] = true;
  }
  char* ws = static_cast<char*>(workspace);
  __nv_bfloat16* ap = reinterpret_cast<__nv_bfloat16*>(ws + L.a_off);
  __nv_bfloat16* bp = reinterpret_cast<__nv_bfloat16*>(ws + L.b_off);
  const int64_t kp = kpad(K);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const int sb = sm_count() * 4;
  k_gemm_split<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div((int64_t)M * kp, 256), sb)),
                 256, 0, st>>>(static_cast<const float*>(A), M, K, (int)kp, sam, sak, ap);
  TLGB_LAUNCH_CHECK();
  k_gemm_split<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div((int64_t)N * kp, 256), sb)),
                 256, 0, st>>>(static_cast<const float*>(B), N, K, (int)kp, sbn, sbk, bp);
  TLGB_LAUNCH_CHECK();
  CUtensorMap ma, mb;
  int rc = encode_planes(&ma, ap, M, kp);
  if (rc) return rc;
  rc = encode_planes(&mb, bp, N, kp);
  if (rc) return rc;
  GemmArgs g{};
  g.M = M;
  g.N = N;
  g.ksteps = L.ksteps;
  g.kps = L.kps;
  g.partial = L.splits > 1 ? reinterpret_cast<float*>(ws + L.p_off) : nullptr;
  g.C = static_cast<float*>(C);
  g.ldc = ldc;
  g.bias = static_cast<const float*>(bias);
  g.relu = relu;
  g.mask = static_cast<const float*>(mask);
  g.err = reinterpret_cast<int*>(ws);
  dim3 grid((unsigned)ceil_div((int64_t)N, (int64_t)kGN), (unsigned)ceil_div((int64_t)M, (int64_t)kGM),
            (unsigned)L.splits);
  k_gemm_tc<<<grid, kGThreads, kGSmem, st>>>(ma, mb, g);
  TLGB_LAUNCH_CHECK();
  if (L.splits > 1) {
    const int64_t n_el = (int64_t)M * N;
    k_gemm_reduce<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n_el, 256), sm_count() * 8)),
                    256, 0, st>>>(g.partial, L.splits, M, N, g.C, ldc, g.bias, relu, g.mask);
    TLGB_LAUNCH_CHECK();
  }
  return TLGB_OK;
}
