// BF16 tensor-core MTTKRP for sm_103a: TMA-staged tcgen05 GEMM of the tensor
// against the inner factor, accumulated in TMEM, and an epilogue that scales
// each outer slice's 128 x R tile by the Khatri-Rao row of the remaining
// factors and sums it in registers.  The Khatri-Rao product is never formed.
//
// Formulation (same as the SIMT path, mttkrp_simt.cuh):
//   M(i, r) = sum_o s(o, r) * sum_c X[o, i, c] * F(c, r)
//   c = inner mode (N-1, or N-2 when the output mode is N-1), F its factor,
//   s(o, r) = w_r * prod_{outer k} A_k(i_k, r)  (f32, from the f32 factors).
//
// One CTA owns one 128-row output tile and a contiguous range of the
// flattened (o, 64-wide c chunk) steps of that tile.  Warp roles:
//   warp 0      TMA producer: the inner factor (bf16 hi/lo split, K-major)
//               once, then one 128 x 64 tensor tile per step into a ring of
//               3-12 stages (as many as shared memory leaves room for)
//   warp 1      TMEM allocation and the single-thread tcgen05.mma issue
//               (M = 128, N = 2 x padded rank, K = 16, four per step) into one
//               of two TMEM accumulators (double buffered across outer slices)
//   warps 2-5   epilogue: tcgen05.ld of the finished slice, scale by s(o, :),
//               accumulate one output row per thread in registers; finally
//               write the CTA's partial tile (summed in a fixed order later)
// Every mbarrier wait is bounded (about 2 s of wall time): on expiry the
// kernel records TLGB_ETIMEOUT in *err, stops waiting, frees its TMEM and
// returns, so a broken pipeline can never hang the GPU.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "mttkrp_tc.cuh"
#include "tc_ptx.cuh"

namespace tlgb {
namespace {

constexpr int kMaxStages = 12;
constexpr int kMinStages = 3;
constexpr int kTileM = 128;
constexpr int kChunk = 64;                       // bf16 elements per 128-byte swizzle row
constexpr int kStageBytes = kTileM * kChunk * 2;  // 16 KiB
constexpr int kSmemBudget = 225 * 1024;          // dynamic shared memory used at most
constexpr int kThreads = 192;

struct TcArgs {
  int stages;                 // depth of the tensor-tile ring
  const float* outer_f[kMaxModes];
  int64_t outer_dim[kMaxModes];
  int n_outer;
  int64_t g2;                 // size of TMA dim 2 (faster outer run)
  const float* weights;
  int R;
  int64_t I_out;
  int kc_total;               // 64-wide chunks of the inner mode
  int kcg;                    // chunks per inner-mode group (blockIdx.y selects the group)
  int64_t O;                  // outer slices
  int64_t steps_per_split;    // (o, chunk) steps per CTA within a group
  int gsplits;                // CTAs per (output tile, group)
  float* partial;
  int* err;
  const int* skip;
  // Test of the timeout path (tuning key "tc_test_starve"): the producer
  // issues no copies, and the MMA and epilogue waits give up after 1 ms.
  int starve;
  int l2_stream;   // tensor tiles loaded with an evict-first L2 policy
};
constexpr unsigned long long kStarveWaitNs = 1000000ull;  // 1 ms

// Instruction descriptor, kind::f16: f32 accumulate, bf16 A and B, B K-major,
// A K-major (a_mn = 0) or MN-major (a_mn = 1), M = 128, N = n (<= 256).
__host__ __device__ constexpr uint32_t make_idesc(int n, int a_mn) {
  return (1u << 4)                      // D format f32
         | (1u << 7)                    // A bf16
         | (1u << 10)                   // B bf16
         | ((uint32_t)a_mn << 15)       // A major
         | (0u << 16)                   // B K-major
         | ((uint32_t)(n >> 3) << 17)   // N / 8
         | ((uint32_t)(kTileM >> 4) << 24);  // M / 16
}

// TMEM columns of one accumulator buffer (a power of two >= the MMA N).
__host__ __device__ constexpr int tmem_stride(int nb) {
  return nb <= 32 ? 32 : nb <= 64 ? 64 : nb <= 128 ? 128 : nb <= 256 ? 256 : 512;
}

// B operand = the first NPL bf16 planes of the inner factor, F = f0 + f1 + f2
// with f0 = bf16(F), f1 = bf16(F - f0), f2 = bf16(F - f0 - f1), stacked as
// NPL*RP rows, so one MMA with N = NPL*RP forms X.f0, X.f1, ... side by side
// in TMEM and the epilogue adds them.
//  * bf16 sweeps: NPL = 2, the factor enters with ~16 mantissa bits (with a
//    single bf16 rounding of the factor, ALS stalls at a worse stationary
//    point in swamp phases; rounding only the tensor to bf16 does not).
//  * f32-faithful MTTKRP: the f32 tensor is split exactly into x0 + x1 + x2
//    (same construction) and contracted in three launches, x0 with NPL = 3,
//    x1 with NPL = 2, x2 with NPL = 1: every product x_i f_j with i + j <= 2.
//    The dropped terms are below 2^-26 of |x||f|, under one f32 rounding.
template <int RP, bool MN, int NPL>
__global__ void __launch_bounds__(kThreads, RP <= 64 ? 2 : 1)   // RP <= 64: at most 168 registers
mttkrp_tc_kernel(const __grid_constant__ CUtensorMap tmX, const __grid_constant__ CUtensorMap tmF,
                 const TcArgs a) {
  constexpr int NB = NPL * RP;             // MMA N (one RP-wide block per factor plane)
  constexpr int TS = tmem_stride(NB);      // TMEM columns per accumulator buffer
  static_assert(NB <= 256 && 2 * TS <= 512, "accumulators exceed one MMA or TMEM");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  const int S = a.stages;
  unsigned char* sA = base;                                   // S x 16 KiB
  unsigned char* sB = sA + S * kStageBytes;                   // KC x NB x 128 B
  const int split = blockIdx.x;
  const int cg = blockIdx.y;                                  // inner-mode group
  const int64_t m0 = (int64_t)blockIdx.z * kTileM;
  const int kc0 = cg * a.kcg;
  const int KC = min(a.kcg, a.kc_total - kc0);                // chunks of this group
  const int b_bytes = KC * NB * 128;
  uint64_t* full = reinterpret_cast<uint64_t*>(sB + b_bytes); // [S]
  uint64_t* empty = full + kMaxStages;                        // [S]
  uint64_t* dfull = empty + kMaxStages;   // [2]
  uint64_t* dempty = dfull + 2;           // [2]
  uint64_t* bfull = dempty + 2;           // [1]
  uint64_t* mdrain = bfull + 1;           // [1] MMA completion before teardown
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mdrain + 1);
  int* ep_ok = reinterpret_cast<int*>(tmem_slot + 1);         // [2] epilogue wait outcome
  int* s_skip = reinterpret_cast<int*>(tmem_slot + 3);        // the epilogue's stop flag
  float* s_sm = reinterpret_cast<float*>(tmem_slot + 4);      // [2][RP]

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t t_begin = (int64_t)split * a.steps_per_split;
  const int64_t t_end = min(t_begin + a.steps_per_split, a.O * KC);
  // partial tile index: every (group, split) CTA of an output tile writes its own
  const int64_t pidx = (int64_t)cg * a.gsplits + split;

  if (threadIdx.x == 32) {
    // the tensor maps live in parameter space: fetch them while the CTA sets up
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmX)) : "memory");
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(&tmF)) : "memory");
  }
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&dfull[b], 1);
      mbar_init(&dempty[b], 128);
    }
    mbar_init(bfull, 1);
    mbar_init(mdrain, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(2 * TS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  bool failed = false;
  // The next kernel of the stream may be scheduled now.  Everything below
  // that reads an earlier kernel's output (the factors, the stop flag) or
  // writes the partial tiles (which the previous solve reads) comes after
  // griddep_wait(); only the tensor tiles of the first ring stages are
  // fetched before it (the tensor is never written during a run).
  griddep_launch_dependents();

  if (t_begin < t_end) {
    if (warp == 0) {
      // ------------------------------------------------------------ producer
      if (lane == 0) {
        // Coordinates advance incrementally (no 64-bit division per step:
        // this single thread's issue rate bounds the whole CTA's bandwidth).
        const int64_t o0 = t_begin / KC;
        int kc = (int)(t_begin - o0 * KC);
        int c2 = (int)(o0 % a.g2), c3 = (int)(o0 / a.g2);
        int stage = 0;
        uint32_t phase = 0;
        int64_t i = 0;
        const uint64_t pol = l2_policy_evict_first();
        auto issue = [&]() -> bool {   // the tensor tile of the next step
          if (!mbar_wait(&empty[stage], phase ^ 1u, a.err, failed)) return false;
          mbar_expect_tx(&full[stage], kStageBytes);
          unsigned char* dst = sA + stage * kStageBytes;
          const int cx = (kc0 + kc) * kChunk;
          if (a.l2_stream) {
            if (!MN) {
              tma_load_4d_hint(dst, &tmX, &full[stage], cx, (int)m0, c2, c3, pol);
            } else {
              tma_load_4d_hint(dst, &tmX, &full[stage], (int)m0, cx, c2, c3, pol);
              tma_load_4d_hint(dst + kStageBytes / 2, &tmX, &full[stage], (int)m0 + 64, cx, c2,
                               c3, pol);
            }
          } else if (!MN) {
            tma_load_4d(dst, &tmX, &full[stage], cx, (int)m0, c2, c3);
          } else {
            tma_load_4d(dst, &tmX, &full[stage], (int)m0, cx, c2, c3);
            tma_load_4d(dst + kStageBytes / 2, &tmX, &full[stage], (int)m0 + 64, cx, c2, c3);
          }
          if (++kc == KC) {
            kc = 0;
            if (++c2 == a.g2) { c2 = 0; ++c3; }
          }
          if (++stage == S) { stage = 0; phase ^= 1u; }
          ++i;
          return true;
        };
        const int64_t pre = a.starve ? 0 : min((int64_t)S, t_end - t_begin);
        int64_t t = t_begin;
        for (; t < t_begin + pre; ++t)
          if (!issue()) break;
        griddep_wait();
        const bool skipped = a.skip && *a.skip;
        if (!skipped && !failed && !a.starve) {
          mbar_expect_tx(bfull, (uint32_t)b_bytes);
          for (int kcb = 0; kcb < KC; ++kcb) {
            unsigned char* dst = sB + kcb * NB * 128;
#pragma unroll
            for (int pl = 0; pl < NPL; ++pl)   // rows of factor plane pl
              tma_load_3d(dst + pl * RP * 128, &tmF, bfull, (kc0 + kcb) * kChunk, 0, pl);
          }
          for (; t < t_end; ++t)
            if (!issue()) break;
          // every issued copy has landed before the CTA may exit
          mbar_drain(bfull, 0);
        }
        {
          const int n = (int)(i < S ? i : S);
          int st_j = stage, ph_j = (int)phase;   // walk back over the last n issued steps
          for (int j = 0; j < n; ++j) {
            if (--st_j < 0) { st_j = S - 1; ph_j ^= 1; }
            mbar_drain(&full[st_j], (uint32_t)ph_j);
          }
        }
      }
    } else if (warp == 1) {
      // ------------------------------------------------------------ MMA issue
      griddep_wait();
      const bool skipped = a.skip && *a.skip;
      const unsigned long long lim = a.starve ? kStarveWaitNs : kWaitNs;
      if (lane == 0 && !skipped) {
        constexpr uint32_t idesc = make_idesc(NB, MN ? 1 : 0);
        mbar_wait(bfull, 0, a.err, failed, lim);
        int64_t oc = 0;
        int kc = (int)(t_begin % KC);
        int stage = 0;
        uint32_t phase = 0;
        for (int64_t t = t_begin; t < t_end && !failed; ++t) {
          const bool first_of_o = (t == t_begin) || (kc == 0);
          const bool last_of_o = (t + 1 == t_end) || (kc == KC - 1);
          const int buf = (int)(oc & 1);
          if (first_of_o) {
            if (!mbar_wait(&dempty[buf], (uint32_t)(((oc >> 1) & 1) ^ 1), a.err, failed, lim))
              break;
            tc_fence_after();
          }
          if (!mbar_wait(&full[stage], phase, a.err, failed, lim)) break;
          tc_fence_after();
          const uint32_t a_base = smem_u32(sA + stage * kStageBytes);
          const uint32_t b_base = smem_u32(sB + kc * NB * 128);
          const uint32_t d = tmem + (uint32_t)(buf * TS);
#pragma unroll
          for (int k = 0; k < kChunk / 16; ++k) {
            const uint64_t adesc = MN ? smem_desc(a_base + k * 2048, kStageBytes / 2, 1024)
                                      : smem_desc(a_base + k * 32, 16, 1024);
            const uint64_t bdesc = smem_desc(b_base + k * 32, 16, 1024);
            umma_bf16(d, adesc, bdesc, idesc, (first_of_o && k == 0) ? 0u : 1u);
          }
          umma_commit(&empty[stage]);
          if (last_of_o) {
            umma_commit(&dfull[buf]);
            ++oc;
          }
          if (++kc == KC) kc = 0;
          if (++stage == S) { stage = 0; phase ^= 1u; }
        }
        // all issued MMAs have completed before TMEM is freed
        umma_commit(mdrain);
        mbar_drain(mdrain, 0);
      }
    } else {
      // ------------------------------------------------------------ epilogue
      griddep_wait();   // the scales read the factors; the partial tiles are rewritten
      // one read of the stop flag for the four epilogue warps, which meet at
      // named barriers below (the flag is stable while this kernel runs)
      if (threadIdx.x == 64) *s_skip = (a.skip && *a.skip) ? 1 : 0;
      asm volatile("bar.sync 1, 128;" ::: "memory");
      const bool skip_ep = *s_skip != 0;
      if (!skip_ep) {
        const int e = threadIdx.x - 64;            // 0..127
        const int q = warp & 3;                    // TMEM lane quarter of this warp
        const int row = 32 * q + lane;
        float acc[RP];
#pragma unroll
        for (int r = 0; r < RP; ++r) acc[r] = 0.f;
        const int64_t o_first = t_begin / KC, o_last = (t_end - 1) / KC;
        // s(o, r) = w_r * prod_{outer k} A_k(i_k, r) for r = e (one entry per thread)
        // outer multi-index of the next slice, advanced with carries (no division)
        int64_t nidx[kMaxModes];
        {
          int64_t rem = o_first;
          for (int k = a.n_outer - 1; k >= 0; --k) {
            nidx[k] = rem % a.outer_dim[k];
            rem /= a.outer_dim[k];
          }
        }
        auto scale_of = [&](int64_t) -> float {
          float s = 0.f;
          if (e < a.R) {
            s = a.weights ? a.weights[e] : 1.f;
            for (int k = 0; k < a.n_outer; ++k) s *= a.outer_f[k][nidx[k] * a.R + e];
          }
          for (int k = a.n_outer - 1; k >= 0; --k) {
            if (++nidx[k] < a.outer_dim[k]) break;
            nidx[k] = 0;
          }
          return s;
        };
        float s_next = (e < RP) ? scale_of(o_first) : 0.f;
        bool ep_broken = false;   // a wait expired (the same value in every epilogue thread)
        int64_t oc = 0;
        for (int64_t o = o_first; o <= o_last; ++o, ++oc) {
          const int buf = (int)(oc & 1);
          if (e < RP) s_sm[buf * RP + e] = s_next;
          // the next slice's scale loads overlap this slice's TMEM traffic
          if (e < RP && o < o_last) s_next = scale_of(o + 1);
          if (e == 0)
            ep_ok[buf] = mbar_wait(&dfull[buf], (uint32_t)((oc >> 1) & 1), a.err, failed,
                                   a.starve ? kStarveWaitNs : kWaitNs) ? 1 : 0;
          asm volatile("bar.sync 1, 128;" ::: "memory");
          if (!ep_ok[buf]) { ep_broken = true; break; }  // uniform across the four epilogue warps
          __syncwarp();            // tcgen05.ld is warp-collective
          tc_fence_after();
          const uint32_t lane_addr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(buf * TS);
          if constexpr (RP >= 32) {
            // 16 columns of every plane at a time: fewer live registers, so
            // the kernel fits 168 a thread (two of its warps per SM
            // sub-partition beside a small solve CTA)
#pragma unroll
            for (int c = 0; c < RP / 16; ++c) {
              uint32_t pv[NPL][16];
#pragma unroll
              for (int pl = 0; pl < NPL; ++pl)
                tmem_ld16_nowait(lane_addr + (uint32_t)(pl * RP + c * 16), pv[pl]);
              tmem_wait_ld();
#pragma unroll
              for (int j = 0; j < 16; ++j) {
                float v = __uint_as_float(pv[NPL - 1][j]);   // smallest plane first
#pragma unroll
                for (int pl = NPL - 2; pl >= 0; --pl) v += __uint_as_float(pv[pl][j]);
                acc[c * 16 + j] = fmaf(s_sm[buf * RP + c * 16 + j], v, acc[c * 16 + j]);
              }
            }
          } else {
            float pv[NPL][16];
#pragma unroll
            for (int pl = 0; pl < NPL; ++pl) tmem_ld16(lane_addr + (uint32_t)(pl * RP), pv[pl]);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              float v = pv[NPL - 1][j];
#pragma unroll
              for (int pl = NPL - 2; pl >= 0; --pl) v += pv[pl][j];
              acc[j] = fmaf(s_sm[buf * RP + j], v, acc[j]);
            }
          }
          tc_fence_before();
          mbar_arrive(&dempty[buf]);
        }
        // The partial tile leaves through shared memory: a thread holds one
        // output row, so direct stores would put 32 rows (32 lines) in every
        // warp store.  Staged in the idle operand buffers (every MMA and copy
        // has completed once the last accumulator was read) with row stride
        // RP + 1 (conflict-free), then written with consecutive threads on
        // consecutive addresses.  The tile's rows are contiguous in `partial`.
        if (!ep_broken) {
          constexpr int SR = RP + 1;
          float* stile = reinterpret_cast<float*>(sA);
#pragma unroll
          for (int r = 0; r < RP; ++r)
            if (r < a.R) stile[row * SR + r] = acc[r];
          asm volatile("bar.sync 1, 128;" ::: "memory");
          const int rows = (int)(a.I_out - m0 < kTileM ? a.I_out - m0 : kTileM);
          const int n = rows * a.R;
          float* out = a.partial + (pidx * a.I_out + m0) * a.R;
          int rr = e / a.R, cc = e - (e / a.R) * a.R;
          const int dr = kTileM / a.R, dc = kTileM - dr * a.R;   // advance of the flat index by 128
          for (int idx = e; idx < n; idx += kTileM) {
            out[idx] = stile[rr * SR + cc];
            rr += dr;
            cc += dc;
            if (cc >= a.R) { cc -= a.R; ++rr; }
          }
        }
      }
    }
  } else if (warp >= 2) {
    // empty range: this split contributes zeros
    griddep_wait();
    const int q = warp & 3;
    const int64_t m = m0 + 32 * q + lane;
    if (m < a.I_out && !(a.skip && *a.skip))
      for (int r = 0; r < a.R; ++r) a.partial[(pidx * a.I_out + m) * a.R + r] = 0.f;
  }

  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * TS)
                 : "memory");
  }
}

__global__ void k_to_bf16(const float* __restrict__ X, int64_t n, __nv_bfloat16* __restrict__ Y) {
  const int64_t n4 = n / 4;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n4;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = reinterpret_cast<const float4*>(X)[i];
    reinterpret_cast<__nv_bfloat162*>(Y)[2 * i] = __floats2bfloat162_rn(v.x, v.y);
    reinterpret_cast<__nv_bfloat162*>(Y)[2 * i + 1] = __floats2bfloat162_rn(v.z, v.w);
  }
  for (int64_t i = n4 * 4 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    Y[i] = __float2bfloat16_rn(X[i]);
}

// Exact three-term bf16 split of an f32 tensor: x = x0 + x1 + x2 with
// x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1).  The residuals are
// exact in f32 and x2 holds the last <= 8 significant bits, so the sum is x
// (for normal numbers).
// Neumaier step of the f32 sum of squares: x*x split exactly into hi + lo.
__device__ __forceinline__ void sumsq_add(float x, float& s, float& c) {
  const float hi = x * x;
  const float lo = fmaf(x, x, -hi);
  const float t = s + hi;
  c += ((fabsf(s) >= hi) ? ((s - t) + hi) : ((hi - t) + s)) + lo;
  s = t;
}

// part (optional, gridDim.x doubles): the block's share of ||X||^2, summed
// as in the stand-alone sum-of-squares kernel, so the split's pass over X
// also gives the norm.
__global__ void __launch_bounds__(256)
k_split3_bf16(const float* __restrict__ X, int64_t n, __nv_bfloat16* __restrict__ y0,
              __nv_bfloat16* __restrict__ y1, __nv_bfloat16* __restrict__ y2, double* part) {
  float s = 0.f, c = 0.f;
  // four elements an iteration (16-byte loads, 8-byte stores a plane) when
  // every pointer allows it, else two
  const bool v4 = ((reinterpret_cast<uintptr_t>(X) & 15) | (reinterpret_cast<uintptr_t>(y0) & 7) |
                   (reinterpret_cast<uintptr_t>(y1) & 7) |
                   (y2 ? (reinterpret_cast<uintptr_t>(y2) & 7) : 0)) == 0;
  const int W = v4 ? 4 : 2;
  const int64_t nv = n / W;
  auto split2 = [&](float x, float y, __nv_bfloat162& a0, __nv_bfloat162& a1,
                    __nv_bfloat162& a2) {
    a0 = __floats2bfloat162_rn(x, y);
    const float2 r1 = make_float2(x - __low2float(a0), y - __high2float(a0));
    a1 = __floats2bfloat162_rn(r1.x, r1.y);
    a2 = __floats2bfloat162_rn(r1.x - __low2float(a1), r1.y - __high2float(a1));
  };
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nv;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (v4) {
      const float4 v = reinterpret_cast<const float4*>(X)[i];
      if (part) {
        sumsq_add(v.x, s, c);
        sumsq_add(v.y, s, c);
        sumsq_add(v.z, s, c);
        sumsq_add(v.w, s, c);
      }
      __nv_bfloat162 p0, p1, p2, q0, q1, q2;
      split2(v.x, v.y, p0, p1, p2);
      split2(v.z, v.w, q0, q1, q2);
      auto pack = [](__nv_bfloat162 lo, __nv_bfloat162 hi) {
        return make_uint2(*reinterpret_cast<const unsigned*>(&lo),
                          *reinterpret_cast<const unsigned*>(&hi));
      };
      reinterpret_cast<uint2*>(y0)[i] = pack(p0, q0);
      reinterpret_cast<uint2*>(y1)[i] = pack(p1, q1);
      if (y2) reinterpret_cast<uint2*>(y2)[i] = pack(p2, q2);   // the third plane is optional
    } else {
      const float2 v = reinterpret_cast<const float2*>(X)[i];
      if (part) {
        sumsq_add(v.x, s, c);
        sumsq_add(v.y, s, c);
      }
      __nv_bfloat162 p0, p1, p2;
      split2(v.x, v.y, p0, p1, p2);
      reinterpret_cast<__nv_bfloat162*>(y0)[i] = p0;
      reinterpret_cast<__nv_bfloat162*>(y1)[i] = p1;
      if (y2) reinterpret_cast<__nv_bfloat162*>(y2)[i] = p2;
    }
  }
  // the last n mod W elements, one a thread of block 0
  if (blockIdx.x == 0 && threadIdx.x < n - nv * W) {
    const int64_t e = nv * W + threadIdx.x;
    const float x = X[e];
    const __nv_bfloat16 a0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(a0);
    const __nv_bfloat16 a1 = __float2bfloat16_rn(r1);
    y0[e] = a0;
    y1[e] = a1;
    if (y2) y2[e] = __float2bfloat16_rn(r1 - __bfloat162float(a1));
    if (part) sumsq_add(x, s, c);
  }
  if (part) {   // block total in a fixed order
    __shared__ double red[8];
    double t = (double)s + (double)c;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x == 0) {
      double b = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) b += red[w];
      part[blockIdx.x] = b;
    }
  }
}

// Transposed bf16 split of a factor into `planes` (2 or 3) planes, each
// R x rows: out[0] = bf16(A^T), out[1] = bf16(A^T - out[0]),
// out[2] = bf16(A^T - out[0] - out[1]).
__global__ void k_factor_bf16t(const float* __restrict__ A, int64_t rows, int64_t R, int planes,
                               __nv_bfloat16* __restrict__ out) {
  const int64_t n = rows * R;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / R, r = e % R;
    const float x = A[e];
    const __nv_bfloat16 p0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p0);
    const __nv_bfloat16 p1 = __float2bfloat16_rn(r1);
    out[r * rows + i] = p0;
    out[n + r * rows + i] = p1;
    if (planes > 2) out[2 * n + r * rows + i] = __float2bfloat16_rn(r1 - __bfloat162float(p1));
  }
}

__global__ void k_sum_partials(const float* __restrict__ partial, int splits, int64_t n,
                               float* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < splits; ++k) s += (double)partial[(int64_t)k * n + e];
    out[e] = (float)s;
  }
}

// ------------------------------------------------------------ host side
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() { return tma_encode_fn(); }
}  // namespace

PFN_cuTensorMapEncodeTiled_v12000 tma_encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  });
  return fn;
}

namespace {

// barriers, TMEM slot, flags and the per-slice scale rows after the operands
size_t tail_bytes(int n_pad) {
  return (2 * kMaxStages + 6) * sizeof(uint64_t) + 16 + 2 * (size_t)n_pad * sizeof(float);
}
size_t b_bytes_for(int64_t kc, int npl, int n_pad) { return (size_t)kc * npl * n_pad * 128; }
size_t smem_for(const TcPlan& p) {
  return 1024 + (size_t)p.stages * kStageBytes + b_bytes_for(p.kcg, p.npl, p.n_pad) +
         tail_bytes(p.n_pad);
}

template <int RP, bool MN, int NPL>
int set_attr_one() {
  TLGB_CUDA_TRY(cudaFuncSetAttribute(mttkrp_tc_kernel<RP, MN, NPL>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBudget));
  return TLGB_OK;
}

// Instantiated kernels: NPL = 2 for every padded rank; NPL = 1 and 3 (the
// f32-faithful split) for padded ranks <= 64, where 3 planes fit one MMA.
template <bool MN>
int set_attrs_mn() {
  int rc = set_attr_one<16, MN, 2>();
  if (!rc) rc = set_attr_one<32, MN, 2>();
  if (!rc) rc = set_attr_one<64, MN, 2>();
  if (!rc) rc = set_attr_one<128, MN, 2>();
  if (!rc) rc = set_attr_one<16, MN, 1>();
  if (!rc) rc = set_attr_one<32, MN, 1>();
  if (!rc) rc = set_attr_one<64, MN, 1>();
  if (!rc) rc = set_attr_one<16, MN, 3>();
  if (!rc) rc = set_attr_one<32, MN, 3>();
  if (!rc) rc = set_attr_one<64, MN, 3>();
  return rc;
}

template <int RP, bool MN, int NPL>
int launch_tc(const TcPlan& p, const CUtensorMap& tx, const CUtensorMap& tf, const TcArgs& a,
              cudaStream_t st) {
  dim3 grid((unsigned)p.gsplits, (unsigned)p.n_cg, (unsigned)p.m_tiles);
  TLGB_CUDA_TRY(launch_maybe_pdl(p.pdl && !tc_tuning().no_pdl, mttkrp_tc_kernel<RP, MN, NPL>,
                                 grid, dim3(kThreads), smem_for(p), st, tx, tf, a));
  return TLGB_OK;
}

template <int RP, int NPL>
int launch_mn(const TcPlan& p, const CUtensorMap& tx, const CUtensorMap& tf, const TcArgs& a,
              cudaStream_t st) {
  return p.out_contig ? launch_tc<RP, true, NPL>(p, tx, tf, a, st)
                      : launch_tc<RP, false, NPL>(p, tx, tf, a, st);
}

}  // namespace

int mttkrp_tc_prepare() {
  static std::atomic<bool> done[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && done[dev]) return TLGB_OK;
  if (!encode_fn()) return set_error(TLGB_EUNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  int rc = set_attrs_mn<false>();
  if (!rc) rc = set_attrs_mn<true>();
  if (!rc && dev >= 0 && dev < 64) done[dev] = true;
  return rc;
}

TcTuning& tc_tuning() {
  static TcTuning t;
  return t;
}

int mttkrp_tc_make_plan(const Shape& sh, int64_t rank, int mode, int npl, int free_sms,
                        TcPlan* plan) {
  TcPlan p{};
  p.npl = npl;
  const int N = sh.ndim;
  if (N < 2 || N > kMaxModes || mode < 0 || mode >= N)
    return set_error(TLGB_EINVAL, "mttkrp_bf16: bad mode");
  p.ndim = N;
  for (int k = 0; k < N; ++k) p.dim[k] = sh.dim[k];
  p.R = rank;
  p.I_out = sh.dim[mode];
  p.out_contig = (mode == N - 1) ? 1 : 0;
  p.out_mode = mode;
  p.inner_mode = p.out_contig ? N - 2 : N - 1;
  p.C = sh.dim[p.inner_mode];
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
  p.n_pad = rank <= 16 ? 16 : rank <= 32 ? 32 : rank <= 64 ? 64 : 128;
  p.kc = ceil_div(p.C, kChunk);
  p.m_tiles = (int)ceil_div(p.I_out, kTileM);
  // Inner-mode groups: a CTA keeps only its group's slice of the split factor
  // resident (about 64 KiB), which leaves room for a deep tensor-tile ring.
  const int per_chunk = npl * p.n_pad * 128;
  const int resident = tc_tuning().group_kib > 0 ? tc_tuning().group_kib : 64;
  const int max_g = std::max(1, (resident * 1024) / per_chunk);
  int kcg = 1;
  for (int g = 1; g <= std::min<int64_t>(max_g, p.kc); ++g)
    if (p.kc % g == 0) kcg = g;
  p.kcg = kcg;
  p.n_cg = (int)ceil_div(p.kc, kcg);
  p.total_steps = p.O * p.kc;
  const size_t bbytes = b_bytes_for(p.kcg, p.npl, p.n_pad);
  const int64_t room = (int64_t)kSmemBudget - 1024 - (int64_t)bbytes - (int64_t)tail_bytes(p.n_pad);
  p.stages = (int)std::min<int64_t>(kMaxStages, room > 0 ? room / kStageBytes : 0);
  if (tc_tuning().stages > 0) p.stages = std::min(p.stages, tc_tuning().stages);
  // the epilogue stages the 128 x (n_pad + 1) f32 partial tile in the operand buffers
  const bool stage_fits = (size_t)kTileM * (p.n_pad + 1) * sizeof(float) <=
                          (size_t)p.stages * kStageBytes + bbytes;
  bool ok = stage_fits && rank <= 128 && npl >= 1 && npl <= 3 && (npl == 2 || p.n_pad <= 64) && (p.C % 8 == 0) && (p.I_out % (p.out_contig ? 8 : 1) == 0) &&
            p.stages >= kMinStages && p.I_out < (1ll << 31) && p.C < (1ll << 31) &&
            p.O < (1ll << 31) && p.m_tiles <= 65535 && p.n_cg <= 65535;
  if (!ok) {
    p.valid = 0;
    *plan = p;
    return TLGB_OK;
  }
  // one wave: (output tiles x groups x splits) CTAs <= SM count when possible
  const int64_t pairs = (int64_t)p.m_tiles * p.n_cg;
  const int64_t ctas =
      std::max<int64_t>(1, (int64_t)(sm_count() - (tc_tuning().reserve_sms > 0
                                                        ? tc_tuning().reserve_sms
                                                        : free_sms)) *
                               (tc_tuning().waves > 0 ? tc_tuning().waves : 1));
  int64_t gs = std::max<int64_t>(1, ctas / pairs);
  const int64_t gsteps = p.O * p.kcg;
  gs = std::max<int64_t>(1, std::min<int64_t>(gs, gsteps));
  p.steps_per_split = ceil_div(gsteps, gs);
  p.gsplits = (int)std::min<int64_t>(65535, ceil_div(gsteps, p.steps_per_split));
  p.splits = p.n_cg * p.gsplits;   // partial tiles per output tile
  p.partial_bytes = (size_t)p.splits * p.I_out * p.R * sizeof(float);
  p.valid = 1;
  *plan = p;
  return TLGB_OK;
}

int mttkrp_tc_encode(const TcPlan& p, const __nv_bfloat16* Xbf, __nv_bfloat16* const* fbt,
                     int fplanes, TcMaps* maps) {
  if (!p.valid) return set_error(TLGB_EUNSUPPORTED, "mttkrp_bf16: shape not supported");
  auto enc = encode_fn();
  if (!enc) return set_error(TLGB_EUNSUPPORTED, "cuTensorMapEncodeTiled unavailable");
  TLGB_CHECK_ARG((reinterpret_cast<uintptr_t>(Xbf) % 16) == 0, "mttkrp_bf16: X not 16-byte aligned");
  const __nv_bfloat16* F = fbt[p.inner_mode];
  TLGB_CHECK_ARG((reinterpret_cast<uintptr_t>(F) % 16) == 0, "mttkrp_bf16: factor not aligned");
  Shape sh = make_shape(p.ndim, p.dim);
  // outer runs: consecutive outer modes merge into one TMA dimension
  int64_t run_size[2] = {1, 1}, run_stride[2] = {0, 0};
  int nrun = 0, prev = -2;
  for (int j = 0; j < p.n_outer; ++j) {
    const int k = p.outer_mode[j];
    if (k != prev + 1 || nrun == 0) {
      if (nrun == 2) return set_error(TLGB_EUNSUPPORTED, "mttkrp_bf16: too many outer runs");
      run_size[nrun] = 1;
      ++nrun;
    }
    run_size[nrun - 1] *= sh.dim[k];
    run_stride[nrun - 1] = sh.stride[k];
    prev = k;
  }
  // TMA dim 2 = the faster run (the later one), dim 3 = the slower run
  int64_t g2 = 1, g3 = 1, s2 = 0, s3 = 0;
  if (nrun == 1) { g2 = run_size[0]; s2 = run_stride[0]; }
  if (nrun == 2) { g2 = run_size[1]; s2 = run_stride[1]; g3 = run_size[0]; s3 = run_stride[0]; }
  cuuint64_t gdim[4];
  cuuint64_t gstride[3];
  cuuint32_t box[4];
  const cuuint32_t estride[4] = {1, 1, 1, 1};
  if (!p.out_contig) {   // dim0 = inner mode (contiguous), dim1 = output mode
    gdim[0] = (cuuint64_t)p.C;
    gdim[1] = (cuuint64_t)p.I_out;
    gstride[0] = (cuuint64_t)sh.stride[p.out_mode] * 2;
    box[0] = kChunk;
    box[1] = kTileM;
  } else {               // dim0 = output mode (contiguous), dim1 = inner mode
    gdim[0] = (cuuint64_t)p.I_out;
    gdim[1] = (cuuint64_t)p.C;
    gstride[0] = (cuuint64_t)sh.stride[p.inner_mode] * 2;
    box[0] = 64;
    box[1] = kChunk;
  }
  gdim[2] = (cuuint64_t)g2;
  gdim[3] = (cuuint64_t)g3;
  gstride[1] = (cuuint64_t)(s2 ? s2 : 1) * 2;
  gstride[2] = (cuuint64_t)(s3 ? s3 : 1) * 2;
  // unit dimensions still need a legal (16-byte multiple) stride
  if (g2 == 1) gstride[1] = gstride[0] * (cuuint64_t)gdim[1];
  if (g3 == 1) gstride[2] = gstride[1] * (cuuint64_t)gdim[2];
  box[2] = 1;
  box[3] = 1;
  for (int j = 0; j < 3; ++j)
    if (gstride[j] % 16 != 0) return set_error(TLGB_EUNSUPPORTED, "mttkrp_bf16: stride not 16-byte aligned");
  CUtensorMap& tx = maps->x;
  CUtensorMap& tf = maps->f;
  maps->g2 = g2;
  CUresult cr = enc(&tx, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(Xbf), gdim,
                    gstride, box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(TLGB_ECUDA, "mttkrp_bf16: tensor map for X failed");
  TLGB_CHECK_ARG(fplanes >= p.npl && fplanes <= 3, "mttkrp_bf16: too few factor planes");
  // inner factor as (C, R, planes): the planes of the transposed bf16 split
  cuuint64_t fdim[3] = {(cuuint64_t)p.C, (cuuint64_t)p.R, (cuuint64_t)fplanes};
  cuuint64_t fstride[2] = {(cuuint64_t)p.C * 2, (cuuint64_t)p.C * (cuuint64_t)p.R * 2};
  cuuint32_t fbox[3] = {(cuuint32_t)kChunk, (cuuint32_t)p.n_pad, 1};
  cr = enc(&tf, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<__nv_bfloat16*>(F), fdim, fstride,
           fbox, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (cr != CUDA_SUCCESS) return set_error(TLGB_ECUDA, "mttkrp_bf16: tensor map for F failed");
  return TLGB_OK;
}

int mttkrp_tc_launch_maps(const TcPlan& p, const TcMaps& maps, const float* const* factors,
                          const float* weights, float* partial, const int* skip_flag, int* err,
                          cudaStream_t st) {
  if (!p.valid) return set_error(TLGB_EUNSUPPORTED, "mttkrp_bf16: shape not supported");
  const CUtensorMap& tx = maps.x;
  const CUtensorMap& tf = maps.f;
  TcArgs a{};
  a.stages = p.stages;
  for (int j = 0; j < p.n_outer; ++j) {
    a.outer_f[j] = factors[p.outer_mode[j]];
    a.outer_dim[j] = p.outer_dim[j];
  }
  a.n_outer = p.n_outer;
  a.g2 = maps.g2;
  a.weights = weights;
  a.R = (int)p.R;
  a.I_out = p.I_out;
  a.kc_total = (int)p.kc;
  a.kcg = p.kcg;
  a.O = p.O;
  a.steps_per_split = p.steps_per_split;
  a.gsplits = p.gsplits;
  a.partial = partial;
  a.err = err;
  a.skip = skip_flag;
  a.starve = tc_tuning().test_starve;
  a.l2_stream = tc_tuning().l2_keep ? 0 : 1;
  if (p.npl == 2) {
    switch (p.n_pad) {
      case 16: return launch_mn<16, 2>(p, tx, tf, a, st);
      case 32: return launch_mn<32, 2>(p, tx, tf, a, st);
      case 64: return launch_mn<64, 2>(p, tx, tf, a, st);
      default: return launch_mn<128, 2>(p, tx, tf, a, st);
    }
  }
  if (p.n_pad > 64) return set_error(TLGB_EUNSUPPORTED, "mttkrp_tc: 1 or 3 planes need rank <= 64");
  if (p.npl == 1) {
    switch (p.n_pad) {
      case 16: return launch_mn<16, 1>(p, tx, tf, a, st);
      case 32: return launch_mn<32, 1>(p, tx, tf, a, st);
      default: return launch_mn<64, 1>(p, tx, tf, a, st);
    }
  }
  switch (p.n_pad) {
    case 16: return launch_mn<16, 3>(p, tx, tf, a, st);
    case 32: return launch_mn<32, 3>(p, tx, tf, a, st);
    default: return launch_mn<64, 3>(p, tx, tf, a, st);
  }
}

int mttkrp_tc_launch(const TcPlan& p, const __nv_bfloat16* Xbf, const float* const* factors,
                     __nv_bfloat16* const* fbt, int fplanes, const float* weights,
                     float* partial, const int* skip_flag, int* err, cudaStream_t st) {
  TcMaps maps;
  int rc = mttkrp_tc_encode(p, Xbf, fbt, fplanes, &maps);
  if (rc) return rc;
  return mttkrp_tc_launch_maps(p, maps, factors, weights, partial, skip_flag, err, st);
}

int tc_launch_sum_partials(const TcPlan& p, const float* partial, float* out, cudaStream_t st) {
  const int64_t n = p.I_out * p.R;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), sm_count() * 4));
  k_sum_partials<<<blocks, 256, 0, st>>>(partial, p.splits, n, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int tc_launch_to_bf16(const float* X, int64_t n, __nv_bfloat16* out, cudaStream_t st) {
  TLGB_CHECK_ARG((reinterpret_cast<uintptr_t>(X) % 16) == 0 &&
                     (reinterpret_cast<uintptr_t>(out) % 8) == 0,
                 "to_bf16: misaligned buffers");
  k_to_bf16<<<sm_count() * 8, 256, 0, st>>>(X, n, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int tc_launch_split3(const float* X, int64_t n, __nv_bfloat16* x0, __nv_bfloat16* x1,
                     __nv_bfloat16* x2, cudaStream_t st) {
  TLGB_CHECK_ARG((reinterpret_cast<uintptr_t>(X) % 8) == 0 &&
                     (reinterpret_cast<uintptr_t>(x0) % 4) == 0 &&
                     (reinterpret_cast<uintptr_t>(x1) % 4) == 0 &&
                     (reinterpret_cast<uintptr_t>(x2) % 4) == 0,   // x2 may be null
                 "split3: misaligned buffers");
  k_split3_bf16<<<sm_count() * 8, 256, 0, st>>>(X, n, x0, x1, x2, nullptr);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int tc_launch_split3_sumsq(const float* X, int64_t n, __nv_bfloat16* x0, __nv_bfloat16* x1,
                           __nv_bfloat16* x2, double* part, int nparts, cudaStream_t st) {
  k_split3_bf16<<<nparts, 256, 0, st>>>(X, n, x0, x1, x2, part);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int tc_launch_factor_bf16t(const float* A, int64_t rows, int64_t R, int planes,
                           __nv_bfloat16* out, cudaStream_t st) {
  const int64_t n = rows * R;
  const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), sm_count() * 4));
  k_factor_bf16t<<<blocks, 256, 0, st>>>(A, rows, R, planes, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

int split_mttkrp_plan(const Shape& sh, int64_t R, SplitMttkrp* s) {
  *s = SplitMttkrp{};
  s->sh = sh;
  s->R = R;
  if (tc_tuning().split_simt || R > 64) return TLGB_OK;
  for (int k = 0; k < sh.ndim; ++k)
    for (int j = 0; j < 3; ++j) {
      int rc = mttkrp_tc_make_plan(sh, R, k, 3 - j, 0, &s->plan[k][j]);
      if (rc) return rc;
      if (!s->plan[k][j].valid) return TLGB_OK;
    }
  s->valid = true;
  return TLGB_OK;
}

size_t split_mttkrp_bytes(const SplitMttkrp& s) {
  if (!s.valid) return 0;
  size_t b = 3 * align_up(sizeof(__nv_bfloat16) * (size_t)s.sh.numel, 256);
  size_t pmax = 0;
  for (int k = 0; k < s.sh.ndim; ++k) {
    b += align_up(sizeof(__nv_bfloat16) * 3 * (size_t)s.R * s.sh.dim[k], 256);
    pmax = std::max(pmax, s.plan[k][0].partial_bytes + s.plan[k][1].partial_bytes +
                              s.plan[k][2].partial_bytes);
  }
  return b + align_up(pmax, 256);
}

int split_mttkrp_setup(SplitMttkrp* s, const float* X, const float* const* factors, void* base,
                       int* err, cudaStream_t st) {
  if (!s->valid) return set_error(TLGB_EINVAL, "split_mttkrp: no valid plan");
  TLGB_CHECK_ARG((reinterpret_cast<uintptr_t>(base) & 255) == 0, "split_mttkrp: misaligned base");
  int rc = mttkrp_tc_prepare();
  if (rc) return rc;
  char* p = static_cast<char*>(base);
  for (int j = 0; j < 3; ++j) {
    s->xp[j] = reinterpret_cast<__nv_bfloat16*>(p);
    p += align_up(sizeof(__nv_bfloat16) * (size_t)s->sh.numel, 256);
  }
  for (int k = 0; k < s->sh.ndim; ++k) {
    s->fbt[k] = reinterpret_cast<__nv_bfloat16*>(p);
    p += align_up(sizeof(__nv_bfloat16) * 3 * (size_t)s->R * s->sh.dim[k], 256);
  }
  s->partial = reinterpret_cast<float*>(p);
  s->err = err;
  rc = tc_launch_split3(X, s->sh.numel, s->xp[0], s->xp[1], s->xp[2], st);
  if (rc) return rc;
  for (int k = 0; k < s->sh.ndim; ++k) {
    rc = split_mttkrp_refresh(*s, k, factors[k], st);
    if (rc) return rc;
    for (int j = 0; j < 3; ++j) {
      rc = mttkrp_tc_encode(s->plan[k][j], s->xp[j], s->fbt, 3, &s->maps[k][j]);
      if (rc) return rc;
    }
  }
  return TLGB_OK;
}

int split_mttkrp_refresh(const SplitMttkrp& s, int mode, const float* A, cudaStream_t st) {
  return tc_launch_factor_bf16t(A, s.sh.dim[mode], s.R, 3, s.fbt[mode], st);
}

int split_mttkrp_launch(const SplitMttkrp& s, int mode, const float* const* factors,
                        const float* weights, const int* skip, cudaStream_t st) {
  int splits = 0;
  for (int j = 0; j < 3; ++j) {
    const TcPlan& tp = s.plan[mode][j];
    int rc = mttkrp_tc_launch_maps(tp, s.maps[mode][j], factors, weights,
                                   s.partial + (size_t)splits * tp.I_out * tp.R, skip, s.err, st);
    if (rc) return rc;
    splits += tp.splits;
  }
  return TLGB_OK;
}

}  // namespace tlgb

// ---------------------------------------------------------------------------
// C ABI: standalone bf16 tensor-core MTTKRP
// ---------------------------------------------------------------------------
using namespace tlgb;

namespace {
int tc_plan_for(int ndim, const int64_t* shape, int64_t rank, int mode, TcPlan* p) {
  TLGB_CHECK_ARG(shape != nullptr, "mttkrp_bf16: null shape");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "mttkrp_bf16: ndim must be in [2, 8]");
  TLGB_CHECK_ARG(mode >= 0 && mode < ndim, "mttkrp_bf16: mode out of range");
  TLGB_CHECK_ARG(rank >= 1, "mttkrp_bf16: rank must be >= 1");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(shape[k] >= 1, "mttkrp_bf16: empty mode");
  Shape sh = make_shape(ndim, shape);
  int rc = mttkrp_tc_make_plan(sh, rank, mode, 2, 0, p);
  if (rc) return rc;
  if (!p->valid)
    return set_error(TLGB_EUNSUPPORTED,
                     "mttkrp_bf16: needs rank <= 128 and the inner mode (and a last output "
                     "mode) a multiple of 8");
  return TLGB_OK;
}
}  // namespace

extern "C" int tlgb_mttkrp_bf16_workspace_size(int ndim, const int64_t* shape, int64_t rank,
                                               int mode, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(bytes != nullptr, "mttkrp_bf16_workspace_size: null pointer");
  TcPlan p;
  int rc = tc_plan_for(ndim, shape, rank, mode, &p);
  if (rc) return rc;
  *bytes = 256 + align_up(p.partial_bytes, 256);
  return TLGB_OK;
}

extern "C" int tlgb_mttkrp_bf16(const void* X, int ndim, const int64_t* shape,
                                const void* const* factors, const void* const* factors_bf16_t,
                                const void* weights, int64_t rank, int mode, void* out,
                                void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TcPlan p;
  int rc = tc_plan_for(ndim, shape, rank, mode, &p);
  if (rc) return rc;
  TLGB_CHECK_ARG(X && factors && factors_bf16_t && out, "mttkrp_bf16: null pointer");
  TLGB_CHECK_ARG(factors_bf16_t[p.inner_mode] != nullptr, "mttkrp_bf16: missing inner factor");
  for (int j = 0; j < p.n_outer; ++j)
    TLGB_CHECK_ARG(factors[p.outer_mode[j]] != nullptr, "mttkrp_bf16: missing factor");
  if (!workspace || workspace_bytes < 256 + p.partial_bytes)
    return set_error(TLGB_EWORKSPACE, "mttkrp_bf16: workspace too small");
  rc = mttkrp_tc_prepare();
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int* err = static_cast<int*>(workspace);
  float* partial = reinterpret_cast<float*>(static_cast<char*>(workspace) + 256);
  TLGB_CUDA_TRY(cudaMemsetAsync(err, 0, sizeof(int), st));
  rc = mttkrp_tc_launch(p, static_cast<const __nv_bfloat16*>(X), (const float* const*)factors,
                        (__nv_bfloat16* const*)factors_bf16_t, 2,
                        static_cast<const float*>(weights), partial, nullptr, err, st);
  if (rc) return rc;
  return tc_launch_sum_partials(p, partial, static_cast<float*>(out), st);
}

extern "C" int tlgb_workspace_status(const void* workspace, void* stream, int* status) {
  clear_error();
  TLGB_CHECK_ARG(workspace && status, "workspace_status: null pointer");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  TLGB_CUDA_TRY(cudaMemcpyAsync(status, workspace, sizeof(int), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  return TLGB_OK;
}

// Tuning knobs of the tensor-core MTTKRP plan (0 restores the default).
extern "C" int tlgb_set_tuning(const char* key, int value) {
  clear_error();
  TLGB_CHECK_ARG(key != nullptr && value >= 0, "set_tuning: bad argument");
  const std::string k(key);
  if (k == "tc_group_kib") tc_tuning().group_kib = value;
  else if (k == "tc_stages") tc_tuning().stages = value;
  else if (k == "tc_waves") tc_tuning().waves = value;
  else if (k == "refine_simt") tc_tuning().refine_simt = value;
  else if (k == "tc_reserve_sms") tc_tuning().reserve_sms = value;
  else if (k == "f64_factorize") tc_tuning().f64_factorize = value;
  else if (k == "no_pdl") tc_tuning().no_pdl = value;
  else if (k == "tc_test_starve") tc_tuning().test_starve = value;
  else if (k == "split_simt") tc_tuning().split_simt = value;
  else if (k == "full_solve") tc_tuning().full_solve = value;
  else if (k == "closing_planes") tc_tuning().closing_planes = value;
  else if (k == "cp_graph_sweeps") tc_tuning().graph_sweeps = value;
  else if (k == "cp_inline_fit") tc_tuning().inline_fit = value;
  else if (k == "tc_l2_keep") tc_tuning().l2_keep = value;
  else if (k == "cp_lite_correction") tc_tuning().lite_correction = value;

  else return batched_set_tuning(k, value);   // the batched CP-ALS variants
  return TLGB_OK;
}
