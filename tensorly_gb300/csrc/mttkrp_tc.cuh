// BF16 tensor-core MTTKRP (tcgen05 + TMA, sm_103a).
#pragma once
#include <cuda.h>
#include <vector>
#include "common.cuh"
#include "mttkrp_simt.cuh"

namespace tlgb {

struct TcPlan {
  int valid;
  int64_t I_out, C, O, R;
  int inner_mode;
  int out_mode;
  int n_outer;
  int outer_mode[kMaxModes];
  int64_t outer_dim[kMaxModes], outer_stride[kMaxModes];
  int out_contig;
  int n_pad;            // rank padded to 16/32/64/128 (MMA N = npl * n_pad)
  int npl;              // factor planes in the B operand (2: bf16 sweeps; 3, 2, 1: f32 split)
  int stages;           // tensor-tile ring depth that fits next to the resident factor
  int m_tiles;
  int64_t kc;           // 64-element chunks of the inner mode
  int64_t total_steps;  // O * kc per output tile
  int kcg;              // chunks per inner-mode group (resident factor slice)
  int n_cg;             // inner-mode groups
  int gsplits;          // CTAs per (output tile, group)
  int64_t steps_per_split;
  int splits;           // partial tiles per output tile (= n_cg * gsplits)
  size_t partial_bytes;
  int ndim;
  int64_t dim[kMaxModes];
  int pdl;              // launch with programmatic stream serialisation (inside CP-ALS sweeps)
};

// Plan knobs set by tlgb_set_tuning (0 = default): resident factor slice per
// CTA in KiB, ring depth cap, CTAs per SM.
struct TcTuning {
  int group_kib = 0;
  int stages = 0;
  int waves = 0;
  int refine_simt = 0;  // 1: CP-ALS refinement sweeps use the SIMT f32 MTTKRP
  int reserve_sms = 0;  // overrides the SMs a plan leaves free (0 = the plan's own)
  int f64_factorize = 0;      // 1: every CP-ALS factorisation takes the f64 Cholesky / LU path
  int no_pdl = 0;             // 1: CP-ALS sweep kernels launch without programmatic dependence
  int test_starve = 0;        // 1: tensor-core MTTKRP issues no copies (timeout-path test)
  int split_simt = 0;         // 1: non-negative / constrained CP keep the SIMT f32 MTTKRP
  int full_solve = 0;         // 1: bf16 CP-ALS sweeps solve with the double-float refinement
  int closing_planes = 0;     // 3: the closing sweeps also contract the third tensor plane
  int graph_sweeps = 0;       // > 0: at most this many CP-ALS sweeps per CUDA graph
  int inline_fit = 0;         // 1: every CP-ALS sweep runs its last mode's fit in line
  int l2_keep = 0;            // 1: tensor tiles loaded without the evict-first L2 policy
  int lite_correction = 0;    // 1: the bf16 sweeps' solve adds one f32 correction pass to x = m W
};
TcTuning& tc_tuning();

int mttkrp_tc_prepare();
// npl: factor planes contracted with the tensor (1..3; 1 and 3 need rank <= 64).
// free_sms: SMs the one-wave grid leaves free for kernels that run concurrently
// on another stream (a CTA of this kernel needs nearly a whole SM, so one busy
// SM would otherwise delay the whole launch by that kernel's duration).
int mttkrp_tc_make_plan(const Shape& sh, int64_t rank, int mode, int npl, int free_sms,
                        TcPlan* plan);

// partial[split][I_out][R] (f32) from a bf16 tensor, the f32 factors (outer
// scales) and the bf16 split transposed factors (inner operand: `fplanes`
// planes of rank x rows each, the first p.npl of which are contracted).
// err: device int that receives TLGB_ETIMEOUT if a bounded wait expired.
int mttkrp_tc_launch(const TcPlan& p, const __nv_bfloat16* Xbf, const float* const* factors,
                     __nv_bfloat16* const* fbt, int fplanes, const float* weights,
                     float* partial, const int* skip_flag, int* err, cudaStream_t st);

// The launch split in two: the TMA descriptors of a plan and its operands
// (host work, done once per run by callers that launch the same plan many
// times), then the launch itself.
struct TcMaps {
  CUtensorMap x, f;
  int64_t g2;
};
int mttkrp_tc_encode(const TcPlan& p, const __nv_bfloat16* Xbf, __nv_bfloat16* const* fbt,
                     int fplanes, TcMaps* maps);
int mttkrp_tc_launch_maps(const TcPlan& p, const TcMaps& maps, const float* const* factors,
                          const float* weights, float* partial, const int* skip_flag, int* err,
                          cudaStream_t st);

// out = sum over splits of partial (I_out x R, f32).
int tc_launch_sum_partials(const TcPlan& p, const float* partial, float* out, cudaStream_t st);

int tc_launch_to_bf16(const float* X, int64_t n, __nv_bfloat16* out, cudaStream_t st);
// Exact split X = x0 + x1 + x2 into three bf16 tensors (x2 may be null: only
// the first two planes are written).
int tc_launch_split3(const float* X, int64_t n, __nv_bfloat16* x0, __nv_bfloat16* x1,
                     __nv_bfloat16* x2, cudaStream_t st);
// The same split, which also writes each of its `nparts` blocks' share of
// ||X||^2 to part (f32 compensated sums, f64 block totals).
int tc_launch_split3_sumsq(const float* X, int64_t n, __nv_bfloat16* x0, __nv_bfloat16* x1,
                           __nv_bfloat16* x2, double* part, int nparts, cudaStream_t st);
// out (planes x R x rows bf16, planes 2 or 3): the bf16 split of A^T,
// plane 0 = bf16(A^T), plane k = bf16(A^T - planes before k).
int tc_launch_factor_bf16t(const float* A, int64_t rows, int64_t R, int planes,
                           __nv_bfloat16* out, cudaStream_t st);

// f32-faithful MTTKRP of an f32 tensor on the tensor cores, for loops that
// update factors with their own kernels (non-negative and constrained CP):
// the exact split X = x0 + x1 + x2 and A_k = f0 + f1 + f2 into bf16 planes,
// and per mode three launches x0.(f0+f1+f2) + x1.(f0+f1) + x2.f0 (the
// dropped terms are below 2^-26 of |x||f|), each writing its own run of
// partial tiles, so the result is partial[split][I][R] in the layout of the
// SIMT MTTKRP with splits(mode) tiles.  The tensor cores' f32 accumulation
// rounds toward zero (about -2e-7 of |M|).
struct SplitMttkrp {
  bool valid = false;
  Shape sh{};
  int64_t R = 0;
  TcPlan plan[kMaxModes][3];
  TcMaps maps[kMaxModes][3];
  __nv_bfloat16* xp[3] = {nullptr, nullptr, nullptr};
  __nv_bfloat16* fbt[kMaxModes] = {};
  float* partial = nullptr;
  int* err = nullptr;     // device int: TLGB_ETIMEOUT if a bounded wait expired
  int splits(int mode) const {
    return plan[mode][0].splits + plan[mode][1].splits + plan[mode][2].splits;
  }
};
// Plans every mode; s->valid stays false when a plan does not fit (shape,
// rank > 64) or the split_simt knob is set: the caller keeps the SIMT kernel.
int split_mttkrp_plan(const Shape& sh, int64_t R, SplitMttkrp* s);
// Workspace of the planes, the factor planes and the partial tiles (0 if !valid).
size_t split_mttkrp_bytes(const SplitMttkrp& s);
// Carves `base` (split_mttkrp_bytes, 256-byte aligned), splits X and every
// factor into planes and encodes the tensor maps.
int split_mttkrp_setup(SplitMttkrp* s, const float* X, const float* const* factors, void* base,
                       int* err, cudaStream_t st);
// The planes of factor `mode` after the caller rewrote it.
int split_mttkrp_refresh(const SplitMttkrp& s, int mode, const float* A, cudaStream_t st);
// partial[splits(mode)][I_mode][R]; skip: the loop's device stop flag.
int split_mttkrp_launch(const SplitMttkrp& s, int mode, const float* const* factors,
                        const float* weights, const int* skip, cudaStream_t st);

// The MTTKRP of a loop that updates its factors itself (non-negative and
// constrained CP): the f32-faithful tensor-core split (SplitMttkrp) for an
// f32 tensor whose plans fit, else the SIMT kernel; partial() and splits()
// name the partial tiles either way.  refresh() after a factor changes.
template <typename T>
struct LoopMttkrp {
  SplitMttkrp stc;
  bool tc = false;
  const T* X;
  const std::vector<MttkrpPlan>* plans;
  T* simt_partial;

  int setup(const T* X_, const Shape& sh, int64_t R, T* const* factors,
            const std::vector<MttkrpPlan>* plans_, T* simt_partial_, char* tcs_base, int* err,
            cudaStream_t st) {
    X = X_;
    plans = plans_;
    simt_partial = simt_partial_;
    if constexpr (sizeof(T) == 4) {
      int rc = split_mttkrp_plan(sh, R, &stc);
      if (rc) return rc;
      if (stc.valid) {
        rc = split_mttkrp_setup(&stc, reinterpret_cast<const float*>(X), 
                                reinterpret_cast<const float* const*>(factors), tcs_base, err, st);
        if (rc) return rc;
        tc = true;
      }
    }
    return TLGB_OK;
  }
  int launch(int mode, const T* const* cf, const T* w, const int* done, cudaStream_t st) {
    if (tc)
      return split_mttkrp_launch(stc, mode, reinterpret_cast<const float* const*>(cf),
                                 reinterpret_cast<const float*>(w), done, st);
    return mttkrp_launch_partials<T>((*plans)[mode], X, cf, w, simt_partial, done, st);
  }
  const T* partial() const { return tc ? reinterpret_cast<const T*>(stc.partial) : simt_partial; }
  int splits(int mode) const { return tc ? stc.splits(mode) : (*plans)[mode].splits; }
  int refresh(int mode, const T* A, cudaStream_t st) {
    return tc ? split_mttkrp_refresh(stc, mode, reinterpret_cast<const float*>(A), st) : TLGB_OK;
  }
};

}  // namespace tlgb
