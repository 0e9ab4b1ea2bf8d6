// BF16 tensor-core MTTKRP (tcgen05 + TMA, sm_103a).
#pragma once
#include "common.cuh"

namespace tlgb {

struct TcPlan {
  int valid;
  int64_t I_out, C, O, R;
  int inner_mode;
  int n_outer;
  int outer_mode[kMaxModes];
  int64_t outer_dim[kMaxModes], outer_stride[kMaxModes];
  int out_contig;
  int n_pad;            // rank padded to the MMA N granularity
  int m_tiles;
  int64_t kc;           // 64-element chunks of the inner mode
  int64_t total_steps;  // O * kc per output tile
  int64_t steps_per_split;
  int splits;           // splits per output tile
  size_t partial_bytes;
  int ndim;
  int64_t dim[kMaxModes];
};

int mttkrp_tc_prepare();
int mttkrp_tc_make_plan(const Shape& sh, int64_t rank, int mode, TcPlan* plan);

// partial[split][I_out][R] (f32) from the bf16 tensor, the f32 factors (outer
// scales) and the bf16 transposed factors (inner operand, rank x rows).
int mttkrp_tc_launch(const TcPlan& p, const __nv_bfloat16* Xbf, const float* const* factors,
                     __nv_bfloat16* const* fbt, const float* weights, float* partial,
                     const int* skip_flag, cudaStream_t st);

int tc_launch_to_bf16(const float* X, int64_t n, __nv_bfloat16* out, cudaStream_t st);
int tc_launch_factor_bf16t(const float* A, int64_t rows, int64_t R, __nv_bfloat16* out,
                           cudaStream_t st);

}  // namespace tlgb
