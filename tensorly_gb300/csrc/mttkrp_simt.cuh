// SIMT MTTKRP (f32 / f64) without forming the Khatri-Rao product.
//
// For mode n of an N-way tensor the reference computes
//   M = unfold(X, n) . KR(factors != n)          (core_tenalg/mttkrp.py:48-49)
// where the unfolding's columns run in C order over the other modes
// (base.py:53) and the KR rows run with the first matrix slowest
// (_khatri_rao.py:101-105).  Both orders agree, so
//   M(i, r) = sum_{o, c} X[o, i, c] * F(c, r) * s(o, r)
// with c the "inner" mode (N-1, or N-2 when n == N-1), F its factor, and o
// running over the remaining "outer" modes with s(o, r) = w_r prod_k A_k(i_k, r).
// For every o the kernel forms the GEMM tile P = X[o] . F over c, then adds
// s(o, :) * P into its accumulator; work is split over the flattened (o, c-chunk)
// sequence and each split writes a partial [I x R] tile that a second pass
// sums in a fixed order (deterministic).
#pragma once
#include "common.cuh"

namespace tlgb {

template <typename T>
struct MttkrpArgs {
  const T* X;
  const T* F;                    // inner factor, C x R
  const T* outer_f[kMaxModes];   // outer factors (row-major, rows x R)
  const T* weights;              // R or null
  int64_t I_out, C, O, R;
  int64_t s_out, s_c;            // element strides of the output and inner modes
  int n_outer;
  int64_t outer_dim[kMaxModes];
  int64_t outer_stride[kMaxModes];
  int64_t KC;                    // number of c-chunks
  int64_t steps_per_split;
  int64_t total_steps;           // O * KC
  int splits;
  int out_contig;                // 1 if the output mode is the contiguous one
  int vec_x, vec_f;              // 16-byte vector loads allowed
  T* partial;                    // [splits][I_out][R]
  const int* skip_flag;          // kernel returns at once if *skip_flag != 0 (may be null)
  int l2_stream;                 // f32 tensor loads with an evict-first L2 policy
};

struct MttkrpPlan {
  int64_t I_out, C, O, R;
  int64_t s_out, s_c;
  int inner_mode;
  int n_outer;
  int outer_mode[kMaxModes];
  int64_t outer_dim[kMaxModes], outer_stride[kMaxModes];
  int out_contig;
  int64_t KC, total_steps, steps_per_split;
  int splits;
  int bm, bn, bk;
  int r_tiles, m_tiles;
  size_t partial_bytes;
};

// Sets kernel attributes once per device (call before stream capture).
int mttkrp_prepare(int dtype);

// Builds the geometry and the split count for one mode (no launch).
// out = sum over `splits` partial tiles of n entries each (partial[split][n]).
template <typename T, typename TO>
int mttkrp_launch_reduce_n(const T* partial, int splits, int64_t n, TO* out, cudaStream_t stream);

int mttkrp_make_plan(int dtype, const Shape& sh, int64_t rank, int mode, MttkrpPlan* plan);

// Enqueues the split kernel (writes `partial`, which must hold plan.partial_bytes).
template <typename T>
int mttkrp_launch_partials(const MttkrpPlan& p, const T* X, const T* const* factors,
                           const T* weights, T* partial, const int* skip_flag,
                           cudaStream_t stream);

// Sums the partials into `out` (I_out x R, type TO).
template <typename T, typename TO>
int mttkrp_launch_reduce(const MttkrpPlan& p, const T* partial, TO* out, cudaStream_t stream);

}  // namespace tlgb
