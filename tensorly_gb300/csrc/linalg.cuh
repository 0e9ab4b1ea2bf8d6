// Dense linear-algebra pieces shared by the SVD / Tucker paths.
#pragma once
#include "common.cuh"

namespace tlgb {

// ---- symmetric eigensolver (eig.cu): the k largest eigenpairs of an n x n
// symmetric matrix, descending, eigenvector signs as svd_flip (optional).
int sym_eig_max_n(int dtype);
size_t sym_eig_workspace(int dtype, int64_t n, int64_t k);
template <typename T>
int sym_eig_launch(const T* A, int n, int k, T* U, T* lam, int flip, void* ws, cudaStream_t st);
// `batch` independent matrices, consecutive in A (n x n each), U (n x k), lam
// (k); the workspace is `batch` times sym_eig_workspace (6 k n elements each).
template <typename T>
int sym_eig_batched_launch(const T* A, int n, int k, int batch, T* U, T* lam, int flip, void* ws,
                           cudaStream_t st);

// ---- Gram matrix of a tensor unfolding (svd.cu).  side 0: M M^T
// (shape[mode] x shape[mode]); side 1: M^T M (J x J, J = numel / shape[mode]),
// with M = unfold(X, mode).
struct GramPlan {
  int64_t Na, Nk;          // Gram order and contraction length
  int64_t aD, aS1, aS0;    // element offset of row a: (a / aD) * aS1 + (a % aD) * aS0
  int64_t kD, kS1, kS0;    // element offset of column k, same form
  int nt, npairs, splits;
  int64_t chunks, cps;     // BK-chunks of the contraction, chunks per split
  size_t partial_bytes;    // f64 partial tiles
};
int gram_make_plan(const Shape& sh, int mode, int side, GramPlan* p);
template <typename T>
int gram_launch(const GramPlan& p, const T* X, T* G, double* partial, cudaStream_t st);

// ---- mode-n product (ttm.cu)
template <typename T>
int ttm_launch(const T* X, const Shape& sh, const T* U, int64_t J, int transpose, int mode, T* Y,
               cudaStream_t st);

// ---- left singular vectors of an unfolding (svd.cu): U (I x k), S (k).
// `input_done` (optional) is recorded on st once X is no longer read.
size_t svd_unfolding_workspace(int dtype, const Shape& sh, int mode, int64_t k);
template <typename T>
int svd_unfolding_launch(const T* X, const Shape& sh, int mode, int k, T* U, T* S, int flip,
                         void* ws, size_t ws_bytes, cudaStream_t st,
                         cudaEvent_t input_done = nullptr);

}  // namespace tlgb
