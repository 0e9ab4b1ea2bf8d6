// Column-wise and rank-based proximal operators (prox_columns.cu).
#pragma once
#include "common.cuh"

namespace tlgb {

// TLGB_CONS_UNIMODALITY .. TLGB_CONS_HARD_SPARSITY
bool prox_is_matrix_kind(int kind);
// TLGB_EUNSUPPORTED when a column does not fit one CTA (or too many entries
// for the rank count of hard thresholding).
int prox_matrix_check(int dtype, int64_t rows, int64_t cols, int kind);
size_t prox_matrix_scratch_bytes(int dtype, int64_t rows, int64_t cols, int kind);
// P = prox(Y) for a rows x cols row-major matrix; every kernel returns at
// once when *stop is set (stop may be null).
template <typename T>
int prox_matrix_launch(const T* Y, T* P, int64_t rows, int64_t cols, int kind, double param,
                       void* scratch, const int* stop, cudaStream_t st);

}  // namespace tlgb
