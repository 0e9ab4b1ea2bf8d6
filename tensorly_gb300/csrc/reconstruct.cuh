// Fused CP reconstruction entry points shared with other drivers.
#pragma once
#include "common.cuh"

namespace tlgb {

int cp_full_check(int dtype, int ndim, const int64_t* shape, int64_t rank);

// Workspace of cp_full_run: transposed factors and one double per CTA.
size_t cp_full_ws_bytes(int dtype, int ndim, const int64_t* shape, int64_t rank);

// out = [[weights; factors]] (C order, mask optional), or with X != nullptr
// *resid (device) = ||X - [[weights; factors]]||_F and nothing stored.
int cp_full_run(int dtype, int ndim, const int64_t* shape, int64_t rank,
                const void* const* factors, const void* weights, const void* mask, void* out,
                const void* X, double* resid, void* workspace, size_t workspace_bytes,
                cudaStream_t st);

}  // namespace tlgb
