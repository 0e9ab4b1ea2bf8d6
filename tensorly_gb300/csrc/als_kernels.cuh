// f64 normal-equation, Gram, fit and normalisation kernels of the CP-ALS sweep.
#pragma once
#include "common.cuh"

namespace tlgb {

// Device-side state of one CP-ALS run (lives in the workspace).
struct AlsCtrl {
  int done;      // stop flag: every sweep kernel returns at once when set
  int iter;      // sweeps whose error has been recorded
  int status;    // TLGB_OK or TLGB_ESINGULAR
  int fac_kind;  // 0: Cholesky factor, 1: LU factors with row permutation
  double norm_x2;
  int tc_err;    // TLGB_ETIMEOUT if a tensor-core pipeline wait expired
  int red_count; // blocks of the fused Gram reduction + fit that finished (reset by the last)
  // Stop raised by a fit deferred to the side stream, which runs beside the
  // next sweep's first MTTKRP (whose threads read `done`, so `done` may not
  // change under it); the first solve after it, ordered after it, promotes
  // it to `done`.
  int done_pending;
};

constexpr int kMaxAlsRank = 160;     // f64 factorisation held in one CTA's shared memory
constexpr int kSolveWarps = 8;       // warps per solve CTA

int als_launch_sumsq(int dtype, const void* X, int64_t n, double* part, int nblocks,
                     AlsCtrl* ctrl, cudaStream_t st);
// ||X||^2 into the control block from `nblocks` partial sums (fixed order).
int als_launch_sumsq_final(const double* part, int nblocks, AlsCtrl* ctrl, cudaStream_t st);

// G32 (optional, 2 R^2 floats): the Gram's f32 (hi, lo) planes, the operand
// of the factorisation's double-float V (see als_launch_factorize).
template <typename T>
int als_launch_gram(const T* A, int64_t I, int R, double* gpart, int nparts_max, double* G,
                    const int* done, cudaStream_t st, float* G32 = nullptr);

// vmat (R*R f64) and w32 (R*R f32) receive V and its f32 inverse for the
// refinement path; fac/perm the f64 Cholesky or LU fallback.
// G32 (optional; ndim x 2 R^2 floats, the (hi, lo) planes of every Gram as
// written by the Gram reductions): for f32 factors with R <= kSolveDfMaxRank,
// V is then formed in double-float on the f32 pipe and vmat is not written
// (the solve reads only w32's V planes there).
template <typename T>
int als_launch_factorize(const double* G, int ndim, int mode, int R, const T* weights,
                         double l2_reg, double* fac, int* perm, double* vmat,
                         float* w32 /* 3 R^2: W, then V's f32 hi and lo planes */,
                         AlsCtrl* ctrl, cudaStream_t st, const float* G32 = nullptr);

// Sums the MTTKRP partials of each row, solves with the factorisation, stores
// the factor (and optionally its bf16 transpose), and writes per-CTA Gram and
// <M, A> partial sums.  Returns the number of CTAs used via *nblocks.  pdl:
// programmatic dependent launch behind the MTTKRP that wrote `partial`.
template <typename T>
// max_passes: refinement passes allowed on the f32-inverse path (each pass
// stops early once the correction is below 1e-12 of the solution).
// lite (f32 factors): the refinement residual and the block's Gram in plain
// f32 instead of double-float, for sweeps whose MTTKRP is itself only
// accurate to ~1e-6 (the bf16 tensor-core sweeps).
int als_launch_solve(const T* partial, int splits, int64_t I, int R, const double* fac,
                     const int* perm, const double* vmat, const float* w32, T* A,
                     __nv_bfloat16* A_bf16_t, double* gpart, double* ipart, AlsCtrl* ctrl,
                     int max_passes, int* nblocks, cudaStream_t st, bool pdl = false,
                     bool lite = false);

constexpr int kIrMaxPasses = 4;

// df: the partials are (hi, lo) f32 planes (written by k_solve for f32 factors
// with rank <= kSolveDfMaxRank), 2: the hi planes only (a lite solve's Gram,
// whose lo planes are zero; its substitution fallback's lo planes are
// dropped), else f64.
int als_launch_gram_reduce(const double* gpart, int nparts, int R, double* G, const int* done,
                           int df, cudaStream_t st, float* G32 = nullptr);
constexpr int kSolveDfMaxRank = 96;

template <typename T>
int als_launch_fit(const double* G, int ndim, int R, const T* weights, const double* ipart,
                   int nip, AlsCtrl* ctrl, double* errors, int n_iter_max, double tol,
                   int cvg_criterion, cudaStream_t st);

// Gram reduction of `mode` (into G_all + mode * R^2) fused with the fit of
// als_launch_fit: one launch instead of two at the end of a sweep.  fpart:
// scratch of ceil(R^2 / 32) doubles.
template <typename T>
int als_launch_gram_reduce_fit(const double* gpart, int nparts, int R, double* G_all, int mode,
                               int ndim, int df, const T* weights, const double* ipart, int nip,
                               double* fpart, AlsCtrl* ctrl, double* errors, int n_iter_max,
                               double tol, int cvg_criterion, cudaStream_t st, bool pdl = false,
                               float* G32_all = nullptr, bool deferred = false);

template <typename T>
int als_launch_normalize(T* const* factors, const int64_t* rows, int ndim, int R, T* weights,
                         const int* done, cudaStream_t st);

template <typename T>
int als_launch_cp_norm(const double* G, int ndim, int R, const T* weights, double* out,
                       cudaStream_t st);

// Relative error of the current model from an MTTKRP of the last mode
// (split partials) and the Grams; result (f64) to *out on the device.
template <typename T>
int als_launch_probe_error(const T* partial, int splits, int64_t I, int R, const T* A,
                           const double* G, int ndim, const T* weights, double* ipart,
                           int nip_max, const AlsCtrl* ctrl, double* out, cudaStream_t st);

int solve_blocks_for(int64_t I);

// Sets kernel attributes once per device (call before stream capture).
int als_prepare(int dtype);

}  // namespace tlgb
