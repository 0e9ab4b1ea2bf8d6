/*
 * tensorly_gb300 — C ABI of the GB300 (sm_103a) CP-ALS / Tucker-HOOI library.
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as void*, i.e. a cudaStream_t; NULL = legacy default stream).
 * Tensors are dense, C-contiguous (row-major, last mode fastest) and live in
 * device memory unless a parameter says "host".  Factor matrices are
 * row-major (rows x rank).  Nothing here allocates device memory: entry points
 * that need scratch space take a caller-provided workspace whose size comes
 * from the matching *_workspace_size query.  Work is enqueued on `stream`;
 * functions return before the GPU finishes unless documented otherwise.
 *
 * Return value: TLGB_OK (0) or an error code; tlgb_last_error() gives the
 * message of the last failure on the calling thread.
 *
 * Each entry point names the TensorLy 0.9.0 function it replaces
 * (file:line inside the TensorLy source tree).
 */
#ifndef TENSORLY_GB300_H
#define TENSORLY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TLGB_MAX_MODES 8

/* status codes */
#define TLGB_OK 0
#define TLGB_EINVAL 1        /* bad argument (shape, dtype, size, mode) */
#define TLGB_ECUDA 2         /* CUDA runtime or launch error */
#define TLGB_ESINGULAR 3     /* normal equations singular (LAPACK gesv would fail too) */
#define TLGB_EUNSUPPORTED 4  /* valid request this library does not implement */
#define TLGB_ETIMEOUT 5      /* a bounded device-side wait gave up */
#define TLGB_EWORKSPACE 6    /* workspace smaller than the size query returned */

/* element types */
#define TLGB_F32 0
#define TLGB_F64 1
#define TLGB_BF16 2

/* CP-ALS precision modes */
#define TLGB_PREC_NATIVE 0   /* every sweep in the tensor dtype (f32 or f64) */
#define TLGB_PREC_BF16 1     /* bf16 tensor + tensor-core MTTKRP, then f32 refinement sweeps */

/* Library version, e.g. 100 for 0.1.0. */
int tlgb_version(void);

/* Message of the last failure on this thread ("" if none). */
const char* tlgb_last_error(void);

/*
 * Khatri-Rao product of `n_mats` matrices (rows[k] x rank each), first matrix
 * varying slowest; optional `weights` (rank) scale the first matrix and the
 * optional `mask` (prod(rows)) scales output rows.  out: prod(rows) x rank.
 * Replaces tensorly/tenalg/core_tenalg/_khatri_rao.py:9-109 (khatri_rao).
 * dtype: TLGB_F32 or TLGB_F64.  weights/mask may be NULL.
 */
int tlgb_khatri_rao(int dtype, int n_mats, const void* const* mats, const int64_t* rows,
                    int64_t rank, const void* weights, const void* mask, void* out,
                    void* stream);

/*
 * MTTKRP: out = unfold(X, mode) . khatri_rao(factors, weights, skip_matrix=mode)
 * without forming the Khatri-Rao product or the unfolding.
 * X: shape[0..ndim) dense; factors[k]: shape[k] x rank (factors[mode] unused,
 * may be NULL); weights: rank or NULL; out: shape[mode] x rank.
 * Replaces tensorly/tenalg/core_tenalg/mttkrp.py:9-50
 * (unfolding_dot_khatri_rao).  dtype: TLGB_F32 or TLGB_F64 (SIMT kernels;
 * f64 accumulation for f64, f32 accumulation with f64 split reduction for f32).
 */
int tlgb_mttkrp_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                               int mode, size_t* bytes);
int tlgb_mttkrp(int dtype, const void* X, int ndim, const int64_t* shape,
                const void* const* factors, const void* weights, int64_t rank, int mode,
                void* out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * tlgb_mttkrp without a workspace, for callers that own no device allocator
 * (a plain C, cgo or ctypes binding): the partial tiles live in one fixed
 * 16 MiB device array inside the library (TLGB_NOALLOC_SCRATCH_BYTES), and
 * nothing is allocated.  Same plan and kernels as tlgb_mttkrp, so the result
 * is bitwise identical.  Shapes whose partial tiles
 * (tlgb_mttkrp_workspace_size) exceed the array return TLGB_EWORKSPACE.  The
 * first call on a device performs that device's set-up: make it before any
 * stream capture.  Nothing needs to start at zero.  The array is shared by
 * all calls on a device: calls in flight at the same time (other streams or
 * threads) race, so serialise them on one stream.
 * No counterpart in TensorLy (its MTTKRP allocates through the backend).
 */
#define TLGB_NOALLOC_SCRATCH_BYTES (16u << 20)
int tlgb_mttkrp_noalloc(int dtype, const void* X, int ndim, const int64_t* shape,
                        const void* const* factors, const void* weights, int64_t rank,
                        int mode, void* out, void* stream);

/*
 * MTTKRP on the bf16 tensor cores (tcgen05, TMA): same contraction as
 * tlgb_mttkrp with X stored in bf16 and f32 accumulation.
 * X: bf16 tensor; factors[k]: f32 (shape[k] x rank) for the scaling modes;
 * factors_bf16_t[k]: the contracted inner factor (mode ndim-1, or ndim-2 when
 * mode == ndim-1) transposed and split into two bf16 planes, each rank x
 * shape[k] row-major: hi = bf16(A^T), then lo = bf16(A^T - hi); the kernel
 * contracts with hi + lo (about 16 significant bits).  Pointers of other
 * modes may be NULL.  weights: f32 rank or NULL.
 * out: f32 shape[mode] x rank.  Requirements (else TLGB_EUNSUPPORTED):
 * rank <= 128, the inner mode a multiple of 8 (and shape[ndim-1] a multiple
 * of 8 when mode == ndim-1).
 * The first int of the workspace receives TLGB_ETIMEOUT if the kernel's
 * bounded pipeline waits expired (read it with tlgb_workspace_status).
 * Replaces tensorly/tenalg/core_tenalg/mttkrp.py:9-50 for bf16 storage.
 */
int tlgb_mttkrp_bf16_workspace_size(int ndim, const int64_t* shape, int64_t rank, int mode,
                                    size_t* bytes);
int tlgb_mttkrp_bf16(const void* X, int ndim, const int64_t* shape, const void* const* factors,
                     const void* const* factors_bf16_t, const void* weights, int64_t rank,
                     int mode, void* out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Tile-plan knobs of the bf16 tensor-core MTTKRP (used by the autotuner;
 * value 0 restores the default): "tc_group_kib" = bytes of the split inner
 * factor kept resident per CTA (KiB; sets how the inner mode is partitioned
 * across CTAs), "tc_stages" = cap on the tensor-tile ring depth,
 * "tc_waves" = CTAs per SM in the grid, "tc_reserve_sms" = SMs the grid
 * leaves free (CP-ALS leaves 1 for its concurrent factorisation kernel),
 * "refine_simt" = 1 makes the f32
 * refinement sweeps of TLGB_PREC_BF16 use the SIMT f32 MTTKRP instead of the
 * tensor-core one on the exact three-plane bf16 split of the f32 tensor;
 * "f64_factorize" = 1
 * sends every CP-ALS normal-equation factorisation to the f64 Cholesky (LU
 * when Cholesky fails) that otherwise serves only ill-conditioned V;
 * "no_pdl" = 1 launches the kernels of a CP-ALS sweep without programmatic
 * dependent launch (each then starts only when its predecessor has ended);
 * "tc_test_starve" = 1 is for testing the timeout path: the tensor-core
 * MTTKRP issues no copies, its waits give up after 1 ms, and the workspace
 * status (tlgb_workspace_status) reads TLGB_ETIMEOUT;
 * "split_simt" = 1 keeps the SIMT f32 MTTKRP in the non-negative and
 * constrained CP loops (instead of the exact bf16 split on the tensor cores);
 * "full_solve" = 1 gives the bf16 CP-ALS sweeps the double-float refinement
 * solve of the closing sweeps; "closing_planes" = 3 makes the closing sweeps
 * also contract the third bf16 plane of the f32 tensor;
 * "cp_graph_sweeps" = n caps the sweeps of one CUDA graph (use_graph = 1);
 * "cp_inline_fit" = 1 runs every sweep's last Gram reduction and fit on the
 * main stream instead of deferring it to the side stream under the next
 * sweep; "cp_lite_correction" = 1 adds one f32 correction pass to the bf16
 * sweeps' solve x = m V^-1; "tc_l2_keep" = 1 loads the tensor-core MTTKRP's
 * tensor tiles without the evict-first L2 policy;
 * "batched_threads_small" / "_medium" / "_large" = threads per CTA (128, 256
 * or 512; 4, 2 or 1 CTAs per SM) of tlgb_cp_als_batched for the tensors
 * whose padded size fits 128-, 256-thread CTAs' shared memory, or neither;
 * "batched_outer_tile_small" / "_medium" / "_large" = outer slices per
 * MTTKRP work tile of those classes (0..64, 0: spread over the threads).
 * Process-wide; no counterpart in TensorLy.
 */
int tlgb_set_tuning(const char* key, int value);

/* Synchronises `stream` and reads the status int at the start of a workspace. */
int tlgb_workspace_status(const void* workspace, void* stream, int* status);

/*
 * Tensor-times-matrix: out = X x_mode U, i.e. fold(U . unfold(X, mode)).
 * U is J x shape[mode] (row-major); with transpose != 0, U is shape[mode] x J
 * and U^T is applied.  out has shape[mode] replaced by J.
 * Replaces tensorly/tenalg/core_tenalg/n_mode_product.py:5-76 (mode_dot,
 * matrix case; the vector case is J = 1 with the mode squeezed by the caller).
 */
int tlgb_mode_dot(int dtype, const void* X, int ndim, const int64_t* shape, const void* U,
                  int64_t J, int transpose, int mode, void* out, void* stream);

/*
 * The k largest eigenpairs of a symmetric n x n matrix A (row-major, both
 * triangles), eigenvalues descending in `evals` (k), eigenvectors as the
 * columns of U (n x k, row-major).  With flip_sign != 0 every column's
 * largest-magnitude entry (first one on ties) is made positive, the sign rule
 * of tensorly/tenalg/svd.py:13-65 (svd_flip, u_based_decision).  One CTA:
 * Householder tridiagonalisation, multisection, inverse iteration.
 * dtype TLGB_F64 (n <= 160) or TLGB_F32 (n <= 224), else TLGB_EUNSUPPORTED.
 * Stands in for the LAPACK eigen/SVD drivers behind
 * tensorly/tenalg/svd.py:211-235 (truncated_svd).
 */
int tlgb_sym_eig_workspace_size(int dtype, int64_t n, int64_t k, size_t* bytes);
int tlgb_sym_eig(int dtype, const void* A, int64_t n, int64_t k, void* U, void* evals,
                 int flip_sign, void* workspace, size_t workspace_bytes, void* stream);

/*
 * Gram matrix of the mode-`mode` unfolding M = unfold(X, mode) without
 * forming it: side 0 -> G = M M^T (shape[mode] x shape[mode]), side 1 ->
 * G = M^T M (J x J, J = numel / shape[mode]).  f32 tensors: compensated f32
 * sums with an f64 split reduction; f64 tensors: f64.  Deterministic.
 * No direct counterpart in TensorLy (it is the first half of the SVD below).
 */
int tlgb_gram_unfolding_workspace_size(int ndim, const int64_t* shape, int mode, int side,
                                       size_t* bytes);
int tlgb_gram_unfolding(int dtype, const void* X, int ndim, const int64_t* shape, int mode,
                        int side, void* G, void* workspace, size_t workspace_bytes, void* stream);

/*
 * svd_interface(unfold(X, mode), n_eigenvecs=k) for method 'truncated_svd'
 * (tensorly/tenalg/svd.py:366-447, :211-235): the leading k left singular
 * vectors U (shape[mode] x k, row-major) and singular values S (k,
 * descending) of the unfolding, from the eigenpairs of its smaller Gram
 * matrix; flip_sign applies svd_flip to U.  Requires k <= min(shape[mode], J)
 * and that order of the Gram matrix within tlgb_sym_eig's limit.
 */
int tlgb_svd_unfolding_workspace_size(int dtype, int ndim, const int64_t* shape, int mode,
                                      int64_t k, size_t* bytes);
int tlgb_svd_unfolding(int dtype, const void* X, int ndim, const int64_t* shape, int mode,
                       int64_t k, void* U, void* S, int flip_sign, void* workspace,
                       size_t workspace_bytes, void* stream);

/*
 * Dense CP-ALS (the sweep loop of tensorly/decomposition/_cp.py:394-530,
 * parafac).  On entry factors[k] (shape[k] x rank, tensor dtype) and weights
 * (rank) hold the initial CP tensor; on exit the result.  Per sweep and mode:
 * the Hadamard product of the other factors' Grams (+ l2_reg I, scaled by
 * w w^T) is factorised in f64 (Cholesky, LU with partial pivoting if not
 * positive definite), the MTTKRP is formed without the Khatri-Rao product,
 * and the factor is the f64 solve.  The error uses the last mode's MTTKRP
 * (tensorly/decomposition/_cp.py:217-225) in f64; the stop test mirrors
 * _cp.py:505-524.  errors (host, n_iter_max entries) receive the relative
 * errors, *n_errors their count.  The call returns after the GPU finished.
 */
typedef int (*tlgb_sweep_callback)(void* user, int iteration, double rec_error);

typedef struct tlgb_cp_als_options {
  int n_iter_max;          /* parafac n_iter_max */
  double tol;              /* parafac tol (0 disables the stop test) */
  double l2_reg;           /* parafac l2_reg */
  int cvg_criterion;       /* 0 = 'abs_rec_error', 1 = 'rec_error' */
  int normalize_factors;   /* parafac normalize_factors */
  uint32_t fixed_modes;    /* bit k set: mode k is kept fixed (parafac fixed_modes) */
  int precision;           /* TLGB_PREC_NATIVE or TLGB_PREC_BF16 (f32 tensors only) */
  int refine_sweeps;       /* TLGB_PREC_BF16: closing sweeps with an f32-accurate MTTKRP
                              (tensor cores on the exact 3-plane bf16 split of X and
                              the factor when rank <= 64, else the SIMT f32 kernel); 1 by default */
  int check_every;         /* sweeps between host reads of the device stop flag (>= 1) */
  int use_graph;           /* 1: replay groups of captured sweeps as CUDA graphs; 0 (default):
                              launch the sweeps directly, a group ahead of the host's reads */
  tlgb_sweep_callback callback;  /* per-sweep hook (parafac callback) or NULL */
  void* callback_user;
  /* Optional (NULL = off), host, TLGB_CP_ALS_SWEEP_KINDS x TLGB_MAX_MODES
   * doubles: entry [kind * TLGB_MAX_MODES + mode] receives the duration (ms,
   * CUDA events recorded around the MTTKRP launch on the stream) of that
   * mode's MTTKRP in the last sweep of each kind that ran, 0 if none, -1 if
   * the events could not be read.  Setting it disables use_graph (events
   * recorded inside a graph cannot be timed).  Kinds: 0 native SIMT, 1 bf16 tensor-core,
   * 2 three-plane f32 split on the tensor cores, 3 the closing sweep.  No
   * counterpart in TensorLy. */
  double* mttkrp_ms;
} tlgb_cp_als_options;
#define TLGB_CP_ALS_SWEEP_KINDS 4

void tlgb_cp_als_default_options(tlgb_cp_als_options* opts);
int tlgb_cp_als_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                               const tlgb_cp_als_options* opts, size_t* bytes);
int tlgb_cp_als(int dtype, const void* X, int ndim, const int64_t* shape, int64_t rank,
                void* const* factors, void* weights, const tlgb_cp_als_options* opts,
                double* errors, int* n_errors, void* workspace, size_t workspace_bytes,
                void* stream);

/*
 * Tucker decomposition by HOOI: the loop of
 * tensorly/decomposition/_tucker.py:105-221 (partial_tucker) after
 * initialize_tucker (:25-102).  modes[i] (n_modes ascending modes, NULL =
 * 0..n_modes-1) is decomposed with rank ranks[i]; factors[i]
 * (shape[modes[i]] x ranks[i], tensor dtype) receives the factor (and holds
 * the initial one on entry when init_svd == 0); core receives the core
 * (shape with modes[i] replaced by ranks[i]).  Per iteration and mode: the
 * factors of the other modes applied transposed (ascending mode order, the
 * skipped position counted in that order as the reference does), then the
 * leading ranks[i] left singular vectors of that unfolding (svd_flip signs);
 * the error is sqrt(|norm(X)^2 - norm(core)^2|) / norm(X) and the run stops
 * after iteration index > 1 when it changed by less than tol.  errors (host,
 * n_iter_max) and *n_errors receive the errors.  Returns after the GPU
 * finished.  Each unfolding's Gram matrix must be within tlgb_sym_eig's size.
 */
typedef struct tlgb_tucker_options {
  int n_iter_max;   /* partial_tucker n_iter_max */
  double tol;       /* partial_tucker tol (0 disables the stop test) */
  int init_svd;     /* 1: factors from the SVD of the unfoldings of X ('svd') */
} tlgb_tucker_options;

void tlgb_tucker_default_options(tlgb_tucker_options* opts);
int tlgb_tucker_workspace_size(int dtype, int ndim, const int64_t* shape, int n_modes,
                               const int* modes, const int64_t* ranks, size_t* bytes);
int tlgb_tucker_hooi(int dtype, const void* X, int ndim, const int64_t* shape, int n_modes,
                     const int* modes, const int64_t* ranks, void* const* factors, void* core,
                     const tlgb_tucker_options* opts, double* errors, int* n_errors,
                     void* workspace, size_t workspace_bytes, void* stream);

/*
 * Batched CP-ALS of many small 3-way f32 tensors of uneven shape and rank:
 * for every item, the sweep loop of tensorly/decomposition/_cp.py:394-440
 * (parafac with normalize_factors=False), weights all one: exactly
 * n_iter_max sweeps when tol is 0, else each tensor stops after the first
 * sweep s >= 1 with |e_{s-1} - e_s| < tol (_cp.py:505-522, cvg_criterion
 * 'abs_rec_error'), e_s the relative error from the residual.  items (host array): device pointers to the
 * tensor (C order) and to the three factors (dims[k] x rank, row-major; the
 * initial factors on entry, the result on exit).  Mode sizes 1..64, rank
 * 1..16.  One persistent kernel per `sweeps_per_launch` sweeps (<= 0: all in
 * one launch); each CTA takes the next tensor from a work queue ordered by
 * decreasing work and keeps it in shared memory when it fits.
 * final_errors (device, n_tensors doubles): relative error of the final
 * model from the residual; sweep_errors (device, n_tensors x n_iter_max, or
 * NULL): per-sweep errors from the reference's expansion (_cp.py:217-225),
 * or from the residual when flags has TLGB_BATCH_EXACT_SWEEP_ERRORS or tol
 * is positive (rows are left unwritten past a tensor's stop); sweeps_done
 * (device, n_tensors ints, or NULL): the sweeps each tensor ran.
 * The call returns after the GPU finished.  No direct counterpart in TensorLy
 * (its users loop over parafac).
 */
typedef struct tlgb_batch_item {
  const void* X;
  void* factors[3];
  int64_t dims[3];
  int64_t rank;
} tlgb_batch_item;

int tlgb_cp_als_batched_workspace_size(int n_tensors, size_t* bytes);
#define TLGB_BATCH_EXACT_SWEEP_ERRORS 1
int tlgb_cp_als_batched(int n_tensors, const tlgb_batch_item* items, int n_iter_max,
                        int sweeps_per_launch, int flags, double tol, double* final_errors,
                        double* sweep_errors, int* sweeps_done, void* workspace,
                        size_t workspace_bytes, void* stream);

/*
 * Non-negative CP by multiplicative updates: the loop of
 * tensorly/decomposition/_nn_cp.py:26-183 (non_negative_parafac) with weights
 * all one, normalize_factors=False and no mask.  factors: the initial
 * non-negative factors on entry, the result on exit (dtype of X, row-major
 * shape[k] x rank).  free_modes: ascending, ending with ndim - 1 (the
 * reference frees the last mode).  With tol > 0 the relative error of every
 * iteration goes to errors (host, n_iter_max doubles) and the run stops at
 * the reference's test (cvg_criterion 0 'abs_rec_error', 1 'rec_error');
 * *n_errors receives how many were recorded (0 when tol is 0, as the
 * reference records none then).
 */
int tlgb_cp_nn_mu_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                                 int n_iter_max, size_t* bytes);
int tlgb_cp_nn_mu(int dtype, const void* X, int ndim, const int64_t* shape, void* const* factors,
                  int64_t rank, const int* free_modes, int n_free, int n_iter_max, double tol,
                  int cvg_criterion, double* errors, int* n_errors, void* workspace,
                  size_t workspace_bytes, void* stream);

/*
 * Non-negative CP by HALS: the loop of tensorly/decomposition/_nn_cp.py:186-377
 * (non_negative_parafac_hals) and its inner solver
 * tensorly/solvers/nnls.py:5-150 (hals_nnls, 100 iterations or, with exact,
 * 50000 at tol 1e-16).  Arguments as tlgb_cp_nn_mu, plus: weights: device,
 * rank entries, in/out, or NULL for weights all one (required when
 * normalize_factors is set); nn_modes_mask: bit k set = mode k is updated by
 * HALS, else by the least-squares solve of CP-ALS (the reference's nn_modes);
 * normalize_factors: cp_normalize after every updated mode but the last and
 * after every iteration.  sparsity: host array of ndim coefficients (NaN =
 * none) or NULL.  The workspace is tlgb_cp_nn_mu_workspace_size's.
 */
int tlgb_cp_nn_hals(int dtype, const void* X, int ndim, const int64_t* shape,
                    void* const* factors, void* weights, int64_t rank, const int* free_modes,
                    int n_free, unsigned nn_modes_mask, int normalize_factors, int n_iter_max,
                    double tol, int cvg_criterion, const double* sparsity, int exact,
                    double* errors, int* n_errors, void* workspace, size_t workspace_bytes,
                    void* stream);

/*
 * Pieces of the non-negative SVD (NNDSVD, tensorly/tenalg/svd.py:68-134):
 *   tlgb_sum             sum of n elements into *out (device f64); workspace
 *                        >= 256 doubles
 *   tlgb_nndsvd_columns  W (I x k) from U (I x k), S (k) and Y = U^T M viewed as
 *                        (L, k, Tt) (the mode-n product of the tensor with U^T);
 *                        fill 1: 'nndsvda' (entries below eps become avg),
 *                        0: 'nndsvd' (soft threshold); workspace >= 2 k elements
 */
int tlgb_sum(int dtype, const void* X, int64_t n, double* out, void* workspace,
             size_t workspace_bytes, void* stream);
int tlgb_nndsvd_columns(int dtype, const void* U, const void* S, const void* Y, int64_t I,
                        int64_t k, int64_t L, int64_t Tt, int fill, double avg, void* W,
                        void* workspace, size_t workspace_bytes, void* stream);

/*
 * Learned warm start for CP-ALS (no counterpart in TensorLy; its fallback is
 * TensorLy's init='svd', tensorly/decomposition/_cp.py:70-96).  Fixed problem
 * family: 32 x 32 x 32 f32 tensors of rank 8 (factor columns with pairwise
 * congruence c ~ U(0, 0.9) per mode, 1 % noise), generated from a seed by a
 * counter-based SplitMix64 generator; the network maps the three sketches
 * unfold(X, n) Omega_n (Omega_n: 1024 x 16 Gaussian, fixed) divided by ||X||
 * to the three 32 x 8 factors divided by ||X||^(1/3).
 *   tlgb_ws_omega      Omega (3 x 1024 x 16 f32)
 *   tlgb_ws_generate   tensors (batch x 32768), sketch features (batch x 1536)
 *                      and ||X|| (batch) of the tensors with the given seeds
 *   tlgb_ws_sketch     sketch features and ||X|| of tensors given in memory
 *   tlgb_ws_gemm       C(m, n) = epi(sum_k A[m sam + k sak] B[k sbk + n sbn])
 *                      (+ bias[n], ReLU if relu, zeroed where mask(m, n) <= 0)
 *   tlgb_ws_colsum     out[n] = sum_m Y[m ld + n]
 *   tlgb_ws_cp_loss    loss (batch) = min_a ||X - a [[A]]||^2 / ||X||^2 with
 *                      A = out * ||X||^(1/3) (= 1 - <X,[[A]]>^2 / (||X||^2 ||[[A]]||^2)),
 *                      its gradient with respect to out divided by batch (dout
 *                      may be NULL) and the best scale a (alpha, may be NULL)
 *   tlgb_ws_lift       initial factors = out * (||X|| alpha)^(1/3)
 *   tlgb_ws_sketch_skip out (batch x 3 x 32 x 8) += the first 8 columns of each
 *                      32 x 16 sketch block of feats (the network's fixed skip)
 *   tlgb_ws_adam       one Adam step on a flat parameter buffer
 *   tlgb_ws_svd_init   init='svd' factors (batch x 3 x 32 x 8) of the tensors
 * All pointers are device memory; all f32.
 */
int tlgb_ws_omega(void* omega, void* stream);
int tlgb_ws_generate(const int64_t* seeds, int batch, void* X, void* feats, void* xnorm,
                     const void* omega, void* stream);
int tlgb_ws_sketch(const void* X, int batch, void* feats, void* xnorm, const void* omega,
                   void* stream);
int tlgb_ws_gemm(int M, int N, int K, const void* A, int64_t sam, int64_t sak, const void* B,
                 int64_t sbk, int64_t sbn, void* C, int64_t ldc, const void* bias, int relu,
                 const void* mask, void* stream);
/*
 * ws_gemm_tc: the same product on the tensor cores (tcgen05): A and B split
 * exactly into three bf16 planes stored K-major in the workspace, each
 * 128 x 128 output tile accumulates the products a_i b_j with i + j <= 2
 * with f32 accumulation (the dropped terms are below 2^-26 of |a||b|).
 * Workspace
 * (tlgb_ws_gemm_tc_workspace_size, 256-byte aligned): its first int is a
 * status word that receives TLGB_ETIMEOUT if a bounded pipeline wait expired
 * (the caller zeroes it; read it with tlgb_workspace_status).
 */
int tlgb_ws_gemm_tc_workspace_size(int M, int N, int K, size_t* bytes);
int tlgb_ws_gemm_tc(int M, int N, int K, const void* A, int64_t sam, int64_t sak, const void* B,
                    int64_t sbk, int64_t sbn, void* C, int64_t ldc, const void* bias, int relu,
                    const void* mask, void* workspace, size_t workspace_bytes, void* stream);
int tlgb_ws_colsum(const void* Y, int M, int N, int64_t ld, void* out, void* stream);
int tlgb_ws_cp_loss(const void* X, const void* out, const void* xnorm, int batch, void* loss,
                    void* dout, void* alpha, void* stream);
int tlgb_ws_sketch_skip(const void* feats, int batch, void* out, void* stream);
int tlgb_ws_lift(const void* out, const void* xnorm, const void* alpha, int batch, void* factors,
                 void* stream);
int tlgb_ws_adam(void* params, const void* grads, void* m, void* v, int64_t n, float lr,
                 float beta1, float beta2, float eps, int step, void* stream);
int tlgb_ws_svd_init_workspace_size(int batch, size_t* bytes);
int tlgb_ws_svd_init(const void* X, int batch, void* factors, void* workspace,
                     size_t workspace_bytes, void* stream);

/*
 * cp_normalize: unit-norm factor columns, norms multiplied into weights
 * (factor 0 first absorbs the weights).  In place on factors and weights.
 * Replaces tensorly/cp_tensor.py:278-321 (cp_normalize).
 */
int tlgb_cp_normalize(int dtype, int ndim, const int64_t* rows, int64_t rank,
                      void* const* factors, void* weights, void* stream);

/*
 * cp_norm: ||[[weights; factors]]||_F from the Hadamard product of the factor
 * Grams (f64).  out: one double in device memory.  weights may be NULL.
 * Replaces tensorly/cp_tensor.py:614-644 (cp_norm).
 */
int tlgb_cp_norm_workspace_size(int ndim, const int64_t* rows, int64_t rank, size_t* bytes);
int tlgb_cp_norm(int dtype, int ndim, const int64_t* rows, int64_t rank,
                 const void* const* factors, const void* weights, double* out,
                 void* workspace, size_t workspace_bytes, void* stream);

/*
 * cp_to_tensor: the full C-order tensor (shape[0] x ... x shape[ndim-1]) of
 * [[weights; factors]], factors[k] row-major shape[k] x rank, computed as the
 * mode-0 unfolding (factors[0] * weights) . khatri_rao(factors[1:])^T without
 * forming the Khatri-Rao matrix.  weights (rank) and mask (the full shape,
 * multiplies the result) may be NULL.  ndim 1 gives sum_r w_r factors[0][:, r].
 * Replaces tensorly/cp_tensor.py:433-485 (cp_to_tensor); cp_to_unfolded
 * (:488-521) and cp_to_vec (:524-546) are this call on reordered factors and
 * a reshape.  dtype: TLGB_F32 or TLGB_F64.  The workspace holds the factors
 * transposed (sum_k shape[k] * rank elements).
 */
int tlgb_cp_to_tensor_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                                     size_t* bytes);
int tlgb_cp_to_tensor(int dtype, int ndim, const int64_t* shape, int64_t rank,
                      const void* const* factors, const void* weights, const void* mask,
                      void* out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * mask_impute: x = x * mask + rec * (1 - mask) in place (n entries, x, mask
 * and rec in the same dtype), and out[0] = ||x||_F, out[1] = ||x - rec||_F
 * (two doubles, device) of the refilled tensor.  Workspace:
 * tlgb_mask_impute_workspace_bytes().  Replaces the mask branch of
 * error_calc, tensorly/decomposition/_cp.py:194-207 (with rec =
 * cp_to_tensor((weights, factors))), and the refill at :441-446.
 */
size_t tlgb_mask_impute_workspace_bytes(void);
int tlgb_mask_impute(int dtype, void* x, const void* mask, const void* rec, int64_t n,
                     double* out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * mask_where: x = where(mask == 0, rec, x) in place, or the constant `fill`
 * in place of rec when rec is NULL (n entries, x, mask and rec in one dtype).
 * Replaces _update_imputed of tensorly/decomposition/_parafac2.py:21-65
 * (the "factors" and "mode-2" refills of masked slices).
 */
int tlgb_mask_where(int dtype, void* x, const void* mask, const void* rec, double fill,
                    int64_t n, void* stream);

/*
 * masked_sq_diff: *out (one double, device) = sum((mask * x - mask * rec)^2),
 * the per-slice term of the masked error of
 * tensorly/decomposition/_parafac2.py:389-396.  Workspace:
 * tlgb_dot_workspace_bytes().
 */
int tlgb_masked_sq_diff(int dtype, const void* x, const void* mask, const void* rec, int64_t n,
                        double* out, void* workspace, size_t workspace_bytes, void* stream);

/*
 * clip_min: x = max(x, lo) in place (NaN kept); tl.clip(x, 0) of the PARAFAC2
 * line search for non-negative modes (tensorly/decomposition/_parafac2.py:282-286).
 */
int tlgb_clip_min(int dtype, void* x, int64_t n, double lo, void* stream);

/*
 * cp_residual_norm: *out (one double, device) = ||X - [[weights; factors]]||_F
 * by the cp_to_tensor kernels with X read in place of the store (the full
 * tensor is never written).  Workspace: tlgb_cp_to_tensor_workspace_size.
 * Replaces tl.norm(tensor - cp_to_tensor(cp), 2) in
 * tensorly/decomposition/_cp.py:723-726 (randomised_parafac's error).
 */
int tlgb_cp_residual_norm(int dtype, const void* X, int ndim, const int64_t* shape, int64_t rank,
                          const void* const* factors, const void* weights, double* out,
                          void* workspace, size_t workspace_bytes, void* stream);

/*
 * sample_khatri_rao: out (n_samples x rank) = rows of khatri_rao(mats) at the
 * given positions, out[s, r] = prod_k mats[k][indices[k * n_samples + s], r]
 * in matrix order (indices: device int64, n_mats x n_samples, each in
 * [0, rows[k]); out-of-range indices read row 0).
 * Replaces the product of tensorly/decomposition/_cp.py:546-630
 * (sample_khatri_rao); the indices are drawn by the caller.
 */
int tlgb_sample_khatri_rao(int dtype, int n_mats, const void* const* mats, const int64_t* rows,
                           int64_t rank, int64_t n_samples, const int64_t* indices, void* out,
                           void* stream);

/*
 * One iteration of randomised CP-ALS (tensorly/decomposition/_cp.py:633-762):
 * for each mode in order, the factor becomes the least-squares solution
 * from n_samples sampled rows, solve(KR_s^T KR_s, KR_s^T X_s)^T, with KR_s
 * the sampled Khatri-Rao rows of the other factors and X_s the matching
 * rows of the unfolding; then *rec_error (host) = ||X - [[factors]]||_F
 * (weights one).  indices: device int64, ndim x (ndim-1) x n_samples: for
 * each mode the rows of the other modes in ascending mode order (the
 * reference's per-mode sample_khatri_rao draws).  Synchronises `stream`.
 * Returns TLGB_EINVAL for an out-of-range index, TLGB_ESINGULAR for
 * singular sampled normal equations.  rank <= 160.
 */
int tlgb_cp_randomised_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                                      int64_t n_samples, size_t* bytes);
int tlgb_cp_randomised_iteration(int dtype, const void* X, int ndim, const int64_t* shape,
                                 int64_t rank, void* const* factors, int64_t n_samples,
                                 const int64_t* indices, double* rec_error, void* workspace,
                                 size_t workspace_bytes, void* stream);
/*
 * The same iteration in two calls: cp_randomised_launch enqueues it on
 * `stream` and returns (indices must stay valid until it has run);
 * cp_randomised_finish waits for it and returns its checks and *rec_error,
 * so the host can draw the next iteration's indices in between.
 */
int tlgb_cp_randomised_launch(int dtype, const void* X, int ndim, const int64_t* shape,
                              int64_t rank, void* const* factors, int64_t n_samples,
                              const int64_t* indices, void* workspace, size_t workspace_bytes,
                              void* stream);
int tlgb_cp_randomised_finish(int dtype, int ndim, const int64_t* shape, int64_t rank,
                              int64_t n_samples, void* workspace, size_t workspace_bytes,
                              double* rec_error, void* stream);

/* constraint kinds of tlgb_cp_constrained / tlgb_proximal */
#define TLGB_CONS_NONE 0
#define TLGB_CONS_NON_NEGATIVE 1   /* clip(x, 0, max(x)) */
#define TLGB_CONS_L1 2             /* soft thresholding by param */
#define TLGB_CONS_L2 3             /* x - x * param / max(||x||, param) */
#define TLGB_CONS_L2_SQUARE 4      /* x / (1 + 2 param) */
#define TLGB_CONS_NORMALIZE 5      /* x / max |x| */
/* column-wise and rank-based operators (tlgb_proximal_matrix, tlgb_cp_constrained) */
#define TLGB_CONS_UNIMODALITY 6    /* unimodal fit of each column */
#define TLGB_CONS_SIMPLEX 7        /* projection of each column on the simplex of size param */
#define TLGB_CONS_NORM_SPARSITY 8  /* the param largest |x| kept, then x / ||x|| */
#define TLGB_CONS_SOFT_SPARSITY 9  /* simplex projection of |x| (size param) times sign(x) */
#define TLGB_CONS_SMOOTHNESS 10    /* (I (1 + 2 param) - param (sub + super diagonal))^-1 x */
#define TLGB_CONS_MONOTONICITY 11  /* non-decreasing fit of each column (param != 0: non-increasing) */
#define TLGB_CONS_HARD_SPARSITY 12 /* the param largest |x| kept, the rest set to 0 */

/*
 * Constrained CP by AO-ADMM (tensorly/decomposition/_constrained_cp.py:166-435,
 * ADMM tensorly/solvers/admm.py:5-135).  factors[k] (shape[k] x rank) hold
 * the initial factors (already passed through their proximal operator, as
 * initialize_constrained_parafac does) and receive the result; the dual
 * variables start at zero.  kinds/params: per mode, the TLGB_CONS_* kind and
 * its parameter (the proximal operators of tensorly/tenalg/proximal.py that
 * act on the whole matrix).  free_modes ascending, the last mode free.
 * errors (host, n_iter_max) receive the relative errors; *n_errors their
 * count.  Synchronises `stream` once per outer iteration.
 */
int tlgb_cp_constrained_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                                       size_t* bytes);
int tlgb_cp_constrained(int dtype, const void* X, int ndim, const int64_t* shape,
                        void* const* factors, int64_t rank, const int* free_modes, int n_free,
                        const int* kinds, const double* params, int n_iter_max,
                        int n_iter_max_inner, double tol_outer, double tol_inner,
                        int cvg_criterion, double* errors, int* n_errors, void* workspace,
                        size_t workspace_bytes, void* stream);

/*
 * proximal: out = the proximal operator `kind` (TLGB_CONS_*) with `param` of
 * the n values of X (tensorly/tenalg/proximal.py:148-267, the whole-matrix
 * operators).  Workspace of tlgb_proximal_workspace_bytes() bytes for
 * non_negative, l2 and normalize (a global max or norm), else may be NULL.
 */
size_t tlgb_proximal_workspace_bytes(void);
int tlgb_proximal(int dtype, const void* X, int64_t n, int kind, double param, void* out,
                  void* workspace, size_t workspace_bytes, void* stream);

/*
 * proximal_matrix: out = the proximal operator `kind` of a rows x cols
 * row-major matrix Y (a factor matrix; tensorly/tenalg/proximal.py:148-628),
 * including the column-wise operators unimodality_prox (:359-441),
 * simplex_prox (:558-599), soft_sparsity_prox (:529-555), smoothness_prox
 * (:270-289), monotonicity_prox (:292-356) and the rank-based
 * hard_thresholding (:602-628) and normalized_sparsity_prox (:496-526);
 * the whole-matrix kinds are tlgb_proximal's.  A column must fit one CTA's
 * shared memory (else TLGB_EUNSUPPORTED).  Entries of equal magnitude at the
 * hard-thresholding cut are kept in index order (the reference's argsort
 * leaves that order unspecified).  out must not alias Y.
 */
int tlgb_proximal_matrix_workspace_size(int dtype, int64_t rows, int64_t cols, int kind,
                                        size_t* bytes);
int tlgb_proximal_matrix(int dtype, const void* Y, int64_t rows, int64_t cols, int kind,
                         double param, void* out, void* workspace, size_t workspace_bytes,
                         void* stream);

/*
 * gemm: C (M x N, row-major) = sum_k A[m*sam + k*sak] * B[k*sbk + n*sbn]
 * (any transposition through the strides), accumulated in the input type.
 * For the core-sized products of the Tucker updates (tl.dot on unfolded
 * cores and factor Grams); not a tuned large GEMM.
 */
int tlgb_gemm(int dtype, int64_t M, int64_t N, int64_t K, const void* A, int64_t sam,
              int64_t sak, const void* B, int64_t sbk, int64_t sbn, void* C, void* stream);

/*
 * mu_update: A <- A * max(num, eps) / max(den, eps), elementwise over n
 * values (the multiplicative updates of tensorly/decomposition/_tucker.py:
 * 396-418, clip(a_min=eps)).
 */
int tlgb_mu_update(int dtype, void* A, const void* num, const void* den, int64_t n, double eps,
                   void* stream);

/* dot: *out (device double) = sum_e a[e] * b[e], f64, in a fixed order. */
size_t tlgb_dot_workspace_bytes(void);
int tlgb_dot(int dtype, const void* a, const void* b, int64_t n, double* out, void* workspace,
             size_t workspace_bytes, void* stream);

/*
 * hals_nnls: the reference's HALS non-negative least squares
 * (tensorly/solvers/nnls.py:5-175) on the transposed layout: V (I x R, in/out)
 * is its V^T, MtU (I x R) its UtM^T, UtU (R x R) its UtU (symmetrised from the
 * upper triangle).  Up to n_iter_max iterations with its stop test (tol), an
 * optional sparsity coefficient (NaN for none).  Synchronises `stream`
 * between chunks of 100 iterations.  rank <= 160.
 */
int tlgb_hals_nnls_workspace_size(int dtype, int64_t I, int64_t R, size_t* bytes);
int tlgb_hals_nnls(int dtype, const void* MtU, const void* UtU, void* V, int64_t I, int64_t R,
                   int n_iter_max, double tol, double sparsity, void* workspace,
                   size_t workspace_bytes, void* stream);

/*
 * sparse_residual: with R = X - L (n entries), *out (device double) =
 * ||R - sparsify(R, k)||_F, where sparsify keeps the entries of R whose
 * magnitude is at least the k-th largest |R| and zeroes the rest
 * (tensorly/decomposition/_cp.py:140-159, the sparse-component error of
 * error_calc, :202-215); k > n keeps everything (error 0).  When `sparse` is
 * given it receives sparsify(R, k).  The k-th largest magnitude comes from a
 * radix select on the device (4 passes for f32, 8 for f64).  Workspace:
 * tlgb_sparse_residual_workspace_bytes().
 */
size_t tlgb_sparse_residual_workspace_bytes(void);
int tlgb_sparse_residual(int dtype, const void* X, const void* L, int64_t n, int64_t k,
                         double* out, void* sparse, void* workspace, size_t workspace_bytes,
                         void* stream);

/*
 * kronecker: out = mats[0] (x) mats[1] (x) ... (row-major matrices of
 * rows[k] x cols[k]), the first varying slowest
 * (tensorly/tenalg/core_tenalg/_kronecker.py).
 */
int tlgb_kronecker(int dtype, int n_mats, const void* const* mats, const int64_t* rows,
                   const int64_t* cols, void* out, void* stream);

/*
 * tucker_normalize: in place, every column of factor k (rows[k] x ranks[k],
 * row-major) divided by its norm (a zero column kept) and the core
 * (ranks[0] x ... , row-major) multiplied along each mode by those norms.
 * Replaces tensorly/tucker_tensor.py:78-102 (tucker_normalize).
 */
int tlgb_tucker_normalize_workspace_size(int ndim, const int64_t* ranks, size_t* bytes);
int tlgb_tucker_normalize(int dtype, int ndim, const int64_t* rows, const int64_t* ranks,
                          void* const* factors, void* core, void* workspace,
                          size_t workspace_bytes, void* stream);

/*
 * active_set_nnls: x (n, device, in/out, the start) minimises
 * ||Utm - UtU x|| subject to x >= 0 by the active-set method of
 * tensorly/solvers/nnls.py:275-406, at most n_iter_max iterations, stop when
 * the largest gradient entry on the active set is <= tol.  One CTA; n <= 128
 * (else TLGB_EUNSUPPORTED).  *status (device int) receives TLGB_OK, or
 * TLGB_ESINGULAR where the reference's solve would raise.
 */
int tlgb_active_set_nnls(int dtype, const void* UtU, const void* Utm, void* x, int64_t n,
                         int n_iter_max, double tol, int* status, void* stream);

/*
 * fista_tucker_core: the reference's FISTA (tensorly/solvers/nnls.py:177-272,
 * non_negative, no ridge) for a Tucker core: x (the core, shape[], in/out)
 * minimises 1/2 <x, x x_k G_k> - <UtM, x> (+ sparsity sum x), gradient
 * -UtM + x x_k grams[k] + sparsity, step lr, floor eps, the momentum of the
 * reference, stop when |sum(x - x_new)| < tol * its first value.  No host
 * round trip (a device stop flag).
 */
int tlgb_fista_tucker_core_workspace_size(int dtype, int ndim, const int64_t* shape,
                                          size_t* bytes);
int tlgb_fista_tucker_core(int dtype, const void* UtM, int ndim, const int64_t* shape,
                           const void* const* grams, void* x, int n_iter_max, double sparsity,
                           double lr, double tol, double eps, void* workspace,
                           size_t workspace_bytes, void* stream);

/* inv_sqrt: out = 1 / sqrt(x) over n values (PARAFAC2 polar factors). */
int tlgb_inv_sqrt(int dtype, const void* x, int64_t n, void* out, void* stream);

/* lerp: out = x + (y - x) * s over n values (PARAFAC2 line search). */
int tlgb_lerp(int dtype, const void* x, const void* y, int64_t n, double s, void* out,
              void* stream);

/*
 * qr: Q (m x n, row-major) of the Householder QR of A (m x n, m >= n,
 * n <= 256) in LAPACK's conventions (dgeqr2 reflectors, dorg2r's explicit Q),
 * so its column signs are NumPy's linalg.qr.  One CTA; for the small tall
 * matrices of tensorly/random/base.py:18-61 (random_parafac2's projections).
 */
int tlgb_qr_workspace_size(int dtype, int64_t m, int64_t n, size_t* bytes);
int tlgb_qr(int dtype, const void* A, int64_t m, int64_t n, void* Q, void* workspace,
            size_t workspace_bytes, void* stream);

/*
 * unfold: out (shape[mode] x prod(other modes)) = the mode-`mode` unfolding of
 * the C-order tensor X, columns in the C order of the other modes
 * (tensorly/base.py:39-53, moveaxis(X, mode, 0).reshape(shape[mode], -1)).
 * fold: its inverse, out = the tensor of `shape` (tensorly/base.py:56-79).
 */
int tlgb_unfold(int dtype, const void* X, int ndim, const int64_t* shape, int mode, void* out,
                void* stream);
int tlgb_fold(int dtype, const void* unfolded, int ndim, const int64_t* shape, int mode,
              void* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TENSORLY_GB300_H */
