// Native CP-ALS driver: the sweep loop of tensorly/decomposition/_cp.py:394-530
// (parafac) run entirely on the GPU.
//
// One sweep = for each non-fixed mode: f64 factorisation of the normal
// equations (k_factorize), split MTTKRP, fused partial-sum + f64 solve + Gram
// partials (k_solve), Gram reduction; then the fit (k_fit) and, if asked,
// cp_normalize.  The stop test runs on the device: k_fit raises a `done`
// flag that makes every later sweep kernel return at once, so the host can
// enqueue several sweeps (one CUDA graph launch each) and read the flag only
// every `check_every` sweeps.  With a callback the host syncs every sweep.
#include <cstring>
#include <vector>

#include "als_kernels.cuh"
#include "mttkrp_simt.cuh"
#include "mttkrp_tc.cuh"

namespace tlgb {
namespace {

struct AlsBuffers {
  AlsCtrl* ctrl;
  double* errors;
  double* G;
  float* G32;                           // (hi, lo) f32 planes of every Gram (f32 factors)
  double* fac;
  int* perm;
  double* vmat;                         // V of the current mode (f64)
  float* w32;                           // f32 inverse of V (refinement path)
  void* partial;
  double* gpart;
  double* ipart;
  double* sumsq_part;
  __nv_bfloat16* xbf;                   // bf16 copy of X (mixed precision) = split plane x0
  __nv_bfloat16* xsplit[2];             // planes x1, x2 of the exact split (f32 refinement)
  __nv_bfloat16* fbt[kMaxModes];        // bf16 split transposed factors (3 x rank x rows)
  void* tc_partial;
  double* probe;                        // one f64 result slot (initial error)
  double* fpart;                        // per-block cp_norm^2 terms of the fused fit
  size_t bytes;
};

constexpr int kSumsqBlocks = 1024;

constexpr int kFactorPlanes = 3;
// The factorisation of the next normal equations runs on a side stream during
// each MTTKRP (one CTA): the tensor-core MTTKRP grid leaves this many SMs free
// for it (measured at 512^3: 86 us -> 55 us per MTTKRP).
constexpr int kAuxSms = 1;

struct Plans {
  MttkrpPlan simt[kMaxModes];
  TcPlan tc[kMaxModes];          // bf16 sweeps (2 factor planes)
  TcPlan tcr[kMaxModes][3];      // closing sweeps: x0, x1 (, x2) with 3, 2 (, 1) factor planes
  bool refine_tc = false;        // refinement sweeps run on the tensor cores
  int xplanes = 2;               // tensor planes the closing sweeps contract (2 or 3)
};

int layout(int dtype, const Shape& sh, int64_t R, const tlgb_cp_als_options& o,
           const Plans& P, void* base, AlsBuffers* B) {
  const MttkrpPlan* plans = P.simt;
  Carver c(base);
  const int64_t RR = R * R;
  const int esz = dtype == TLGB_F64 ? 8 : 4;
  B->ctrl = c.take<AlsCtrl>(1);
  B->errors = c.take<double>(std::max(1, o.n_iter_max));
  B->G = c.take<double>((size_t)sh.ndim * RR);
  B->G32 = (dtype == TLGB_F32) ? c.take<float>((size_t)sh.ndim * 2 * RR) : nullptr;
  B->fac = c.take<double>((size_t)RR + R);
  B->perm = c.take<int>(R);
  B->vmat = c.take<double>((size_t)RR);
  B->w32 = c.take<float>((size_t)3 * RR);   // W = V^-1 (f32), then V's f32 hi and lo planes
  size_t pmax = 0;
  int64_t imax = 0;
  for (int k = 0; k < sh.ndim; ++k) {
    pmax = std::max(pmax, plans[k].partial_bytes);
    imax = std::max(imax, sh.dim[k]);
  }
  B->partial = c.take<char>(pmax);
  const int nparts = solve_blocks_for(imax);
  B->gpart = c.take<double>((size_t)nparts * RR);
  B->ipart = c.take<double>(nparts);
  B->sumsq_part = c.take<double>(kSumsqBlocks);
  B->probe = c.take<double>(1);
  B->fpart = c.take<double>((size_t)ceil_div(RR, 32));   // per-block fit terms of k_gram_reduce_fit
  B->xbf = nullptr;
  B->xsplit[0] = B->xsplit[1] = nullptr;
  for (int k = 0; k < kMaxModes; ++k) B->fbt[k] = nullptr;
  B->tc_partial = nullptr;
  if (o.precision == TLGB_PREC_BF16) {
    B->xbf = c.take<__nv_bfloat16>((size_t)sh.numel);
    if (P.refine_tc) {
      B->xsplit[0] = c.take<__nv_bfloat16>((size_t)sh.numel);
      if (P.xplanes == 3) B->xsplit[1] = c.take<__nv_bfloat16>((size_t)sh.numel);
    }
    for (int k = 0; k < sh.ndim; ++k)
      B->fbt[k] = c.take<__nv_bfloat16>((size_t)kFactorPlanes * R * sh.dim[k]);
    size_t tmax = 0;
    for (int k = 0; k < sh.ndim; ++k) {
      if (P.tc[k].valid) tmax = std::max(tmax, P.tc[k].partial_bytes);
      if (P.refine_tc) {
        size_t sum = 0;
        for (int j = 0; j < P.xplanes; ++j) sum += P.tcr[k][j].partial_bytes;
        tmax = std::max(tmax, sum);
      }
    }
    B->tc_partial = c.take<char>(tmax);
  }
  (void)esz;
  B->bytes = c.used();
  return TLGB_OK;
}

int validate(int dtype, int ndim, const int64_t* shape, int64_t rank,
             const tlgb_cp_als_options* o) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "cp_als: dtype must be f32 or f64");
  TLGB_CHECK_ARG(shape != nullptr && o != nullptr, "cp_als: null pointer");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "cp_als: ndim must be in [2, 8]");
  TLGB_CHECK_ARG(rank >= 1, "cp_als: rank must be >= 1");
  if (rank > kMaxAlsRank)
    return set_error(TLGB_EUNSUPPORTED, "cp_als: rank above 160 is not supported");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(shape[k] >= 1, "cp_als: empty mode");
  TLGB_CHECK_ARG(o->n_iter_max >= 0, "cp_als: n_iter_max must be >= 0");
  TLGB_CHECK_ARG(o->cvg_criterion == 0 || o->cvg_criterion == 1, "cp_als: bad cvg_criterion");
  if (o->precision == TLGB_PREC_BF16) {
    if (dtype != TLGB_F32)
      return set_error(TLGB_EUNSUPPORTED, "cp_als: bf16 precision needs an f32 tensor");
    TLGB_CHECK_ARG(o->refine_sweeps >= 0, "cp_als: refine_sweeps must be >= 0");
  } else {
    TLGB_CHECK_ARG(o->precision == TLGB_PREC_NATIVE, "cp_als: unknown precision");
  }
  return TLGB_OK;
}

int make_plans(int dtype, const Shape& sh, int64_t R, const tlgb_cp_als_options& o, Plans* P) {
  const bool mixed = o.precision == TLGB_PREC_BF16;
  P->refine_tc = mixed && o.refine_sweeps > 0 && !tc_tuning().refine_simt;
  P->xplanes = tc_tuning().closing_planes == 3 ? 3 : 2;
  for (int k = 0; k < sh.ndim; ++k) {
    int rc = mttkrp_make_plan(dtype, sh, R, k, &P->simt[k]);
    if (rc) return rc;
    P->tc[k] = TcPlan{};
    for (int j = 0; j < 3; ++j) P->tcr[k][j] = TcPlan{};
    if (mixed) {
      rc = mttkrp_tc_make_plan(sh, R, k, 2, kAuxSms, &P->tc[k]);
      if (rc) return rc;
      P->tc[k].pdl = 1;   // programmatic launch behind the previous solve
    }
    if (P->refine_tc) {
      for (int j = 0; j < P->xplanes; ++j) {
        rc = mttkrp_tc_make_plan(sh, R, k, 3 - j, kAuxSms, &P->tcr[k][j]);
        if (rc) return rc;
        if (!P->tcr[k][j].valid) P->refine_tc = false;
        P->tcr[k][j].pdl = 1;
      }
    }
  }
  return TLGB_OK;
}

constexpr int kSweepNative = 0;
constexpr int kSweepBf16 = 1;
constexpr int kSweepF32Tc = 2;
constexpr int kSweepF32TcFinal = 3;
constexpr int kCpAlsSweepKinds = TLGB_CP_ALS_SWEEP_KINDS;

template <typename T>
struct Runner {
  const T* X;
  Shape sh;
  int64_t R;
  T* const* factors;
  T* weights;
  tlgb_cp_als_options o;
  Plans* P;
  AlsBuffers B;
  std::vector<int> modes;
  // The last mode's Gram reduction and fit of the previous sweep when that
  // sweep deferred it (mode < 0: none pending).
  int fit_mode = -1, fit_nb = 0, fit_df = 0;
  // The factorisation of mode n's normal equations needs only the Grams, so
  // it runs on `aux` concurrently with mode n's MTTKRP (fork/join by events,
  // captured into the graph as parallel branches).
  cudaStream_t aux = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  // optional timing events around each mode's MTTKRP (recorded into the graph)
  cudaEvent_t ev_mt[2][kMaxModes] = {};
  // TMA descriptors of the tensor-core MTTKRPs, encoded once per run
  TcMaps tc_maps[kMaxModes];
  TcMaps tcr_maps[kMaxModes][3];

  int encode_maps() {
    const __nv_bfloat16* planes[3] = {B.xbf, B.xsplit[0], B.xsplit[1]};
    for (int k = 0; k < sh.ndim; ++k) {
      if (P->tc[k].valid) {
        int rc = mttkrp_tc_encode(P->tc[k], B.xbf, B.fbt, kFactorPlanes, &tc_maps[k]);
        if (rc) return rc;
      }
      if (P->refine_tc)
        for (int j = 0; j < P->xplanes; ++j) {
          int rc = mttkrp_tc_encode(P->tcr[k][j], planes[j], B.fbt, kFactorPlanes,
                                    &tcr_maps[k][j]);
          if (rc) return rc;
        }
    }
    return TLGB_OK;
  }

  // Enqueues one sweep.  kind: kSweepNative (SIMT MTTKRP in the tensor dtype),
  // kSweepBf16 (bf16 tensor, two-plane factor, tensor cores), kSweepF32Tc
  // (the split f32 tensor and three-plane factor on the tensor cores) or
  // kSweepF32TcFinal (the same, but the last mode's MTTKRP on the SIMT f32
  // kernel).  The tensor cores' f32 accumulation rounds toward zero (measured
  // bias about -2e-7 of |M| at 512^3, against ~1e-10 for the SIMT kernel) and
  // the fit's cancellation amplifies an error in <M_last, A_last> by about
  // ||X||^2 / rec_error^2; the closing sweep's last MTTKRP feeds the reported
  // error, so it runs unbiased.
  //
  // defer_fit: the last mode's Gram reduction and the fit are left to the
  // next sweep, which runs them on the aux stream in front of its first
  // factorisation (their only consumer besides the stop test), so the next
  // sweep's first MTTKRP follows the last solve directly.  The stop flag the
  // fit raises is then seen one sweep late: every kernel of that next sweep
  // that writes a factor or the Grams runs after the fit (its solves wait for
  // the aux stream) and returns at once, so the factors stay those of the
  // converged sweep.  Not used with normalize_factors (the normalisation
  // rewrites the Grams and the weights the fit reads).
  int sweep(int kind, cudaStream_t st, bool defer_fit = false) {
    const bool tc = kind == kSweepBf16;
    const int N = sh.ndim;
    const int RR = (int)(R * R);
    const int* done = &B.ctrl->done;
    const T* cf[kMaxModes];
    for (int k = 0; k < N; ++k) cf[k] = factors[k];
    // The reference's Khatri-Rao of a single remaining factor drops the
    // weights (tensorly/tenalg/core_tenalg/_khatri_rao.py:71-73), so a 2-way
    // MTTKRP is unweighted there; kept for parity.
    const T* mw = (N == 2) ? nullptr : weights;
    const int df = (sizeof(T) == 4 && R <= kSolveDfMaxRank) ? 1 : 0;
    // Main-stream kernels that follow a kernel of this sweep start by
    // programmatic dependent launch: they are scheduled while their
    // predecessor drains and wait for it on the device.
    const bool pdl = !tc_tuning().no_pdl;
    // The Gram reduction of a mode other than the last runs on the aux
    // stream in front of the next mode's factorisation (the only consumer of
    // that Gram), so the next MTTKRP does not wait for it.
    int pending_mode = -1, pending_nb = 0, pending_df = 0;
    for (size_t mi = 0; mi < modes.size(); ++mi) {
      const int mode = modes[mi];
      const bool last = (mi + 1 == modes.size());
      TLGB_CUDA_TRY(cudaEventRecord(ev_fork, st));
      TLGB_CUDA_TRY(cudaStreamWaitEvent(aux, ev_fork, 0));
      int rc;
      if (fit_mode >= 0) {   // the previous sweep's deferred fit
        rc = als_launch_gram_reduce_fit<T>(B.gpart, fit_nb, (int)R, B.G, fit_mode, N, fit_df,
                                           weights, B.ipart, fit_nb, B.fpart, B.ctrl, B.errors,
                                           o.n_iter_max, o.tol, o.cvg_criterion, aux, false,
                                           B.G32, true);
        if (rc) return rc;
        fit_mode = -1;
      }
      if (pending_mode >= 0) {
        rc = als_launch_gram_reduce(B.gpart, pending_nb, (int)R,
                                    B.G + (size_t)pending_mode * RR, done, pending_df, aux,
                                    B.G32 ? B.G32 + (size_t)pending_mode * 2 * RR : nullptr);
        if (rc) return rc;
        pending_mode = -1;
      }
      rc = als_launch_factorize<T>(B.G, N, mode, (int)R, weights, o.l2_reg, B.fac, B.perm,
                                   B.vmat, B.w32, B.ctrl, aux, B.G32);
      if (rc) return rc;
      TLGB_CUDA_TRY(cudaEventRecord(ev_join, aux));
      if (ev_mt[0][mode]) TLGB_CUDA_TRY(cudaEventRecord(ev_mt[0][mode], st));
      int splits;
      const void* partial;
      if (tc && P->tc[mode].valid) {
        if constexpr (sizeof(T) == 4) {
          rc = mttkrp_tc_launch_maps(P->tc[mode], tc_maps[mode], (const float* const*)cf,
                                     (const float*)mw, (float*)B.tc_partial, done,
                                     &B.ctrl->tc_err, st);
        }
        if (rc) return rc;
        splits = P->tc[mode].splits;
        partial = B.tc_partial;
      } else if (kind == kSweepF32Tc || (kind == kSweepF32TcFinal && !last)) {
        // x0 . (f0 + f1 + f2) + x1 . (f0 + f1) (+ x2 . f0 with three tensor
        // planes), each launch writing its own run of partial tiles; the solve
        // sums all of them
        splits = 0;
        if constexpr (sizeof(T) == 4) {
          for (int j = 0; j < P->xplanes && !rc; ++j) {
            const TcPlan& tp = P->tcr[mode][j];
            rc = mttkrp_tc_launch_maps(tp, tcr_maps[mode][j], (const float* const*)cf,
                                       (const float*)mw,
                                       (float*)B.tc_partial + (size_t)splits * tp.I_out * tp.R,
                                       done, &B.ctrl->tc_err, st);
            splits += tp.splits;
          }
        }
        if (rc) return rc;
        partial = B.tc_partial;
      } else {
        rc = mttkrp_launch_partials<T>(P->simt[mode], X, cf, mw, (T*)B.partial, done, st);
        if (rc) return rc;
        splits = P->simt[mode].splits;
        partial = B.partial;
      }
      if (ev_mt[1][mode]) TLGB_CUDA_TRY(cudaEventRecord(ev_mt[1][mode], st));
      TLGB_CUDA_TRY(cudaStreamWaitEvent(st, ev_join, 0));
      int nb = 0;
      // the bf16 sweeps' solve keeps its Gram in plain f32 (one plane)
      const bool lite = tc && P->tc[mode].valid && !tc_tuning().full_solve;
      const int gdf = (df && lite) ? 2 : df;
      rc = als_launch_solve<T>((const T*)partial, splits, sh.dim[mode], (int)R, B.fac, B.perm,
                               B.vmat, B.w32, factors[mode], B.fbt[mode], B.gpart,
                               last ? B.ipart : nullptr, B.ctrl,
                               // the bf16 sweeps take x = m W (f32 inverse) with no
                               // correction pass: their MTTKRP is itself only accurate
                               // to ~1e-6, and the closing sweeps solve in double-float
                               (tc && P->tc[mode].valid) ? (tc_tuning().lite_correction ? 1 : 0)
                                                         : kIrMaxPasses,
                               &nb, st, pdl, lite);
      if (rc) return rc;
      if (last && defer_fit && !o.normalize_factors && !tc_tuning().inline_fit) {
        fit_mode = mode;
        fit_nb = nb;
        fit_df = gdf;
      } else if (last) {   // the last mode's Gram reduction also computes the fit (in order)
        rc = als_launch_gram_reduce_fit<T>(B.gpart, nb, (int)R, B.G, mode, N, gdf, weights,
                                           B.ipart, nb, B.fpart, B.ctrl, B.errors,
                                           o.n_iter_max, o.tol, o.cvg_criterion, st, pdl, B.G32);
        if (rc) return rc;
      } else {      // reduced on the aux stream before the next factorisation
        pending_mode = mode;
        pending_nb = nb;
        pending_df = gdf;
      }
    }
    int rc = TLGB_OK;
    if (o.normalize_factors) {
      rc = als_launch_normalize<T>(factors, sh.dim, N, (int)R, weights, done, st);
      if (rc) return rc;
      rc = grams(done, st);
      if (rc) return rc;
      if (kind != kSweepNative) {
        rc = bf16_factors(st);
        if (rc) return rc;
      }
    }
    return TLGB_OK;
  }

  // A fit still deferred when a phase ends early (the host saw the stop flag
  // and launched no further sweep) runs here, on the main stream before the
  // next phase clears the flag: it then finds the flag set and records
  // nothing, instead of running in the next phase on the partials of a
  // sweep that did no work.
  int flush_fit(cudaStream_t st) {
    if (fit_mode < 0) return TLGB_OK;
    const int mode = fit_mode;
    fit_mode = -1;
    return als_launch_gram_reduce_fit<T>(B.gpart, fit_nb, (int)R, B.G, mode, sh.ndim, fit_df,
                                         weights, B.ipart, fit_nb, B.fpart, B.ctrl, B.errors,
                                         o.n_iter_max, o.tol, o.cvg_criterion, st, false, B.G32);
  }

  int grams(const int* done, cudaStream_t st) {
    const int RR = (int)(R * R);
    int64_t imax = 0;
    for (int k = 0; k < sh.ndim; ++k) imax = std::max(imax, sh.dim[k]);
    for (int k = 0; k < sh.ndim; ++k) {
      int rc = als_launch_gram<T>(factors[k], sh.dim[k], (int)R, B.gpart, solve_blocks_for(imax),
                                  B.G + (size_t)k * RR, done, st,
                                  B.G32 ? B.G32 + (size_t)k * 2 * RR : nullptr);
      if (rc) return rc;
    }
    return TLGB_OK;
  }

  // Relative error of the initial model (what the reference's callback gets
  // before the first sweep, tensorly/decomposition/_cp.py:379-392).
  int initial_error(cudaStream_t st, double* host_err) {
    const int N = sh.ndim;
    const int last = N - 1;
    const T* cf[kMaxModes];
    for (int k = 0; k < N; ++k) cf[k] = factors[k];
    int rc = mttkrp_launch_partials<T>(P->simt[last], X, cf, weights, (T*)B.partial, nullptr, st);
    if (rc) return rc;
    int64_t imax = 0;
    for (int k = 0; k < N; ++k) imax = std::max(imax, sh.dim[k]);
    rc = als_launch_probe_error<T>((const T*)B.partial, P->simt[last].splits, sh.dim[last], (int)R,
                                   factors[last], B.G, N, weights, B.ipart, solve_blocks_for(imax),
                                   B.ctrl, B.probe, st);
    if (rc) return rc;
    TLGB_CUDA_TRY(cudaMemcpyAsync(host_err, B.probe, sizeof(double), cudaMemcpyDeviceToHost, st));
    TLGB_CUDA_TRY(cudaStreamSynchronize(st));
    return TLGB_OK;
  }

  // bf16 transposed copies of every factor (tensor-core operand B)
  int bf16_factors(cudaStream_t st) {
    for (int k = 0; k < sh.ndim; ++k) {
      int rc = tc_launch_factor_bf16t((const float*)factors[k], sh.dim[k], R, kFactorPlanes,
                                      B.fbt[k], st);
      if (rc) return rc;
    }
    return TLGB_OK;
  }
};

class StreamGuard {
 public:
  cudaStream_t s = nullptr;
  ~StreamGuard() { if (s) cudaStreamDestroy(s); }
};
class EventGuard {
 public:
  cudaEvent_t e = nullptr;
  ~EventGuard() { if (e) cudaEventDestroy(e); }
};
class GraphGuard {
 public:
  cudaGraph_t g = nullptr;
  cudaGraphExec_t e = nullptr;
  GraphGuard() = default;
  GraphGuard(const GraphGuard&) = delete;
  GraphGuard& operator=(const GraphGuard&) = delete;
  ~GraphGuard() {
    if (e) cudaGraphExecDestroy(e);
    if (g) cudaGraphDestroy(g);
  }
};

template <typename T>
int run(const T* X, const Shape& sh, int64_t R, T* const* factors, T* weights,
        const tlgb_cp_als_options& o, double* errors_host, int* n_errors, void* ws,
        size_t ws_bytes, cudaStream_t st) {
  Plans P;
  int rc = make_plans(TypeCode<T>::value, sh, R, o, &P);
  if (rc) return rc;
  Runner<T> run{};
  run.X = X; run.sh = sh; run.R = R; run.factors = factors; run.weights = weights; run.o = o;
  run.P = &P;
  rc = layout(TypeCode<T>::value, sh, R, o, P, ws, &run.B);
  if (rc) return rc;
  if (ws_bytes < run.B.bytes) return set_error(TLGB_EWORKSPACE, "cp_als: workspace too small");
  for (int k = 0; k < sh.ndim; ++k)
    if (!((o.fixed_modes >> k) & 1u) || k == sh.ndim - 1) run.modes.push_back(k);
  if (n_errors) *n_errors = 0;
  rc = mttkrp_prepare(TypeCode<T>::value);
  if (rc) return rc;
  rc = als_prepare(TypeCode<T>::value);
  if (rc) return rc;
  const bool mixed = o.precision == TLGB_PREC_BF16;
  if (mixed) {
    rc = mttkrp_tc_prepare();
    if (rc) return rc;
    rc = run.encode_maps();
    if (rc) return rc;
  }

  StreamGuard aux;
  EventGuard ev_fork, ev_join;
  TLGB_CUDA_TRY(cudaStreamCreateWithFlags(&aux.s, cudaStreamNonBlocking));
  TLGB_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork.e, cudaEventDisableTiming));
  TLGB_CUDA_TRY(cudaEventCreateWithFlags(&ev_join.e, cudaEventDisableTiming));
  run.aux = aux.s;
  run.ev_fork = ev_fork.e;
  run.ev_join = ev_join.e;
  EventGuard ev_mt[2][kMaxModes];
  if (o.mttkrp_ms) {
    for (int i = 0; i < kCpAlsSweepKinds * kMaxModes; ++i) o.mttkrp_ms[i] = 0.0;
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < sh.ndim; ++k) {
        TLGB_CUDA_TRY(cudaEventCreate(&ev_mt[j][k].e));
        run.ev_mt[j][k] = ev_mt[j][k].e;
      }
  }

  // ---- set-up: control block, ||X||^2, Grams, bf16 operands
  TLGB_CUDA_TRY(cudaMemsetAsync(run.B.ctrl, 0, sizeof(AlsCtrl), st));
  if (mixed) {
    // The Grams and the factors' bf16 planes on the side stream, beside the
    // pass over X that writes its bf16 planes (and, with the closing sweeps'
    // split, ||X||^2 in the same pass).
    TLGB_CUDA_TRY(cudaEventRecord(run.ev_fork, st));
    TLGB_CUDA_TRY(cudaStreamWaitEvent(aux.s, run.ev_fork, 0));
    rc = run.grams(nullptr, aux.s);
    if (rc) return rc;
    rc = run.bf16_factors(aux.s);
    if (rc) return rc;
    TLGB_CUDA_TRY(cudaEventRecord(run.ev_join, aux.s));
    if (P.refine_tc) {   // x2 only with three planes
      rc = tc_launch_split3_sumsq((const float*)X, sh.numel, run.B.xbf, run.B.xsplit[0],
                                  run.B.xsplit[1], run.B.sumsq_part, kSumsqBlocks, st);
      if (rc) return rc;
      rc = als_launch_sumsq_final(run.B.sumsq_part, kSumsqBlocks, run.B.ctrl, st);
    } else {
      rc = als_launch_sumsq(TypeCode<T>::value, X, sh.numel, run.B.sumsq_part, kSumsqBlocks,
                            run.B.ctrl, st);
      if (rc) return rc;
      rc = tc_launch_to_bf16((const float*)X, sh.numel, run.B.xbf, st);
    }
    if (rc) return rc;
    TLGB_CUDA_TRY(cudaStreamWaitEvent(st, run.ev_join, 0));
  } else {
    rc = als_launch_sumsq(TypeCode<T>::value, X, sh.numel, run.B.sumsq_part, kSumsqBlocks,
                          run.B.ctrl, st);
    if (rc) return rc;
    rc = run.grams(nullptr, st);
    if (rc) return rc;
  }
  if (o.callback) {
    double e0 = 0.0;
    rc = run.initial_error(st, &e0);
    if (rc) return rc;
    if (o.callback(o.callback_user, -1, e0) != 0) {
      // the reference ignores the return value of this first call
    }
  }
  if (o.n_iter_max == 0) {
    TLGB_CUDA_TRY(cudaStreamSynchronize(st));
    return TLGB_OK;
  }

  // ---- phases: (bf16 sweeps, then native refinement) or native sweeps only
  struct Phase { int kind; int sweeps; };
  std::vector<Phase> phases;
  if (mixed) {
    const int refine = std::min(o.refine_sweeps, o.n_iter_max);
    if (o.n_iter_max - refine > 0) phases.push_back({kSweepBf16, o.n_iter_max - refine});
    if (refine > 0 && !P.refine_tc) phases.push_back({kSweepNative, refine});
    if (refine > 1 && P.refine_tc) phases.push_back({kSweepF32Tc, refine - 1});
    if (refine > 0 && P.refine_tc) phases.push_back({kSweepF32TcFinal, 1});
  } else {
    phases.push_back({kSweepNative, o.n_iter_max});
  }
  const int check_every = (o.callback != nullptr) ? 1 : std::max(1, o.check_every);

  StreamGuard cap;
  // Timing events recorded inside a graph cannot be read back, so timed runs
  // launch the sweeps directly (kernel durations are the same).
  // Without graphs (the default), the sweeps are launched directly, a group
  // ahead of the host's read of the control block (which then waits for the
  // previous group only, on a side stream), so the GPU never waits for the
  // host between groups and programmatic launch and the deferred fit bridge
  // every sweep of a phase.  The host sees a converged run up to two groups
  // late; the sweeps launched meanwhile return at once on the device's stop
  // flag.  A callback (which sees every sweep) and the timing events read
  // the control block after every group instead.
  const bool use_graph = o.use_graph && !o.mttkrp_ms;
  const bool lookahead = !use_graph && !o.mttkrp_ms && !o.callback;
  if (use_graph) TLGB_CUDA_TRY(cudaStreamCreateWithFlags(&cap.s, cudaStreamNonBlocking));
  StreamGuard peek;
  EventGuard ev_grp[2];
  if (lookahead) {
    TLGB_CUDA_TRY(cudaStreamCreateWithFlags(&peek.s, cudaStreamNonBlocking));
    for (int j = 0; j < 2; ++j)
      TLGB_CUDA_TRY(cudaEventCreateWithFlags(&ev_grp[j].e, cudaEventDisableTiming));
  }

  AlsCtrl hc{};
  int launched = 0;
  int reported = 0;
  bool stopped = false;
  for (size_t pi = 0; pi < phases.size() && !stopped; ++pi) {
    const Phase ph = phases[pi];
    if (pi > 0 && phases[pi - 1].kind == kSweepBf16) {
      // A converged bf16 phase still gets its refinement sweeps: clear the flag.
      TLGB_CUDA_TRY(cudaMemsetAsync(&run.B.ctrl->done, 0, sizeof(int), st));
      TLGB_CUDA_TRY(cudaMemsetAsync(&run.B.ctrl->done_pending, 0, sizeof(int), st));
    }
    // The sweeps run in groups of check_every (the last group of a phase may
    // be shorter); the host reads the control block after each group.  A
    // group is launched as CUDA graphs of up to gmax sweeps (one graph per
    // length, captured when first needed), so programmatic launch and the
    // deferred fit also bridge the sweeps inside a graph; a graph's last
    // sweep runs its fit in line.
    const int gsize = std::min(check_every, ph.sweeps);
    const int gmax = tc_tuning().graph_sweeps > 0 ? std::min(tc_tuning().graph_sweeps, gsize)
                                                  : gsize;
    std::vector<GraphGuard> gg(gmax + 1);   // [n]: the graph of n sweeps
    auto capture = [&](int n, GraphGuard& g) -> int {
      TLGB_CUDA_TRY(cudaStreamBeginCapture(cap.s, cudaStreamCaptureModeThreadLocal));
      int rc2 = TLGB_OK;
      for (int j = 0; j < n && !rc2; ++j) rc2 = run.sweep(ph.kind, cap.s, j + 1 < n);
      cudaGraph_t graph = nullptr;
      cudaError_t ce = cudaStreamEndCapture(cap.s, &graph);
      g.g = graph;
      if (rc2) return rc2;
      if (ce != cudaSuccess)
        return set_error(TLGB_ECUDA, std::string("cp_als: graph capture: ") + cudaGetErrorString(ce));
      TLGB_CUDA_TRY(cudaGraphInstantiate(&g.e, g.g, 0));
      return TLGB_OK;
    };
    if (use_graph) {
      rc = capture(gmax, gg[gmax]);
      if (rc) return rc;
    }
    if (lookahead) {
      int cur = 0;
      bool have_prev = false;
      for (int s = 0; s < ph.sweeps;) {
        const int n = std::min(gsize, ph.sweeps - s);
        for (int j = 0; j < n; ++j) {
          // the phase's last sweep runs its fit in line: the next phase (or
          // the final read) follows it in stream order
          rc = run.sweep(ph.kind, st, s + j + 1 < ph.sweeps);
          if (rc) return rc;
        }
        s += n;
        launched += n;
        TLGB_CUDA_TRY(cudaEventRecord(ev_grp[cur].e, st));
        if (have_prev) {   // the control block as of the previous group
          TLGB_CUDA_TRY(cudaStreamWaitEvent(peek.s, ev_grp[cur ^ 1].e, 0));
          TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, run.B.ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost,
                                        peek.s));
          TLGB_CUDA_TRY(cudaStreamSynchronize(peek.s));
          // errors are reported after the final synchronisation below
          if (hc.tc_err != 0 || hc.status != TLGB_OK || hc.done || hc.done_pending) break;
        }
        have_prev = true;
        cur ^= 1;
      }
      rc = run.flush_fit(st);
      if (rc) return rc;
      if (hc.tc_err != 0 || hc.status != TLGB_OK) break;
      continue;
    }
    for (int s = 0; s < ph.sweeps;) {
      const int n = std::min(gsize, ph.sweeps - s);
      for (int left = n; left > 0;) {
        const int k = std::min(gmax, left);
        if (use_graph) {
          if (!gg[k].e) {
            rc = capture(k, gg[k]);
            if (rc) return rc;
          }
          TLGB_CUDA_TRY(cudaGraphLaunch(gg[k].e, st));
        } else {
          for (int j = 0; j < k; ++j) {
            rc = run.sweep(ph.kind, st, j + 1 < k);
            if (rc) return rc;
          }
        }
        left -= k;
      }
      launched += n;
      s += n;
      {   // end of a group: read the control block
        TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, run.B.ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
        TLGB_CUDA_TRY(cudaStreamSynchronize(st));
        // a timed-out MTTKRP leaves garbage partials behind it, so it is
        // reported before anything that garbage may have caused
        if (hc.tc_err != 0)
          return set_error(TLGB_ETIMEOUT, "cp_als: tensor-core MTTKRP pipeline wait timed out");
        if (hc.status != TLGB_OK)
          return set_error(hc.status, "cp_als: singular normal equations (LU found a zero pivot)");
        if (o.callback) {
          while (reported < hc.iter) {
            double e = 0.0;
            TLGB_CUDA_TRY(cudaMemcpy(&e, run.B.errors + reported, sizeof(double),
                                     cudaMemcpyDeviceToHost));
            const int ret = o.callback(o.callback_user, reported, e);
            ++reported;
            if (ret != 0) { stopped = true; break; }
          }
        }
        if (stopped || hc.done || hc.done_pending) break;  // callback asked to stop, or converged
      }
    }
    rc = run.flush_fit(st);
    if (rc) return rc;
    if (o.mttkrp_ms) {  // durations of this phase's last sweep (the host synced above)
      for (int k : run.modes) {
        float ms = 0.f;
        const cudaError_t e = cudaEventElapsedTime(&ms, run.ev_mt[0][k], run.ev_mt[1][k]);
        if (e != cudaSuccess) cudaGetLastError();
        o.mttkrp_ms[ph.kind * kMaxModes + k] = (e == cudaSuccess) ? (double)ms : -1.0;
      }
    }
    // only the bf16 phase hands a converged run on to further sweeps
    if ((hc.done || hc.done_pending) && ph.kind != kSweepBf16) break;
  }
  TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, run.B.ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  if (hc.tc_err != 0)
    return set_error(TLGB_ETIMEOUT, "cp_als: tensor-core MTTKRP pipeline wait timed out");
  if (hc.status != TLGB_OK)
    return set_error(hc.status, "cp_als: singular normal equations (LU found a zero pivot)");
  const int n = std::min(hc.iter, o.n_iter_max);
  if (errors_host && n > 0)
    TLGB_CUDA_TRY(cudaMemcpy(errors_host, run.B.errors, sizeof(double) * n, cudaMemcpyDeviceToHost));
  if (n_errors) *n_errors = n;
  (void)launched;
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" void tlgb_cp_als_default_options(tlgb_cp_als_options* o) {
  if (!o) return;
  std::memset(o, 0, sizeof(*o));
  o->n_iter_max = 100;
  o->tol = 1e-8;
  o->l2_reg = 0.0;
  o->cvg_criterion = 0;
  o->normalize_factors = 0;
  o->fixed_modes = 0;
  o->precision = TLGB_PREC_NATIVE;
  o->refine_sweeps = 1;
  o->check_every = 8;
  o->use_graph = 0;
  o->callback = nullptr;
  o->callback_user = nullptr;
}

extern "C" int tlgb_cp_als_workspace_size(int dtype, int ndim, const int64_t* shape, int64_t rank,
                                          const tlgb_cp_als_options* opts, size_t* bytes) {
  clear_error();
  int rc = validate(dtype, ndim, shape, rank, opts);
  if (rc) return rc;
  TLGB_CHECK_ARG(bytes != nullptr, "cp_als_workspace_size: null pointer");
  Shape sh = make_shape(ndim, shape);
  Plans P;
  rc = make_plans(dtype, sh, rank, *opts, &P);
  if (rc) return rc;
  AlsBuffers B;
  rc = layout(dtype, sh, rank, *opts, P, nullptr, &B);
  if (rc) return rc;
  *bytes = B.bytes;
  return TLGB_OK;
}

extern "C" int tlgb_cp_als(int dtype, const void* X, int ndim, const int64_t* shape, int64_t rank,
                           void* const* factors, void* weights, const tlgb_cp_als_options* opts,
                           double* errors, int* n_errors, void* workspace, size_t workspace_bytes,
                           void* stream) {
  clear_error();
  int rc = validate(dtype, ndim, shape, rank, opts);
  if (rc) return rc;
  TLGB_CHECK_ARG(X && factors && weights && workspace, "cp_als: null pointer");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(factors[k] != nullptr, "cp_als: null factor");
  Shape sh = make_shape(ndim, shape);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    return run<float>((const float*)X, sh, rank, (float* const*)factors, (float*)weights, *opts,
                      errors, n_errors, workspace, workspace_bytes, st);
  return run<double>((const double*)X, sh, rank, (double* const*)factors, (double*)weights, *opts,
                     errors, n_errors, workspace, workspace_bytes, st);
}

extern "C" int tlgb_cp_normalize(int dtype, int ndim, const int64_t* rows, int64_t rank,
                                 void* const* factors, void* weights, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "cp_normalize: dtype must be f32 or f64");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes && rows && factors && weights,
                 "cp_normalize: bad arguments");
  TLGB_CHECK_ARG(rank >= 1, "cp_normalize: rank must be >= 1");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(factors[k] != nullptr, "cp_normalize: null factor");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    return als_launch_normalize<float>((float* const*)factors, rows, ndim, (int)rank,
                                       (float*)weights, nullptr, st);
  return als_launch_normalize<double>((double* const*)factors, rows, ndim, (int)rank,
                                      (double*)weights, nullptr, st);
}

extern "C" int tlgb_cp_norm_workspace_size(int ndim, const int64_t* rows, int64_t rank,
                                           size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes && rows && bytes, "cp_norm: bad arguments");
  TLGB_CHECK_ARG(rank >= 1 && rank <= kMaxAlsRank, "cp_norm: rank must be in [1, 160]");
  int64_t imax = 0;
  for (int k = 0; k < ndim; ++k) imax = std::max(imax, rows[k]);
  Carver c(nullptr);
  c.take<double>((size_t)ndim * rank * rank);
  c.take<double>((size_t)solve_blocks_for(imax) * rank * rank);
  *bytes = c.used();
  return TLGB_OK;
}

extern "C" int tlgb_cp_norm(int dtype, int ndim, const int64_t* rows, int64_t rank,
                            const void* const* factors, const void* weights, double* out,
                            void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  size_t need = 0;
  int rc = tlgb_cp_norm_workspace_size(ndim, rows, rank, &need);
  if (rc) return rc;
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "cp_norm: dtype must be f32 or f64");
  TLGB_CHECK_ARG(factors && out, "cp_norm: null pointer");
  if (!workspace || workspace_bytes < need)
    return set_error(TLGB_EWORKSPACE, "cp_norm: workspace too small");
  int64_t imax = 0;
  for (int k = 0; k < ndim; ++k) imax = std::max(imax, rows[k]);
  Carver c(workspace);
  double* G = c.take<double>((size_t)ndim * rank * rank);
  double* gpart = c.take<double>((size_t)solve_blocks_for(imax) * rank * rank);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  rc = als_prepare(dtype);
  if (rc) return rc;
  const int R = (int)rank;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(factors[k] != nullptr, "cp_norm: null factor");
    rc = (dtype == TLGB_F32)
             ? als_launch_gram<float>((const float*)factors[k], rows[k], R, gpart,
                                      solve_blocks_for(imax), G + (size_t)k * R * R, nullptr, st)
             : als_launch_gram<double>((const double*)factors[k], rows[k], R, gpart,
                                       solve_blocks_for(imax), G + (size_t)k * R * R, nullptr, st);
    if (rc) return rc;
  }
  return (dtype == TLGB_F32) ? als_launch_cp_norm<float>(G, ndim, R, (const float*)weights, out, st)
                             : als_launch_cp_norm<double>(G, ndim, R, (const double*)weights, out, st);
}
