// Constrained CP by AO-ADMM (tensorly/decomposition/_constrained_cp.py:166-435)
// with the ADMM solver tensorly/solvers/admm.py:5-135 and the proximal
// operators tensorly/tenalg/proximal.py:148-671: those that act on a whole
// factor matrix entry by entry (non_negative, l1_reg (soft thresholding),
// l2_reg, l2_square_reg, normalize) here, the column-wise and rank-based ones
// (unimodality, simplex, soft / normalized / hard sparsity, smoothness,
// monotonicity) by the kernels of prox_columns.cu.
//
// Per free mode: V = (Hadamard of the other Grams) + rho I, rho = trace / R,
// factorised once (the CP-ALS factorisation, f64); M = MTTKRP; then up to
// n_inner ADMM iterations without a host round trip:
//   B = M + rho (x + dual);  S = B V^-1            (the CP-ALS solve)
//   x = prox(S - dual);      dual += x - S
//   stop when ||x - S|| < tol ||x|| and ||x - x_old|| < tol ||dual||
// (a device flag; the kernels of later iterations return at once).  The outer
// error uses the Grams and <M_last, A_last> and is tested on the host once
// per outer iteration, with the constraint error sum ||x - S|| / ||x||.
#include <algorithm>
#include <cmath>
#include <vector>

#include "als_kernels.cuh"
#include "mttkrp_simt.cuh"
#include "mttkrp_tc.cuh"
#include "prox_columns.cuh"

namespace tlgb {
namespace {

enum ConsKind { kConsNone = 0, kConsNonNeg, kConsL1, kConsL2, kConsL2Sq, kConsNormalize };

constexpr int kConsBlocks = 128;   // CTAs of the reduction kernels (fixed order)
constexpr int kConsThreads = 256;

struct ConsState {   // device scalars of one mode's ADMM
  double rho;
  double glob;       // global value of the prox input (max, norm or max |.|)
  double dres, xnorm;  // last ||x - S||, ||x||
  double cerr;       // sum over the modes of ||x - S|| / ||x||
  int stop;
};

__device__ double cta_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  return t;
}

// V = Hadamard of the Grams other than `mode`; rho = trace(V) / R; V += rho I.
__global__ void k_cons_v(const double* __restrict__ G, int ndim, int mode, int R, double* V,
                         ConsState* cs) {
  const int RR = R * R;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    double v = 1.0;
    for (int k = 0; k < ndim; ++k)
      if (k != mode) v *= G[(size_t)k * RR + e];
    V[e] = v;
  }
  __syncthreads();
  __shared__ double rho;
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int r = 0; r < R; ++r) t += V[r * R + r];
    rho = t / R;
    cs->rho = rho;
    cs->stop = 0;
  }
  __syncthreads();
  for (int r = threadIdx.x; r < R; r += blockDim.x) V[r * R + r] += rho;
}

// B = M + rho (x + dual)
template <typename T>
__global__ void k_cons_rhs(const T* __restrict__ M, const T* __restrict__ x,
                           const T* __restrict__ dual, int64_t n, const ConsState* cs,
                           T* __restrict__ B) {
  if (cs->stop) return;
  const T rho = (T)cs->rho;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    B[e] = M[e] + rho * (x[e] + dual[e]);
}

// Global value of y = S - dual that the prox needs: max(y) (non_negative,
// the reference's clip upper bound), ||y||^2 (l2_reg) or max |y| (normalize):
// per-CTA partials.
// (dual may be null: y = S; cs may be null: no stop flag.)
template <typename T>
__global__ void k_cons_glob(const T* __restrict__ S, const T* __restrict__ dual, int64_t n,
                            int kind, const ConsState* cs, double* part) {
  if (cs && cs->stop) return;
  __shared__ double red[kConsThreads / 32];
  double acc = kind == kConsL2 ? 0.0 : -INFINITY;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const double y = (double)(dual ? S[e] - dual[e] : S[e]);
    if (kind == kConsL2) acc += y * y;
    else if (kind == kConsNonNeg) acc = fmax(acc, y);
    else acc = fmax(acc, fabs(y));
  }
  if (kind == kConsL2) {
    const double t = cta_sum(acc, red);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  } else {
    for (int o = 16; o > 0; o >>= 1) acc = fmax(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = -INFINITY;
      for (int w = 0; w < kConsThreads / 32; ++w) t = fmax(t, red[w]);
      part[blockIdx.x] = t;
    }
  }
}

__global__ void k_cons_glob_final(const double* part, int nb, int kind, ConsState* cs) {
  if (cs->stop) return;
  if (threadIdx.x == 0) {
    double t = kind == kConsL2 ? 0.0 : -INFINITY;
    for (int b = 0; b < nb; ++b) t = kind == kConsL2 ? t + part[b] : fmax(t, part[b]);
    cs->glob = kind == kConsL2 ? sqrt(t) : t;
  }
}

template <typename T>
__device__ __forceinline__ T cons_prox(T y, int kind, T param, T glob) {
  switch (kind) {
    case kConsNonNeg: {                       // clip(y, 0, max(y))
      const T lo = y > (T)0 ? y : (T)0;
      return lo < glob ? lo : glob;
    }
    case kConsL1: {                           // sign(y) * clip(|y| - t, 0)
      const T a = fabs(y) - param;
      const T m = a > (T)0 ? a : (T)0;
      return y > (T)0 ? m : (y < (T)0 ? -m : (T)0);
    }
    case kConsL2: {                           // y - y * reg / max(||y||, reg)
      const T big = glob > param ? glob : param;
      return y - (y * param) / big;
    }
    case kConsL2Sq: return y / ((T)1 + (T)2 * param);
    case kConsNormalize: return y / glob;     // y / max |y|
    default: return y;
  }
}

// x = prox(S - dual); dual += x - S; per-CTA sums of ||x - S||^2,
// ||x - x_old||^2, ||x||^2, ||dual||^2.
template <typename T>
__global__ void k_cons_prox(const T* __restrict__ S, T* __restrict__ x, T* __restrict__ dual,
                            int64_t n, int kind, double param, const ConsState* cs,
                            double* part) {
  if (cs->stop) return;
  __shared__ double red[kConsThreads / 32];
  const T glob = (T)cs->glob;
  const T p = (T)param;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T s = S[e];
    const T xo = x[e];
    const T xn = cons_prox<T>(s - dual[e], kind, p, glob);
    const T dn = (dual[e] + xn) - s;
    x[e] = xn;
    dual[e] = dn;
    const double dr = (double)(xn - s), pr = (double)(xn - xo);
    a0 += dr * dr;
    a1 += pr * pr;
    a2 += (double)xn * (double)xn;
    a3 += (double)dn * (double)dn;
  }
  const double t0 = cta_sum(a0, red), t1 = cta_sum(a1, red), t2 = cta_sum(a2, red),
               t3 = cta_sum(a3, red);
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x + 0] = t0;
    part[4 * blockIdx.x + 1] = t1;
    part[4 * blockIdx.x + 2] = t2;
    part[4 * blockIdx.x + 3] = t3;
  }
}

// The ADMM stop test (tensorly/solvers/admm.py:128-133); keeps ||x - S|| and
// ||x|| of the last iteration run for the constraint error.
__global__ void k_cons_check(const double* part, int nb, double tol, ConsState* cs) {
  if (cs->stop) return;
  if (threadIdx.x == 0) {
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = 0; b < nb; ++b)
      for (int q = 0; q < 4; ++q) s[q] += part[4 * b + q];
    const double dres = sqrt(s[0]), pres = sqrt(s[1]), xn = sqrt(s[2]), dn = sqrt(s[3]);
    cs->dres = dres;
    cs->xnorm = xn;
    if (dres < tol * xn && pres < tol * dn) cs->stop = 1;
  }
}

__global__ void k_cons_cerr(ConsState* cs) {
  if (threadIdx.x == 0) cs->cerr += cs->dres / cs->xnorm;
}

// <M, A> partial sums in a fixed order.
template <typename T>
__global__ void k_cons_inner(const T* __restrict__ M, const T* __restrict__ A, int64_t n,
                             double* part) {
  __shared__ double red[kConsThreads / 32];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    s += (double)M[e] * (double)A[e];
  const double t = cta_sum(s, red);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// y = S - dual, the input of a column-wise proximal operator.
template <typename T>
__global__ void k_cons_diff(const T* __restrict__ S, const T* __restrict__ dual, int64_t n,
                            const ConsState* cs, T* __restrict__ Y) {
  if (cs->stop) return;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    Y[e] = S[e] - dual[e];
}

// As k_cons_prox, with x = P, the proximal operator already applied.
template <typename T>
__global__ void k_cons_take(const T* __restrict__ S, T* __restrict__ x, T* __restrict__ dual,
                            const T* __restrict__ P, int64_t n, const ConsState* cs,
                            double* part) {
  if (cs->stop) return;
  __shared__ double red[kConsThreads / 32];
  double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    const T s = S[e];
    const T xo = x[e];
    const T xn = P[e];
    const T dn = (dual[e] + xn) - s;
    x[e] = xn;
    dual[e] = dn;
    const double dr = (double)(xn - s), pr = (double)(xn - xo);
    a0 += dr * dr;
    a1 += pr * pr;
    a2 += (double)xn * (double)xn;
    a3 += (double)dn * (double)dn;
  }
  const double t0 = cta_sum(a0, red), t1 = cta_sum(a1, red), t2 = cta_sum(a2, red),
               t3 = cta_sum(a3, red);
  if (threadIdx.x == 0) {
    part[4 * blockIdx.x + 0] = t0;
    part[4 * blockIdx.x + 1] = t1;
    part[4 * blockIdx.x + 2] = t2;
    part[4 * blockIdx.x + 3] = t3;
  }
}

// Whole-matrix proximal operator out = prox(X) (no ADMM state).
template <typename T>
__global__ void k_prox_apply(const T* __restrict__ X, int64_t n, int kind, double param,
                             const double* glob, T* __restrict__ out) {
  const T g = glob ? (T)*glob : (T)0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x)
    out[e] = cons_prox<T>(X[e], kind, (T)param, g);
}

struct ConsLayout {
  size_t ctrl, cs, G, V2, fac, perm, vmat, w32, gpart, partial, M, B, S, dual, part, bytes;
  size_t P, pscratch;   // column-wise operators: their output and scratch
  size_t tcs;           // f32 tensors: the split tensor-core MTTKRP's buffers
};

template <typename T>
int cons_layout(const Shape& sh, int64_t R, std::vector<MttkrpPlan>* plans, ConsLayout* L) {
  const int dtype = TypeCode<T>::value;
  plans->resize(sh.ndim);
  size_t pmax = 0;
  int64_t imax = 0, dual_total = 0;
  for (int k = 0; k < sh.ndim; ++k) {
    int rc = mttkrp_make_plan(dtype, sh, R, k, &(*plans)[k]);
    if (rc) return rc;
    pmax = std::max(pmax, (*plans)[k].partial_bytes);
    imax = std::max(imax, sh.dim[k]);
    dual_total += sh.dim[k] * R;
  }
  size_t off = 0;
  auto take = [&](size_t b) { off = align_up(off, 256); const size_t o = off; off += b; return o; };
  const size_t RR = (size_t)R * R;
  L->ctrl = take(sizeof(AlsCtrl));
  L->cs = take(sizeof(ConsState));
  L->G = take(sizeof(double) * RR * sh.ndim);
  L->V2 = take(sizeof(double) * 2 * RR);
  L->fac = take(sizeof(double) * (RR + R));
  L->perm = take(sizeof(int) * R);
  L->vmat = take(sizeof(double) * RR);
  L->w32 = take(sizeof(float) * 3 * RR);
  L->gpart = take(sizeof(double) * RR * (size_t)solve_blocks_for(imax));
  L->partial = take(pmax);
  L->M = take(sizeof(T) * (size_t)imax * R);
  L->B = take(sizeof(T) * (size_t)imax * R);
  L->S = take(sizeof(T) * (size_t)imax * R);
  L->dual = take(sizeof(T) * (size_t)dual_total);
  L->part = take(sizeof(double) * 4 * kConsBlocks);
  L->P = take(sizeof(T) * (size_t)imax * R);
  L->pscratch = take(std::max(prox_matrix_scratch_bytes(dtype, imax, R, TLGB_CONS_UNIMODALITY),
                              prox_matrix_scratch_bytes(dtype, imax, R, TLGB_CONS_HARD_SPARSITY)));
  size_t tcs_bytes = 0;
  if (dtype == TLGB_F32) {
    SplitMttkrp stc;
    int rc = split_mttkrp_plan(sh, R, &stc);
    if (rc) return rc;
    tcs_bytes = split_mttkrp_bytes(stc);
  }
  L->tcs = take(tcs_bytes);
  L->bytes = align_up(off, 256);
  return TLGB_OK;
}

template <typename T>
int cons_run(const T* X, const Shape& sh, T* const* factors, int64_t R, const int* free_modes,
             int n_free, const int* kinds, const double* params, int n_iter_max, int n_inner,
             double tol_outer, double tol_inner, int crit, double* errors, int* n_errors,
             void* ws, size_t ws_bytes, cudaStream_t st) {
  std::vector<MttkrpPlan> plans;
  ConsLayout L;
  int rc = cons_layout<T>(sh, R, &plans, &L);
  if (rc) return rc;
  if (!ws || ws_bytes < L.bytes)
    return set_error(TLGB_EWORKSPACE, "constrained_parafac: workspace too small");
  rc = als_prepare(TypeCode<T>::value);
  if (rc) return rc;
  char* base = static_cast<char*>(ws);
  AlsCtrl* ctrl = reinterpret_cast<AlsCtrl*>(base + L.ctrl);
  ConsState* cs = reinterpret_cast<ConsState*>(base + L.cs);
  double* G = reinterpret_cast<double*>(base + L.G);
  double* V2 = reinterpret_cast<double*>(base + L.V2);
  double* fac = reinterpret_cast<double*>(base + L.fac);
  int* perm = reinterpret_cast<int*>(base + L.perm);
  double* vmat = reinterpret_cast<double*>(base + L.vmat);
  float* w32 = reinterpret_cast<float*>(base + L.w32);
  double* gpart = reinterpret_cast<double*>(base + L.gpart);
  T* partial = reinterpret_cast<T*>(base + L.partial);
  T* M = reinterpret_cast<T*>(base + L.M);
  T* B = reinterpret_cast<T*>(base + L.B);
  T* S = reinterpret_cast<T*>(base + L.S);
  T* dual0 = reinterpret_cast<T*>(base + L.dual);
  double* part = reinterpret_cast<double*>(base + L.part);
  T* Pbuf = reinterpret_cast<T*>(base + L.P);
  void* pscratch = base + L.pscratch;
  const int N = sh.ndim;
  for (int q = 0; q < n_free; ++q) {
    const int mode = free_modes[q];
    if (prox_is_matrix_kind(kinds[mode])) {
      rc = prox_matrix_check(TypeCode<T>::value, sh.dim[mode], R, kinds[mode]);
      if (rc) return rc;
    }
  }
  const int RR = (int)(R * R);
  const int nparts = solve_blocks_for([&] {
    int64_t m = 0;
    for (int k = 0; k < N; ++k) m = std::max(m, sh.dim[k]);
    return m;
  }());
  std::vector<T*> dual(N);
  {
    int64_t o = 0;
    for (int k = 0; k < N; ++k) {
      dual[k] = dual0 + o;
      o += sh.dim[k] * R;
    }
    TLGB_CUDA_TRY(cudaMemsetAsync(dual0, 0, sizeof(T) * (size_t)o, st));
  }
  TLGB_CUDA_TRY(cudaMemsetAsync(ctrl, 0, sizeof(AlsCtrl), st));
  TLGB_CUDA_TRY(cudaMemsetAsync(cs, 0, sizeof(ConsState), st));
  TLGB_CUDA_TRY(cudaMemsetAsync(V2, 0, sizeof(double) * 2 * RR, st));
  const int* done = &ctrl->done;
  for (int k = 0; k < N; ++k) {
    rc = als_launch_gram<T>(factors[k], sh.dim[k], (int)R, gpart, nparts, G + (size_t)k * RR,
                            done, st);
    if (rc) return rc;
  }
  // ||X||^2 (f64, fixed order)
  rc = als_launch_sumsq(TypeCode<T>::value, X, sh.numel, part, kConsBlocks, ctrl, st);
  if (rc) return rc;
  LoopMttkrp<T> mk;
  rc = mk.setup(X, sh, R, factors, &plans, partial, base + L.tcs, &ctrl->tc_err, st);
  if (rc) return rc;
  const T* cf[kMaxModes];
  for (int k = 0; k < N; ++k) cf[k] = factors[k];
  const int last = free_modes[n_free - 1];
  std::vector<double> hG((size_t)N * RR);
  std::vector<double> hip(kConsBlocks);
  double prev = 0.0;
  int ne = 0;
  for (int it = 0; it < n_iter_max; ++it) {
    TLGB_CUDA_TRY(cudaMemsetAsync(&cs->cerr, 0, sizeof(double), st));
    for (int q = 0; q < n_free; ++q) {
      const int mode = free_modes[q];
      const int64_t I = sh.dim[mode];
      const int64_t IR = I * R;
      k_cons_v<<<1, 1024, 0, st>>>(G, N, mode, (int)R, V2 + RR, cs);
      TLGB_LAUNCH_CHECK();
      rc = als_launch_factorize<T>(V2, 2, 0, (int)R, nullptr, 0.0, fac, perm, vmat, w32, ctrl,
                                   st);
      if (rc) return rc;
      rc = mk.launch(mode, cf, nullptr, done, st);
      if (rc) return rc;
      rc = mttkrp_launch_reduce_n<T, T>(mk.partial(), mk.splits(mode), I * R, M, st);
      if (rc) return rc;
      const int kind = kinds[mode];
      const bool glob = kind == kConsNonNeg || kind == kConsL2 || kind == kConsNormalize;
      const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(IR, (int64_t)kConsThreads),
                                                      kConsBlocks);
      for (int t = 0; t < n_inner; ++t) {
        k_cons_rhs<T><<<nb, kConsThreads, 0, st>>>(M, factors[mode], dual[mode], IR, cs, B);
        TLGB_LAUNCH_CHECK();
        int sb = 0;
        rc = als_launch_solve<T>(B, 1, I, (int)R, fac, perm, vmat, w32, S, nullptr, gpart,
                                 nullptr, ctrl, kIrMaxPasses, &sb, st);
        if (rc) return rc;
        if (prox_is_matrix_kind(kind)) {
          k_cons_diff<T><<<nb, kConsThreads, 0, st>>>(S, dual[mode], IR, cs, B);
          TLGB_LAUNCH_CHECK();
          rc = prox_matrix_launch<T>(B, Pbuf, I, R, kind, params[mode], pscratch, &cs->stop, st);
          if (rc) return rc;
          k_cons_take<T><<<nb, kConsThreads, 0, st>>>(S, factors[mode], dual[mode], Pbuf, IR,
                                                      cs, part);
          TLGB_LAUNCH_CHECK();
        } else {
          if (glob) {
            k_cons_glob<T><<<nb, kConsThreads, 0, st>>>(S, dual[mode], IR, kind, cs, part);
            TLGB_LAUNCH_CHECK();
            k_cons_glob_final<<<1, 32, 0, st>>>(part, (int)nb, kind, cs);
            TLGB_LAUNCH_CHECK();
          }
          k_cons_prox<T><<<nb, kConsThreads, 0, st>>>(S, factors[mode], dual[mode], IR, kind,
                                                      params[mode], cs, part);
          TLGB_LAUNCH_CHECK();
        }
        k_cons_check<<<1, 32, 0, st>>>(part, (int)nb, tol_inner, cs);
        TLGB_LAUNCH_CHECK();
      }
      k_cons_cerr<<<1, 32, 0, st>>>(cs);
      TLGB_LAUNCH_CHECK();
      rc = mk.refresh(mode, factors[mode], st);
      if (rc) return rc;
      rc = als_launch_gram<T>(factors[mode], I, (int)R, gpart, nparts, G + (size_t)mode * RR,
                              done, st);
      if (rc) return rc;
      if (mode == last) {
        k_cons_inner<T><<<kConsBlocks, kConsThreads, 0, st>>>(M, factors[mode], IR, part);
        TLGB_LAUNCH_CHECK();
      }
    }
    AlsCtrl hc{};
    ConsState hs{};
    TLGB_CUDA_TRY(cudaMemcpyAsync(hG.data(), G, sizeof(double) * hG.size(),
                                  cudaMemcpyDeviceToHost, st));
    TLGB_CUDA_TRY(cudaMemcpyAsync(hip.data(), part, sizeof(double) * kConsBlocks,
                                  cudaMemcpyDeviceToHost, st));
    TLGB_CUDA_TRY(cudaMemcpyAsync(&hc, ctrl, sizeof(AlsCtrl), cudaMemcpyDeviceToHost, st));
    TLGB_CUDA_TRY(cudaMemcpyAsync(&hs, cs, sizeof(ConsState), cudaMemcpyDeviceToHost, st));
    TLGB_CUDA_TRY(cudaStreamSynchronize(st));
    if (hc.status == TLGB_ESINGULAR)
      return set_error(TLGB_ESINGULAR, "constrained_parafac: normal equations singular");
    if (hc.tc_err != 0)
      return set_error(TLGB_ETIMEOUT, "constrained_parafac: a tensor-core MTTKRP wait timed out");
    // error (tensorly/decomposition/_constrained_cp.py:391-396), weights one
    double fn2 = 0.0;
    for (int e = 0; e < RR; ++e) {
      double v = 1.0;
      for (int k = 0; k < N; ++k) v *= hG[(size_t)k * RR + e];
      fn2 += v;
    }
    double iprod = 0.0;
    for (int b = 0; b < kConsBlocks; ++b) iprod += hip[b];
    const double nx2 = hc.norm_x2;
    const double err = std::sqrt(std::fabs(nx2 + fn2 - 2.0 * iprod)) / std::sqrt(nx2);
    if (errors) errors[ne] = err;
    ++ne;
    if (tol_outer > 0.0 && it >= 1) {
      const double dec = prev - err;
      if (hs.cerr < tol_outer) break;
      const bool stop = crit == 0 ? std::fabs(dec) < tol_outer : dec < tol_outer;
      if (stop) break;
    }
    prev = err;
  }
  if (n_errors) *n_errors = ne;
  return TLGB_OK;
}

int cons_check_args(int dtype, const int64_t* shape, int ndim, int64_t rank) {
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "constrained_parafac: f32 or f64");
  TLGB_CHECK_ARG(shape != nullptr, "constrained_parafac: null shape");
  TLGB_CHECK_ARG(ndim >= 2 && ndim <= kMaxModes, "constrained_parafac: ndim must be in [2, 8]");
  TLGB_CHECK_ARG(rank >= 1 && rank <= kMaxAlsRank, "constrained_parafac: rank must be in [1, 160]");
  for (int k = 0; k < ndim; ++k) TLGB_CHECK_ARG(shape[k] >= 1, "constrained_parafac: empty mode");
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" size_t tlgb_proximal_workspace_bytes(void) {
  return sizeof(double) * kConsBlocks + sizeof(ConsState);
}

extern "C" int tlgb_cp_constrained_workspace_size(int dtype, int ndim, const int64_t* shape,
                                                  int64_t rank, size_t* bytes) {
  clear_error();
  int rc = cons_check_args(dtype, shape, ndim, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(bytes != nullptr, "constrained_parafac: null bytes");
  Shape sh = make_shape(ndim, shape);
  std::vector<MttkrpPlan> plans;
  ConsLayout L;
  rc = dtype == TLGB_F64 ? cons_layout<double>(sh, rank, &plans, &L)
                         : cons_layout<float>(sh, rank, &plans, &L);
  if (rc) return rc;
  *bytes = L.bytes;
  return TLGB_OK;
}

extern "C" int tlgb_cp_constrained(int dtype, const void* X, int ndim, const int64_t* shape,
                                   void* const* factors, int64_t rank, const int* free_modes,
                                   int n_free, const int* kinds, const double* params,
                                   int n_iter_max, int n_iter_max_inner, double tol_outer,
                                   double tol_inner, int cvg_criterion, double* errors,
                                   int* n_errors, void* workspace, size_t workspace_bytes,
                                   void* stream) {
  clear_error();
  int rc = cons_check_args(dtype, shape, ndim, rank);
  if (rc) return rc;
  TLGB_CHECK_ARG(X && factors && free_modes && kinds && params, "constrained_parafac: null pointer");
  TLGB_CHECK_ARG(n_free >= 1 && n_free <= ndim && free_modes[n_free - 1] == ndim - 1,
                 "constrained_parafac: the last mode must be free");
  for (int q = 0; q < n_free; ++q)
    TLGB_CHECK_ARG(free_modes[q] >= 0 && free_modes[q] < ndim &&
                       (q == 0 || free_modes[q] > free_modes[q - 1]),
                   "constrained_parafac: free modes must be ascending and in range");
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(factors[k] != nullptr, "constrained_parafac: null factor");
    TLGB_CHECK_ARG(kinds[k] >= TLGB_CONS_NONE && kinds[k] <= TLGB_CONS_HARD_SPARSITY,
                   "constrained_parafac: unknown constraint kind");
  }
  TLGB_CHECK_ARG(n_iter_max >= 0 && n_iter_max_inner >= 1, "constrained_parafac: bad iterations");
  TLGB_CHECK_ARG(cvg_criterion == 0 || cvg_criterion == 1, "constrained_parafac: bad criterion");
  Shape sh = make_shape(ndim, shape);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F64)
    return cons_run<double>(static_cast<const double*>(X), sh,
                            reinterpret_cast<double* const*>(factors), rank, free_modes, n_free,
                            kinds, params, n_iter_max, n_iter_max_inner, tol_outer, tol_inner,
                            cvg_criterion, errors, n_errors, workspace, workspace_bytes, st);
  return cons_run<float>(static_cast<const float*>(X), sh, reinterpret_cast<float* const*>(factors),
                         rank, free_modes, n_free, kinds, params, n_iter_max, n_iter_max_inner,
                         tol_outer, tol_inner, cvg_criterion, errors, n_errors, workspace,
                         workspace_bytes, st);
}

extern "C" int tlgb_proximal(int dtype, const void* X, int64_t n, int kind, double param,
                             void* out, void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "proximal: dtype must be f32 or f64");
  TLGB_CHECK_ARG(X && out && n >= 0, "proximal: bad argument");
  TLGB_CHECK_ARG(kind >= kConsNone && kind <= kConsNormalize, "proximal: unknown kind");
  if (n == 0) return TLGB_OK;
  const bool glob = kind == kConsNonNeg || kind == kConsL2 || kind == kConsNormalize;
  if (glob && (!workspace || workspace_bytes < tlgb_proximal_workspace_bytes()))
    return set_error(TLGB_EWORKSPACE, "proximal: workspace too small");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const unsigned nb = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)kConsThreads), kConsBlocks);
  double* part = static_cast<double*>(workspace);
  ConsState* cs = glob ? reinterpret_cast<ConsState*>(part + kConsBlocks) : nullptr;
  const unsigned ab = (unsigned)std::min<int64_t>(ceil_div(n, (int64_t)256), 152 * 8);
  if (glob) TLGB_CUDA_TRY(cudaMemsetAsync(cs, 0, sizeof(ConsState), st));
  if (dtype == TLGB_F64) {
    const double* x = static_cast<const double*>(X);
    if (glob) {
      k_cons_glob<double><<<nb, kConsThreads, 0, st>>>(x, nullptr, n, kind, nullptr, part);
      TLGB_LAUNCH_CHECK();
      k_cons_glob_final<<<1, 32, 0, st>>>(part, (int)nb, kind, cs);
      TLGB_LAUNCH_CHECK();
    }
    k_prox_apply<double><<<ab, 256, 0, st>>>(x, n, kind, param, glob ? &cs->glob : nullptr,
                                             static_cast<double*>(out));
  } else {
    const float* x = static_cast<const float*>(X);
    if (glob) {
      k_cons_glob<float><<<nb, kConsThreads, 0, st>>>(x, nullptr, n, kind, nullptr, part);
      TLGB_LAUNCH_CHECK();
      k_cons_glob_final<<<1, 32, 0, st>>>(part, (int)nb, kind, cs);
      TLGB_LAUNCH_CHECK();
    }
    k_prox_apply<float><<<ab, 256, 0, st>>>(x, n, kind, param, glob ? &cs->glob : nullptr,
                                            static_cast<float*>(out));
  }
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
