// Tucker decomposition by higher-order orthogonal iteration on the GPU:
// the loop of tensorly/decomposition/_tucker.py:105-221 (partial_tucker)
// after initialize_tucker (:25-102).
//
// Per iteration and decomposed mode (index i of `modes`):
//   Y = multi_mode_dot(X, factors, modes, skip=i, transpose=True)
//       (core_tenalg/n_mode_product.py:79-135: the factors are applied in
//       ascending mode order and `skip` is a position in that order; `modes`
//       must be ascending, the only order in which the reference's skip and
//       factor indices agree)
//   factors[i] = svd_interface(unfold(Y, modes[i]), n_eigenvecs=rank[i]).U
// then core = multi_mode_dot(X, factors, modes, transpose=True) and
//   rec_error = sqrt(|norm(X)^2 - norm(core)^2|) / norm(X),
// stopping when iteration > 1 and |rec_errors[-2] - rec_errors[-1]| < tol.
// The chain intermediates ping-pong between two workspace buffers; the SVDs
// come from the Gram eigensolver (svd.cu, eig.cu); one host sync per
// iteration reads norm(core)^2 for the stop test, like the reference's.
//
// Overlap: a chain applies the factor updated just before it last.  Its other
// products do not depend on that update, so they run on a second stream as
// soon as the previous SVD has read its input (its Gram is done), underneath
// the previous SVD's eigensolver, which occupies one SM.  The products are
// the same; only their order differs from the reference's ascending order.
#include <algorithm>
#include <cmath>
#include <vector>

#include "als_kernels.cuh"
#include "linalg.cuh"

namespace tlgb {
namespace {

struct TuckerGeom {
  int ndim;
  int64_t dim[kMaxModes];
  int n_modes;
  int modes[kMaxModes];
  int64_t ranks[kMaxModes];
  // sorted application order: positions into modes[]
  int order[kMaxModes];
};

// The factor indices a chain applies: ascending mode order without position
// `skip` (-1: none), with index `last` (-1: none) moved to the end.
int chain_list(const TuckerGeom& g, int skip, int last, int* list) {
  int cnt = 0;
  bool has_last = false;
  for (int q = 0; q < g.n_modes; ++q) {
    if (q == skip) continue;
    const int idx = g.order[q];
    if (idx == last) { has_last = true; continue; }
    list[cnt++] = idx;
  }
  if (has_last) list[cnt++] = last;
  return cnt;
}

// Shapes along a chain; returns the largest intermediate element count.
int64_t chain_max(const TuckerGeom& g, int skip, int last, int64_t* final_dims) {
  int list[kMaxModes];
  const int cnt = chain_list(g, skip, last, list);
  int64_t cur[kMaxModes];
  for (int k = 0; k < g.ndim; ++k) cur[k] = g.dim[k];
  int64_t best = 0;
  for (int q = 0; q < cnt; ++q) {
    const int idx = list[q];
    cur[g.modes[idx]] = g.ranks[idx];
    int64_t n = 1;
    for (int k = 0; k < g.ndim; ++k) n *= cur[k];
    best = std::max(best, n);
  }
  if (final_dims)
    for (int k = 0; k < g.ndim; ++k) final_dims[k] = cur[k];
  return best;
}

// The factor updated just before position i's chain (-1: none pending).
int prev_index(const TuckerGeom& g, int i) { return (i == 0) ? -1 : i - 1; }

struct TuckerLayout {
  size_t buf_elems;      // each ping-pong buffer
  size_t svd_bytes;      // largest SVD workspace over the modes
  size_t bytes;
  size_t off_buf0, off_buf1, off_svd, off_s, off_ctrl, off_part;
};

constexpr int kNormBlocks = 256;

template <typename T>
int layout(const TuckerGeom& g, TuckerLayout* L) {
  const int dtype = TypeCode<T>::value;
  int64_t mx = 1;
  for (int i = 0; i < g.n_modes; ++i) {   // the chains as run: mode i's, and the core's
    int pos = 0;
    while (g.order[pos] != i) ++pos;
    mx = std::max(mx, chain_max(g, pos, prev_index(g, i), nullptr));
    mx = std::max(mx, chain_max(g, pos, -1, nullptr));
  }
  mx = std::max(mx, chain_max(g, -1, g.n_modes - 1, nullptr));
  mx = std::max(mx, chain_max(g, -1, -1, nullptr));
  L->buf_elems = (size_t)mx;
  size_t svdb = 0;
  int64_t kmax = 1;
  for (int i = 0; i < g.n_modes; ++i) {
    // the SVD input of position i: the chain with that position skipped
    int64_t d[kMaxModes];
    int64_t cur[kMaxModes];
    for (int k = 0; k < g.ndim; ++k) cur[k] = g.dim[k];
    for (int q = 0; q < g.n_modes; ++q) {
      const int idx = g.order[q];
      if (idx == i) continue;
      cur[g.modes[idx]] = g.ranks[idx];
    }
    for (int k = 0; k < g.ndim; ++k) d[k] = cur[k];
    Shape sh = make_shape(g.ndim, d);
    const size_t w = svd_unfolding_workspace(dtype, sh, g.modes[i], g.ranks[i]);
    if (w == 0) return -1 - i;   // unsupported SVD shape for this position
    svdb = std::max(svdb, w);
    kmax = std::max(kmax, g.ranks[i]);
    // the initial SVD works on X itself
    Shape shx = make_shape(g.ndim, g.dim);
    const size_t wx = svd_unfolding_workspace(dtype, shx, g.modes[i], g.ranks[i]);
    if (wx == 0) return -1 - i;
    svdb = std::max(svdb, wx);
  }
  L->svd_bytes = svdb;
  size_t off = 0;
  auto take = [&](size_t b) { off = align_up(off, 256); const size_t o = off; off += b; return o; };
  L->off_buf0 = take(L->buf_elems * sizeof(T));
  L->off_buf1 = take(L->buf_elems * sizeof(T));
  L->off_svd = take(L->svd_bytes);
  L->off_s = take((size_t)kmax * sizeof(T));
  L->off_ctrl = take(2 * sizeof(AlsCtrl));
  L->off_part = take(kNormBlocks * sizeof(double));
  L->bytes = align_up(off, 256);
  return 0;
}

int make_geom(int ndim, const int64_t* shape, int n_modes, const int* modes, const int64_t* ranks,
              TuckerGeom* g) {
  TLGB_CHECK_ARG(shape && ranks, "tucker: null pointer");
  TLGB_CHECK_ARG(ndim >= 1 && ndim <= kMaxModes, "tucker: ndim must be in [1, 8]");
  TLGB_CHECK_ARG(n_modes >= 1 && n_modes <= ndim, "tucker: bad number of modes");
  g->ndim = ndim;
  for (int k = 0; k < ndim; ++k) {
    TLGB_CHECK_ARG(shape[k] >= 1, "tucker: empty mode");
    g->dim[k] = shape[k];
  }
  g->n_modes = n_modes;
  bool seen[kMaxModes] = {};
  for (int i = 0; i < n_modes; ++i) {
    const int m = modes ? modes[i] : i;
    TLGB_CHECK_ARG(m >= 0 && m < ndim && !seen[m], "tucker: modes must be distinct and in range");
    TLGB_CHECK_ARG(i == 0 || m > g->modes[i - 1], "tucker: modes must be in ascending order");
    seen[m] = true;
    g->modes[i] = m;
    TLGB_CHECK_ARG(ranks[i] >= 1, "tucker: ranks must be >= 1");
    g->ranks[i] = ranks[i];
    g->order[i] = i;
  }
  std::stable_sort(g->order, g->order + n_modes,
                   [&](int a, int b) { return g->modes[a] < g->modes[b]; });
  return TLGB_OK;
}

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

template <typename T>
struct Hooi {
  const TuckerGeom& g;
  const T* X;
  T* const* factors;
  T* buf[2];
  void* svdws;
  size_t svd_bytes;
  T* S;
  cudaStream_t st;
  cudaStream_t aux;          // independent products of a chain
  cudaEvent_t ev_in_free;    // the last SVD has read its input
  cudaEvent_t ev_part;       // the aux part of a chain is done
  bool pending = false;      // ev_in_free was recorded by the last SVD

  // Applies the factors (transposed), ascending mode order without position
  // `skip` (-1: none), factor index `last` at the end; the products before it
  // run on the aux stream when an SVD is pending.  Returns the result and dims.
  int chain(int skip, int last, const T** out, int64_t* dims) {
    int list[kMaxModes];
    const int cnt = chain_list(g, skip, last, list);
    const bool split = pending && cnt >= 2 && list[cnt - 1] == last;
    int64_t cur[kMaxModes];
    for (int k = 0; k < g.ndim; ++k) cur[k] = g.dim[k];
    const T* src = X;
    int which = 0;
    if (split) TLGB_CUDA_TRY(cudaStreamWaitEvent(aux, ev_in_free, 0));
    for (int q = 0; q < cnt; ++q) {
      const int idx = list[q];
      const int mode = g.modes[idx];
      const bool on_aux = split && q + 1 < cnt;
      if (split && q + 1 == cnt) {
        TLGB_CUDA_TRY(cudaEventRecord(ev_part, aux));
        TLGB_CUDA_TRY(cudaStreamWaitEvent(st, ev_part, 0));
      }
      Shape sh = make_shape(g.ndim, cur);
      T* dst = buf[which];
      int rc = ttm_launch<T>(src, sh, factors[idx], g.ranks[idx], /*transpose=*/1, mode, dst,
                             on_aux ? aux : st);
      if (rc) return rc;
      cur[mode] = g.ranks[idx];
      src = dst;
      which ^= 1;
    }
    pending = false;
    *out = src;
    for (int k = 0; k < g.ndim; ++k) dims[k] = cur[k];
    return TLGB_OK;
  }

  int svd_into(const T* Y, const int64_t* dims, int idx) {
    Shape sh = make_shape(g.ndim, dims);
    int rc = svd_unfolding_launch<T>(Y, sh, g.modes[idx], (int)g.ranks[idx], factors[idx], S, 1,
                                     svdws, svd_bytes, st, ev_in_free);
    pending = (rc == TLGB_OK);
    return rc;
  }
};

template <typename T>
int run(const T* X, const TuckerGeom& g, T* const* factors, T* core,
        const tlgb_tucker_options& o, double* errors, int* n_errors, void* ws, size_t ws_bytes,
        cudaStream_t st) {
  TuckerLayout L;
  if (layout<T>(g, &L) != 0)
    return set_error(TLGB_EUNSUPPORTED,
                     "tucker: an unfolding's SVD is outside the eigensolver's limits (order of "
                     "its Gram matrix, or a rank above min(unfolding shape))");
  if (!ws || ws_bytes < L.bytes) return set_error(TLGB_EWORKSPACE, "tucker: workspace too small");
  for (int i = 0; i < g.n_modes; ++i)
    TLGB_CHECK_ARG(factors[i] != nullptr, "tucker: missing factor pointer");
  TLGB_CHECK_ARG(core != nullptr, "tucker: null core");
  char* base = static_cast<char*>(ws);
  StreamGuard aux;
  EventGuard ev_in_free, ev_part;
  TLGB_CUDA_TRY(cudaStreamCreateWithFlags(&aux.s, cudaStreamNonBlocking));
  TLGB_CUDA_TRY(cudaEventCreateWithFlags(&ev_in_free.e, cudaEventDisableTiming));
  TLGB_CUDA_TRY(cudaEventCreateWithFlags(&ev_part.e, cudaEventDisableTiming));
  Hooi<T> h{g, X, factors, {reinterpret_cast<T*>(base + L.off_buf0),
                            reinterpret_cast<T*>(base + L.off_buf1)},
            base + L.off_svd, L.svd_bytes, reinterpret_cast<T*>(base + L.off_s), st,
            aux.s, ev_in_free.e, ev_part.e};
  AlsCtrl* ctrl = reinterpret_cast<AlsCtrl*>(base + L.off_ctrl);
  double* part = reinterpret_cast<double*>(base + L.off_part);
  const int dtype = TypeCode<T>::value;
  if (n_errors) *n_errors = 0;

  TLGB_CUDA_TRY(cudaMemsetAsync(ctrl, 0, 2 * sizeof(AlsCtrl), st));
  int64_t numel = 1;
  for (int k = 0; k < g.ndim; ++k) numel *= g.dim[k];
  int rc = als_launch_sumsq(dtype, X, numel, part, kNormBlocks, &ctrl[0], st);
  if (rc) return rc;

  if (o.init_svd) {   // initialize_tucker 'svd': U of each unfolding of X itself
    for (int i = 0; i < g.n_modes; ++i) {
      rc = h.svd_into(X, g.dim, i);
      if (rc) return rc;
    }
  }
  double nx2 = 0.0;
  TLGB_CUDA_TRY(cudaMemcpyAsync(&nx2, &ctrl[0].norm_x2, sizeof(double), cudaMemcpyDeviceToHost, st));
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  const double norm_x = std::sqrt(nx2);

  std::vector<double> errs;
  int64_t cdims[kMaxModes];
  for (int it = 0; it < o.n_iter_max; ++it) {
    for (int i = 0; i < g.n_modes; ++i) {
      // skip = the sorted position of modes[i]
      int pos = 0;
      while (g.order[pos] != i) ++pos;
      const T* Y;
      int64_t dims[kMaxModes];
      rc = h.chain(pos, prev_index(g, i), &Y, dims);
      if (rc) return rc;
      rc = h.svd_into(Y, dims, i);
      if (rc) return rc;
    }
    const T* C;
    rc = h.chain(-1, g.n_modes - 1, &C, cdims);
    if (rc) return rc;
    int64_t cn = 1;
    for (int k = 0; k < g.ndim; ++k) cn *= cdims[k];
    TLGB_CUDA_TRY(cudaMemcpyAsync(core, C, (size_t)cn * sizeof(T), cudaMemcpyDeviceToDevice, st));
    rc = als_launch_sumsq(dtype, core, cn, part, kNormBlocks, &ctrl[1], st);
    if (rc) return rc;
    double nc2 = 0.0;
    TLGB_CUDA_TRY(cudaMemcpyAsync(&nc2, &ctrl[1].norm_x2, sizeof(double), cudaMemcpyDeviceToHost, st));
    TLGB_CUDA_TRY(cudaStreamSynchronize(st));
    const double nc = std::sqrt(nc2);
    const double rec = std::sqrt(std::fabs(norm_x * norm_x - nc * nc)) / norm_x;
    errs.push_back(rec);
    if (errors && it < o.n_iter_max) errors[it] = rec;
    if (n_errors) *n_errors = (int)errs.size();
    if (it > 1 && o.tol > 0.0 && std::fabs(errs[errs.size() - 2] - errs.back()) < o.tol) break;
  }
  if (o.n_iter_max <= 0) {   // no iteration: the core of the initial factors
    const T* C;
    h.pending = false;
    rc = h.chain(-1, -1, &C, cdims);
    if (rc) return rc;
    int64_t cn = 1;
    for (int k = 0; k < g.ndim; ++k) cn *= cdims[k];
    TLGB_CUDA_TRY(cudaMemcpyAsync(core, C, (size_t)cn * sizeof(T), cudaMemcpyDeviceToDevice, st));
    TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  }
  return TLGB_OK;
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" void tlgb_tucker_default_options(tlgb_tucker_options* o) {
  if (!o) return;
  o->n_iter_max = 100;
  o->tol = 10e-5;
  o->init_svd = 1;
}

extern "C" int tlgb_tucker_workspace_size(int dtype, int ndim, const int64_t* shape, int n_modes,
                                          const int* modes, const int64_t* ranks,
                                          size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(bytes != nullptr, "tucker_workspace_size: null pointer");
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "tucker: dtype must be f32 or f64");
  TuckerGeom g;
  int rc = make_geom(ndim, shape, n_modes, modes, ranks, &g);
  if (rc) return rc;
  TuckerLayout L;
  const int bad = (dtype == TLGB_F32) ? layout<float>(g, &L) : layout<double>(g, &L);
  if (bad != 0)
    return set_error(TLGB_EUNSUPPORTED,
                     "tucker: an unfolding's SVD is outside the eigensolver's limits (order of "
                     "its Gram matrix, or a rank above min(unfolding shape))");
  *bytes = L.bytes;
  return TLGB_OK;
}

extern "C" int tlgb_tucker_hooi(int dtype, const void* X, int ndim, const int64_t* shape,
                                int n_modes, const int* modes, const int64_t* ranks,
                                void* const* factors, void* core,
                                const tlgb_tucker_options* opts, double* errors, int* n_errors,
                                void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(dtype == TLGB_F32 || dtype == TLGB_F64, "tucker: dtype must be f32 or f64");
  TLGB_CHECK_ARG(X && factors && opts, "tucker: null pointer");
  TuckerGeom g;
  int rc = make_geom(ndim, shape, n_modes, modes, ranks, &g);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (dtype == TLGB_F32)
    return run<float>((const float*)X, g, (float* const*)factors, (float*)core, *opts, errors,
                      n_errors, workspace, workspace_bytes, st);
  return run<double>((const double*)X, g, (double* const*)factors, (double*)core, *opts, errors,
                     n_errors, workspace, workspace_bytes, st);
}
