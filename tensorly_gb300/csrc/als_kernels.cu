// f64 kernels of the CP-ALS sweep: tensor norm, factor Grams, the normal-
// equation factorisation and solve, the fit, and column normalisation.
//
// Reference steps (tensorly/decomposition/_cp.py):
//   :411-422  V = (prod_{i != mode} A_i^H A_i + l2_reg I) scaled by w w^T
//   :425-428  A_mode = solve(V^H, M^T)^T            (LAPACK gesv there)
//   :217-225  ||X - [[w; A]]||^2 = ||X||^2 + cp_norm^2 - 2 sum(M_last * A_last)
//   :529-530  cp_normalize (tensorly/cp_tensor.py:278-321)
// V is symmetric positive (semi)definite, so it is factorised by Cholesky;
// if a pivot is not positive the kernel falls back to LU with partial
// pivoting (what gesv does), and an exactly zero LU pivot reports
// TLGB_ESINGULAR.  All of this runs in f64 regardless of the tensor dtype.
#include "als_kernels.cuh"
#include "mttkrp_tc.cuh"

namespace tlgb {
namespace {

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block-wide sum for blockDim.x a multiple of 32 (<= 1024); result valid in all threads.
__device__ double block_sum(double v, double* scratch /* >= 32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  const int nw = blockDim.x >> 5;
  double t = (threadIdx.x < nw) ? scratch[threadIdx.x] : 0.0;
  if (warp == 0) t = warp_sum(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  const double r = scratch[0];
  __syncthreads();
  return r;
}

// ---------------------------------------------------------------- sum of squares
// f32 tensors: each square is split exactly into hi + lo (TwoProd by FMA) and
// summed with Neumaier compensation in f32, so the thread total is accurate
// to ~2^-40 relative without touching the (much slower) f64 pipe per element.
__global__ void k_sumsq_f32(const float* __restrict__ X, int64_t n, double* part) {
  __shared__ double scratch[32];
  float s = 0.f, c = 0.f;
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += step) {
    const float x = X[i];
    const float hi = x * x;
    const float lo = fmaf(x, x, -hi);
    const float t = s + hi;
    c += ((fabsf(s) >= hi) ? ((s - t) + hi) : ((hi - t) + s)) + lo;
    s = t;
  }
  const double tot = block_sum((double)s + (double)c, scratch);
  if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

template <typename T>
__global__ void k_sumsq(const T* __restrict__ X, int64_t n, double* part) {
  __shared__ double scratch[32];
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;  // independent f64 chains
  const int64_t step = (int64_t)gridDim.x * blockDim.x;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (; i + 3 * step < n; i += 4 * step) {
    const double x0 = (double)X[i], x1 = (double)X[i + step];
    const double x2 = (double)X[i + 2 * step], x3 = (double)X[i + 3 * step];
    s0 = fma(x0, x0, s0);
    s1 = fma(x1, x1, s1);
    s2 = fma(x2, x2, s2);
    s3 = fma(x3, x3, s3);
  }
  for (; i < n; i += step) {
    const double x = (double)X[i];
    s0 = fma(x, x, s0);
  }
  double s = block_sum((s0 + s1) + (s2 + s3), scratch);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

__global__ void k_sumsq_final(const double* part, int n, AlsCtrl* ctrl) {
  __shared__ double scratch[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += part[i];
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) ctrl->norm_x2 = s;
}

// ---------------------------------------------------------------- Gram partials
constexpr int kGramRows = 8;  // rows staged per pass (keeps R = 160 under 227 KB)

// CTA b owns rows [b*rpb, (b+1)*rpb); writes sum_rows a a^T (full square) to gpart[b].
template <typename T>
__global__ void k_gram_partial(const T* __restrict__ A, int64_t I, int R, int64_t rpb,
                               double* gpart, const int* done) {
  if (done && *done) return;
  extern __shared__ double sm[];
  const int RR = R * R;
  double* gacc = sm;        // [R][R]
  double* rows = sm + RR;   // [kGramRows][R]
  const int64_t r0 = blockIdx.x * rpb;
  const int64_t r1 = min(r0 + rpb, I);
  for (int e = threadIdx.x; e < RR; e += blockDim.x) gacc[e] = 0.0;
  for (int64_t base = r0; base < r1; base += kGramRows) {
    const int nrow = (int)((r1 - base) < kGramRows ? (r1 - base) : kGramRows);
    __syncthreads();
    for (int e = threadIdx.x; e < kGramRows * R; e += blockDim.x) {
      const int i = e / R, r = e % R;
      rows[e] = (i < nrow) ? (double)A[(base + i) * R + r] : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < RR; e += blockDim.x) {
      const int r = e / R, s = e % R;
      if (s > r) continue;
      double g = gacc[e];
      for (int i = 0; i < nrow; ++i) g = fma(rows[i * R + r], rows[i * R + s], g);
      gacc[e] = g;
    }
  }
  __syncthreads();
  double* out = gpart + (int64_t)blockIdx.x * RR;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    out[e] = (s <= r) ? gacc[r * R + s] : gacc[s * R + r];
  }
}

// G[e] = sum_p gpart[p][e] over the lower triangle, mirrored into the upper
// one.  Block b owns 32 consecutive row-major entries (one per lane) and
// reduces those on or below the diagonal, so every load is coalesced; its 8
// warps take every 8th partial, then the warps' sums are combined in a fixed
// order.  df: the partials are (hi, lo) f32 planes, summed on the f32 pipe
// (Neumaier for hi, plain for lo) with one conversion at the end; df == 2:
// only the hi planes were written (the lite solve's f32 Gram).
// G32 (optional): the entry's f32 (hi, lo) split as well, hi at G32[e] and lo
// at G32[R^2 + e].
// Returns the reduced entry in warp 0's lanes that own one (0 elsewhere).
__device__ __forceinline__ double gram_reduce_block(const double* __restrict__ gpart, int nparts,
                                                   int R, double* G, int df,
                                                   float* G32 = nullptr) {
  __shared__ double red[8][33];
  const int RR = R * R;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int e = blockIdx.x * 32 + lane;
  const int r = e / R, s = e - (e / R) * R;
  const bool mine = e < RR && s <= r;
  double part = 0.0;
  if (df) {
    // sixteen partials of a warp in flight per batch (one L2 round trip each)
    float h = 0.f, c = 0.f, l = 0.f;
    if (mine) {
      const float* gp = reinterpret_cast<const float*>(gpart);
      for (int p0 = warp; p0 < nparts; p0 += 8 * 16) {
        float v[16], lo[16];
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const int p = p0 + 8 * u;
          v[u] = (p < nparts) ? gp[(int64_t)p * 2 * RR + e] : 0.f;
          lo[u] = (p < nparts && df == 1) ? gp[(int64_t)p * 2 * RR + RR + e] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          l += lo[u];
          const float t = h + v[u];
          c += (fabsf(h) >= fabsf(v[u])) ? ((h - t) + v[u]) : ((v[u] - t) + h);
          h = t;
        }
      }
    }
    part = (double)h + (double)(c + l);
  } else {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (mine) {
      int p = warp;
      for (; p + 56 < nparts; p += 64)
#pragma unroll
        for (int u = 0; u < 8; ++u) acc[u] += gpart[(int64_t)(p + 8 * u) * RR + e];
      for (; p < nparts; p += 8) acc[0] += gpart[(int64_t)p * RR + e];
    }
    part = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + ((acc[4] + acc[5]) + (acc[6] + acc[7]));
  }
  red[warp][lane] = part;
  __syncthreads();
  double t = 0.0;
  if (warp == 0 && mine) {
#pragma unroll
    for (int w = 0; w < 8; ++w) t += red[w][lane];
    G[e] = t;
    if (s < r) G[s * R + r] = t;
    if (G32) {
      const float h = (float)t, l = (float)(t - (double)h);
      G32[e] = h;
      G32[RR + e] = l;
      if (s < r) {
        G32[s * R + r] = h;
        G32[RR + s * R + r] = l;
      }
    }
  }
  return t;
}

__global__ void __launch_bounds__(256, 4)   // <= 64 registers: fits beside an MTTKRP CTA
k_gram_reduce(const double* __restrict__ gpart, int nparts, int R, double* G, const int* done,
              int df, float* G32) {
  if (done && *done) return;
  gram_reduce_block(gpart, nparts, R, G, df, G32);
}

// ---------------------------------------------------------------- factorisation
template <typename T>
__device__ void build_v(double* V, const double* G, int ndim, int mode, int R, const T* w,
                        double l2) {
  const int RR = R * R;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k)
      if (k != mode) v = v * G[(int64_t)k * RR + e];
    if (r == s) v = v + l2;
    if (w) v = ((double)w[r] * v) * (double)w[s];
    V[e] = v;
  }
}

// ---- fast path: f32 Gauss-Jordan inverse of V, matrix held in registers.
// Thread (ti, tj) of a TI x TJ grid owns rows ti + TI*u and columns tj + TJ*v
// of the matrix padded to n = TI*NI = TJ*NJ (identity beyond R).  Pivots of
// Gauss-Jordan are the Schur complement pivots, so their spread bounds
// cond(V) from below; a spread above kIrMaxPivotRatio (or a non-positive
// pivot) hands V to the f64 kernel.
//
// Blocked by kGjBlock pivots: one warp inverts the diagonal block D of the
// current Schur complement with shuffles (no block barrier between its
// pivots), then with the block column C and block row P (shared memory)
// every thread applies the block step to the elements it owns:
//   block rows: D^-1 P (and D^-1 in the block's columns);
//   other rows: A - C (D^-1 P), and -C D^-1 in the block's columns.
// Four barriers per block instead of two per pivot.
//
// V: in double-float on the f32 pipe from the Grams' f32 (hi, lo) planes when
// they are given and the solve takes V's planes only (f32 factors with
// R <= kSolveDfMaxRank), else in f64 (this GPU's f64 pipe is far slower, so
// the f64 build is most of the kernel's time when it runs).
constexpr float kIrMaxPivotRatio = 1e5f;
constexpr int kGjBlock = 16;

// (h, l) *= (bh, bl), double-float product (~2^-46 relative).
__device__ __forceinline__ void df_mul(float& h, float& l, float bh, float bl) {
  const float p = h * bh;
  float e = fmaf(h, bh, -p);
  e = fmaf(h, bl, e);
  e = fmaf(l, bh, e);
  const float t = p + e;
  l = e - (t - p);
  h = t;
}
// (h, l) += (bh, bl), double-float sum.
__device__ __forceinline__ void df_add(float& h, float& l, float bh, float bl) {
  const float t = h + bh;
  const float bb = t - h;
  float e = (h - (t - bb)) + (bh - bb);
  e += l + bl;
  const float u = t + e;
  l = e - (u - t);
  h = u;
}

template <typename T>
__device__ void factorize_f64(const double* G, int ndim, int mode, int R, const T* w, double l2,
                              double* fac, int* perm, double* V, AlsCtrl* ctrl);

// Stop test of the kernels that run after a deferred fit in stream order (the
// solves, the factorisations, the fits): true when either flag is set; a
// solve (promote) raises `done` from `done_pending` for the kernels after it.
__device__ __forceinline__ bool als_stopped(AlsCtrl* ctrl, bool promote = false) {
  if (ctrl->done) return true;
  if (ctrl->done_pending) {
    if (promote && blockIdx.x == 0 && threadIdx.x == 0) ctrl->done = 1;
    return true;
  }
  return false;
}

template <typename T, int TI, int TJ, int NI, int NJ>
__global__ void __launch_bounds__(TI * TJ)
k_factorize_fast(const double* __restrict__ G, const float* __restrict__ G32, int ndim, int mode,
                 int R, const T* __restrict__ w, double l2, double* __restrict__ vmat,
                 float* __restrict__ w32, AlsCtrl* ctrl, double* fac, int* perm) {
  constexpr int N = TI * NI;
  constexpr int B = kGjBlock;
  constexpr int NT = TI * TJ;
  static_assert(TJ * NJ == N && N % B == 0, "padded order must be a multiple of the block");
  if (als_stopped(ctrl)) return;
  __shared__ __align__(16) float sC[N][B];   // block column of the current Schur complement
  __shared__ __align__(16) float sP[B][N];   // block row
  __shared__ __align__(16) float sT[B][N];   // D^-1 P (D^-1 itself in the block's columns)
  __shared__ float sD[B][B];                 // D^-1
  __shared__ double wsh[N];
  __shared__ int s_ok;
  const int tid = threadIdx.x;
  const int ti = tid / TJ, tj = tid - (tid / TJ) * TJ;
  const int RR = R * R;
  const bool dfv = (sizeof(T) == 4) && G32 != nullptr && R <= kSolveDfMaxRank;
  float a[NI][NJ];
  if (dfv) {
    // V = (prod_{k != mode} G_k + l2 I) * w w^T in double-float; the planes of
    // a row chunk are all loaded before the products that use them
    const float l2h = (float)l2, l2l = (float)(l2 - (double)l2h);
    constexpr int UB = (16 / NJ) > 0 ? (16 / NJ) : 1;
#pragma unroll
    for (int u0 = 0; u0 < NI; u0 += UB) {
      float vh[UB][NJ], vl[UB][NJ];
#pragma unroll
      for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int v = 0; v < NJ; ++v) { vh[u][v] = 1.f; vl[u][v] = 0.f; }
      for (int k = 0; k < ndim; ++k) {
        if (k == mode) continue;
        const float* gh = G32 + (int64_t)k * 2 * RR;
        float bh[UB][NJ], bl[UB][NJ];
#pragma unroll
        for (int u = 0; u < UB; ++u)
#pragma unroll
          for (int v = 0; v < NJ; ++v) {
            const int i = ti + TI * (u0 + u), j = tj + TJ * v;
            const bool in = u0 + u < NI && i < R && j < R;
            bh[u][v] = in ? gh[i * R + j] : 1.f;
            bl[u][v] = in ? gh[RR + i * R + j] : 0.f;
          }
#pragma unroll
        for (int u = 0; u < UB; ++u)
#pragma unroll
          for (int v = 0; v < NJ; ++v) df_mul(vh[u][v], vl[u][v], bh[u][v], bl[u][v]);
      }
#pragma unroll
      for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int v = 0; v < NJ; ++v) {
          if (u0 + u >= NI) continue;
          const int i = ti + TI * (u0 + u), j = tj + TJ * v;
          float h = 0.f;
          if (i < R && j < R) {
            float l = vl[u][v];
            h = vh[u][v];
            if (i == j) df_add(h, l, l2h, l2l);
            if (w) {
              df_mul(h, l, (float)w[i], 0.f);
              df_mul(h, l, (float)w[j], 0.f);
            }
            w32[RR + i * R + j] = h;
            w32[2 * RR + i * R + j] = l;
          }
          a[u0 + u][v] = h;
        }
    }
  } else {
    for (int t = tid; t < R; t += NT) wsh[t] = w ? (double)w[t] : 1.0;
    __syncthreads();
    // V in f64, a chunk of rows at a time with every Gram load of the chunk
    // issued before any use (they come from L2; issued one by one they would
    // serialise on its latency)
    constexpr int UB = (32 / NJ) > 0 ? (32 / NJ) : 1;
#pragma unroll
    for (int u0 = 0; u0 < NI; u0 += UB) {
      double g[UB][NJ];
#pragma unroll
      for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int v = 0; v < NJ; ++v) g[u][v] = 1.0;
      for (int k = 0; k < ndim; ++k) {
        if (k == mode) continue;
        const double* Gk = G + (int64_t)k * RR;
#pragma unroll
        for (int u = 0; u < UB; ++u)
#pragma unroll
          for (int v = 0; v < NJ; ++v) {
            const int i = ti + TI * (u0 + u), j = tj + TJ * v;
            if (u0 + u < NI && i < R && j < R) g[u][v] *= Gk[i * R + j];
          }
      }
#pragma unroll
      for (int u = 0; u < UB; ++u)
#pragma unroll
        for (int v = 0; v < NJ; ++v) {
          if (u0 + u >= NI) continue;
          const int i = ti + TI * (u0 + u), j = tj + TJ * v;
          float val = 0.f;
          if (i < R && j < R) {
            double gv = g[u][v];
            if (i == j) gv = gv + l2;
            gv = (wsh[i] * gv) * wsh[j];
            vmat[i * R + j] = gv;
            val = (float)gv;
            // f32 (hi, lo) planes of V after W in w32, for the double-float solve
            w32[RR + i * R + j] = val;
            w32[2 * RR + i * R + j] = (float)(gv - (double)val);
          }
          a[u0 + u][v] = val;
        }
    }
  }
  // identity beyond R
#pragma unroll
  for (int u = 0; u < NI; ++u)
#pragma unroll
    for (int v = 0; v < NJ; ++v) {
      const int i = ti + TI * u, j = tj + TJ * v;
      if (i >= R || j >= R) a[u][v] = (i == j) ? 1.f : 0.f;
    }
  if (tid == 0) s_ok = 1;
  float pmin = 3.0e38f, pmax = 0.f;   // warp 0
  const int warp = tid >> 5, lane = tid & 31;
  for (int k0 = 0; k0 < N; k0 += B) {
    // the block column and row of the current Schur complement
#pragma unroll
    for (int u = 0; u < NI; ++u) {
      const int i = ti + TI * u;
#pragma unroll
      for (int v = 0; v < NJ; ++v) {
        const int j = tj + TJ * v;
        if ((unsigned)(j - k0) < (unsigned)B) sC[i][j - k0] = a[u][v];
        if ((unsigned)(i - k0) < (unsigned)B) sP[i - k0][j] = a[u][v];
      }
    }
    __syncthreads();
    if (warp == 0) {
      // D^-1 by scalar Gauss-Jordan: lane l holds row l & 15, columns
      // (l >> 4) * 8 .. + 7; entry (x, y) lives in lane x + 16 * (y >> 3),
      // register y & 7
      const int r = lane & 15, c0 = (lane >> 4) * 8;
      float d[8];
#pragma unroll
      for (int m = 0; m < 8; ++m) d[m] = sP[r][k0 + c0 + m];
      bool ok = true;
#pragma unroll
      for (int k = 0; k < B; ++k) {
        const int hi = (k >> 3) << 4;
        const float dk = d[k & 7];
        const float p = __shfl_sync(0xffffffffu, dk, k + hi);
        const float ck = __shfl_sync(0xffffffffu, dk, r + hi);
        float rk[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) rk[m] = __shfl_sync(0xffffffffu, d[m], k + (lane & 16));
        if (!(p > 0.f)) ok = false;   // the same p in every lane
        if (k0 + k < R) {
          pmin = fminf(pmin, p);
          pmax = fmaxf(pmax, p);
        }
        const float inv = __frcp_rn(p);
        const float fi = ck * inv;
#pragma unroll
        for (int m = 0; m < 8; ++m) {
          const int col = c0 + m;
          const float upd = fmaf(-fi, rk[m], d[m]);
          d[m] = (r == k) ? ((col == k) ? inv : d[m] * inv) : ((col == k) ? -fi : upd);
        }
      }
#pragma unroll
      for (int m = 0; m < 8; ++m) sD[r][c0 + m] = d[m];
      if (lane == 0 && !ok) s_ok = 0;
    }
    __syncthreads();
    if (!s_ok) break;   // uniform
    for (int e = tid; e < B * N; e += NT) {
      const int m = e / N, j = e - (e / N) * N;
      float t;
      if ((unsigned)(j - k0) < (unsigned)B) {
        t = sD[m][j - k0];
      } else {
        float t0 = 0.f, t1 = 0.f;
#pragma unroll
        for (int q = 0; q < B; q += 2) {
          t0 = fmaf(sD[m][q], sP[q][j], t0);
          t1 = fmaf(sD[m][q + 1], sP[q + 1][j], t1);
        }
        t = t0 + t1;
      }
      sT[m][j] = t;
    }
    __syncthreads();
#pragma unroll
    for (int u = 0; u < NI; ++u) {
      const int i = ti + TI * u;
      if ((unsigned)(i - k0) < (unsigned)B) continue;
#pragma unroll
      for (int v = 0; v < NJ; ++v) {
        const int j = tj + TJ * v;
        if ((unsigned)(j - k0) < (unsigned)B) a[u][v] = 0.f;
      }
    }
#pragma unroll 4
    for (int m = 0; m < B; ++m) {
      float cv[NI], tv[NJ];
#pragma unroll
      for (int u = 0; u < NI; ++u) cv[u] = sC[ti + TI * u][m];
#pragma unroll
      for (int v = 0; v < NJ; ++v) tv[v] = sT[m][tj + TJ * v];
#pragma unroll
      for (int u = 0; u < NI; ++u)
#pragma unroll
        for (int v = 0; v < NJ; ++v) a[u][v] = fmaf(-cv[u], tv[v], a[u][v]);
    }
#pragma unroll
    for (int u = 0; u < NI; ++u) {
      const int i = ti + TI * u;
      if ((unsigned)(i - k0) < (unsigned)B)
#pragma unroll
        for (int v = 0; v < NJ; ++v) a[u][v] = sT[i - k0][tj + TJ * v];
    }
    __syncthreads();   // sC, sP, sT are rewritten by the next block
  }
  __shared__ float s_pr[2];
  if (tid == 0) { s_pr[0] = pmin; s_pr[1] = pmax; }
  __syncthreads();
  const bool ok = s_ok && !(s_pr[1] > kIrMaxPivotRatio * s_pr[0]);
  if (ok) {
#pragma unroll
    for (int u = 0; u < NI; ++u)
#pragma unroll
      for (int v = 0; v < NJ; ++v) {
        const int i = ti + TI * u, j = tj + TJ * v;
        if (i < R && j < R) w32[i * R + j] = a[u][v];
      }
  }
  if (tid == 0) ctrl->fac_kind = ok ? 2 : 3;
  if (!ok) {   // uniform: the f64 Cholesky / LU in the same launch
    __syncthreads();
    factorize_f64<T>(G, ndim, mode, R, w, l2, fac, perm, vmat, ctrl);
  }
}

// ---- fallback: f64 Cholesky (fac_kind 0) or LU with partial pivoting
// (fac_kind 1) of V when the fast path reported fac_kind 3; fac layout
// [R*R] factor(s) then [R] reciprocal diagonal.  V is factorised in place in
// global memory (`vmat`, which only the refinement path of the solve reads):
// this rare path then needs no dynamic shared memory, so it never keeps an SM
// from hosting a tensor-core MTTKRP CTA that runs concurrently on another
// stream.
template <typename T>
__device__ void factorize_f64(const double* G, int ndim, int mode, int R, const T* w, double l2,
                              double* fac, int* perm, double* V, AlsCtrl* ctrl) {
  if (als_stopped(ctrl) || ctrl->fac_kind != 3) return;
  __shared__ int s_fail;
  __shared__ int s_piv;
  const int RR = R * R;
  build_v<T>(V, G, ndim, mode, R, w, l2);
  if (threadIdx.x == 0) s_fail = 0;
  __syncthreads();
  // right-looking Cholesky on the lower triangle with unscaled columns:
  // after step k, V[i][k] = sqrt(d_k) * L[i][k] and V[k][k] = d_k.
  for (int k = 0; k < R; ++k) {
    const double d = V[k * R + k];
    if (!(d > 0.0)) {
      if (threadIdx.x == 0) s_fail = 1;
      break;  // uniform: every thread read the same d
    }
    const double inv = 1.0 / d;
    const int n = R - k - 1;
    for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
      const int i = k + 1 + e / n, j = k + 1 + e % n;
      if (j <= i) V[i * R + j] -= V[i * R + k] * V[j * R + k] * inv;
    }
    __syncthreads();
  }
  __syncthreads();
  if (!s_fail) {
    for (int e = threadIdx.x; e < RR; e += blockDim.x) {
      const int i = e / R, k = e % R;
      fac[e] = (k <= i) ? V[e] / sqrt(V[k * R + k]) : 0.0;
    }
    for (int k = threadIdx.x; k < R; k += blockDim.x) {
      fac[RR + k] = 1.0 / sqrt(V[k * R + k]);
      perm[k] = k;
    }
    if (threadIdx.x == 0) ctrl->fac_kind = 0;
    return;
  }
  // LU with partial pivoting (row interchanges tracked in perm).
  __syncthreads();
  build_v<T>(V, G, ndim, mode, R, w, l2);
  for (int k = threadIdx.x; k < R; k += blockDim.x) perm[k] = k;
  __syncthreads();
  for (int k = 0; k < R; ++k) {
    if (threadIdx.x == 0) {
      int p = k;
      double best = fabs(V[k * R + k]);
      for (int i = k + 1; i < R; ++i) {
        const double a = fabs(V[i * R + k]);
        if (a > best) { best = a; p = i; }
      }
      s_piv = p;
      if (best == 0.0 && s_fail != 2) s_fail = 2;
      if (p != k) { const int t = perm[k]; perm[k] = perm[p]; perm[p] = t; }
    }
    __syncthreads();
    const int p = s_piv;
    if (p != k)
      for (int j = threadIdx.x; j < R; j += blockDim.x) {
        const double t = V[k * R + j];
        V[k * R + j] = V[p * R + j];
        V[p * R + j] = t;
      }
    __syncthreads();
    const double piv = V[k * R + k];
    if (piv != 0.0) {
      const double inv = 1.0 / piv;
      for (int i = k + 1 + threadIdx.x; i < R; i += blockDim.x) V[i * R + k] *= inv;
      __syncthreads();
      const int n = R - k - 1;
      for (int e = threadIdx.x; e < n * n; e += blockDim.x) {
        const int i = k + 1 + e / n, j = k + 1 + e % n;
        V[i * R + j] -= V[i * R + k] * V[k * R + j];
      }
    }
    __syncthreads();
  }
  for (int e = threadIdx.x; e < RR; e += blockDim.x) fac[e] = V[e];
  for (int k = threadIdx.x; k < R; k += blockDim.x) {
    const double u = V[k * R + k];
    fac[RR + k] = (u != 0.0) ? 1.0 / u : 0.0;
  }
  if (threadIdx.x == 0) {
    ctrl->fac_kind = 1;
    if (s_fail == 2) ctrl->status = TLGB_ESINGULAR;
  }
}

template <typename T>
__global__ void __launch_bounds__(256)
k_factorize(const double* G, int ndim, int mode, int R, const T* w, double l2, double* fac,
            int* perm, double* V, AlsCtrl* ctrl) {
  factorize_f64<T>(G, ndim, mode, R, w, l2, fac, perm, V, ctrl);
}

// ---------------------------------------------------------------- solve
constexpr int kRQ = kMaxAlsRank / 32;  // register slots per lane

__device__ __forceinline__ double pick(const double (&v)[kRQ], int q) {
  double t = v[0];
#pragma unroll
  for (int i = 1; i < kRQ; ++i)
    if (q == i) t = v[i];
  return t;
}
__device__ __forceinline__ void put(double (&v)[kRQ], int q, double x) {
#pragma unroll
  for (int i = 0; i < kRQ; ++i)
    if (q == i) v[i] = x;
}

constexpr int kSolveThreads = 32 * kSolveWarps;
constexpr double kIrStop = 1e-12;   // stop refining once max|correction| <= kIrStop max|x|

// Store one solved row: the factor (tensor dtype), its bf16 split transposed
// copy for the tensor cores, the stored value (f64) for the Gram, and the
// row's contribution to <M, A>.
template <typename T>
__device__ __forceinline__ double store_entry(T* A, __nv_bfloat16* A_bt, int64_t I, int R,
                                              int64_t row, int r, double x, double* rb) {
  const T xv = (T)x;
  A[row * R + r] = xv;
  const double xd = (double)xv;
  rb[r] = xd;
  if (A_bt) {  // three-plane bf16 split, transposed, for the tensor cores
    const float xf = (float)xv;
    const __nv_bfloat16 p0 = __float2bfloat16_rn(xf);
    const float r1 = xf - __bfloat162float(p0);
    const __nv_bfloat16 p1 = __float2bfloat16_rn(r1);
    const int64_t plane = (int64_t)R * I, at = (int64_t)r * I + row;
    A_bt[at] = p0;
    A_bt[plane + at] = p1;
    A_bt[2 * plane + at] = __float2bfloat16_rn(r1 - __bfloat162float(p1));
  }
  return xd;
}

// store_entry for f32 factors with the value already in f32 (the lite solve).
__device__ __forceinline__ void store_entry_f32(float* A, __nv_bfloat16* A_bt, int64_t I, int R,
                                                int64_t row, int r, float x) {
  A[row * R + r] = x;
  if (A_bt) {
    const __nv_bfloat16 p0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(p0);
    const __nv_bfloat16 p1 = __float2bfloat16_rn(r1);
    const int64_t plane = (int64_t)R * I, at = (int64_t)r * I + row;
    A_bt[at] = p0;
    A_bt[plane + at] = p1;
    A_bt[2 * plane + at] = __float2bfloat16_rn(r1 - __bfloat162float(p1));
  }
}

// gacc += sum over `nrows` rows of a a^T, lower triangle only; the entry
// index advances without integer division.
__device__ __forceinline__ void gram_update(double* gacc, const double* rows, int nrows, int R) {
  const int RR = R * R;
  int e = threadIdx.x;
  int r = e / R, s = e - (e / R) * R;
  const int dr = blockDim.x / R, ds = blockDim.x - dr * R;
  for (; e < RR; e += blockDim.x) {
    if (s <= r) {
      double g = gacc[e];
      for (int w = 0; w < nrows; ++w) g = fma(rows[w * R + r], rows[w * R + s], g);
      gacc[e] = g;
    }
    r += dr;
    s += ds;
    if (s >= R) { s -= R; ++r; }
  }
}

// Double-float variant for f32 factor values: g = (gh, gl) f32 pairs; each
// product a*b is split exactly (p + fma(a, b, -p)) and added with a Neumaier
// step, so the block's Gram is accurate to ~2^-48 without the f64 pipe.
__device__ __forceinline__ void gram_update_df(float* g, const float* rows, int nrows, int R) {
  const int RR = R * R;
  float* gh = g;
  float* gl = g + RR;
  int e = threadIdx.x;
  int r = e / R, s = e - (e / R) * R;
  const int dr = blockDim.x / R, ds = blockDim.x - dr * R;
  for (; e < RR; e += blockDim.x) {
    if (s <= r) {
      float h = gh[e], l = gl[e];
      for (int w = 0; w < nrows; ++w) {
        const float a = rows[w * R + r], b = rows[w * R + s];
        const float p = a * b;
        const float t = h + p;
        l += ((fabsf(h) >= fabsf(p)) ? ((h - t) + p) : ((p - t) + h)) + fmaf(a, b, -p);
        h = t;
      }
      gh[e] = h;
      gl[e] = l;
    }
    r += dr;
    s += ds;
    if (s >= R) { s -= R; ++r; }
  }
}

// Plain f32 variant (the lite solve): only the hi plane accumulates, the lo
// plane stays zero; two entries a step for independent chains.
__device__ __forceinline__ void gram_update_f32(float* g, const float* rows, int nrows, int R) {
  const int RR = R * R;
  for (int e = threadIdx.x; e < RR; e += 2 * blockDim.x) {
    const int e2 = e + blockDim.x;
    const int r = e / R, s = e - (e / R) * R;
    const int r2 = e2 / R, s2 = e2 - (e2 / R) * R;
    const bool a1 = s <= r, a2 = e2 < RR && s2 <= r2;
    float h = a1 ? g[e] : 0.f, h2 = a2 ? g[e2] : 0.f;
    for (int w = 0; w < nrows; ++w) {
      if (a1) h = fmaf(rows[w * R + r], rows[w * R + s], h);
      if (a2) h2 = fmaf(rows[w * R + r2], rows[w * R + s2], h2);
    }
    if (a1) g[e] = h;
    if (a2) g[e2] = h2;
  }
}

// Sum of the MTTKRP split partials of one entry.  f32 partials: compensated
// f32 summation (Neumaier), whose error (~splits * 2^-48) is far below the
// partials' own rounding, on the f32 pipe (the f64 pipe is ~70x slower here).
__device__ __forceinline__ void sum_splits_sc(const float* __restrict__ partial, int splits,
                                              int64_t stride, int64_t off, float& s_out,
                                              float& c_out) {
  float s = 0.f, c = 0.f;
  int p = 0;
  // up to 36 loads in flight per batch: the partials come from L2 and a
  // batch costs one round trip (the bf16 sweeps' 36 tiles take one)
  for (; p + 35 < splits; p += 36) {
    float v[36];
#pragma unroll
    for (int u = 0; u < 36; ++u) v[u] = partial[(int64_t)(p + u) * stride + off];
#pragma unroll
    for (int u = 0; u < 36; ++u) {
      const float t = s + v[u];
      c += (fabsf(s) >= fabsf(v[u])) ? ((s - t) + v[u]) : ((v[u] - t) + s);
      s = t;
    }
  }
  for (; p + 17 < splits; p += 18) {
    float v[18];
#pragma unroll
    for (int u = 0; u < 18; ++u) v[u] = partial[(int64_t)(p + u) * stride + off];
#pragma unroll
    for (int u = 0; u < 18; ++u) {
      const float t = s + v[u];
      c += (fabsf(s) >= fabsf(v[u])) ? ((s - t) + v[u]) : ((v[u] - t) + s);
      s = t;
    }
  }
  for (; p + 3 < splits; p += 4) {
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = partial[(int64_t)(p + u) * stride + off];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float t = s + v[u];
      c += (fabsf(s) >= fabsf(v[u])) ? ((s - t) + v[u]) : ((v[u] - t) + s);
      s = t;
    }
  }
  for (; p < splits; ++p) {
    const float x = partial[(int64_t)p * stride + off];
    const float t = s + x;
    c += (fabsf(s) >= fabsf(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
  }
  s_out = s;
  c_out = c;
}
__device__ __forceinline__ double sum_splits(const float* __restrict__ partial, int splits,
                                             int64_t stride, int64_t off) {
  float s, c;
  sum_splits_sc(partial, splits, stride, off, s, c);
  return (double)s + (double)c;
}

// f64 partials: four independent f64 chains.
__device__ __forceinline__ double sum_splits(const double* __restrict__ partial, int splits,
                                             int64_t stride, int64_t off) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int p = 0;
  for (; p + 3 < splits; p += 4) {
    s0 += (double)partial[(int64_t)p * stride + off];
    s1 += (double)partial[(int64_t)(p + 1) * stride + off];
    s2 += (double)partial[(int64_t)(p + 2) * stride + off];
    s3 += (double)partial[(int64_t)(p + 3) * stride + off];
  }
  for (; p < splits; ++p) s0 += (double)partial[(int64_t)p * stride + off];
  return (s0 + s1) + (s2 + s3);
}

// Solves A_mode = M V^-1 for a block of rows (V symmetric), writes the factor
// and the block's Gram and <M, A> partial sums.
//   fac_kind 2: x = M W32 (f32 inverse), then up to kIrMaxPasses passes of
//     mixed-precision iterative refinement x += W32 (m - V x) with the
//     residual in f64; every dot product is split into independent chains
//     (f64 FMA latency is long on this GPU, so long chains would dominate).
//   fac_kind 0/1: forward/back substitution with the f64 Cholesky or LU
//     factors, one warp per row.
// RT > 0: the rank is the compile-time constant RT (R_in == RT), so the
// rank loops unroll and the index arithmetic folds; RT == 0: runtime rank.
template <typename T, int RT>
__global__ void __launch_bounds__(kSolveThreads)
k_solve(const T* __restrict__ partial, int splits, int64_t I, int R_in,
        const double* __restrict__ fac, const int* __restrict__ perm,
        const double* __restrict__ vmat, const float* __restrict__ w32, T* A,
        __nv_bfloat16* A_bt, double* gpart, double* ipart, AlsCtrl* ctrl, int64_t rpb,
        int mats_in_smem, int max_passes, int lite_in) {
  const int R = (RT > 0) ? RT : R_in;
  // Up to the first read of the partials, nothing here reads what the
  // programmatic predecessor (the MTTKRP) writes: the factorisation's W and V
  // and the control block's fac_kind were written by kernels that completed
  // before this one was launched, so their staging overlaps the MTTKRP's tail.
  extern __shared__ double sm[];
  const int RR = R * R;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int kind = ctrl->fac_kind;
  __shared__ double s_ip[kSolveWarps];
  __shared__ unsigned long long s_dmax, s_xmax;
  double* gacc = sm;                          // RR
  for (int e = tid; e < RR; e += blockDim.x) gacc[e] = 0.0;
  const int64_t row0 = blockIdx.x * rpb;
  const int64_t row1 = min(row0 + rpb, I);
  const int64_t IR = I * R;
  double ip = 0.0;

  // f32 tensors with V in shared memory: the residual and the Gram run in
  // double-float arithmetic on the f32 pipe (exact products by FMA, Neumaier
  // sums; ~2^-48 relative), since this GPU's f64 pipe is ~70x slower.  The
  // block's Gram is then kept as f32 (hi, lo) pairs.
  const bool df = (sizeof(T) == 4) && mats_in_smem;
  const bool lite = df && lite_in;
  if (kind == 2) {
    // ------------------------------------------------ refinement path
    const int RB = max(1, kSolveThreads / R);   // rows per round
    const int RBR = RB * R;
    double* mb = gacc + RR;                     // [RB][R] right-hand sides
    double* xb = mb + RBR;                      // [RB][R] solution
    double* rb = xb + RBR;                      // [RB][R] residual, then stored values
    float* mbf = reinterpret_cast<float*>(rb + RBR);   // [RB][R] f32 copy of m
    float* rbf = mbf + RBR;                              // [RB][R] f32 copy of r
    float* xbh = rbf + RBR;                              // [RB][R] x = xbh + xbl (df)
    float* xbl = xbh + RBR;
    float* gbf = xbl + RBR;                              // [RB][R] stored values, f32 (df)
    const double* Vm = vmat;
    const float* Wm = w32;
    const float* VmH = nullptr;                          // V = VmH + VmL (df)
    const float* VmL = nullptr;
    if (mats_in_smem) {
      // 16-byte aligned for the float4 copies below: R * R (the offset of mb
      // in doubles) is odd for odd R, so round up by one double
      double* Vs = rb + RBR + ((5 * RBR + 3) / 4) * 2;
      if (reinterpret_cast<uintptr_t>(Vs) & 15) Vs += 1;
      if (df) {
        // [W | V hi | V lo] as written by the factorisation, copied with
        // 16-byte loads that are all issued before the first store
        float* Ws = reinterpret_cast<float*>(Vs);
        // the lite solve reads W (and, with a correction pass, V's hi plane)
        const int n = (lite ? (max_passes > 0 ? 2 : 1) : 3) * RR;
        const int n4 = ((reinterpret_cast<uintptr_t>(w32) & 15) == 0) ? n / 4 : 0;
        // asynchronous 16-byte copies (cp.async): all in flight at once and
        // overlapped with the partial sums below; waited for before the first
        // product that reads them
        const float4* src = reinterpret_cast<const float4*>(w32);
        for (int e = tid; e < n4; e += blockDim.x) {
          const unsigned dst = (unsigned)__cvta_generic_to_shared(reinterpret_cast<float4*>(Ws) + e);
          asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(src + e)
                       : "memory");
        }
        asm volatile("cp.async.commit_group;\n" ::: "memory");
        for (int f = 4 * n4 + tid; f < n; f += blockDim.x) Ws[f] = w32[f];
        VmH = Ws + RR;
        VmL = Ws + 2 * RR;
        Wm = Ws;
      } else {
        float* Ws = reinterpret_cast<float*>(Vs + RR);
        for (int e = tid; e < RR; e += blockDim.x) { Vs[e] = vmat[e]; Ws[e] = w32[e]; }
        Vm = Vs;
        Wm = Ws;
      }
    }
    if (df) {   // the lite Gram accumulates the hi plane only
      float* gh = reinterpret_cast<float*>(gacc);
      for (int e = tid; e < (lite ? RR : 2 * RR); e += blockDim.x) gh[e] = 0.f;
    }
    __syncthreads();
    griddep_wait();   // the MTTKRP partials (programmatic launch inside a sweep)
    griddep_launch_dependents();
    if (als_stopped(ctrl, true)) {
      asm volatile("cp.async.wait_all;\n" ::: "memory");   // no copy outlives the CTA
      return;
    }
    const int rr = tid / R, c = tid - (tid / R) * R;
    const bool act = tid < RB * R;
    for (int64_t base = row0; base < row1; base += RB) {
      const int64_t row = base + rr;
      const bool live = act && row < row1;
      if constexpr (sizeof(T) == 4) {
        if (lite) {
          // The bf16 sweeps' solve on the f32 pipe alone (this GPU's f64 pipe
          // is ~64x slower): m in f32, x = m W, and with max_passes > 0 one
          // correction x += (m - x V_hi) W.  The MTTKRP it solves for is
          // itself only accurate to ~1e-6.
          float m = 0.f;
          if (live) {
            float sh, sc;
            sum_splits_sc(partial, splits, IR, row * R + c, sh, sc);
            m = sh + sc;
          }
          if (act) mbf[rr * R + c] = m;
          asm volatile("cp.async.wait_all;\n" ::: "memory");   // this thread's copies of W, V
          __syncthreads();
          // four-chain dot products of a row vector in shared memory with a
          // column of an R x R matrix in shared memory
          auto dot_col = [&](const float* v, const float* M) -> float {
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
            int k = 0;
            for (; k + 3 < R; k += 4) {
              a0 = fmaf(v[k], M[k * R + c], a0);
              a1 = fmaf(v[k + 1], M[(k + 1) * R + c], a1);
              a2 = fmaf(v[k + 2], M[(k + 2) * R + c], a2);
              a3 = fmaf(v[k + 3], M[(k + 3) * R + c], a3);
            }
            for (; k < R; ++k) a0 = fmaf(v[k], M[k * R + c], a0);
            return (a0 + a1) + (a2 + a3);
          };
          float x = act ? dot_col(mbf + rr * R, Wm) : 0.f;
          if (max_passes > 0) {
            if (act) xbh[rr * R + c] = x;
            __syncthreads();
            if (act) rbf[rr * R + c] = m - dot_col(xbh + rr * R, VmH);
            __syncthreads();
            if (act) x += dot_col(rbf + rr * R, Wm);
          }
          if (live) {
            store_entry_f32(reinterpret_cast<float*>(A), A_bt, I, R, row, c, x);
            ip += (double)(m * x);
            gbf[rr * R + c] = x;
          } else if (act) {
            gbf[rr * R + c] = 0.f;
          }
          __syncthreads();
          gram_update_f32(reinterpret_cast<float*>(gacc), gbf, RB, R);
          __syncthreads();
          continue;
        }
      }
      if (act) {
        const double mv = live ? sum_splits(partial, splits, IR, row * R + c) : 0.0;
        mb[rr * R + c] = mv;
        mbf[rr * R + c] = (float)mv;
      }
      asm volatile("cp.async.wait_all;\n" ::: "memory");   // this thread's copies of W, V
      __syncthreads();
      if (act) {   // x0 = m W32 (f32)
        const float* m = mbf + rr * R;
        float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        int k = 0;
        for (; k + 3 < R; k += 4) {
          a0 = fmaf(m[k], Wm[k * R + c], a0);
          a1 = fmaf(m[k + 1], Wm[(k + 1) * R + c], a1);
          a2 = fmaf(m[k + 2], Wm[(k + 2) * R + c], a2);
          a3 = fmaf(m[k + 3], Wm[(k + 3) * R + c], a3);
        }
        for (; k < R; ++k) a0 = fmaf(m[k], Wm[k * R + c], a0);
        const float x0 = (a0 + a1) + (a2 + a3);
        xb[rr * R + c] = (double)x0;
        if (df) { xbh[rr * R + c] = x0; xbl[rr * R + c] = 0.f; }
      }
      __syncthreads();
      for (int pass = 0; pass < max_passes; ++pass) {
        if (tid == 0) { s_dmax = 0ull; s_xmax = 0ull; }
        if (act && lite) {   // r = m - x V with x V in f32 (four chains, V's hi plane)
          const float* xh = xbh + rr * R;
          float q[4] = {0.f, 0.f, 0.f, 0.f};
          for (int k = 0; k < R; k += 4) {
#pragma unroll
            for (int u = 0; u < 4; ++u)
              if (k + u < R) q[u] = fmaf(xh[k + u], VmH[(k + u) * R + c], q[u]);
          }
          rbf[rr * R + c] = (float)(mb[rr * R + c] - (double)((q[0] + q[1]) + (q[2] + q[3])));
        } else if (act && df) {   // r = m - x V in double-float (four Neumaier chains)
          const float* xh = xbh + rr * R;
          const float* xl = xbl + rr * R;
          float s[4] = {0.f, 0.f, 0.f, 0.f}, cp[4] = {0.f, 0.f, 0.f, 0.f};
          float low = 0.f;   // exact product errors and the cross terms
          for (int k = 0; k < R; k += 4) {   // R <= 96 here; tail guarded per term
#pragma unroll
            for (int u = 0; u < 4; ++u) {
              if (k + u < R) {
                const float a = xh[k + u], al = xl[k + u];
                const float b = VmH[(k + u) * R + c], bl = VmL[(k + u) * R + c];
                const float p = a * b;
                low += fmaf(a, b, -p) + fmaf(a, bl, al * b);
                const float t = s[u] + p;
                cp[u] += (fabsf(s[u]) >= fabsf(p)) ? ((s[u] - t) + p) : ((p - t) + s[u]);
                s[u] = t;
              }
            }
          }
          const double vx = (((double)s[0] + (double)s[1]) + ((double)s[2] + (double)s[3])) +
                            (double)(((cp[0] + cp[1]) + (cp[2] + cp[3])) + low);
          rbf[rr * R + c] = (float)(mb[rr * R + c] - vx);
        } else if (act) {   // r = m - x V (f64, eight chains)
          const double* x = xb + rr * R;
          double q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
          int k = 0;
          for (; k + 7 < R; k += 8)
#pragma unroll
            for (int u = 0; u < 8; ++u) q[u] = fma(x[k + u], Vm[(k + u) * R + c], q[u]);
          for (; k < R; ++k) q[0] = fma(x[k], Vm[k * R + c], q[0]);
          const double vx = ((q[0] + q[1]) + (q[2] + q[3])) + ((q[4] + q[5]) + (q[6] + q[7]));
          rbf[rr * R + c] = (float)(mb[rr * R + c] - vx);
        }
        __syncthreads();
        if (act) {   // x += r W32 (f32 product of the small residual)
          const float* r = rbf + rr * R;
          float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
          int k = 0;
          for (; k + 3 < R; k += 4) {
            a0 = fmaf(r[k], Wm[k * R + c], a0);
            a1 = fmaf(r[k + 1], Wm[(k + 1) * R + c], a1);
            a2 = fmaf(r[k + 2], Wm[(k + 2) * R + c], a2);
            a3 = fmaf(r[k + 3], Wm[(k + 3) * R + c], a3);
          }
          for (; k < R; ++k) a0 = fmaf(r[k], Wm[k * R + c], a0);
          const double d = (double)((a0 + a1) + (a2 + a3));
          const double xn = xb[rr * R + c] + d;
          xb[rr * R + c] = xn;
          if (df) {
            const float h = (float)xn;
            xbh[rr * R + c] = h;
            xbl[rr * R + c] = (float)(xn - (double)h);
          }
          if (live && pass + 1 < max_passes) {  // non-negative doubles order like their bits
            atomicMax(&s_dmax, (unsigned long long)__double_as_longlong(fabs(d)));
            atomicMax(&s_xmax, (unsigned long long)__double_as_longlong(fabs(xn)));
          }
        }
        __syncthreads();
        if (pass + 1 == max_passes) break;   // no stop test after the last pass
        const bool stop = __longlong_as_double((long long)s_dmax) <=
                          kIrStop * __longlong_as_double((long long)s_xmax);
        __syncthreads();  // everyone has read the maxima before they are reset
        if (stop) break;
      }
      if (live) {
        const double xd = store_entry(A, A_bt, I, R, row, c, xb[rr * R + c], rb + rr * R);
        ip = fma(mb[rr * R + c], xd, ip);
        if (df) gbf[rr * R + c] = (float)xd;   // exact: xd is an f32 value
      } else if (act) {
        rb[rr * R + c] = 0.0;
        if (df) gbf[rr * R + c] = 0.f;
      }
      __syncthreads();
      if (lite) gram_update_f32(reinterpret_cast<float*>(gacc), gbf, RB, R);
      else if (df) gram_update_df(reinterpret_cast<float*>(gacc), gbf, RB, R);
      else gram_update(gacc, rb, RB, R);   // Gram of the stored rows
      __syncthreads();
    }
  } else {
    // ------------------------------------------------ substitution path
    griddep_wait();
    griddep_launch_dependents();
    if (als_stopped(ctrl, true)) return;
    double* rowbuf = gacc + RR;                    // kSolveWarps * R
    double* sfac = rowbuf + kSolveWarps * R;       // RR + R (optional)
    if (mats_in_smem)
      for (int e = tid; e < RR + R; e += blockDim.x) sfac[e] = fac[e];
    __syncthreads();
    const double* F = mats_in_smem ? sfac : fac;
    const double* invd = F + RR;
    for (int64_t base = row0; base < row1; base += kSolveWarps) {
      const int64_t row = base + warp;
      double* rb = rowbuf + warp * R;
      if (row < row1) {
        double v[kRQ], mv[kRQ];
#pragma unroll
        for (int q = 0; q < kRQ; ++q) {
          const int r = lane + 32 * q;
          const double s = (r < R) ? sum_splits(partial, splits, IR, row * R + r) : 0.0;
          mv[q] = s;
          v[q] = s;
        }
        if (kind == 1) {  // b = P m
#pragma unroll
          for (int q = 0; q < kRQ; ++q) {
            const int r = lane + 32 * q;
            if (r < R) rb[r] = v[q];
          }
          __syncwarp();
#pragma unroll
          for (int q = 0; q < kRQ; ++q) {
            const int r = lane + 32 * q;
            if (r < R) v[q] = rb[perm[r]];
          }
          __syncwarp();
        }
        for (int j = 0; j < R; ++j) {   // forward substitution, lower factor
          const int qj = j >> 5;
          double yj = __shfl_sync(0xffffffffu, pick(v, qj), j & 31);
          if (kind == 0) yj *= invd[j];
          if (lane == (j & 31)) put(v, qj, yj);
#pragma unroll
          for (int q = 0; q < kRQ; ++q) {
            const int i = lane + 32 * q;
            if (i > j && i < R) v[q] = fma(-F[i * R + j], yj, v[q]);
          }
        }
        for (int j = R - 1; j >= 0; --j) {   // back substitution, upper factor (L^T for Cholesky)
          const int qj = j >> 5;
          const double xj = __shfl_sync(0xffffffffu, pick(v, qj), j & 31) * invd[j];
          if (lane == (j & 31)) put(v, qj, xj);
#pragma unroll
          for (int q = 0; q < kRQ; ++q) {
            const int i = lane + 32 * q;
            if (i < j) {
              const double u = (kind == 0) ? F[j * R + i] : F[i * R + j];
              v[q] = fma(-u, xj, v[q]);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < kRQ; ++q) {
          const int r = lane + 32 * q;
          if (r < R) {
            const double xd = store_entry(A, A_bt, I, R, row, r, v[q], rb);
            ip = fma(mv[q], xd, ip);
          }
        }
      } else {
        for (int r = lane; r < R; r += 32) rb[r] = 0.0;
      }
      __syncthreads();
      gram_update(gacc, rowbuf, kSolveWarps, R);
      __syncthreads();
    }
  }
  ip = warp_sum(ip);
  if (lane == 0) s_ip[warp] = ip;
  // lower triangle only (the upper one is not accumulated); the reducer mirrors.
  // With df the partial is written as (hi, lo) f32 planes into the same slot
  // (the substitution path splits its f64 sums), which the reducer sums on
  // the f32 pipe.
  double* out = gpart + (int64_t)blockIdx.x * RR;
  if (df) {
    float* o = reinterpret_cast<float*>(out);
    if (kind == 2 && lite) {
      // one plane, lower triangle: the entries the reducer reads (df == 2)
      const float* g = reinterpret_cast<const float*>(gacc);
      for (int e = tid; e < RR; e += blockDim.x)
        if (e - (e / R) * R <= e / R) o[e] = g[e];
    } else if (kind == 2) {
      const float* g = reinterpret_cast<const float*>(gacc);
      for (int e = tid; e < 2 * RR; e += blockDim.x) o[e] = g[e];
    } else {
      for (int e = tid; e < RR; e += blockDim.x) {
        const double g = gacc[e];
        const float h = (float)g;
        o[e] = h;
        o[RR + e] = (float)(g - (double)h);
      }
    }
  } else {
    for (int e = tid; e < RR; e += blockDim.x) out[e] = gacc[e];
  }
  __syncthreads();
  if (ipart && tid == 0) {
    double t = 0.0;
    for (int w = 0; w < kSolveWarps; ++w) t += s_ip[w];
    ipart[blockIdx.x] = t;
  }
}

// ---------------------------------------------------------------- fit
// Hadamard product of all Grams scaled by w w^T, summed (= cp_norm^2); four
// entries per thread in flight so the f64 products do not form one chain.
template <typename T>
__device__ double sum_gram_product(const double* G, int ndim, int R, const T* w) {
  const int RR = R * R;
  double acc = 0.0;
  for (int e0 = threadIdx.x; e0 < RR; e0 += 4 * blockDim.x) {
    double v[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int e = e0 + j * blockDim.x;
      if (e < RR) v[j] = 1.0;
    }
    for (int k = 0; k < ndim; ++k)
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int e = e0 + j * blockDim.x;
        if (e < RR) v[j] = v[j] * G[(int64_t)k * RR + e];
      }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int e = e0 + j * blockDim.x;
      if (e < RR && w) v[j] = v[j] * ((double)w[e / R] * (double)w[e % R]);
    }
    acc += (v[0] + v[1]) + (v[2] + v[3]);
  }
  return acc;
}

template <typename T>
__global__ void k_fit(const double* G, int ndim, int R, const T* w, const double* ipart, int nip,
                      AlsCtrl* ctrl, double* errors, int n_iter_max, double tol, int crit) {
  if (als_stopped(ctrl)) return;
  __shared__ double scratch[32];
  double c = block_sum(sum_gram_product<T>(G, ndim, R, w), scratch);
  double ip = 0.0;
  for (int i = threadIdx.x; i < nip; i += blockDim.x) ip += ipart[i];
  ip = block_sum(ip, scratch);
  if (threadIdx.x == 0) {
    const double nx2 = ctrl->norm_x2;
    const double err = sqrt(fabs(nx2 + c - 2.0 * ip)) / sqrt(nx2);
    const int it = ctrl->iter;
    if (it < n_iter_max) errors[it] = err;
    if (tol > 0.0 && it >= 1) {
      const double dec = errors[it - 1] - err;
      const bool stop = (crit == 0) ? (fabs(dec) < tol) : (dec < tol);
      if (stop) ctrl->done = 1;
    }
    ctrl->iter = it + 1;
  }
}

// The last mode's Gram reduction fused with the fit.  Every block reduces its
// 32 Gram entries and adds their terms of cp_norm^2 = sum_e prod_k G_k[e]
// w_r w_s (an entry below the diagonal counts twice, for its mirror) into
// fpart[block]; the block that finishes last (a device-scope counter in the
// control block, which it resets) sums fpart and the <M, A> partials in a
// fixed order and records the error.  Deterministic whichever block is last.
// At most 64 registers a thread (the second launch bound): a CTA then fits
// beside a tensor-core MTTKRP CTA (192 threads x 253 registers), so on the
// aux stream it does not wait for an idle SM.
template <typename T>
__global__ void __launch_bounds__(256, 4)
k_gram_reduce_fit(const double* __restrict__ gpart, int nparts, int R, double* G_all, int mode,
                  int ndim, int df, const T* w, const double* ipart, int nip, double* fpart,
                  AlsCtrl* ctrl, double* errors, int n_iter_max, double tol, int crit,
                  float* G32_all, int deferred) {
  griddep_wait();   // the solve's Gram and <M, A> partials
  if (als_stopped(ctrl)) return;
  const int RR = R * R;
  const double t = gram_reduce_block(gpart, nparts, R, G_all + (int64_t)mode * RR, df,
                                     G32_all ? G32_all + (int64_t)mode * 2 * RR : nullptr);
  __shared__ int s_last;
  __shared__ double scratch[32];
  if (threadIdx.x < 32) {
    const int e = blockIdx.x * 32 + threadIdx.x;
    const int r = e / R, s = e - (e / R) * R;
    double v = 0.0;
    if (e < RR && s <= r) {
      v = t;
      for (int k = 0; k < ndim; ++k)
        if (k != mode) v = v * G_all[(int64_t)k * RR + e];
      if (w) v = v * ((double)w[r] * (double)w[s]);
      if (s < r) v = 2.0 * v;
    }
    v = warp_sum(v);
    if (threadIdx.x == 0) fpart[blockIdx.x] = v;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) s_last = (atomicAdd(&ctrl->red_count, 1) == (int)gridDim.x - 1) ? 1 : 0;
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double acc = 0.0;
  for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x) acc += __ldcg(&fpart[b]);
  const double c = block_sum(acc, scratch);
  double ip = 0.0;
  for (int i = threadIdx.x; i < nip; i += blockDim.x) ip += ipart[i];
  ip = block_sum(ip, scratch);
  if (threadIdx.x == 0) {
    ctrl->red_count = 0;
    const double nx2 = ctrl->norm_x2;
    const double err = sqrt(fabs(nx2 + c - 2.0 * ip)) / sqrt(nx2);
    const int it = ctrl->iter;
    if (it < n_iter_max) errors[it] = err;
    if (tol > 0.0 && it >= 1) {
      const double dec = errors[it - 1] - err;
      const bool stop = (crit == 0) ? (fabs(dec) < tol) : (dec < tol);
      if (stop) {   // deferred: beside the next sweep's first MTTKRP, which reads done
        if (deferred) ctrl->done_pending = 1;
        else ctrl->done = 1;
      }
    }
    ctrl->iter = it + 1;
  }
}

// <X, [[w; A]]> partials: sum over rows of (sum of MTTKRP split partials) * A.
template <typename T>
__global__ void k_inner_partial(const T* __restrict__ partial, int splits, int64_t n,
                                const T* __restrict__ A, double* ipart) {
  __shared__ double scratch[32];
  double s = 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
       e += (int64_t)gridDim.x * blockDim.x) {
    double m = 0.0;
    for (int p = 0; p < splits; ++p) m += (double)partial[(int64_t)p * n + e];
    s = fma(m, (double)A[e], s);
  }
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) ipart[blockIdx.x] = s;
}

// Relative error of the current model without updating anything:
// sqrt(|nx2 + cp_norm^2 - 2 <X, rec>|) / sqrt(nx2) -> *out.
template <typename T>
__global__ void k_probe_error(const double* G, int ndim, int R, const T* w, const double* ipart,
                              int nip, const AlsCtrl* ctrl, double* out) {
  __shared__ double scratch[32];
  const int RR = R * R;
  double c = 0.0;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k) v = v * G[(int64_t)k * RR + e];
    if (w) v = v * ((double)w[r] * (double)w[s]);
    c += v;
  }
  c = block_sum(c, scratch);
  double ip = 0.0;
  for (int i = threadIdx.x; i < nip; i += blockDim.x) ip += ipart[i];
  ip = block_sum(ip, scratch);
  if (threadIdx.x == 0) {
    const double nx2 = ctrl->norm_x2;
    *out = sqrt(fabs(nx2 + c - 2.0 * ip)) / sqrt(nx2);
  }
}

// cp_norm (tensorly/cp_tensor.py:614-644): sqrt(sum(prod_k G_k * w w^T)).
template <typename T>
__global__ void k_cp_norm(const double* G, int ndim, int R, const T* w, double* out) {
  __shared__ double scratch[32];
  const int RR = R * R;
  double c = 0.0;
  for (int e = threadIdx.x; e < RR; e += blockDim.x) {
    const int r = e / R, s = e % R;
    double v = 1.0;
    for (int k = 0; k < ndim; ++k) v = v * G[(int64_t)k * RR + e];
    if (w) v = v * ((double)w[r] * (double)w[s]);
    c += v;
  }
  c = block_sum(c, scratch);
  if (threadIdx.x == 0) *out = sqrt(c);
}

// ---------------------------------------------------------------- normalisation
template <typename T>
struct FactorPtrs {
  T* f[kMaxModes];
  int64_t rows[kMaxModes];
};

template <typename T>
__global__ void k_normalize(FactorPtrs<T> fp, int ndim, int R, T* weights, const int* done) {
  if (done && *done) return;
  __shared__ double scratch[32];
  const int r = blockIdx.x;
  T wacc = weights ? weights[r] : T(1);
  for (int k = 0; k < ndim; ++k) {
    T* f = fp.f[k];
    const int64_t I = fp.rows[k];
    if (k == 0) {
      for (int64_t i = threadIdx.x; i < I; i += blockDim.x) f[i * R + r] = f[i * R + r] * wacc;
      wacc = T(1);
      __syncthreads();
    }
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < I; i += blockDim.x) {
      const double x = (double)f[i * R + r];
      s = fma(x, x, s);
    }
    s = block_sum(s, scratch);
    const T scale = (T)sqrt(s);
    wacc = wacc * scale;
    const T div = (scale == T(0)) ? T(1) : scale;
    for (int64_t i = threadIdx.x; i < I; i += blockDim.x) f[i * R + r] = f[i * R + r] / div;
    __syncthreads();
  }
  if (threadIdx.x == 0 && weights) weights[r] = wacc;
}

}  // namespace

// ====================================================================== launchers
int solve_blocks_for(int64_t I) {
  const int64_t want = ceil_div(I, 4);  // about four rows per CTA
  return (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)sm_count() * 2));
}

int als_launch_sumsq(int dtype, const void* X, int64_t n, double* part, int nblocks,
                     AlsCtrl* ctrl, cudaStream_t st) {
  if (dtype == TLGB_F32)
    k_sumsq_f32<<<nblocks, 256, 0, st>>>((const float*)X, n, part);
  else
    k_sumsq<double><<<nblocks, 256, 0, st>>>((const double*)X, n, part);
  TLGB_LAUNCH_CHECK();
  return als_launch_sumsq_final(part, nblocks, ctrl, st);
}

int als_launch_sumsq_final(const double* part, int nblocks, AlsCtrl* ctrl, cudaStream_t st) {
  k_sumsq_final<<<1, 256, 0, st>>>(part, nblocks, ctrl);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_gram(const T* A, int64_t I, int R, double* gpart, int nparts_max, double* G,
                    const int* done, cudaStream_t st, float* G32) {
  int nparts = (int)std::min<int64_t>(nparts_max, std::max<int64_t>(1, ceil_div(I, 4)));
  const int64_t rpb = ceil_div(I, nparts);
  nparts = (int)ceil_div(I, rpb);
  const int threads = 256;
  const size_t smem = ((size_t)R * R + (size_t)kGramRows * R) * sizeof(double);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(
        k_gram_partial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)(((size_t)kMaxAlsRank * kMaxAlsRank + kGramRows * kMaxAlsRank) * sizeof(double))));
    attr[dev] = true;
  }
  k_gram_partial<T><<<nparts, threads, smem, st>>>(A, I, R, rpb, gpart, done);
  TLGB_LAUNCH_CHECK();
  return als_launch_gram_reduce(gpart, nparts, R, G, done, 0, st, G32);
}

int als_launch_gram_reduce(const double* gpart, int nparts, int R, double* G, const int* done,
                           int df, cudaStream_t st, float* G32) {
  const int RR = R * R;
  k_gram_reduce<<<(int)ceil_div(RR, 32), 256, 0, st>>>(gpart, nparts, R, G, done, df, G32);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T, int TI, int TJ, int NI, int NJ>
static void launch_fast(const double* G, const float* G32, int ndim, int mode, int R, const T* w,
                        double l2, double* vmat, float* w32, AlsCtrl* ctrl, double* fac, int* perm,
                        cudaStream_t st) {
  k_factorize_fast<T, TI, TJ, NI, NJ><<<1, TI * TJ, 0, st>>>(G, G32, ndim, mode, R, w, l2, vmat,
                                                             w32, ctrl, fac, perm);
}

// Hands every factorisation to the f64 kernel (the "f64_factorize" tuning key).
__global__ void k_force_f64_factorize(AlsCtrl* ctrl) {
  if (!als_stopped(ctrl) && threadIdx.x == 0) ctrl->fac_kind = 3;
}

template <typename T>
int als_launch_factorize(const double* G, int ndim, int mode, int R, const T* weights,
                         double l2_reg, double* fac, int* perm, double* vmat, float* w32,
                         AlsCtrl* ctrl, cudaStream_t st, const float* G32) {
  int rc = als_prepare(TypeCode<T>::value);
  if (rc) return rc;
  if (tc_tuning().f64_factorize)
    k_force_f64_factorize<<<1, 32, 0, st>>>(ctrl);
  else if (R <= 32)
    launch_fast<T, 8, 16, 4, 2>(G, G32, ndim, mode, R, weights, l2_reg, vmat, w32, ctrl, fac,
                                    perm, st);
  else if (R <= 64)
    launch_fast<T, 16, 16, 4, 4>(G, G32, ndim, mode, R, weights, l2_reg, vmat, w32, ctrl, fac,
                                    perm, st);
  else if (R <= 96)
    launch_fast<T, 16, 16, 6, 6>(G, G32, ndim, mode, R, weights, l2_reg, vmat, w32, ctrl, fac,
                                    perm, st);
  else
    launch_fast<T, 16, 16, 10, 10>(G, G32, ndim, mode, R, weights, l2_reg, vmat, w32, ctrl, fac,
                                    perm, st);
  TLGB_LAUNCH_CHECK();
  if (tc_tuning().f64_factorize) {   // (the fast kernel otherwise falls back in its own launch)
    k_factorize<T><<<1, 256, 0, st>>>(G, ndim, mode, R, weights, l2_reg, fac, perm, vmat, ctrl);
    TLGB_LAUNCH_CHECK();
  }
  return TLGB_OK;
}

// Dynamic shared memory of k_solve for rank R (largest of its two paths).
static size_t solve_smem(int R) {
  const size_t RR = (size_t)R * R;
  const bool mats = R <= kSolveDfMaxRank;
  const size_t rb = (size_t)std::max(1, kSolveThreads / R) * R;
  // gacc, mb, xb, rb (f64) + five f32 arrays + V (f64, or two f32 planes) and W (f32),
  // whose start is rounded up to 16 bytes (one more double)
  const size_t ir = RR + 3 * rb + ((5 * rb + 3) / 4) * 2 + (mats ? RR + (RR + 1) / 2 + 1 : 0);
  const size_t direct = RR + (size_t)kSolveWarps * R + (mats ? RR + R : 0);
  return std::max(ir, direct) * sizeof(double);
}

template <typename T>
int als_launch_solve(const T* partial, int splits, int64_t I, int R, const double* fac,
                     const int* perm, const double* vmat, const float* w32, T* A,
                     __nv_bfloat16* A_bt, double* gpart, double* ipart, AlsCtrl* ctrl,
                     int max_passes, int* nblocks, cudaStream_t st, bool pdl, bool lite) {
  const int nb = solve_blocks_for(I);
  const int64_t rpb = ceil_div(I, nb);
  const int nbe = (int)ceil_div(I, rpb);
  int rc = als_prepare(TypeCode<T>::value);
  if (rc) return rc;
  const int mats = R <= kSolveDfMaxRank ? 1 : 0;
  if (R == 64)
    TLGB_CUDA_TRY(launch_maybe_pdl(pdl, k_solve<T, 64>, dim3(nbe), dim3(kSolveThreads),
                                   solve_smem(R), st, partial, splits, I, R, fac, perm, vmat,
                                   w32, A, A_bt, gpart, ipart, ctrl, rpb, mats, max_passes,
                                   lite ? 1 : 0));
  else if (R == 32)
    TLGB_CUDA_TRY(launch_maybe_pdl(pdl, k_solve<T, 32>, dim3(nbe), dim3(kSolveThreads),
                                   solve_smem(R), st, partial, splits, I, R, fac, perm, vmat,
                                   w32, A, A_bt, gpart, ipart, ctrl, rpb, mats, max_passes,
                                   lite ? 1 : 0));
  else
    TLGB_CUDA_TRY(launch_maybe_pdl(pdl, k_solve<T, 0>, dim3(nbe), dim3(kSolveThreads),
                                   solve_smem(R), st, partial, splits, I, R, fac, perm, vmat,
                                   w32, A, A_bt, gpart, ipart, ctrl, rpb, mats, max_passes,
                                   lite ? 1 : 0));
  TLGB_LAUNCH_CHECK();
  *nblocks = nbe;
  return TLGB_OK;
}

template <typename T>
int als_launch_fit(const double* G, int ndim, int R, const T* weights, const double* ipart,
                   int nip, AlsCtrl* ctrl, double* errors, int n_iter_max, double tol,
                   int cvg_criterion, cudaStream_t st) {
  k_fit<T><<<1, 512, 0, st>>>(G, ndim, R, weights, ipart, nip, ctrl, errors, n_iter_max, tol,
                              cvg_criterion);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_gram_reduce_fit(const double* gpart, int nparts, int R, double* G_all, int mode,
                               int ndim, int df, const T* weights, const double* ipart, int nip,
                               double* fpart, AlsCtrl* ctrl, double* errors, int n_iter_max,
                               double tol, int cvg_criterion, cudaStream_t st, bool pdl,
                               float* G32_all, bool deferred) {
  const int RR = R * R;
  TLGB_CUDA_TRY(launch_maybe_pdl(pdl, k_gram_reduce_fit<T>, dim3((unsigned)ceil_div(RR, 32)),
                                 dim3(256), 0, st, gpart, nparts, R, G_all, mode, ndim, df,
                                 weights, ipart, nip, fpart, ctrl, errors, n_iter_max, tol,
                                 cvg_criterion, G32_all, deferred ? 1 : 0));
  return TLGB_OK;
}

template <typename T>
int als_launch_normalize(T* const* factors, const int64_t* rows, int ndim, int R, T* weights,
                         const int* done, cudaStream_t st) {
  FactorPtrs<T> fp{};
  for (int k = 0; k < ndim; ++k) { fp.f[k] = factors[k]; fp.rows[k] = rows[k]; }
  k_normalize<T><<<R, 256, 0, st>>>(fp, ndim, R, weights, done);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

template <typename T>
int als_launch_cp_norm(const double* G, int ndim, int R, const T* weights, double* out,
                       cudaStream_t st) {
  k_cp_norm<T><<<1, 256, 0, st>>>(G, ndim, R, weights, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
template int als_launch_cp_norm<float>(const double*, int, int, const float*, double*, cudaStream_t);
template int als_launch_cp_norm<double>(const double*, int, int, const double*, double*,
                                        cudaStream_t);

template <typename T>
int als_launch_probe_error(const T* partial, int splits, int64_t I, int R, const T* A,
                           const double* G, int ndim, const T* weights, double* ipart,
                           int nip_max, const AlsCtrl* ctrl, double* out, cudaStream_t st) {
  const int64_t n = I * R;
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(nip_max, ceil_div(n, 256)));
  k_inner_partial<T><<<nb, 256, 0, st>>>(partial, splits, n, A, ipart);
  TLGB_LAUNCH_CHECK();
  k_probe_error<T><<<1, 256, 0, st>>>(G, ndim, R, weights, ipart, nb, ctrl, out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
template int als_launch_probe_error<float>(const float*, int, int64_t, int, const float*,
                                           const double*, int, const float*, double*, int,
                                           const AlsCtrl*, double*, cudaStream_t);
template int als_launch_probe_error<double>(const double*, int, int64_t, int, const double*,
                                            const double*, int, const double*, double*, int,
                                            const AlsCtrl*, double*, cudaStream_t);

template <typename T, int TI, int TJ, int NI, int NJ>
static cudaError_t set_carveout_fast() {
  return cudaFuncSetAttribute(k_factorize_fast<T, TI, TJ, NI, NJ>,
                              cudaFuncAttributePreferredSharedMemoryCarveout,
                              cudaSharedmemCarveoutMaxShared);
}

template <typename T>
static int als_prepare_typed() {
  static std::atomic<bool> done[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && done[dev]) return TLGB_OK;
  // The factorisation kernels run on a side stream next to the tensor-core
  // MTTKRP, whose CTAs need nearly all of an SM's shared memory: keep the SMs
  // they land on configured for the maximum shared-memory carveout, so a
  // MTTKRP CTA can start beside them instead of waiting for them to finish.
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_factorize<T>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
  TLGB_CUDA_TRY((set_carveout_fast<T, 8, 16, 4, 2>()));
  TLGB_CUDA_TRY((set_carveout_fast<T, 16, 16, 4, 4>()));
  TLGB_CUDA_TRY((set_carveout_fast<T, 16, 16, 6, 6>()));
  TLGB_CUDA_TRY((set_carveout_fast<T, 16, 16, 10, 10>()));
  // likewise the Gram reductions on the side stream, which share SMs with
  // MTTKRP CTAs (they fit beside one in registers and shared memory), and
  // the solves
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_gram_reduce_fit<T>,
                                     cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_gram_reduce, cudaFuncAttributePreferredSharedMemoryCarveout,
                                     cudaSharedmemCarveoutMaxShared));
  TLGB_CUDA_TRY((cudaFuncSetAttribute(k_solve<T, 64>,
                                      cudaFuncAttributePreferredSharedMemoryCarveout,
                                      cudaSharedmemCarveoutMaxShared)));
  TLGB_CUDA_TRY((cudaFuncSetAttribute(k_solve<T, 32>,
                                      cudaFuncAttributePreferredSharedMemoryCarveout,
                                      cudaSharedmemCarveoutMaxShared)));
  TLGB_CUDA_TRY((cudaFuncSetAttribute(k_solve<T, 0>,
                                      cudaFuncAttributePreferredSharedMemoryCarveout,
                                      cudaSharedmemCarveoutMaxShared)));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(
      k_gram_partial<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      (int)(((size_t)kMaxAlsRank * kMaxAlsRank + kGramRows * kMaxAlsRank) * sizeof(double))));
  size_t smax = 0;
  for (int r = 1; r <= kMaxAlsRank; ++r) smax = std::max(smax, solve_smem(r));
  TLGB_CUDA_TRY(cudaFuncSetAttribute(k_solve<T, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smax));
  TLGB_CUDA_TRY((cudaFuncSetAttribute(k_solve<T, 32>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)solve_smem(32))));
  TLGB_CUDA_TRY((cudaFuncSetAttribute(k_solve<T, 64>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)solve_smem(64))));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return TLGB_OK;
}

int als_prepare(int dtype) {
  return dtype == TLGB_F64 ? als_prepare_typed<double>() : als_prepare_typed<float>();
}

#define TLGB_INST(T)                                                                          \
  template int als_launch_gram<T>(const T*, int64_t, int, double*, int, double*, const int*,  \
                                  cudaStream_t, float*);                                     \
  template int als_launch_factorize<T>(const double*, int, int, int, const T*, double,       \
                                       double*, int*, double*, float*, AlsCtrl*,             \
                                       cudaStream_t, const float*);                          \
  template int als_launch_solve<T>(const T*, int, int64_t, int, const double*, const int*,   \
                                   const double*, const float*, T*, __nv_bfloat16*, double*, \
                                   double*, AlsCtrl*, int, int*, cudaStream_t, bool, bool);  \
  template int als_launch_fit<T>(const double*, int, int, const T*, const double*, int,      \
                                 AlsCtrl*, double*, int, double, int, cudaStream_t);         \
  template int als_launch_gram_reduce_fit<T>(const double*, int, int, double*, int, int, int,  \
                                             const T*, const double*, int, double*, AlsCtrl*, \
                                             double*, int, double, int, cudaStream_t, bool, \
                                             float*, bool);                                   \
  template int als_launch_normalize<T>(T* const*, const int64_t*, int, int, T*, const int*,  \
                                       cudaStream_t);
TLGB_INST(float)
TLGB_INST(double)
#undef TLGB_INST

}  // namespace tlgb
