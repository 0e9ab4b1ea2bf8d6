// Batched CP-ALS for many small 3-way tensors of uneven shape and rank: the
// sweep of tensorly/decomposition/_cp.py:394-440 (parafac, normalize_factors
// False, weights all one) run for every tensor of the batch by one
// persistent kernel.
//
// Each CTA takes the next tensor from a work queue ordered by decreasing
// work (largest first, so the tail is short), keeps the tensor in shared
// memory when it fits (rows padded to odd strides so every access pattern of
// the three MTTKRPs is bank-conflict free; larger tensors are read from
// global memory through the same code), keeps the factors, their Grams and
// the MTTKRP in shared memory, and runs `n_sweeps` sweeps before writing the
// factors back.  Per mode:
//   warp 0      : W = V^-1 for V = Hadamard product of the other Grams
//                 (f32 Gauss-Jordan with partial pivoting, one column per lane,
//                 registers and shuffles only), concurrently with
//   warps 1..15 : M = MTTKRP (threads over (row, 4 rank columns), groups of
//                 threads over the outer mode, partial sums reduced in a
//                 fixed order);
//   then A_n = M W and G_n = A_n^T A_n.
// The last launch of a run also writes the relative error of the final model
// computed from the residual sum(x - rec)^2 (compensated), which is accurate
// where the reference's expansion ||X||^2 + ||rec||^2 - 2<M, A> (_cp.py:217-225)
// cancels (1 % noise leaves 1e-4 of ||X||^2); per-sweep errors use the
// expansion in f64.
#include <algorithm>
#include <utility>
#include <vector>

#include "common.cuh"

namespace tlgb {
namespace {

constexpr int kBThreads = 512;
constexpr int kBMaxDim = 64;
constexpr int kBMaxRank = 16;
constexpr int kBSmemTotal = 226 * 1024;   // dynamic shared memory of one SM's CTAs

// Variants: NT threads per CTA and kBThreads / NT CTAs per SM sharing the SM's
// shared memory (more small tensors in flight, or more room per tensor).
template <int NT> constexpr int red_slots() { return NT > 256 ? NT : 256; }
template <int NT> constexpr int smem_bytes() {
  return (kBSmemTotal / (kBThreads / NT)) & ~1023;
}
template <int NT> constexpr int fixed_bytes() {
  return (3 * kBMaxDim * kBMaxRank + kBMaxDim * kBMaxRank + 3 * kBMaxRank * kBMaxRank +
          2 * kBMaxRank * kBMaxRank + 4 * red_slots<NT>()) * (int)sizeof(float) +
         32 * (int)sizeof(double);
}
template <int NT> constexpr int x_cap() { return (smem_bytes<NT>() - fixed_bytes<NT>()) / 4; }

struct BItem {
  const float* X;
  float* F[3];
  int I[3];
  int R;
  int pad;
};

struct BArgs {
  const BItem* items;
  const int* order;
  int n;
  int n_sweeps;        // sweeps in this launch
  int sweep0;          // index of the first sweep of this launch
  int n_iter;          // sweeps of the whole run (row length of sweep_err)
  int last;            // this launch ends the run: write the final errors
  int* counter;        // work queue head (zeroed before the launch)
  int x_cap;           // floats of shared memory available for the tensor
  double* final_err;   // [n] (item order)
  double* sweep_err;   // [n][n_iter] or null
  int exact_sweep_err; // per-sweep errors from the residual instead of the expansion
  double tol;          // > 0: stop a tensor once |e_{s-1} - e_s| < tol (s >= 1)
  int* sweeps_done;    // [n] sweeps run per tensor, or null
  int* conv;           // [n] converged in an earlier launch (workspace, zeroed per run)
  int otile;           // outer-mode slices per MTTKRP work item (0: as many groups as fit)
};

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

template <int NT>
__device__ double block_sum_d(double v, double* scratch) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_d(v);
  __syncthreads();
  if (lane == 0) scratch[warp] = v;
  __syncthreads();
  double t = (threadIdx.x < (NT >> 5)) ? scratch[threadIdx.x] : 0.0;
  if (warp == 0) t = warp_sum_d(t);
  if (threadIdx.x == 0) scratch[0] = t;
  __syncthreads();
  const double r = scratch[0];
  __syncthreads();
  return r;
}

// W = V^-1 (RP x RP, V padded with the identity) by warp 0: lane c < 2*RP
// holds column c of [V | I]; the pivot row is chosen by |value| (first
// maximum), rows are swapped and eliminated through shuffles.
__device__ void gj_inverse_warp(const float* V, float* W, int RP) {
  const int lane = threadIdx.x & 31;
  float col[kBMaxRank];
#pragma unroll
  for (int i = 0; i < kBMaxRank; ++i) {
    float v = 0.f;
    if (i < RP) {
      if (lane < RP) v = V[i * RP + lane];
      else if (lane < 2 * RP) v = (lane - RP == i) ? 1.f : 0.f;
    }
    col[i] = v;
  }
#pragma unroll
  for (int k = 0; k < kBMaxRank; ++k) {
    if (k < RP) {
      // pivot search in column k (held by lane k)
      int p = k;
      float best = -1.f;
#pragma unroll
      for (int i = 0; i < kBMaxRank; ++i)
        if (i >= k && i < RP && fabsf(col[i]) > best) { best = fabsf(col[i]); p = i; }
      p = __shfl_sync(0xffffffffu, p, k);
      // swap rows k and p in every column
      float rk = 0.f, rp = 0.f;
#pragma unroll
      for (int i = 0; i < kBMaxRank; ++i) {
        if (i == k) rk = col[i];
        if (i == p) rp = col[i];
      }
#pragma unroll
      for (int i = 0; i < kBMaxRank; ++i) {
        if (i == k) col[i] = rp;
        else if (i == p) col[i] = rk;
      }
      float piv = 0.f;
#pragma unroll
      for (int i = 0; i < kBMaxRank; ++i)
        if (i == k) piv = col[i];
      piv = __shfl_sync(0xffffffffu, piv, k);
      if (piv == 0.f) piv = 1e-30f;
      const float inv = 1.f / piv;
      float rowk = 0.f;
#pragma unroll
      for (int i = 0; i < kBMaxRank; ++i)
        if (i == k) { col[i] *= inv; rowk = col[i]; }
#pragma unroll
      for (int i = 0; i < kBMaxRank; ++i) {
        if (i != k && i < RP) {
          const float f = __shfl_sync(0xffffffffu, col[i], k);   // column k, row i
          col[i] = fmaf(-f, rowk, col[i]);
        }
      }
    }
  }
  if (lane >= RP && lane < 2 * RP) {
#pragma unroll
    for (int i = 0; i < kBMaxRank; ++i)
      if (i < RP) W[i * RP + (lane - RP)] = col[i];
  }
}

// Copies the block X[i][j][k] (i < d0, j < d1, k < d2 <= 64; rows of d2
// contiguous floats, `pitch_i` floats between consecutive i, d2 between
// consecutive j) into shared memory at i * si + j * sj + k.  One warp per
// (i, j) row with the lanes across k (coalesced), four rows in flight per
// warp, and one division per row rather than per element.
template <int NT>
__device__ __forceinline__ void stage_block(const float* __restrict__ src, int d0, int d1, int d2,
                                            int64_t pitch_i, float* dst, int si, int sj) {
  constexpr int NW = NT / 32, U = 4;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int rows = d0 * d1;
  for (int r0 = warp; r0 < rows; r0 += NW * U) {
    float v0[U], v1[U];
    int off[U];
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int row = r0 + u * NW;
      v0[u] = 0.f;
      v1[u] = 0.f;
      off[u] = -1;
      if (row < rows) {
        const int i = row / d1, j = row - (row / d1) * d1;
        const float* s = src + i * pitch_i + (int64_t)j * d2;
        if (lane < d2) v0[u] = __ldg(s + lane);
        if (lane + 32 < d2) v1[u] = __ldg(s + lane + 32);
        off[u] = i * si + j * sj;
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      if (off[u] >= 0) {
        if (lane < d2) dst[off[u] + lane] = v0[u];
        if (lane + 32 < d2) dst[off[u] + lane + 32] = v1[u];
      }
    }
  }
}

// One thread's four rank columns of an MTTKRP row: sum over the outer
// slices b = g, g + ngrp, ... of S[b] * (sum over c of X[row, b, c] * F[c]),
// with F and S already offset to the thread's columns (rows RP apart).
template <typename Idx>
__device__ __forceinline__ float4 mttkrp_rows(const float* __restrict__ X, Idx row, Idx s_o,
                                              Idx s_c, int g, int ngrp, int no, int nc,
                                              const float* __restrict__ F,
                                              const float* __restrict__ S, int RP) {
  float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
  for (int b = g; b < no; b += ngrp) {
    const float* xp = X + row + (Idx)b * s_o;
    const float* fp = F;
    float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
#pragma unroll 4
    for (int c = 0; c < nc; ++c) {
      const float x = *xp;
      const float4 f = *reinterpret_cast<const float4*>(fp);
      p0 = fmaf(x, f.x, p0);
      p1 = fmaf(x, f.y, p1);
      p2 = fmaf(x, f.z, p2);
      p3 = fmaf(x, f.w, p3);
      xp += s_c;
      fp += RP;
    }
    const float4 sv = *reinterpret_cast<const float4*>(S + b * RP);
    a0 = fmaf(sv.x, p0, a0);
    a1 = fmaf(sv.y, p1, a1);
    a2 = fmaf(sv.z, p2, a2);
    a3 = fmaf(sv.w, p3, a3);
  }
  return make_float4(a0, a1, a2, a3);
}

// sum over the tensor of (x - [[A0, A1, A2]])^2, compensated f32 per thread
// then f64 across the block; one warp per (i, j) row of X (global memory).
template <int NT>
__device__ double residual2(const float* __restrict__ X, const float* Fs, int I0, int I1, int I2,
                            int R, int RP, double* scratch) {
  const float* A0 = Fs;
  const float* A1 = Fs + kBMaxDim * kBMaxRank;
  const float* A2 = Fs + 2 * kBMaxDim * kBMaxRank;
  float s = 0.f, c = 0.f;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int row = warp; row < I0 * I1; row += NT / 32) {
    const int i = row / I1, j = row - (row / I1) * I1;
    const float* xr = X + (int64_t)row * I2;
    for (int k = lane; k < I2; k += 32) {
      float rec = 0.f;
      for (int r = 0; r < R; ++r) rec = fmaf(A0[i * RP + r] * A1[j * RP + r], A2[k * RP + r], rec);
      const float d = __ldg(&xr[k]) - rec;
      const float h = d * d, l = fmaf(d, d, -h);
      const float u = s + h;
      c += ((fabsf(s) >= h) ? ((s - u) + h) : ((h - u) + s)) + l;
      s = u;
    }
  }
  return block_sum_d<NT>((double)s + (double)c, scratch);
}

template <int NT>
__global__ void __launch_bounds__(NT, kBThreads / NT) k_cp_als_batched(const BArgs a) {
  extern __shared__ __align__(16) float sm[];
  float* Fs = sm;                                  // [3][64 * 16]
  float* M = Fs + 3 * kBMaxDim * kBMaxRank;        // [64 * 16]
  float* G = M + kBMaxDim * kBMaxRank;             // [3][16 * 16]
  float* V = G + 3 * kBMaxRank * kBMaxRank;        // [16 * 16]
  float* W = V + kBMaxRank * kBMaxRank;            // [16 * 16]
  float* red = W + kBMaxRank * kBMaxRank;          // [4 * red_slots<NT>()]
  double* scratch = reinterpret_cast<double*>(red + 4 * red_slots<NT>());   // [32]
  float* Xs = reinterpret_cast<float*>(scratch + 32);
  __shared__ int s_t;
  const int tid = threadIdx.x;

  while (true) {
    __syncthreads();
    if (tid == 0) s_t = atomicAdd(a.counter, 1);
    __syncthreads();
    const int t = s_t;
    if (t >= a.n) break;
    const int idx = a.order[t];
    if (a.tol > 0.0 && a.sweep0 > 0 && a.conv[idx]) continue;   // stopped in an earlier launch
    const BItem it = a.items[idx];
    const int I0 = it.I[0], I1 = it.I[1], I2 = it.I[2], R = it.R;
    const int RP = (R + 3) & ~3, NQ = RP / 4;
    const int64_t numel = (int64_t)I0 * I1 * I2;

    // ---- tensor placement: padded odd strides in shared memory, or global
    int sJ = I2 | 1;
    int64_t sI = (int64_t)I1 * sJ;
    if ((sI & 1) == 0) sI += 1;
    const bool resident = (int64_t)I0 * sI <= a.x_cap;
    if (resident) {
      stage_block<NT>(it.X, I0, I1, I2, (int64_t)I1 * I2, Xs, (int)sI, sJ);
    } else {
      sJ = I2;
      sI = (int64_t)I1 * I2;
    }
    const int dims[3] = {I0, I1, I2};
    for (int k = 0; k < 3; ++k)
      for (int e = tid; e < kBMaxDim * kBMaxRank; e += NT) {
        const int i = e / RP, r = e - (e / RP) * RP;
        float v = 0.f;
        if (i < dims[k] && r < R) v = it.F[k][i * R + r];
        Fs[k * kBMaxDim * kBMaxRank + e] = (i < dims[k]) ? v : 0.f;
      }
    // ||X||^2, compensated f32 per thread
    double nx2;
    {
      float s = 0.f, c = 0.f;
      for (int64_t e0 = tid; e0 < numel; e0 += 4 * NT) {
        float xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t e = e0 + (int64_t)u * NT;
          xv[u] = (e < numel) ? __ldg(&it.X[e]) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float x = xv[u];
          const float h = x * x, l = fmaf(x, x, -h);
          const float t2 = s + h;
          c += ((fabsf(s) >= h) ? ((s - t2) + h) : ((h - t2) + s)) + l;
          s = t2;
        }
      }
      nx2 = block_sum_d<NT>((double)s + (double)c, scratch);
    }
    // Grams of the initial factors
    __syncthreads();
    for (int k = 0; k < 3; ++k) {
      for (int e = tid; e < RP * RP; e += NT) {
        const int r = e / RP, c = e - (e / RP) * RP;
        const float* F = Fs + k * kBMaxDim * kBMaxRank;
        float g = 0.f;
        for (int i = 0; i < dims[k]; ++i) g = fmaf(F[i * RP + r], F[i * RP + c], g);
        G[k * kBMaxRank * kBMaxRank + e] = g;
      }
    }
    __syncthreads();

    // tol: the error of the previous sweep is carried between launches in final_err
    double prev = (a.tol > 0.0 && a.sweep0 > 0) ? a.final_err[idx] : -1.0;
    double e_last = -1.0;
    int n_done = a.n_sweeps;
    bool stopped = false;
    for (int sw = 0; sw < a.n_sweeps; ++sw) {
      for (int n = 0; n < 3; ++n) {
        // V = Hadamard product of the other Grams (identity on the padding)
        for (int e = tid; e < RP * RP; e += NT) {
          const int r = e / RP, c = e - (e / RP) * RP;
          float v;
          if (r < R && c < R) {
            v = 1.f;
            for (int k = 0; k < 3; ++k)
              if (k != n) v *= G[k * kBMaxRank * kBMaxRank + e];
          } else {
            v = (r == c) ? 1.f : 0.f;
          }
          V[e] = v;
        }
        __syncthreads();
        // out / outer / inner modes and their strides
        const int o_mode = (n == 0) ? 1 : 0;
        const int c_mode = (n == 2) ? 1 : 2;
        const int64_t s_out = (n == 0) ? sI : (n == 1) ? (int64_t)sJ : 1;
        const int64_t s_o = (o_mode == 1) ? (int64_t)sJ : sI;
        const int64_t s_c = (c_mode == 2) ? 1 : (int64_t)sJ;
        const int na = dims[n], no = dims[o_mode], nc = dims[c_mode];
        const float* Fc = Fs + c_mode * kBMaxDim * kBMaxRank;
        const float* So = Fs + o_mode * kBMaxDim * kBMaxRank;
        const int per = na * NQ;                       // outputs (row, 4 columns)
        const int workers = NT - 32;                   // warps 1.. (warp 0 inverts V)
        // the MTTKRP's work tile: one row, four rank columns and every ngrp-th
        // outer slice; otile sets how many outer slices a tile covers
        int ngrp = max(1, min(no, workers / per));
        if (a.otile > 0) ngrp = max(1, min(ngrp, (no + a.otile - 1) / a.otile));
        if (resident) {
          if (tid < 32) {
            gj_inverse_warp(V, W, RP);
          } else {
            for (int item = tid - 32; item < ngrp * per; item += workers) {
              const int g = item / per, rem = item - (item / per) * per;
              const int ai = rem % na, q = rem / na;
              *reinterpret_cast<float4*>(red + 4 * item) =
                  mttkrp_rows<int>(Xs, ai * (int)s_out, (int)s_o, (int)s_c, g, ngrp, no, nc,
                                   Fc + 4 * q, So + 4 * q, RP);
            }
          }
        } else {
          // The tensor does not fit: panels of the outer mode are staged into
          // shared memory with coalesced loads (same odd padded strides) and
          // their contributions accumulated in `red`.
          if (tid < 32) gj_inverse_warp(V, W, RP);
          for (int item = tid; item < ngrp * per; item += NT)
            *reinterpret_cast<float4*>(red + 4 * item) = make_float4(0.f, 0.f, 0.f, 0.f);
          const bool pan_i = (o_mode == 0);   // modes 1, 2: panels of i; mode 0: panels of j
          const int ps_j = I2 | 1;
          int ps_i, P;
          if (pan_i) {
            ps_i = I1 * ps_j;
            if ((ps_i & 1) == 0) ps_i += 1;
            P = max(1, min(no, a.x_cap / ps_i));
          } else {
            P = max(1, min(no, (a.x_cap / I0 - 1) / ps_j));
            ps_i = P * ps_j;
            if ((ps_i & 1) == 0) ps_i += 1;
          }
          const int s_out_p = (n == 0) ? ps_i : (n == 1) ? ps_j : 1;
          const int s_o_p = pan_i ? ps_i : ps_j;
          const int s_c_p = (c_mode == 2) ? 1 : ps_j;
          const int64_t IJK = (int64_t)I1 * I2;
          for (int b0 = 0; b0 < no; b0 += P) {
            const int pb = min(P, no - b0);
            __syncthreads();   // the previous panel has been consumed
            if (pan_i)         // X[b0 : b0 + pb, :, :] is contiguous
              stage_block<NT>(it.X + (int64_t)b0 * IJK, pb, I1, I2, IJK, Xs, ps_i, ps_j);
            else               // X[:, b0 : b0 + pb, :]: one contiguous run per i
              stage_block<NT>(it.X + (int64_t)b0 * I2, I0, pb, I2, IJK, Xs, ps_i, ps_j);
            __syncthreads();
            if (tid >= 32) {
              for (int item = tid - 32; item < ngrp * per; item += workers) {
                const int g = item / per, rem = item - (item / per) * per;
                const int ai = rem % na, q = rem / na;
                const float4 acc = mttkrp_rows<int>(Xs, ai * s_out_p, s_o_p, s_c_p, g, ngrp, pb,
                                                    nc, Fc + 4 * q, So + b0 * RP + 4 * q, RP);
                float4* dst = reinterpret_cast<float4*>(red + 4 * item);
                float4 cur = *dst;
                cur.x += acc.x; cur.y += acc.y; cur.z += acc.z; cur.w += acc.w;
                *dst = cur;
              }
            }
          }
        }
        __syncthreads();
        // M = sum of the groups' partials in group order
        for (int e = tid; e < per; e += NT) {
          const int ai = e % na, q = e / na;
          float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
          for (int g = 0; g < ngrp; ++g) {
            const float* src = red + 4 * (g * per + e);
            s0 += src[0]; s1 += src[1]; s2 += src[2]; s3 += src[3];
          }
          float* m = M + ai * RP + 4 * q;
          m[0] = s0; m[1] = s1; m[2] = s2; m[3] = s3;
        }
        __syncthreads();
        // A_n = M W
        float* An = Fs + n * kBMaxDim * kBMaxRank;
        for (int e = tid; e < na * RP; e += NT) {
          const int i = e / RP, r = e - (e / RP) * RP;
          float v = 0.f;
          if (r < R)
            for (int s = 0; s < R; ++s) v = fmaf(M[i * RP + s], W[s * RP + r], v);
          An[e] = v;
        }
        __syncthreads();
        // G_n = A_n^T A_n
        for (int e = tid; e < RP * RP; e += NT) {
          const int r = e / RP, c = e - (e / RP) * RP;
          float g = 0.f;
          for (int i = 0; i < na; ++i) g = fmaf(An[i * RP + r], An[i * RP + c], g);
          G[n * kBMaxRank * kBMaxRank + e] = g;
        }
        __syncthreads();
      }
      if (a.tol > 0.0 || (a.sweep_err && a.exact_sweep_err)) {
        const double res2 = residual2<NT>(it.X, Fs, I0, I1, I2, R, RP, scratch);
        const double e = sqrt(res2) / sqrt(nx2);
        e_last = e;
        if (a.sweep_err && tid == 0) a.sweep_err[(int64_t)idx * a.n_iter + a.sweep0 + sw] = e;
        // _cp.py:505-522 (cvg_criterion 'abs_rec_error'); e is uniform over the block
        if (a.tol > 0.0) {
          if (a.sweep0 + sw >= 1 && fabs(prev - e) < a.tol) {
            n_done = sw + 1;
            stopped = true;
            break;
          }
          prev = e;
        }
      } else if (a.sweep_err) {   // expansion of _cp.py:217-225 in f64 from the f32 pieces
        double rec = 0.0, ip = 0.0;
        for (int e = tid; e < RP * RP; e += NT) {
          const int r = e / RP, c = e - (e / RP) * RP;
          if (r < R && c < R)
            rec += (double)G[e] * (double)G[kBMaxRank * kBMaxRank + e] *
                   (double)G[2 * kBMaxRank * kBMaxRank + e];
        }
        for (int e = tid; e < I2 * RP; e += NT) {
          const int r = e % RP;
          if (r < R) ip += (double)M[e] * (double)Fs[2 * kBMaxDim * kBMaxRank + e];
        }
        rec = block_sum_d<NT>(rec, scratch);
        ip = block_sum_d<NT>(ip, scratch);
        if (tid == 0)
          a.sweep_err[(int64_t)idx * a.n_iter + a.sweep0 + sw] =
              sqrt(fabs(nx2 + rec - 2.0 * ip)) / sqrt(nx2);
      }
    }
    // factors back to global memory
    for (int k = 0; k < 3; ++k)
      for (int e = tid; e < dims[k] * R; e += NT) {
        const int i = e / R, r = e - (e / R) * R;
        it.F[k][e] = Fs[k * kBMaxDim * kBMaxRank + i * RP + r];
      }
    if (a.last || a.tol > 0.0) {   // relative error of the current model from the residual
      if (e_last < 0.0) {
        const double res2 = residual2<NT>(it.X, Fs, I0, I1, I2, R, RP, scratch);
        e_last = sqrt(res2) / sqrt(nx2);
      }
      if (tid == 0) a.final_err[idx] = e_last;
    }
    if (tid == 0) {
      if (a.sweeps_done) a.sweeps_done[idx] = a.sweep0 + n_done;
      if (a.tol > 0.0 && stopped) a.conv[idx] = 1;
    }
  }
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

namespace {
struct BatchLayout {
  size_t items_off, order_off, counter_off, conv_off, bytes;
};
BatchLayout batch_layout(int n) {
  BatchLayout L{};
  size_t off = 0;
  auto take = [&](size_t b) { off = align_up(off, 256); const size_t o = off; off += b; return o; };
  L.items_off = take((size_t)n * sizeof(BItem));
  L.order_off = take((size_t)n * sizeof(int));
  L.counter_off = take(256);
  L.conv_off = take((size_t)n * sizeof(int));
  L.bytes = align_up(off, 256);
  return L;
}
}  // namespace

extern "C" int tlgb_cp_als_batched_workspace_size(int n_tensors, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(bytes != nullptr && n_tensors >= 0, "cp_als_batched_workspace_size: bad argument");
  *bytes = batch_layout(n_tensors).bytes;
  return TLGB_OK;
}

namespace {
// Size classes (by the padded shared-memory footprint of the tensor) and the
// kernel variant each one runs; set by tlgb_set_tuning ("batched_threads_small"
// / "_medium" / "_large", 0 = default) and chosen by the autotuner.
int g_batched_nt[3] = {0, 0, 0};
const int kDefaultNt[3] = {128, 256, 512};
int g_batched_otile[3] = {0, 0, 0};   // outer slices per MTTKRP work tile (0 = default)

int64_t padded_elems(const int64_t* d) {
  const int64_t sJ = d[2] | 1;
  int64_t sI = d[1] * sJ;
  if ((sI & 1) == 0) sI += 1;
  return d[0] * sI;
}

template <int NT>
int launch_variant(BArgs a, int grid_max, cudaStream_t st) {
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_cp_als_batched<NT>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       smem_bytes<NT>()));
    attr[dev] = true;
  }
  a.x_cap = x_cap<NT>();
  const int grid = std::min(a.n, grid_max * (kBThreads / NT));
  k_cp_als_batched<NT><<<grid, NT, smem_bytes<NT>(), st>>>(a);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
}  // namespace

namespace tlgb {
int batched_set_tuning(const std::string& key, int value) {
  int cls = -1;
  if (key == "batched_outer_tile_small") cls = 0;
  else if (key == "batched_outer_tile_medium") cls = 1;
  else if (key == "batched_outer_tile_large") cls = 2;
  if (cls >= 0) {
    TLGB_CHECK_ARG(value >= 0 && value <= 64, "set_tuning: batched outer tiles are 0..64");
    g_batched_otile[cls] = value;
    return TLGB_OK;
  }
  if (key == "batched_threads_small") cls = 0;
  else if (key == "batched_threads_medium") cls = 1;
  else if (key == "batched_threads_large") cls = 2;
  if (cls < 0) return set_error(TLGB_EINVAL, "set_tuning: unknown key " + key);
  TLGB_CHECK_ARG(value == 0 || value == 128 || value == 256 || value == 512,
                 "set_tuning: batched thread counts are 128, 256 or 512");
  g_batched_nt[cls] = value;
  return TLGB_OK;
}
}  // namespace tlgb

extern "C" int tlgb_cp_als_batched(int n_tensors, const tlgb_batch_item* items, int n_iter_max,
                                   int sweeps_per_launch, int flags, double tol,
                                   double* final_errors, double* sweep_errors, int* sweeps_done,
                                   void* workspace, size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(n_tensors >= 0 && (n_tensors == 0 || items), "cp_als_batched: bad items");
  TLGB_CHECK_ARG(n_iter_max >= 0, "cp_als_batched: n_iter_max must be >= 0");
  TLGB_CHECK_ARG(final_errors != nullptr || n_tensors == 0, "cp_als_batched: null final_errors");
  TLGB_CHECK_ARG(tol >= 0.0, "cp_als_batched: tol must be >= 0");
  if (n_tensors == 0) return TLGB_OK;
  const BatchLayout L = batch_layout(n_tensors);
  if (!workspace || workspace_bytes < L.bytes)
    return set_error(TLGB_EWORKSPACE, "cp_als_batched: workspace too small");
  std::vector<BItem> hv((size_t)n_tensors);
  std::vector<std::pair<double, int>> work[3];
  const int64_t cap_s = x_cap<128>(), cap_m = x_cap<256>();
  for (int t = 0; t < n_tensors; ++t) {
    const tlgb_batch_item& s = items[t];
    TLGB_CHECK_ARG(s.X && s.factors[0] && s.factors[1] && s.factors[2],
                   "cp_als_batched: null pointer in an item");
    for (int k = 0; k < 3; ++k)
      if (s.dims[k] < 1 || s.dims[k] > kBMaxDim)
        return set_error(TLGB_EUNSUPPORTED, "cp_als_batched: mode sizes must be in [1, 64]");
    if (s.rank < 1 || s.rank > kBMaxRank)
      return set_error(TLGB_EUNSUPPORTED, "cp_als_batched: rank must be in [1, 16]");
    BItem b{};
    b.X = static_cast<const float*>(s.X);
    for (int k = 0; k < 3; ++k) {
      b.F[k] = static_cast<float*>(s.factors[k]);
      b.I[k] = (int)s.dims[k];
    }
    b.R = (int)s.rank;
    hv[t] = b;
    const int64_t pe = padded_elems(s.dims);
    const int cls = pe <= cap_s ? 0 : pe <= cap_m ? 1 : 2;
    work[cls].push_back({-(double)s.dims[0] * s.dims[1] * s.dims[2] * ((s.rank + 3) / 4), t});
  }
  // order: large class first, each class by decreasing work
  std::vector<int> order;
  order.reserve((size_t)n_tensors);
  int off[3], cnt[3];
  for (int c = 2; c >= 0; --c) {
    std::stable_sort(work[c].begin(), work[c].end());
    off[c] = (int)order.size();
    cnt[c] = (int)work[c].size();
    for (auto& w : work[c]) order.push_back(w.second);
  }
  char* base = static_cast<char*>(workspace);
  BItem* d_items = reinterpret_cast<BItem*>(base + L.items_off);
  int* d_order = reinterpret_cast<int*>(base + L.order_off);
  int* d_counter = reinterpret_cast<int*>(base + L.counter_off);
  int* d_conv = reinterpret_cast<int*>(base + L.conv_off);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  TLGB_CUDA_TRY(cudaMemcpyAsync(d_items, hv.data(), hv.size() * sizeof(BItem),
                                cudaMemcpyHostToDevice, st));
  TLGB_CUDA_TRY(cudaMemcpyAsync(d_order, order.data(), order.size() * sizeof(int),
                                cudaMemcpyHostToDevice, st));
  BArgs a{};
  a.items = d_items;
  a.n_iter = std::max(1, n_iter_max);
  a.final_err = final_errors;
  a.sweep_err = sweep_errors;
  a.exact_sweep_err = (flags & TLGB_BATCH_EXACT_SWEEP_ERRORS) ? 1 : 0;
  a.tol = tol;
  a.sweeps_done = sweeps_done;
  a.conv = d_conv;
  if (tol > 0.0)
    TLGB_CUDA_TRY(cudaMemsetAsync(d_conv, 0, (size_t)n_tensors * sizeof(int), st));
  const int spl = sweeps_per_launch > 0 ? sweeps_per_launch : std::max(1, n_iter_max);
  const int sms = sm_count();
  int done = 0;
  do {
    const int ns = std::max(0, std::min(spl, n_iter_max - done));
    a.n_sweeps = ns;
    a.sweep0 = done;
    a.last = (done + ns >= n_iter_max) ? 1 : 0;
    TLGB_CUDA_TRY(cudaMemsetAsync(d_counter, 0, 3 * sizeof(int), st));
    for (int c = 2; c >= 0; --c) {
      if (cnt[c] == 0) continue;
      a.order = d_order + off[c];
      a.n = cnt[c];
      a.counter = d_counter + c;
      const int nt = g_batched_nt[c] ? g_batched_nt[c] : kDefaultNt[c];
      a.otile = g_batched_otile[c];
      int rc = nt == 128 ? launch_variant<128>(a, sms, st)
             : nt == 256 ? launch_variant<256>(a, sms, st)
                         : launch_variant<512>(a, sms, st);
      if (rc) return rc;
    }
    done += ns;
  } while (done < n_iter_max);
  TLGB_CUDA_TRY(cudaStreamSynchronize(st));
  return TLGB_OK;
}
