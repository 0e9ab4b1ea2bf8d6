// Learned warm start for CP-ALS: the data generator, the sketches, the
// network's training and inference kernels and the batched SVD baseline.
//
// Problem family (fixed sizes I = 32, R = 8, sketch width S = 16): tensor t
// is a rank-8 CP model X = [[A0, A1, A2]] + 1 % noise whose factor columns
// have equal pairwise congruence c_n ~ U(0, 0.9) per mode (A_n = Q_n L_n^T,
// Q_n the Gram-Schmidt orthonormalisation of a Gaussian 32 x 8 matrix, L_n
// the Cholesky factor of (1 - c_n) I + c_n 1 1^T), the "swamp" regime of
// ALS.  The network sees the three sketches S_n = unfold(X, n) Omega_n
// (Omega_n a fixed 1024 x 16 Gaussian matrix) divided by ||X|| and predicts
// the three 32 x 8 factors divided by ||X||^(1/3).
//
// Random numbers: counter-based, z = SplitMix64((stream << 40) ^ index)
// (Steele, Lea and Flood, "Fast splittable pseudorandom number generators",
// OOPSLA 2014); a uniform is the top 24 bits + 1/2 scaled into (0, 1), a
// Gaussian is Box-Muller on the uniforms of indices 2i and 2i + 1.  Streams:
// 8 t + n (factor n of tensor t), 8 t + 3 + n (congruence of mode n),
// 8 t + 6 (noise), 2^23 + n (Omega_n).
//
// Network: 1536 -> 1024 -> 512 -> 768, ReLU between layers, plus a fixed skip
// that adds the first 8 columns of each sketch to the output, trained with
// Adam on the relative reconstruction error of [[A0, A1, A2]] at its best
// scale (V_n the Hadamard product of the other factors' Grams and M_n the
// MTTKRP give the gradient).  All layers run on one strided f32
// GEMM kernel (forward X W^T, backward dY W and dY^T X) with the bias, the
// ReLU and the ReLU mask fused into its epilogue.
#include "linalg.cuh"

namespace tlgb {
namespace {

constexpr int kI = 32, kR = 8, kS = 16;
constexpr int kN3 = kI * kI * kI;            // 32768 elements
constexpr int kFeat = 3 * kI * kS;           // 1536 inputs
constexpr int kOut = 3 * kI * kR;            // 768 outputs
constexpr int kLThreads = 256;

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ float rng_uniform(uint64_t stream, uint64_t i) {
  const uint64_t z = splitmix64((stream << 40) ^ i);
  return ((float)(z >> 40) + 0.5f) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float rng_gauss(uint64_t stream, uint64_t i) {
  const float u1 = rng_uniform(stream, 2 * i), u2 = rng_uniform(stream, 2 * i + 1);
  return sqrtf(-2.0f * logf(u1)) * cosf(6.28318530717958647692f * u2);
}

template <typename T>
__device__ __forceinline__ T warp_sum_f(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ float block_sum_f(float v, float* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  v = warp_sum_f(v);
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  float t = (threadIdx.x < kLThreads / 32) ? red[threadIdx.x] : 0.f;
  if (warp == 0) t = warp_sum_f(t);
  if (threadIdx.x == 0) red[0] = t;
  __syncthreads();
  const float r = red[0];
  __syncthreads();
  return r;
}

// ||X|| from the sum of squares and the three sketches S_n = unfold(X, n) Omega_n
// (32 x 16 each) divided by ||X||, of the tensor in shared memory; thread ->
// (two rows, one column) of each sketch.  Omega_n (64 KiB) is staged in shared
// memory (Os) per mode, so the inner loop reads only shared memory.
__device__ void sketch_block(const float* Xs, float sumsq, const float* __restrict__ omega,
                             float* Os, float* fo_base, float* xnorm_out) {
  const int tid = threadIdx.x;
  const float nrm = sqrtf(sumsq);
  if (tid == 0) *xnorm_out = nrm;
  const int s = tid & 15, rp = tid >> 4;   // rp: 0..15 -> rows 2 rp, 2 rp + 1
  for (int n = 0; n < 3; ++n) {
    __syncthreads();   // the previous mode's reads of Os are done
    const float4* src = reinterpret_cast<const float4*>(omega + (int64_t)n * kI * kI * kS);
    float4* dst = reinterpret_cast<float4*>(Os);
    for (int i = tid; i < kI * kI * kS / 4; i += kLThreads) dst[i] = __ldg(src + i);
    __syncthreads();
    float acc0 = 0.f, acc1 = 0.f;
    const int r0 = 2 * rp, r1 = 2 * rp + 1;
    for (int col = 0; col < kI * kI; ++col) {
      const int hi = col >> 5, lo = col & 31;
      int e0, e1;
      if (n == 0) { e0 = r0 * 1024 + col; e1 = r1 * 1024 + col; }
      else if (n == 1) { e0 = hi * 1024 + r0 * 32 + lo; e1 = hi * 1024 + r1 * 32 + lo; }
      else { e0 = hi * 1024 + lo * 32 + r0; e1 = hi * 1024 + lo * 32 + r1; }
      const float w = Os[col * kS + s];
      acc0 = fmaf(Xs[e0], w, acc0);
      acc1 = fmaf(Xs[e1], w, acc1);
    }
    float* fo = fo_base + n * kI * kS;
    fo[r0 * kS + s] = acc0 / nrm;
    fo[r1 * kS + s] = acc1 / nrm;
  }
}

// Copy one 32^3 tensor into shared memory with 16-byte loads, eight in flight
// per thread (one CTA per SM holds a 128 KiB tensor, so each thread must keep
// many loads outstanding to stream at the memory's rate).
__device__ __forceinline__ void load_tensor_smem(const float* __restrict__ Xg, float* Xs) {
  const float4* src = reinterpret_cast<const float4*>(Xg);
  float4* dst = reinterpret_cast<float4*>(Xs);
  constexpr int n4 = kN3 / 4, per = n4 / kLThreads;   // 32 per thread
#pragma unroll 8
  for (int k = 0; k < per; ++k) dst[threadIdx.x + k * kLThreads] = __ldg(src + threadIdx.x + k * kLThreads);
}

__global__ void k_omega(float* omega) {   // 3 x 1024 x 16
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= 3 * kI * kI * kS) return;
  const int n = e / (kI * kI * kS), r = e - n * (kI * kI * kS);
  omega[e] = rng_gauss((1ull << 23) + n, (uint64_t)r);
}

// One CTA per tensor: factors, tensor, noise, sketches.
__global__ void __launch_bounds__(kLThreads)
k_generate(const int64_t* seeds, int batch, float* X, float* feats, float* xnorm,
           const float* __restrict__ omega) {
  extern __shared__ __align__(16) float lsm[];
  float* Xs = lsm;                     // 32768
  float* F = Xs + kN3;                 // [3][32][8]
  float* red = F + 3 * kI * kR;        // 32
  float* Os = red + 32;                // 16384 (Omega of one mode)
  const int b = blockIdx.x;
  const uint64_t t = (uint64_t)seeds[b];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (warp < 3) {   // factor n = warp; lane = row
    const int n = warp;
    float g[kR];
#pragma unroll
    for (int r = 0; r < kR; ++r) g[r] = rng_gauss(8 * t + n, (uint64_t)(lane * kR + r));
    // modified Gram-Schmidt on the columns
#pragma unroll
    for (int r = 0; r < kR; ++r) {
#pragma unroll
      for (int s2 = 0; s2 < r; ++s2) {
        const float d = warp_sum_f(g[s2] * g[r]);
        g[r] -= d * g[s2];
      }
      const float nr = sqrtf(warp_sum_f(g[r] * g[r]));
      g[r] /= nr;
    }
    // L = chol((1 - c) I + c 1 1^T), A = Q L^T
    const float c = 0.9f * rng_uniform(8 * t + 3 + n, 0);
    float L[kR][kR];
#pragma unroll
    for (int i = 0; i < kR; ++i)
#pragma unroll
      for (int j = 0; j < kR; ++j) L[i][j] = 0.f;
#pragma unroll
    for (int j = 0; j < kR; ++j) {
      float s = 1.f;   // diagonal of C
#pragma unroll
      for (int k = 0; k < j; ++k) s -= L[j][k] * L[j][k];
      const float d = sqrtf(s);
      L[j][j] = d;
#pragma unroll
      for (int i = j + 1; i < kR; ++i) {
        float v = c;   // off-diagonal of C
#pragma unroll
        for (int k = 0; k < j; ++k) v -= L[i][k] * L[j][k];
        L[i][j] = v / d;
      }
    }
#pragma unroll
    for (int r = 0; r < kR; ++r) {
      float a = 0.f;
#pragma unroll
      for (int s2 = 0; s2 <= r; ++s2) a += g[s2] * L[r][s2];
      F[n * kI * kR + lane * kR + r] = a;
    }
  }
  __syncthreads();
  // clean tensor and the norms of it and of the noise
  float sx = 0.f, sn = 0.f;
  for (int e = tid; e < kN3; e += kLThreads) {
    const int i = e >> 10, j = (e >> 5) & 31, k = e & 31;
    float v = 0.f;
#pragma unroll
    for (int r = 0; r < kR; ++r)
      v += F[i * kR + r] * F[kI * kR + j * kR + r] * F[2 * kI * kR + k * kR + r];
    Xs[e] = v;
    sx += v * v;
    const float z = rng_gauss(8 * t + 6, (uint64_t)e);
    sn += z * z;
  }
  sx = block_sum_f(sx, red);
  sn = block_sum_f(sn, red);
  const float scale = 0.01f * sqrtf(sx) / sqrtf(sn);
  float sf = 0.f;
  float* Xg = X + (int64_t)b * kN3;
  for (int e = tid; e < kN3; e += kLThreads) {
    const float v = Xs[e] + scale * rng_gauss(8 * t + 6, (uint64_t)e);
    Xs[e] = v;
    Xg[e] = v;
    sf += v * v;
  }
  sf = block_sum_f(sf, red);
  sketch_block(Xs, sf, omega, Os, feats + (int64_t)b * kFeat, xnorm + b);
}

// Sketch features and norm of tensors already in memory (batch x 32768).
__global__ void __launch_bounds__(kLThreads)
k_sketch(const float* __restrict__ X, float* feats, float* xnorm, const float* __restrict__ omega) {
  extern __shared__ __align__(16) float lsm[];
  float* Xs = lsm;
  float* red = Xs + kN3;
  float* Os = red + 32;                // 16384 (Omega of one mode)
  const int b = blockIdx.x, tid = threadIdx.x;
  load_tensor_smem(X + (int64_t)b * kN3, Xs);
  __syncthreads();
  float sf = 0.f;   // the same per-thread order as the generator's, so ||X|| agrees bitwise
  for (int e = tid; e < kN3; e += kLThreads) {
    const float v = Xs[e];
    sf += v * v;
  }
  sf = block_sum_f(sf, red);
  sketch_block(Xs, sf, omega, Os, feats + (int64_t)b * kFeat, xnorm + b);
}

// C(m, n) = epi(sum_k A(m, k) B(k, n)), A(m, k) = A[m sam + k sak],
// B(k, n) = B[k sbk + n sbn]; epilogue: + bias[n], ReLU, times (mask(m, n) > 0).
constexpr int kGB = 64, kGK2 = 16;
__global__ void __launch_bounds__(256)
k_gemm(int M, int N, int K, const float* __restrict__ A, int64_t sam, int64_t sak,
       const float* __restrict__ B, int64_t sbk, int64_t sbn, float* C, int64_t ldc,
       const float* __restrict__ bias, int relu, const float* __restrict__ mask) {
  __shared__ float As[kGK2][kGB + 1];
  __shared__ float Bs[kGK2][kGB + 1];
  const int tid = threadIdx.x, ty = tid >> 4, tx = tid & 15;
  const int m0 = blockIdx.y * kGB, n0 = blockIdx.x * kGB;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += kGK2) {
    // consecutive threads walk the operand's contiguous index (k when its
    // stride is 1, else m / n) so the loads coalesce
    for (int e = tid; e < kGB * kGK2; e += 256) {
      int kk, mm;
      if (sak == 1) { kk = e & (kGK2 - 1); mm = e / kGK2; } else { kk = e / kGB; mm = e & (kGB - 1); }
      const int m = m0 + mm, k = k0 + kk;
      As[kk][mm] = (m < M && k < K) ? A[m * sam + k * sak] : 0.f;
    }
    for (int e = tid; e < kGB * kGK2; e += 256) {
      int kk, nn;
      if (sbk == 1) { kk = e & (kGK2 - 1); nn = e / kGK2; } else { kk = e / kGB; nn = e & (kGB - 1); }
      const int n = n0 + nn, k = k0 + kk;
      Bs[kk][nn] = (n < N && k < K) ? B[k * sbk + n * sbn] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kGK2; ++kk) {
      float av[4], bv[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) av[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int m = m0 + ty + 16 * i;
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int n = n0 + tx + 16 * j;
      if (n >= N) continue;
      float v = acc[i][j];
      if (bias) v += bias[n];
      if (relu) v = fmaxf(v, 0.f);
      if (mask && !(mask[(int64_t)m * ldc + n] > 0.f)) v = 0.f;
      C[(int64_t)m * ldc + n] = v;
    }
  }
}

// Column sums (bias gradients): out[n] = sum_m Y[m * ld + n].
__global__ void k_colsum(const float* Y, int M, int N, int64_t ld, float* out) {
  const int n = blockIdx.x * blockDim.x + threadIdx.x;
  if (n >= N) return;
  float s = 0.f;
  for (int m = 0; m < M; ++m) s += Y[(int64_t)m * ld + n];
  out[n] = s;
}

// Scale-free reconstruction loss of one tensor and its gradient with respect
// to the network output.  out: 768 = three 32 x 8 factors divided by
// ||X||^(1/3); A_n = out_n ||X||^(1/3), p = <X, [[A]]> = <M_0, A_0>,
// q = ||[[A]]||^2 = sum G0 * G1 * G2.  The loss is the relative error at the
// best scale of the model, 1 - p^2 / (||X||^2 q) (no saddle at out = 0), with
// gradient (2 p / (||X||^2 q)) ((p / q) A_n V_n - M_n) per factor; alpha = p / q
// is that best scale.
__global__ void __launch_bounds__(kLThreads)
k_cp_loss(const float* __restrict__ X, const float* __restrict__ out,
          const float* __restrict__ xnorm, int batch, float* loss, float* dout, float* alpha) {
  extern __shared__ __align__(16) float lsm[];
  float* Xs = lsm;                    // 32768
  float* Ah = Xs + kN3;               // [3][32][8] scaled factors
  float* M = Ah + 3 * kI * kR;        // [3][32][8]
  float* G = M + 3 * kI * kR;         // [3][8][8]
  float* red = G + 3 * kR * kR;       // 32
  const int b = blockIdx.x, tid = threadIdx.x;
  const float nx = xnorm[b];
  const float sc = cbrtf(nx);
  load_tensor_smem(X + (int64_t)b * kN3, Xs);
  for (int e = tid; e < kOut; e += kLThreads) Ah[e] = out[(int64_t)b * kOut + e] * sc;
  __syncthreads();
  for (int e = tid; e < 3 * kR * kR; e += kLThreads) {
    const int n = e / (kR * kR), rs = e - n * kR * kR, r = rs / kR, s = rs - (rs / kR) * kR;
    float g = 0.f;
    for (int i = 0; i < kI; ++i) g += Ah[n * kI * kR + i * kR + r] * Ah[n * kI * kR + i * kR + s];
    G[e] = g;
  }
  // MTTKRPs: thread -> (mode, row, 4 columns) in two passes of 256 of the 3*32*2
  for (int w = tid; w < 3 * kI * 2; w += kLThreads) {
    const int n = w / (kI * 2), rem = w - n * kI * 2, row = rem >> 1, q = rem & 1;
    const int o1 = (n == 0) ? 1 : 0, o2 = (n == 2) ? 1 : 2;   // the other two modes
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    for (int u = 0; u < kI; ++u) {
      float p0 = 0.f, p1 = 0.f, p2 = 0.f, p3 = 0.f;
      for (int v0 = 0; v0 < kI; ++v0) {
        const int v = (v0 + row) & (kI - 1);   // rotated per row: no bank conflicts
        int e;
        if (n == 0) e = row * 1024 + u * 32 + v;
        else if (n == 1) e = u * 1024 + row * 32 + v;
        else e = u * 1024 + v * 32 + row;
        const float x = Xs[e];
        const float* f2 = Ah + o2 * kI * kR + v * kR + 4 * q;
        p0 = fmaf(x, f2[0], p0); p1 = fmaf(x, f2[1], p1);
        p2 = fmaf(x, f2[2], p2); p3 = fmaf(x, f2[3], p3);
      }
      const float* f1 = Ah + o1 * kI * kR + u * kR + 4 * q;
      a0 = fmaf(f1[0], p0, a0); a1 = fmaf(f1[1], p1, a1);
      a2 = fmaf(f1[2], p2, a2); a3 = fmaf(f1[3], p3, a3);
    }
    float* m = M + n * kI * kR + row * kR + 4 * q;
    m[0] = a0; m[1] = a1; m[2] = a2; m[3] = a3;
  }
  __syncthreads();
  float pp = 0.f, qq = 0.f;
  for (int e = tid; e < kI * kR; e += kLThreads) pp += M[e] * Ah[e];
  for (int e = tid; e < kR * kR; e += kLThreads) qq += G[e] * G[kR * kR + e] * G[2 * kR * kR + e];
  const float p = block_sum_f(pp, red);
  const float q = block_sum_f(qq, red);
  const float nx2 = nx * nx;
  const bool ok = q > 0.f;
  if (tid == 0) {
    loss[b] = ok ? 1.f - (p / nx2) * (p / q) : 1.f;
    if (alpha) alpha[b] = ok ? p / q : 0.f;
  }
  if (!dout) return;
  // d loss / d out = ||X||^(1/3) (2 p / (||X||^2 q)) ((p / q) A_n V_n - M_n) / batch
  const float gs = ok ? 2.f * sc * (p / nx2) / (q * (float)batch) : 0.f;
  const float pq = ok ? p / q : 0.f;
  for (int e = tid; e < kOut; e += kLThreads) {
    const int n = e / (kI * kR), rem = e - n * kI * kR, i = rem / kR, r = rem - (rem / kR) * kR;
    float av = 0.f;
    for (int s = 0; s < kR; ++s) {
      float v = 1.f;
      for (int k = 0; k < 3; ++k)
        if (k != n) v *= G[k * kR * kR + s * kR + r];
      av += Ah[n * kI * kR + i * kR + s] * v;
    }
    dout[(int64_t)b * kOut + e] = gs * (pq * av - M[e]);
  }
}

// Fixed skip connection of the network: out_n[i, r] += S_n[i, r] / ||X||, the
// first R columns of mode n's sketch (they lie in the span of factor n).
__global__ void k_sketch_skip(const float* __restrict__ feats, int batch, float* out) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)batch * kOut) return;
  const int b = (int)(e / kOut), rem = (int)(e - (int64_t)b * kOut);
  const int n = rem / (kI * kR), ir = rem - n * kI * kR, i = ir / kR, r = ir - (ir / kR) * kR;
  out[e] += feats[(int64_t)b * kFeat + n * kI * kS + i * kS + r];
}

// Initial factors from the network output: F = out * (||X|| * alpha)^(1/3).
__global__ void k_lift(const float* __restrict__ out, const float* __restrict__ xnorm,
                       const float* __restrict__ alpha, int batch, float* F) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= (int64_t)batch * kOut) return;
  const int b = (int)(e / kOut);
  F[e] = out[e] * cbrtf(xnorm[b]) * cbrtf(alpha[b]);
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Gram matrices of the three unfoldings of each 32^3 tensor (SVD baseline).
__global__ void __launch_bounds__(kLThreads)
k_gram3(const float* __restrict__ X, float* G) {
  extern __shared__ __align__(16) float lsm[];
  float* Xs = lsm;
  const int b = blockIdx.x, tid = threadIdx.x;
  load_tensor_smem(X + (int64_t)b * kN3, Xs);
  __syncthreads();
  for (int w = tid; w < 3 * kI * kI; w += kLThreads) {
    const int n = w / (kI * kI), rem = w - n * kI * kI, r = rem / kI, c = rem - (rem / kI) * kI;
    float acc = 0.f;
    for (int col = 0; col < kI * kI; ++col) {
      const int hi = col >> 5, lo = col & 31;
      int e0, e1;
      if (n == 0) { e0 = r * 1024 + col; e1 = c * 1024 + col; }
      else if (n == 1) { e0 = hi * 1024 + r * 32 + lo; e1 = hi * 1024 + c * 32 + lo; }
      else { e0 = hi * 1024 + lo * 32 + r; e1 = hi * 1024 + lo * 32 + c; }
      acc = fmaf(Xs[e0], Xs[e1], acc);
    }
    G[((int64_t)b * 3 + n) * kI * kI + rem] = acc;
  }
}

// SVD initial factors from the eigenpairs: mode 0 columns times sqrt(lambda).
__global__ void k_svd_init_scale(float* U, const float* lam, int batch) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= batch * kI * kR) return;
  const int b = e / (kI * kR), r = e % kR;
  const float l = lam[(int64_t)b * 3 * kR + r];   // mode 0 of tensor b
  U[(int64_t)b * 3 * kI * kR + (e - b * kI * kR)] *= (l > 0.f ? sqrtf(l) : 0.f);
}

}  // namespace
}  // namespace tlgb

using namespace tlgb;

extern "C" int tlgb_ws_omega(void* omega, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(omega != nullptr, "ws_omega: null pointer");
  const int n = 3 * kI * kI * kS;
  k_omega<<<(n + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>((float*)omega);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_generate(const int64_t* seeds, int batch, void* X, void* feats, void* xnorm,
                                const void* omega, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(seeds && X && feats && xnorm && omega && batch >= 1, "ws_generate: bad argument");
  const size_t smem = (size_t)(kN3 + 3 * kI * kR + 32 + kI * kI * kS) * sizeof(float);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_generate, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr[dev] = true;
  }
  k_generate<<<batch, kLThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      seeds, batch, (float*)X, (float*)feats, (float*)xnorm, (const float*)omega);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_sketch(const void* X, int batch, void* feats, void* xnorm,
                              const void* omega, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(X && feats && xnorm && omega && batch >= 1, "ws_sketch: bad argument");
  const size_t smem = (size_t)(kN3 + 32 + kI * kI * kS) * sizeof(float);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_sketch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr[dev] = true;
  }
  k_sketch<<<batch, kLThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      (const float*)X, (float*)feats, (float*)xnorm, (const float*)omega);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_gemm(int M, int N, int K, const void* A, int64_t sam, int64_t sak,
                            const void* B, int64_t sbk, int64_t sbn, void* C, int64_t ldc,
                            const void* bias, int relu, const void* mask, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(A && B && C && M >= 1 && N >= 1 && K >= 1, "ws_gemm: bad argument");
  dim3 grid((unsigned)((N + kGB - 1) / kGB), (unsigned)((M + kGB - 1) / kGB));
  k_gemm<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      M, N, K, (const float*)A, sam, sak, (const float*)B, sbk, sbn, (float*)C, ldc,
      (const float*)bias, relu, (const float*)mask);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_colsum(const void* Y, int M, int N, int64_t ld, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(Y && out && M >= 1 && N >= 1, "ws_colsum: bad argument");
  k_colsum<<<(N + 255) / 256, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      (const float*)Y, M, N, ld, (float*)out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_cp_loss(const void* X, const void* out, const void* xnorm, int batch,
                               void* loss, void* dout, void* alpha, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(X && out && xnorm && loss && batch >= 1, "ws_cp_loss: bad argument");
  const size_t smem = (size_t)(kN3 + 6 * kI * kR + 3 * kR * kR + 32) * sizeof(float);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_cp_loss, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr[dev] = true;
  }
  k_cp_loss<<<batch, kLThreads, smem, static_cast<cudaStream_t>(stream)>>>(
      (const float*)X, (const float*)out, (const float*)xnorm, batch, (float*)loss, (float*)dout,
      (float*)alpha);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_sketch_skip(const void* feats, int batch, void* out, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(feats && out && batch >= 1, "ws_sketch_skip: bad argument");
  const int64_t n = (int64_t)batch * kOut;
  k_sketch_skip<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      (const float*)feats, batch, (float*)out);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_lift(const void* out, const void* xnorm, const void* alpha, int batch,
                            void* factors, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(out && xnorm && alpha && factors && batch >= 1, "ws_lift: bad argument");
  const int64_t n = (int64_t)batch * kOut;
  k_lift<<<(unsigned)((n + 255) / 256), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      (const float*)out, (const float*)xnorm, (const float*)alpha, batch, (float*)factors);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_adam(void* p, const void* g, void* m, void* v, int64_t n, float lr,
                            float beta1, float beta2, float eps, int step, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(p && g && m && v && n >= 1 && step >= 1, "ws_adam: bad argument");
  const float c1 = 1.f - powf(beta1, (float)step), c2 = 1.f - powf(beta2, (float)step);
  const int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
  k_adam<<<blocks, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      (float*)p, (const float*)g, (float*)m, (float*)v, n, lr, beta1, beta2, eps, c1, c2);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}

extern "C" int tlgb_ws_svd_init_workspace_size(int batch, size_t* bytes) {
  clear_error();
  TLGB_CHECK_ARG(bytes && batch >= 1, "ws_svd_init_workspace_size: bad argument");
  *bytes = align_up((size_t)batch * 3 * kI * kI * sizeof(float), 256) +
           align_up((size_t)batch * 3 * kR * sizeof(float), 256) +
           align_up((size_t)batch * 3 * 6 * kR * kI * sizeof(float), 256);
  return TLGB_OK;
}

extern "C" int tlgb_ws_svd_init(const void* X, int batch, void* factors, void* workspace,
                                size_t workspace_bytes, void* stream) {
  clear_error();
  TLGB_CHECK_ARG(X && factors && batch >= 1, "ws_svd_init: bad argument");
  size_t need = 0;
  tlgb_ws_svd_init_workspace_size(batch, &need);
  if (!workspace || workspace_bytes < need)
    return set_error(TLGB_EWORKSPACE, "ws_svd_init: workspace too small");
  char* base = static_cast<char*>(workspace);
  float* G = reinterpret_cast<float*>(base);
  float* lam = reinterpret_cast<float*>(base + align_up((size_t)batch * 3 * kI * kI * 4, 256));
  void* eigws = base + align_up((size_t)batch * 3 * kI * kI * 4, 256) +
                align_up((size_t)batch * 3 * kR * 4, 256);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const size_t smem = (size_t)kN3 * sizeof(float);
  static std::atomic<bool> attr[64];  // per-device set-up flags, read and set by any host thread
  const int dev = current_device();
  if (dev >= 0 && dev < 64 && !attr[dev]) {
    TLGB_CUDA_TRY(cudaFuncSetAttribute(k_gram3, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
    attr[dev] = true;
  }
  k_gram3<<<batch, kLThreads, smem, st>>>((const float*)X, G);
  TLGB_LAUNCH_CHECK();
  // factors: [batch][3][32][8]; the eigensolver writes U (32 x 8) per matrix
  int rc = sym_eig_batched_launch<float>(G, kI, kR, 3 * batch, (float*)factors, lam, 1, eigws, st);
  if (rc) return rc;
  k_svd_init_scale<<<(batch * kI * kR + 255) / 256, 256, 0, st>>>((float*)factors, lam, batch);
  TLGB_LAUNCH_CHECK();
  return TLGB_OK;
}
