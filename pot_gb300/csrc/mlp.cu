// Kernels of the learned warm-start network (forward, backward, AdamW).
//
// The network (no counterpart in the reference) maps a cloud pair (X, Y) to a
// source potential f: per-point encoders phi_X, phi_Y, mean pooling into
// summaries s_X, s_Y, and a per-point head psi([x_i, s_X, s_Y]).  Its layers
// are dense GEMMs of a few hundred columns over B*n rows; they run as a tiled
// fp32 GEMM with fused bias and ReLU.  All training arithmetic is fp32 except
// the loss, which is accumulated in fp64.
#include <algorithm>
#include "common.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

constexpr int GT = 64;      // output tile
constexpr int GK = 16;      // k tile

// C = alpha * op(A) * op(B) + beta * C (+ bias, ReLU).  op(A) is M x K, op(B)
// is K x N; ta / tb select the transposed storage of A ([K, M]) / B ([N, K]).
template <typename T>
__global__ void __launch_bounds__(256) gemm_tiled_kernel(int ta, int tb, int64_t M, int64_t N, int64_t K, T alpha,
                                                         const T* __restrict__ A, int64_t lda,
                                                         const T* __restrict__ B, int64_t ldb, T beta,
                                                         T* __restrict__ C, int64_t ldc,
                                                         const T* __restrict__ bias, int relu,
                                                         int64_t sA, int64_t sB, int64_t sC, int splitk) {
  __shared__ T As[GK][GT + 4];
  __shared__ T Bs[GK][GT + 4];
  // gridDim.z is either the split-K factor (splitk = 1) or the batch (strides sA, sB, sC)
  if (!splitk) {
    A += blockIdx.z * sA;
    B += blockIdx.z * sB;
    C += blockIdx.z * sC;
  }
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int64_t m0 = (int64_t)blockIdx.y * GT, n0 = (int64_t)blockIdx.x * GT;
  // split-K: CTA z covers k in [kbeg, kend) and adds its partial product
  const int64_t nz = splitk ? gridDim.z : 1, z = splitk ? blockIdx.z : 0;
  const int64_t kper = ((K + nz - 1) / nz + GK - 1) / GK * GK;
  const int64_t kbeg = z * kper, kend = min(K, kbeg + kper);
  const bool split = splitk && nz > 1;
  T acc[4][4] = {};
  for (int64_t k0 = kbeg; k0 < kend; k0 += GK) {
    // load A tile (GT x GK) into As[k][m]
    for (int e = threadIdx.x; e < GT * GK; e += 256) {
      int mm, kk;
      if (ta) { kk = e / GT; mm = e % GT; } else { mm = e / GK; kk = e % GK; }
      const int64_t gm = m0 + mm, gk = k0 + kk;
      T val = 0;
      if (gm < M && gk < kend) val = ta ? A[gk * lda + gm] : A[gm * lda + gk];
      As[kk][mm] = val;
    }
    for (int e = threadIdx.x; e < GT * GK; e += 256) {
      int nn, kk;
      if (tb) { nn = e / GK; kk = e % GK; } else { kk = e / GT; nn = e % GT; }
      const int64_t gn = n0 + nn, gk = k0 + kk;
      T val = 0;
      if (gn < N && gk < kend) val = tb ? B[gn * ldb + gk] : B[gk * ldb + gn];
      Bs[kk][nn] = val;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GK; ++kk) {
      T a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty * 4 + i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx * 4 + j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int64_t gm = m0 + ty * 4 + i;
    if (gm >= M) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gn = n0 + tx * 4 + j;
      if (gn >= N) continue;
      T r = alpha * acc[i][j];
      if (split) { atomicAdd(C + gm * ldc + gn, r); continue; }  // C zeroed, no bias/act
      if (beta != T(0)) r += beta * C[gm * ldc + gn];
      if (bias) r += bias[gn];
      if (relu) r = fmax(r, T(0));
      C[gm * ldc + gn] = r;
    }
  }
}

// dY *= (Y > 0)
__global__ void relu_bwd_kernel(float* dY, const float* Y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (!(Y[i] > 0.f)) dY[i] = 0.f;
}

// out[c] (+)= sum_r X[r, c]  (bias gradients), X is R x C row-major.
__global__ void colsum_kernel(const float* X, int64_t R, int64_t C, float* out, int accumulate) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= C) return;
  float s = 0.f;
  for (int64_t r = blockIdx.y; r < R; r += gridDim.y) s += X[r * C + c];
  atomicAdd(out + c, s);
  (void)accumulate;
}

// Segment mean: out[p, c] = mean_{r in segment p} X[p*n + r, c].
__global__ void segment_mean_kernel(const float* X, int64_t P, int64_t n, int64_t C, float* out) {
  const int64_t p = blockIdx.y;
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= C || p >= P) return;
  float s = 0.f;
  for (int64_t r = 0; r < n; ++r) s += X[(p * n + r) * C + c];
  out[p * C + c] = s / (float)n;
}

// Backward of the segment mean: dX[p*n + r, c] (+)= dS[p, c] / n.
__global__ void segment_mean_bwd_kernel(const float* dS, int64_t P, int64_t n, int64_t C, float* dX, int accumulate) {
  const int64_t total = P * n * C;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e % C, row = e / C, p = row / n;
    const float g = dS[p * C + c] / (float)n;
    dX[e] = accumulate ? dX[e] + g : g;
  }
}

// z[p*n + r] = [x (d), sx[p] (H), sy[p] (H)]
__global__ void concat3_kernel(const float* x, const float* sx, const float* sy, int64_t P, int64_t n, int64_t d,
                               int64_t H, float* z) {
  const int64_t W = d + 2 * H;
  const int64_t total = P * n * W;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = e % W, row = e / W, p = row / n;
    float val;
    if (c < d) val = x[row * d + c];
    else if (c < d + H) val = sx[p * H + (c - d)];
    else val = sy[p * H + (c - d - H)];
    z[e] = val;
  }
}

// Backward of concat3 for the summaries: dsx[p, h] = sum_r dz[p*n+r, d+h], same for dsy.
__global__ void concat3_bwd_kernel(const float* dz, int64_t P, int64_t n, int64_t d, int64_t H, float* dsx, float* dsy) {
  const int64_t p = blockIdx.y;
  const int64_t h = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (h >= 2 * H || p >= P) return;
  const int64_t W = d + 2 * H;
  float s = 0.f;
  for (int64_t r = 0; r < n; ++r) s += dz[(p * n + r) * W + d + h];
  if (h < H) dsx[p * H + h] = s;
  else dsy[p * H + (h - H)] = s;
}

// Gauge-free loss: per segment, e = (f - mean f) - t (targets already centred);
// loss += sum e^2 / (P n); df = 2 (e - mean e) / (P n).
__global__ void centered_mse_kernel(const float* f, const float* t, int64_t P, int64_t n, double* loss, float* df) {
  const int64_t p = blockIdx.x;
  __shared__ double red[32];
  __shared__ float s_mean_f, s_mean_e;
  double s = 0;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) s += f[p * n + r];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) { double q = 0; for (int w = 0; w < (int)(blockDim.x >> 5); ++w) q += red[w]; s_mean_f = (float)(q / n); }
  __syncthreads();
  const float mf = s_mean_f;
  double se = 0, se2 = 0;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) {
    const float e = (f[p * n + r] - mf) - t[p * n + r];
    se += e; se2 += (double)e * e;
  }
  se = warp_sum(se); se2 = warp_sum(se2);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = se;
  __syncthreads();
  if (threadIdx.x == 0) { double q = 0; for (int w = 0; w < (int)(blockDim.x >> 5); ++w) q += red[w]; s_mean_e = (float)(q / n); }
  __syncthreads();
  const double scale = 1.0 / ((double)P * (double)n);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, se2 * scale);
  const float me = s_mean_e;
  for (int64_t r = threadIdx.x; r < n; r += blockDim.x) {
    const float e = (f[p * n + r] - mf) - t[p * n + r];
    df[p * n + r] = (float)(2.0 * scale) * (e - me);
  }
}

// AdamW (decoupled weight decay), bias-corrected.
__global__ void adamw_kernel(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                             float eps, float wd, float bc1, float bc2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi; v[i] = vi;
    const float mh = mi / bc1, vh = vi / bc2;
    w[i] = w[i] - lr * (mh / (sqrtf(vh) + eps) + wd * w[i]);
  }
}

inline int blocks_for(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 16); }

}  // namespace otg

using namespace otg;

template <typename T>
static int gemm_tiled(int ta, int tb, int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, const T* B,
                      int64_t ldb, T beta, T* C, int64_t ldc, const T* bias, int relu, cudaStream_t stream) {
  if (M < 1 || N < 1 || K < 1 || !A || !B || !C) return OTG_ERR_ARG;
  if ((M + GT - 1) / GT > 65535) return OTG_ERR_UNSUPPORTED;
  const int64_t tiles = ((N + GT - 1) / GT) * ((M + GT - 1) / GT);
  int64_t splits = 1;
  // few output tiles and a long K (weight gradients over many rows): split K
  if (tiles < 304 && K >= 4096 && beta == 0.f && !bias && !relu) splits = std::min<int64_t>(K / 1024, 608 / tiles + 1);
  if (splits > 1 && ldc != N) splits = 1;  // split-K accumulates into a zeroed, dense C
  if (splits > 1 && cudaMemsetAsync(C, 0, sizeof(T) * M * N, stream) != cudaSuccess) return OTG_ERR_CUDA;
  dim3 grid((unsigned)((N + GT - 1) / GT), (unsigned)((M + GT - 1) / GT), (unsigned)splits);
  gemm_tiled_kernel<T><<<grid, 256, 0, stream>>>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, bias, relu,
                                                 0, 0, 0, 1);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

template <typename T>
static int gemm_batched(int ta, int tb, int64_t M, int64_t N, int64_t K, T alpha, const T* A, int64_t lda, int64_t sA,
                        const T* B, int64_t ldb, int64_t sB, T beta, T* C, int64_t ldc, int64_t sC, int64_t batch,
                        cudaStream_t stream) {
  if (M < 1 || N < 1 || K < 1 || batch < 1 || !A || !B || !C) return OTG_ERR_ARG;
  if ((M + GT - 1) / GT > 65535 || batch > 65535) return OTG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)((N + GT - 1) / GT), (unsigned)((M + GT - 1) / GT), (unsigned)batch);
  gemm_tiled_kernel<T><<<grid, 256, 0, stream>>>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, nullptr, 0,
                                                 sA, sB, sC, 0);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

// ---------------------------------------------------------------------------
// Fused inference of the warm-start network (no activations in memory).
//
// Encoder + pooling: s[p] = mean_i relu(relu(x_i W1 + b1) W2 + b2) over the
// n points of cloud p; one thread per point, weights in shared memory, the
// block's sum added to s[p] (pre-scaled by 1/n) with one atomic per output.
template <int D, int H1, int H2>
__global__ void __launch_bounds__(256) mlp_encode_pool_kernel(const float* __restrict__ X, int n,
                                                              const float* __restrict__ W1, const float* __restrict__ b1,
                                                              const float* __restrict__ W2, const float* __restrict__ b2,
                                                              float* __restrict__ s) {
  __shared__ float w1[D * H1], sb1[H1], w2[H1 * H2], sb2[H2], acc[H2];
  const int p = blockIdx.y;
  for (int e = threadIdx.x; e < D * H1; e += blockDim.x) w1[e] = W1[e];
  for (int e = threadIdx.x; e < H1 * H2; e += blockDim.x) w2[e] = W2[e];
  for (int e = threadIdx.x; e < H1; e += blockDim.x) sb1[e] = b1[e];
  for (int e = threadIdx.x; e < H2; e += blockDim.x) { sb2[e] = b2[e]; acc[e] = 0.f; }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float h2v[H2];
#pragma unroll
  for (int o = 0; o < H2; ++o) h2v[o] = 0.f;
  if (i < n) {
    float x[D];
#pragma unroll
    for (int q = 0; q < D; ++q) x[q] = X[((int64_t)p * n + i) * D + q];
    float h1v[H1];
#pragma unroll
    for (int o = 0; o < H1; ++o) {
      float a = sb1[o];
#pragma unroll
      for (int q = 0; q < D; ++q) a = fmaf(x[q], w1[q * H1 + o], a);
      h1v[o] = fmaxf(a, 0.f);
    }
    const float inv = 1.f / (float)n;
#pragma unroll
    for (int o = 0; o < H2; ++o) {
      float a = sb2[o];
#pragma unroll
      for (int q = 0; q < H1; ++q) a = fmaf(h1v[q], w2[q * H2 + o], a);
      h2v[o] = fmaxf(a, 0.f) * inv;
    }
  }
#pragma unroll
  for (int o = 0; o < H2; ++o) {
    float v = h2v[o];
    for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(acc + o, v);
  }
  __syncthreads();
  for (int o = threadIdx.x; o < H2; o += blockDim.x) atomicAdd(s + (int64_t)p * H2 + o, acc[o]);
}

// Head: f_i = relu(relu([z_i, sX_p, sY_p] W3 + b3) W4 + b4) W5 + b5.  The
// summaries' part of the first layer is the same for every point of a pair:
// it is folded into a per-pair bias once per block.  One thread per point.
template <int DZ, int H2, int H3>
__global__ void __launch_bounds__(128) mlp_head_kernel(const float* __restrict__ Z, int n,
                                                       const float* __restrict__ sX, const float* __restrict__ sY,
                                                       const float* __restrict__ W3, const float* __restrict__ b3,
                                                       const float* __restrict__ W4, const float* __restrict__ b4,
                                                       const float* __restrict__ W5, const float* __restrict__ b5,
                                                       float* __restrict__ f) {
  __shared__ __align__(16) float w3[DZ * H3];
  __shared__ __align__(16) float w4t[H3 * H3];  // transposed: [out][in]
  __shared__ float cb[H3], sb4[H3], w5[H3];
  const int p = blockIdx.y;
  for (int e = threadIdx.x; e < DZ * H3; e += blockDim.x) w3[e] = W3[e];
  for (int e = threadIdx.x; e < H3 * H3; e += blockDim.x) { const int a = e / H3, b = e % H3; w4t[b * H3 + a] = W4[e]; }
  for (int o = threadIdx.x; o < H3; o += blockDim.x) {
    float a = b3[o];
    for (int q = 0; q < H2; ++q) a = fmaf(sX[(int64_t)p * H2 + q], W3[(DZ + q) * H3 + o], a);
    for (int q = 0; q < H2; ++q) a = fmaf(sY[(int64_t)p * H2 + q], W3[(DZ + H2 + q) * H3 + o], a);
    cb[o] = a;
    sb4[o] = b4[o];
    w5[o] = W5[o];
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float z[DZ];
#pragma unroll
  for (int q = 0; q < DZ; ++q) z[q] = Z[((int64_t)p * n + i) * DZ + q];
  float h3v[H3];
#pragma unroll
  for (int o = 0; o < H3; ++o) h3v[o] = cb[o];
#pragma unroll
  for (int q = 0; q < DZ; ++q) {
#pragma unroll
    for (int o = 0; o < H3; o += 4) {
      const float4 w = *reinterpret_cast<const float4*>(w3 + q * H3 + o);
      h3v[o] = fmaf(z[q], w.x, h3v[o]);
      h3v[o + 1] = fmaf(z[q], w.y, h3v[o + 1]);
      h3v[o + 2] = fmaf(z[q], w.z, h3v[o + 2]);
      h3v[o + 3] = fmaf(z[q], w.w, h3v[o + 3]);
    }
  }
#pragma unroll
  for (int o = 0; o < H3; ++o) h3v[o] = fmaxf(h3v[o], 0.f);
  float out = b5[0];
  for (int o = 0; o < H3; ++o) {
    float a = sb4[o];
#pragma unroll
    for (int q = 0; q < H3; q += 4) {
      const float4 w = *reinterpret_cast<const float4*>(w4t + o * H3 + q);
      a = fmaf(h3v[q], w.x, a);
      a = fmaf(h3v[q + 1], w.y, a);
      a = fmaf(h3v[q + 2], w.z, a);
      a = fmaf(h3v[q + 3], w.w, a);
    }
    out = fmaf(fmaxf(a, 0.f), w5[o], out);
  }
  f[(int64_t)p * n + i] = out;
}

extern "C" {

int otg_gemm_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda,
                 const float* B, int64_t ldb, float beta, float* C, int64_t ldc, const float* bias, int relu,
                 cudaStream_t stream) {
  return gemm_tiled<float>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, bias, relu, stream);
}

int otg_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                 const double* B, int64_t ldb, double beta, double* C, int64_t ldc, cudaStream_t stream) {
  return gemm_tiled<double>(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, nullptr, 0, stream);
}

int otg_gemm_batched(int dtype, int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const void* A,
                     int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, double beta, void* C,
                     int64_t ldc, int64_t sC, int64_t batch, cudaStream_t stream) {
  if (dtype == OTG_F64)
    return gemm_batched<double>(ta, tb, M, N, K, alpha, (const double*)A, lda, sA, (const double*)B, ldb, sB, beta,
                                (double*)C, ldc, sC, batch, stream);
  if (dtype == OTG_F32)
    return gemm_batched<float>(ta, tb, M, N, K, (float)alpha, (const float*)A, lda, sA, (const float*)B, ldb, sB,
                               (float)beta, (float*)C, ldc, sC, batch, stream);
  return OTG_ERR_DTYPE;
}

int otg_mlp_relu_bwd(float* dY, const float* Y, int64_t n, cudaStream_t stream) {
  relu_bwd_kernel<<<blocks_for(n), 256, 0, stream>>>(dY, Y, n);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_colsum(const float* X, int64_t R, int64_t C, float* out, cudaStream_t stream) {
  if (cudaMemsetAsync(out, 0, sizeof(float) * C, stream) != cudaSuccess) return OTG_ERR_CUDA;
  dim3 grid((unsigned)((C + 127) / 128), (unsigned)std::min<int64_t>(R, 256));
  colsum_kernel<<<grid, 128, 0, stream>>>(X, R, C, out, 1);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_encode_pool(const float* X, int64_t P, int64_t n, int32_t d, int32_t h1, int32_t h2, const float* W1,
                        const float* b1, const float* W2, const float* b2, float* s, cudaStream_t stream) {
  if (!X || !W1 || !b1 || !W2 || !b2 || !s || P < 1 || P > 65535 || n < 1) return OTG_ERR_ARG;
  if (!(d == 16 && h1 == 32 && h2 == 32)) return OTG_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(s, 0, sizeof(float) * (size_t)P * h2, stream) != cudaSuccess) return OTG_ERR_CUDA;
  dim3 grid((unsigned)((n + 255) / 256), (unsigned)P);
  mlp_encode_pool_kernel<16, 32, 32><<<grid, 256, 0, stream>>>(X, (int)n, W1, b1, W2, b2, s);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_head(const float* Z, int64_t P, int64_t n, int32_t dz, int32_t h2, int32_t h3, const float* sX,
                 const float* sY, const float* W3, const float* b3, const float* W4, const float* b4, const float* W5,
                 const float* b5, float* f, cudaStream_t stream) {
  if (!Z || !sX || !sY || !W3 || !b3 || !W4 || !b4 || !W5 || !b5 || !f || P < 1 || P > 65535 || n < 1)
    return OTG_ERR_ARG;
  if (!(dz == 22 && h2 == 32 && h3 == 64)) return OTG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)((n + 127) / 128), (unsigned)P);
  mlp_head_kernel<22, 32, 64><<<grid, 128, 0, stream>>>(Z, (int)n, sX, sY, W3, b3, W4, b4, W5, b5, f);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_segment_mean(const float* X, int64_t P, int64_t n, int64_t C, float* out, cudaStream_t stream) {
  if (P > 65535) return OTG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)((C + 127) / 128), (unsigned)P);
  segment_mean_kernel<<<grid, 128, 0, stream>>>(X, P, n, C, out);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_segment_mean_bwd(const float* dS, int64_t P, int64_t n, int64_t C, float* dX, int accumulate,
                             cudaStream_t stream) {
  segment_mean_bwd_kernel<<<blocks_for(P * n * C), 256, 0, stream>>>(dS, P, n, C, dX, accumulate);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_concat3(const float* x, const float* sx, const float* sy, int64_t P, int64_t n, int64_t d, int64_t H,
                    float* z, cudaStream_t stream) {
  concat3_kernel<<<blocks_for(P * n * (d + 2 * H)), 256, 0, stream>>>(x, sx, sy, P, n, d, H, z);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_concat3_bwd(const float* dz, int64_t P, int64_t n, int64_t d, int64_t H, float* dsx, float* dsy,
                        cudaStream_t stream) {
  if (P > 65535) return OTG_ERR_UNSUPPORTED;
  dim3 grid((unsigned)((2 * H + 127) / 128), (unsigned)P);
  concat3_bwd_kernel<<<grid, 128, 0, stream>>>(dz, P, n, d, H, dsx, dsy);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_centered_mse(const float* f, const float* t, int64_t P, int64_t n, double* loss, float* df,
                         cudaStream_t stream) {
  if (cudaMemsetAsync(loss, 0, sizeof(double), stream) != cudaSuccess) return OTG_ERR_CUDA;
  centered_mse_kernel<<<(unsigned)P, 256, 0, stream>>>(f, t, P, n, loss, df);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_mlp_adamw(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                  float wd, int step, cudaStream_t stream) {
  if (step < 1) return OTG_ERR_ARG;
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  adamw_kernel<<<blocks_for(n), 256, 0, stream>>>(w, g, m, v, n, lr, b1, b2, eps, wd, bc1, bc2);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

}  // extern "C"
