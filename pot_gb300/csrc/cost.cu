// Squared-Euclidean cost blocks for a table of point-cloud pairs, and the
// batched plan / value kernel.
//
// Reference behaviour: ot/utils.py:270-305 (euclidean_distances, squared) and
// ot/batch/_linear.py:54-85 (dist_euclidean_batch) compute |x|^2+|y|^2-2x.y;
// here the cost is formed from coordinate differences, sum_k (x_k - y_k)^2,
// which has no cancellation and matches a float64 evaluation more closely.
// Plan and values: ot/batch/_linear.py:326-345 (value_linear = sum M T,
// value = value_linear + reg * sum T log(T + 1e-16) or the KL form).
#include <algorithm>
#include "common.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

// One CTA per (problem, tile of 32 rows); the tile's points are staged in
// shared memory.  With a compile-time dimension D each thread keeps four
// target points in registers and writes four adjacent costs per row as one
// 16-byte store; other dimensions take the generic loop.  Padded columns
// [m, ldm) get +inf.
template <typename T, int D>
__device__ __forceinline__ void sqdist_tile_fixed(const T* xs, int rows, const T* Y, int m, int ldm, T* M, int r0,
                                                  T& local_max) {
  for (int j0 = threadIdx.x * 4; j0 < ldm; j0 += blockDim.x * 4) {
    T y[4][D];
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
      for (int k = 0; k < D; ++k) y[q][k] = (j0 + q < m) ? Y[(int64_t)(j0 + q) * D + k] : T(0);
    for (int r = 0; r < rows; ++r) {
      T acc[4] = {0, 0, 0, 0};
#pragma unroll
      for (int k = 0; k < D; ++k) {
        const T xk = xs[r * D + k];
#pragma unroll
        for (int q = 0; q < 4; ++q) { const T df = xk - y[q][k]; acc[q] = fma(df, df, acc[q]); }
      }
      T* dst = M + (int64_t)(r0 + r) * ldm + j0;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (j0 + q < m) local_max = fmax(local_max, acc[q]);
        else acc[q] = T(INFINITY);
      }
      if (j0 + 4 <= ldm && sizeof(T) == 4) {
        *reinterpret_cast<float4*>(dst) = make_float4((float)acc[0], (float)acc[1], (float)acc[2], (float)acc[3]);
      } else {
#pragma unroll
        for (int q = 0; q < 4; ++q) if (j0 + q < ldm) dst[q] = acc[q];
      }
    }
  }
}

template <typename T>
__global__ void __launch_bounds__(256) batched_sqdist_kernel(OtgCostTable t) {
  constexpr int TR = 32;
  extern __shared__ __align__(16) unsigned char sm_raw[];
  T* xs = reinterpret_cast<T*>(sm_raw);
  const int p = blockIdx.y;
  if (p >= t.nprob) return;
  const int n = t.rows[p], m = t.cols[p], d = t.dim[p], ldm = t.ldm[p];
  const int r0 = blockIdx.x * TR;
  if (r0 >= n) return;
  const int rows = min(TR, n - r0);
  const T* X = static_cast<const T*>(t.X) + t.x_off[p];
  const T* Y = static_cast<const T*>(t.Y) + t.y_off[p];
  T* M = static_cast<T*>(t.M) + t.m_off[p];
  for (int e = threadIdx.x; e < rows * d; e += blockDim.x) xs[e] = X[(int64_t)r0 * d + e];
  __syncthreads();
  T local_max = 0;
  // ldm is a multiple of 16 bytes, so 4-column groups of float rows stay aligned
  if (d == 16 && ldm % 4 == 0) sqdist_tile_fixed<T, 16>(xs, rows, Y, m, ldm, M, r0, local_max);
  else if (d == 8 && ldm % 4 == 0) sqdist_tile_fixed<T, 8>(xs, rows, Y, m, ldm, M, r0, local_max);
  else if (d == 3 && ldm % 4 == 0) sqdist_tile_fixed<T, 3>(xs, rows, Y, m, ldm, M, r0, local_max);
  else if (d == 2 && ldm % 4 == 0) sqdist_tile_fixed<T, 2>(xs, rows, Y, m, ldm, M, r0, local_max);
  else {
    for (int j = threadIdx.x; j < ldm; j += blockDim.x) {
      if (j < m) {
        const T* y = Y + (int64_t)j * d;
        for (int r = 0; r < rows; ++r) {
          const T* x = xs + r * d;
          T acc = 0;
          for (int k = 0; k < d; ++k) { const T df = x[k] - y[k]; acc = fma(df, df, acc); }
          M[(int64_t)(r0 + r) * ldm + j] = acc;
          local_max = fmax(local_max, acc);
        }
      } else {
        for (int r = 0; r < rows; ++r) M[(int64_t)(r0 + r) * ldm + j] = T(INFINITY);
      }
    }
  }
  if (t.max_out) {
    // non-negative floats order like their bit patterns
    local_max = warp_max(local_max);
    if ((threadIdx.x & 31) == 0) {
      if (sizeof(T) == 4) atomicMax(reinterpret_cast<unsigned int*>(static_cast<T*>(t.max_out) + p), __float_as_uint((float)local_max));
      else atomicMax(reinterpret_cast<unsigned long long*>(static_cast<T*>(t.max_out) + p), (unsigned long long)__double_as_longlong((double)local_max));
    }
  }
}

// Register-tiled float32 cost blocks for the common point dimensions: a CTA
// computes 64 rows x 128 columns of one problem, both point tiles staged in
// shared memory dimension-major; each thread owns 8 rows x (2 + 2) columns --
// columns 2l, 2l+1 and 64+2l, 64+2l+1 for lane l -- so each 8-byte store of a
// warp covers 256 contiguous bytes.  Same arithmetic as the kernel above:
// sum_k (x_k - y_k)^2 in order of k, +inf padding.  The tile is sized for
// occupancy: at 32 accumulators a thread fits four CTAs per SM, which hide
// one another's point staging (64 x 256 tiles with 64 accumulators, two CTAs
// per SM: 6.0 ms for 1024 blocks of 2048 x 2048 at d = 16; this shape 4.7 ms,
// bit-identical).
// grid = (column-tile stride, row tiles, problems).
constexpr int SQ_R = 64, SQ_C = 128, SQ_CSTRIDE = 16;
// shared-memory row strides of the staged tiles: +4 floats keeps 16-byte
// alignment and spreads the transposing stores over the banks
constexpr int SQ_RP = SQ_R + 4, SQ_CP = SQ_C + 4;

template <int D>
__device__ __forceinline__ void sqdist_regtile(const float* __restrict__ X, const float* __restrict__ Y, int n, int m,
                                               int ldm, float* __restrict__ M, int r0, float* xt, float* yt,
                                               float& local_max) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // D a multiple of 4: rows of X and Y are 16-byte aligned (the packed clouds
  // start at multiples of D elements), so points are staged as float4 loads
  constexpr bool V4 = D % 4 == 0;
  if constexpr (V4) {
    for (int e = threadIdx.x; e < SQ_R * D / 4; e += blockDim.x) {
      const int r = e / (D / 4), k = (e % (D / 4)) * 4;
      const float4 v = (r0 + r < n) ? *reinterpret_cast<const float4*>(X + (int64_t)(r0 + r) * D + k)
                                    : make_float4(0.f, 0.f, 0.f, 0.f);
      xt[k * SQ_RP + r] = v.x; xt[(k + 1) * SQ_RP + r] = v.y;
      xt[(k + 2) * SQ_RP + r] = v.z; xt[(k + 3) * SQ_RP + r] = v.w;
    }
  } else {
    for (int e = threadIdx.x; e < SQ_R * D; e += blockDim.x) {
      const int r = e / D, k = e % D;
      xt[k * SQ_RP + r] = (r0 + r < n) ? X[(int64_t)(r0 + r) * D + k] : 0.f;
    }
  }
  for (int c0 = blockIdx.x * SQ_C; c0 < ldm; c0 += gridDim.x * SQ_C) {
    __syncthreads();  // previous tile's reads of yt are done (and xt is staged)
    if constexpr (V4) {
      for (int e = threadIdx.x; e < SQ_C * D / 4; e += blockDim.x) {
        const int c = e / (D / 4), k = (e % (D / 4)) * 4;
        const float4 v = (c0 + c < m) ? *reinterpret_cast<const float4*>(Y + (int64_t)(c0 + c) * D + k)
                                      : make_float4(0.f, 0.f, 0.f, 0.f);
        yt[k * SQ_CP + c] = v.x; yt[(k + 1) * SQ_CP + c] = v.y;
        yt[(k + 2) * SQ_CP + c] = v.z; yt[(k + 3) * SQ_CP + c] = v.w;
      }
    } else {
      for (int e = threadIdx.x; e < SQ_C * D; e += blockDim.x) {
        const int c = e / D, k = e % D;
        yt[k * SQ_CP + c] = (c0 + c < m) ? Y[(int64_t)(c0 + c) * D + k] : 0.f;
      }
    }
    __syncthreads();
    // column pairs (j, j+1) in packed fp32x2 registers: one sub.f32x2 and one
    // fma.f32x2 per pair and dimension, each lane rounding as the scalar ops
    unsigned long long acc2[8][2];
#pragma unroll
    for (int i = 0; i < 8; ++i) acc2[i][0] = acc2[i][1] = 0ull;
#pragma unroll
    for (int k = 0; k < D; ++k) {
      const float4 xa = *reinterpret_cast<const float4*>(xt + k * SQ_RP + warp * 8);
      const float4 xb = *reinterpret_cast<const float4*>(xt + k * SQ_RP + warp * 8 + 4);
      const unsigned long long yp[2] = {*reinterpret_cast<const unsigned long long*>(yt + k * SQ_CP + lane * 2),
                                        *reinterpret_cast<const unsigned long long*>(yt + k * SQ_CP + SQ_C / 2 +
                                                                                     lane * 2)};
      const float xv[8] = {xa.x, xa.y, xa.z, xa.w, xb.x, xb.y, xb.z, xb.w};
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const unsigned long long xx =
            (unsigned long long)__float_as_uint(xv[i]) | ((unsigned long long)__float_as_uint(xv[i]) << 32);
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          unsigned long long df;
          asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(df) : "l"(xx), "l"(yp[j]));
          asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(acc2[i][j]) : "l"(df));
        }
      }
    }
    // columns of acc2[i][0]: ca, ca + 1; of acc2[i][1]: cz, cz + 1 (ldm is a
    // multiple of 4, so a pair starting below ldm ends within it)
    const int ca = c0 + lane * 2, cz = c0 + SQ_C / 2 + lane * 2;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const int row = r0 + warp * 8 + i;
      if (row >= n) break;
      float v[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const float x = __uint_as_float((unsigned)(j & 1 ? acc2[i][j >> 1] >> 32 : acc2[i][j >> 1] & 0xffffffffull));
        const int col = (j < 2 ? ca : cz) + (j & 1);
        if (col < m) { v[j] = x; local_max = fmaxf(local_max, x); }
        else v[j] = INFINITY;
      }
      float* dst = M + (int64_t)row * ldm;
      if (ca < ldm) *reinterpret_cast<float2*>(dst + ca) = make_float2(v[0], v[1]);
      if (cz < ldm) *reinterpret_cast<float2*>(dst + cz) = make_float2(v[2], v[3]);
    }
  }
}

__global__ void __launch_bounds__(256, 4) sqdist_regtile_kernel(OtgCostTable t) {
  extern __shared__ __align__(16) float sq_smem[];
  const int p = blockIdx.z;
  if (p >= t.nprob) return;
  const int n = t.rows[p], m = t.cols[p], d = t.dim[p], ldm = t.ldm[p];
  const int r0 = blockIdx.y * SQ_R;
  if (r0 >= n || (int)blockIdx.x * SQ_C >= ldm) return;  // no tile of this problem for this CTA
  const float* X = static_cast<const float*>(t.X) + t.x_off[p];
  const float* Y = static_cast<const float*>(t.Y) + t.y_off[p];
  float* M = static_cast<float*>(t.M) + t.m_off[p];
  float* xt = sq_smem;
  float* yt = sq_smem + SQ_RP * t.max_dim;
  float local_max = 0.f;
  if (d == 16) sqdist_regtile<16>(X, Y, n, m, ldm, M, r0, xt, yt, local_max);
  else if (d == 8) sqdist_regtile<8>(X, Y, n, m, ldm, M, r0, xt, yt, local_max);
  else if (d == 3) sqdist_regtile<3>(X, Y, n, m, ldm, M, r0, xt, yt, local_max);
  else if (d == 2) sqdist_regtile<2>(X, Y, n, m, ldm, M, r0, xt, yt, local_max);
  if (t.max_out) {
    local_max = warp_max(local_max);
    if ((threadIdx.x & 31) == 0)
      atomicMax(reinterpret_cast<unsigned int*>(static_cast<float*>(t.max_out) + p), __float_as_uint(local_max));
  }
}

// Batched transpose through 32 x 32 shared-memory tiles: dst[b][j][i] =
// src[b][i][j] for i < n, j < m, and +inf in the padding columns i in
// [n, ld_dst) of every destination row (they add nothing to any LSE).
// grid = (column tiles of the source, tiles over ld_dst, batch).
template <typename T>
__global__ void __launch_bounds__(256) transpose_batched_kernel(const T* __restrict__ src, int64_t n, int64_t m,
                                                                int64_t ld_src, int64_t bs_src, T* __restrict__ dst,
                                                                int64_t ld_dst, int64_t bs_dst) {
  __shared__ T tile[32][33];
  const int64_t b = blockIdx.z;
  const int64_t j0 = (int64_t)blockIdx.x * 32, i0 = (int64_t)blockIdx.y * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  const T* S = src + b * bs_src;
  T* D = dst + b * bs_dst;
  for (int r = ty; r < 32; r += 8) {
    const int64_t i = i0 + r, j = j0 + tx;
    tile[r][tx] = (i < n && j < m) ? S[i * ld_src + j] : T(INFINITY);
  }
  __syncthreads();
  for (int r = ty; r < 32; r += 8) {
    const int64_t j = j0 + r, i = i0 + tx;
    if (j < m && i < ld_dst) D[j * ld_dst + i] = tile[tx][r];
  }
}

// Plan and values per problem.  grid = (row tiles, problems).
// out_vals[3p+0] = value_linear, [3p+1] = sum T log(T+1e-16) (entropy form)
// or sum T log(T/(a b) + 1e-16) (KL form), [3p+2] = sum T.
template <typename T, int METHOD>
__global__ void __launch_bounds__(256) batched_plan_kernel(OtgPlanTable t) {
  const int p = blockIdx.y;
  if (p >= t.nprob) return;
  const int n = t.rows[p], m = t.cols[p], ldm = t.ldm[p];
  const T* M = static_cast<const T*>(t.M) + t.m_off[p];
  const T* u = static_cast<const T*>(t.u) + t.r_off[p];
  const T* v = static_cast<const T*>(t.v) + t.c_off[p];
  const T* a = static_cast<const T*>(t.a) + t.r_off[p];
  const T* b = static_cast<const T*>(t.b) + t.c_off[p];
  T* P = t.P ? static_cast<T*>(t.P) + t.m_off[p] : nullptr;
  const T c = (T)(-OTG_LOG2E / t.reg[p]);
  const T L2E = T(OTG_LOG2E);
  // sums in the working type within a row, in fp64 across rows: float
  // inputs keep their logarithms in fp32 (GB300's fp64 rate is a small
  // fraction of fp32; a per-element fp64 log made this kernel the batch
  // path's bottleneck), double inputs stay in fp64 throughout
  double lin = 0, reg_term = 0, mass = 0;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const T ui = u[i];
    const T ai = a[i];
    T lr = 0, rr = 0, mr = 0;
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      const T x = M[(int64_t)i * ldm + j];
      T pij;
      if (METHOD == OTG_METHOD_LOG) pij = ex2(fma(x, c, (ui + v[j]) * L2E));
      else pij = ui * ex2(x * c) * v[j];
      if (P) P[(int64_t)i * ldm + j] = pij;
      lr = fma(x, pij, lr);
      mr += pij;
      if (t.kl) rr = fma(pij, log(pij / (ai * b[j]) + T(1e-16)), rr);
      else rr = fma(pij, log(pij + T(1e-16)), rr);
    }
    lin += (double)lr;
    mass += (double)mr;
    reg_term += (double)rr;
  }
  __shared__ double red[3][8];
  lin = warp_sum(lin); reg_term = warp_sum(reg_term); mass = warp_sum(mass);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { red[0][w] = lin; red[1][w] = reg_term; red[2][w] = mass; }
  __syncthreads();
  if (threadIdx.x < 3) {
    double s = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[threadIdx.x][k];
    atomicAdd(t.out_vals + 3 * p + threadIdx.x, s);
  }
}

// Soft-min distances of every source point to the target measure at several
// temperatures, in units of the problem's cost scale:
//   out[r_off[p] + i, k] = -tau_k * ln sum_j b_j exp(g_j - M_ij / (scale_p tau_k)).
// With g = 0 these are c-transforms of the zero potential; with g the
// (natural-log) target potential of a solved problem on the same target
// points and tau = reg/scale, it is that potential's c-transform, i.e. the
// log-domain row update.  One warp per row, all temperatures in one pass.
constexpr int SM_MAXTAU = 8;
__global__ void __launch_bounds__(256) softmin_features_kernel(const float* __restrict__ Mall, const int64_t* m_off,
                                                               const int32_t* rows, const int32_t* cols,
                                                               const int32_t* ldms, const int64_t* r_off,
                                                               const int64_t* c_off, const float* __restrict__ ball,
                                                               const float* scale, const float* taus, int ntau,
                                                               int nprob, const float* __restrict__ gall,
                                                               float* out) {
  const int p = blockIdx.y;
  if (p >= nprob) return;
  const int n = rows[p], m = cols[p], ldm = ldms[p];
  const int lane = threadIdx.x & 31;
  const int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (row >= n) return;
  const float* Mrow = Mall + m_off[p] + (int64_t)row * ldm;
  const float* b = ball + c_off[p];
  const float* g = gall ? gall + c_off[p] : nullptr;
  float ck[SM_MAXTAU], mx[SM_MAXTAU], s[SM_MAXTAU];
#pragma unroll
  for (int k = 0; k < SM_MAXTAU; ++k) {
    ck[k] = k < ntau ? -(float)OTG_LOG2E / (scale[p] * taus[k]) : 0.f;
    mx[k] = -INFINITY;
    s[k] = 0.f;
  }
  for (int j = lane; j < m; j += 32) {
    const float x = Mrow[j];
    const float lb = lg2(b[j]) + (g ? g[j] * (float)OTG_LOG2E : 0.f);
#pragma unroll
    for (int k = 0; k < SM_MAXTAU; ++k) {
      if (k < ntau) {
        const float t = fmaf(x, ck[k], lb);
        const float nm = fmaxf(mx[k], t);
        s[k] = s[k] * ex2(mx[k] - nm) + ex2(t - nm);
        mx[k] = nm;
      }
    }
  }
#pragma unroll
  for (int k = 0; k < SM_MAXTAU; ++k) {
    if (k < ntau) {
      warp_lse(mx[k], s[k]);
      if (lane == 0) out[(r_off[p] + row) * ntau + k] = -taus[k] * (float)OTG_LN2 * lse_value(mx[k], s[k]);
    }
  }
}

// Soft-min of every source point over the k weighted atoms of its pair, the
// squared distances computed on the fly (no cost block): one thread per
// point, the pair's atoms in shared memory.  One sweep over the atoms in
// chunks of SP_CHUNK: the chunk's distances, then per temperature one
// rescale of the running (max, sum) to the chunk's max and the chunk's
// exponentials (1 + 1/SP_CHUNK exponentials and one distance per term).
// Slot 0 of the result is the c-transform of the atoms' potential g at
// temperature g_tau (if g is given), slots 1.. the soft-mins of the zero
// potential at taus[]; all in units of scale[p], as softmin_features_kernel
// computes them from a cost block.  NT: the temperature slots handled (1:
// slot 0 only).  Every thread reads the same atom at the same time
// (broadcast), so the atoms are stored densely and read as float4 when D is
// a multiple of 4.
constexpr int SP_CHUNK = 8;
constexpr int SP_PTS_PRIOR = 2;  // points per thread of the c-transform-only form

template <int D, int NT, int PTS>
__global__ void __launch_bounds__(256) softmin_points_kernel(const float* __restrict__ X, const float* __restrict__ C,
                                                             int n, int k, int64_t sx, int64_t sc,
                                                             const float* __restrict__ bw,
                                                             const float* __restrict__ gw, float g_tau,
                                                             const float* __restrict__ scale,
                                                             const float* __restrict__ taus, int ntau,
                                                             float* __restrict__ out_f, float* __restrict__ out_F) {
  extern __shared__ __align__(16) float sp_smem[];
  const int p = blockIdx.y;
  float* cs = sp_smem;                         // [k][D]
  float* lb = cs + (size_t)k * D;              // log2 b
  float* lg = lb + k;                          // log2 b + g log2 e
  const float* Cp = C + p * sc;
  for (int e = threadIdx.x; e < k * D; e += blockDim.x) cs[e] = Cp[e];
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    const float l = lg2(bw[(int64_t)p * k + c]);
    lb[c] = l;
    lg[c] = gw ? l + gw[(int64_t)p * k + c] * (float)OTG_LOG2E : l;
  }
  __syncthreads();
  // points i0 + r * blockDim.x, r < PTS: every atom read from shared memory
  // serves all of them
  const int i0 = blockIdx.x * blockDim.x * PTS + threadIdx.x;
  if (i0 >= n) return;
  float x[PTS][D];
#pragma unroll
  for (int r = 0; r < PTS; ++r) {
    const int i = min(i0 + r * (int)blockDim.x, n - 1);
#pragma unroll
    for (int q = 0; q < D; ++q) x[r][q] = X[p * sx + (int64_t)i * D + q];
  }
  const int nt = NT == 1 ? 1 : ntau + 1;       // slot 0: the c-transform of g
  float ck[NT], mx[PTS][NT], s[PTS][NT];
#pragma unroll
  for (int t = 0; t < NT; ++t) {
    const float tau = t == 0 ? g_tau : (t <= ntau ? taus[t - 1] : 1.f);
    ck[t] = -(float)OTG_LOG2E / (scale[p] * tau);
#pragma unroll
    for (int r = 0; r < PTS; ++r) { mx[r][t] = -INFINITY; s[r][t] = 0.f; }
  }
  for (int c0 = 0; c0 < k; c0 += SP_CHUNK) {
    float d2[PTS][SP_CHUNK];
#pragma unroll
    for (int j = 0; j < SP_CHUNK; ++j) {
      const int c = min(c0 + j, k - 1);
      const float* y = cs + c * D;
#pragma unroll
      for (int r = 0; r < PTS; ++r) d2[r][j] = 0.f;
      if (D % 4 == 0) {
#pragma unroll
        for (int q = 0; q < D; q += 4) {
          const float4 w = *reinterpret_cast<const float4*>(y + q);
#pragma unroll
          for (int r = 0; r < PTS; ++r) {
            float df = x[r][q] - w.x; d2[r][j] = fmaf(df, df, d2[r][j]);
            df = x[r][q + 1] - w.y; d2[r][j] = fmaf(df, df, d2[r][j]);
            df = x[r][q + 2] - w.z; d2[r][j] = fmaf(df, df, d2[r][j]);
            df = x[r][q + 3] - w.w; d2[r][j] = fmaf(df, df, d2[r][j]);
          }
        }
      } else {
#pragma unroll
        for (int q = 0; q < D; ++q) {
          const float yq = y[q];
#pragma unroll
          for (int r = 0; r < PTS; ++r) { const float df = x[r][q] - yq; d2[r][j] = fmaf(df, df, d2[r][j]); }
        }
      }
    }
#pragma unroll
    for (int t = 0; t < NT; ++t) {
      if (NT > 1 && t >= nt) break;
      const float* l = t == 0 ? lg : lb;
      float lc[SP_CHUNK];
#pragma unroll
      for (int j = 0; j < SP_CHUNK; ++j) lc[j] = c0 + j < k ? l[c0 + j] : -INFINITY;
#pragma unroll
      for (int r = 0; r < PTS; ++r) {
        float v[SP_CHUNK];
        float cm = -INFINITY;
#pragma unroll
        for (int j = 0; j < SP_CHUNK; ++j) {
          v[j] = fmaf(d2[r][j], ck[t], lc[j]);
          cm = fmaxf(cm, v[j]);
        }
        const float nm = fmaxf(mx[r][t], cm);
        if (nm > -INFINITY) {  // (atoms of zero mass add nothing)
          float acc = s[r][t] * ex2(mx[r][t] - nm);
#pragma unroll
          for (int j = 0; j < SP_CHUNK; ++j) acc += ex2(v[j] - nm);
          s[r][t] = acc;
          mx[r][t] = nm;
        }
      }
    }
  }
#pragma unroll
  for (int r = 0; r < PTS; ++r) {
    const int i = i0 + r * (int)blockDim.x;
    if (i >= n) break;
    const int64_t row = (int64_t)p * n + i;
    if (out_f) out_f[row] = -g_tau * (float)OTG_LN2 * lse_value(mx[r][0], s[r][0]);
#pragma unroll
    for (int t = 1; t < NT; ++t)
      if (t < nt) out_F[row * ntau + (t - 1)] = -taus[t - 1] * (float)OTG_LN2 * lse_value(mx[r][t], s[r][t]);
  }
}

// Voronoi cell masses: for every point of cloud p (n points, rows of X), the
// nearest of its k centres (the first k points of the paired centre cloud)
// gains weight 1/n.  Centres and their squared norms are staged in shared
// memory; each thread ranks the centres for NM_PTS points (every centre read
// from shared memory serves them all) by |c|^2 - 2 x.c (|x - c|^2 less the
// point's own |x|^2: one FMA per coordinate; the first of equal values wins).
constexpr int NM_PTS = 2;

template <int D>
__global__ void __launch_bounds__(256) nearest_mass_kernel(const float* __restrict__ X, const float* __restrict__ Cc,
                                                           int n, int k, int64_t sx, int64_t sc, float* w) {
  extern __shared__ __align__(16) float cs[];
  float* cn = cs + (size_t)k * D;  // [k] squared norms
  const int p = blockIdx.y;
  const float* C = Cc + p * sc;
  for (int e = threadIdx.x; e < k * D; e += blockDim.x) cs[e] = C[e];
  __syncthreads();
  for (int c = threadIdx.x; c < k; c += blockDim.x) {
    float q2 = 0.f;
    for (int q = 0; q < D; ++q) q2 = fmaf(cs[c * D + q], cs[c * D + q], q2);
    cn[c] = q2;
  }
  __syncthreads();
  // points i0 + r * blockDim.x, r < NM_PTS (coalesced rows of X per r)
  const int i0 = blockIdx.x * blockDim.x * NM_PTS + threadIdx.x;
  float x[NM_PTS][D];
#pragma unroll
  for (int r = 0; r < NM_PTS; ++r) {
    const int i = min(i0 + r * (int)blockDim.x, n - 1);
#pragma unroll
    for (int q = 0; q < D; ++q) x[r][q] = -2.f * X[p * sx + (int64_t)i * D + q];
  }
  float best[NM_PTS];
  int arg[NM_PTS];
#pragma unroll
  for (int r = 0; r < NM_PTS; ++r) { best[r] = INFINITY; arg[r] = 0; }
  for (int c = 0; c < k; ++c) {
    float v[NM_PTS];
#pragma unroll
    for (int r = 0; r < NM_PTS; ++r) v[r] = cn[c];
    if (D % 4 == 0) {  // every thread reads centre c: broadcast float4 loads
#pragma unroll
      for (int q = 0; q < D; q += 4) {
        const float4 y = *reinterpret_cast<const float4*>(cs + c * D + q);
#pragma unroll
        for (int r = 0; r < NM_PTS; ++r) {
          v[r] = fmaf(x[r][q], y.x, v[r]);
          v[r] = fmaf(x[r][q + 1], y.y, v[r]);
          v[r] = fmaf(x[r][q + 2], y.z, v[r]);
          v[r] = fmaf(x[r][q + 3], y.w, v[r]);
        }
      }
    } else {
#pragma unroll
      for (int q = 0; q < D; ++q) {
        const float y = cs[c * D + q];
#pragma unroll
        for (int r = 0; r < NM_PTS; ++r) v[r] = fmaf(x[r][q], y, v[r]);
      }
    }
#pragma unroll
    for (int r = 0; r < NM_PTS; ++r)
      if (v[r] < best[r]) { best[r] = v[r]; arg[r] = c; }
  }
#pragma unroll
  for (int r = 0; r < NM_PTS; ++r)
    if (i0 + r * (int)blockDim.x < n) atomicAdd(w + (int64_t)p * k + arg[r], 1.0f / (float)n);
}

// Loss of a lazy plan: sum_ij C_ij exp(f_i + g_j - C_ij / reg) with C the
// squared distance of points x_i, y_j (natural-log potentials f, g), the
// value ot/bregman/_empirical.py:470-478 accumulates block by block.  One CTA
// per tile of LL_ROWS points (staged in shared memory); each thread walks
// columns; fp64 accumulation, one atomic per CTA.
constexpr int LL_ROWS = 16;

template <typename T>
__global__ void __launch_bounds__(256) lazy_loss_kernel(const T* __restrict__ X, const T* __restrict__ Y, int64_t n,
                                                        int64_t m, int d, const T* __restrict__ f,
                                                        const T* __restrict__ g, T c, double* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char ll_raw[];
  T* xs = reinterpret_cast<T*>(ll_raw);
  T* fs = xs + LL_ROWS * d;
  const int64_t r0 = (int64_t)blockIdx.x * LL_ROWS;
  const int rows = (n - r0) < LL_ROWS ? (int)(n - r0) : LL_ROWS;
  const T L2E = T(OTG_LOG2E);
  for (int e = threadIdx.x; e < rows * d; e += blockDim.x) xs[e] = X[r0 * d + e];
  for (int r = threadIdx.x; r < rows; r += blockDim.x) fs[r] = f[r0 + r] * L2E;
  __syncthreads();
  double acc = 0.0;
  for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
    const T* y = Y + j * d;
    const T gj = g[j] * L2E;
    for (int r = 0; r < rows; ++r) {
      const T* x = xs + r * d;
      T cij = 0;
      for (int k = 0; k < d; ++k) { const T df = x[k] - y[k]; cij = fma(df, df, cij); }
      acc += (double)cij * (double)ex2(fma(cij, c, fs[r] + gj));
    }
  }
  __shared__ double red[8];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    atomicAdd(out, t);
  }
}

}  // namespace otg

using namespace otg;

extern "C" {

int otg_batched_sqdist(const OtgCostTable* t, int32_t max_rows, cudaStream_t stream) {
  if (!t || !t->X || !t->Y || !t->M || !t->rows || !t->cols || !t->dim || !t->ldm || !t->x_off || !t->y_off ||
      !t->m_off || t->nprob < 1 || max_rows < 1 || t->max_dim < 1)
    return OTG_ERR_ARG;
  if (t->nprob > 65535) return OTG_ERR_UNSUPPORTED;
  if (t->fixed_dim && t->fixed_dim != 2 && t->fixed_dim != 3 && t->fixed_dim != 8 && t->fixed_dim != 16)
    return OTG_ERR_ARG;
  if (t->fixed_dim && t->fixed_dim != t->max_dim) return OTG_ERR_ARG;
  dim3 grid((max_rows + 31) / 32, t->nprob);
  if (t->max_out) {
    size_t es = t->dtype == OTG_F64 ? 8 : 4;
    if (cudaMemsetAsync(t->max_out, 0, es * t->nprob, stream) != cudaSuccess) return OTG_ERR_CUDA;
  }
  if (t->dtype == OTG_F64) {
    batched_sqdist_kernel<double><<<grid, 256, 32 * t->max_dim * sizeof(double), stream>>>(*t);
  } else if (t->dtype == OTG_F32 && t->fixed_dim &&
             (t->fixed_dim % 4 != 0 || ((uintptr_t)t->X % 16 == 0 && (uintptr_t)t->Y % 16 == 0))) {
    // every problem has the same dimension, one of 2, 3, 8, 16: register tiles
    const dim3 g2(SQ_CSTRIDE, (unsigned)((max_rows + SQ_R - 1) / SQ_R), (unsigned)t->nprob);
    sqdist_regtile_kernel<<<g2, 256, (SQ_RP + SQ_CP) * t->max_dim * sizeof(float), stream>>>(*t);
  } else if (t->dtype == OTG_F32) {
    batched_sqdist_kernel<float><<<grid, 256, 32 * t->max_dim * sizeof(float), stream>>>(*t);
  } else {
    return OTG_ERR_DTYPE;
  }
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_batched_plan(const OtgPlanTable* t, int32_t max_rows, cudaStream_t stream) {
  if (!t || !t->M || !t->u || !t->v || !t->a || !t->b || !t->reg || !t->out_vals || t->nprob < 1 || max_rows < 1)
    return OTG_ERR_ARG;
  if (t->nprob > 65535) return OTG_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(t->out_vals, 0, 3 * sizeof(double) * t->nprob, stream) != cudaSuccess) return OTG_ERR_CUDA;
  dim3 grid(std::min(max_rows, 64), t->nprob);
  if (t->dtype == OTG_F64) {
    if (t->method == OTG_METHOD_LOG) batched_plan_kernel<double, OTG_METHOD_LOG><<<grid, 256, 0, stream>>>(*t);
    else batched_plan_kernel<double, OTG_METHOD_KNOPP><<<grid, 256, 0, stream>>>(*t);
  } else if (t->dtype == OTG_F32) {
    if (t->method == OTG_METHOD_LOG) batched_plan_kernel<float, OTG_METHOD_LOG><<<grid, 256, 0, stream>>>(*t);
    else batched_plan_kernel<float, OTG_METHOD_KNOPP><<<grid, 256, 0, stream>>>(*t);
  } else {
    return OTG_ERR_DTYPE;
  }
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_nearest_mass(const float* X, const float* C, int32_t nprob, int32_t n, int32_t k, int32_t d, int64_t sx,
                     int64_t sc, float* w, cudaStream_t stream) {
  if (!X || !C || !w || nprob < 1 || nprob > 65535 || n < 1 || k < 1) return OTG_ERR_ARG;
  if (cudaMemsetAsync(w, 0, sizeof(float) * (size_t)nprob * k, stream) != cudaSuccess) return OTG_ERR_CUDA;
  dim3 grid((unsigned)((n + 256 * NM_PTS - 1) / (256 * NM_PTS)), (unsigned)nprob);
  const size_t sm = sizeof(float) * ((size_t)k * d + (size_t)k);
  if (sm > 48 * 1024) return OTG_ERR_UNSUPPORTED;
  if (d == 16) nearest_mass_kernel<16><<<grid, 256, sm, stream>>>(X, C, n, k, sx, sc, w);
  else if (d == 8) nearest_mass_kernel<8><<<grid, 256, sm, stream>>>(X, C, n, k, sx, sc, w);
  else if (d == 3) nearest_mass_kernel<3><<<grid, 256, sm, stream>>>(X, C, n, k, sx, sc, w);
  else if (d == 2) nearest_mass_kernel<2><<<grid, 256, sm, stream>>>(X, C, n, k, sx, sc, w);
  else return OTG_ERR_UNSUPPORTED;
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_softmin_points(const float* X, const float* C, int32_t nprob, int32_t n, int32_t k, int32_t d, int64_t sx,
                       int64_t sc, const float* b, const float* g, float g_tau, const float* scale,
                       const float* taus, int32_t ntau, float* out_f, float* out_F, cudaStream_t stream) {
  if (!X || !C || !b || !scale || nprob < 1 || nprob > 65535 || n < 1 || k < 1) return OTG_ERR_ARG;
  if (ntau < 0 || ntau > SM_MAXTAU || (ntau > 0 && (!taus || !out_F)) || (!out_f && ntau == 0)) return OTG_ERR_ARG;
  if (out_f && !(g_tau > 0)) return OTG_ERR_ARG;
  const size_t sm = sizeof(float) * ((size_t)k * d + 2 * (size_t)k);
  if (sm > 48 * 1024) return OTG_ERR_UNSUPPORTED;
  const int pts = ntau == 0 ? SP_PTS_PRIOR : 1;  // points per thread
  dim3 grid((unsigned)((n + 256 * pts - 1) / (256 * pts)), (unsigned)nprob);
  const float gt = out_f ? g_tau : 1.f;
#define OTG_SOFTMIN_POINTS(DD)                                                                                     \
  if (ntau == 0)                                                                                                   \
    softmin_points_kernel<DD, 1, SP_PTS_PRIOR><<<grid, 256, sm, stream>>>(X, C, n, k, sx, sc, b, g, gt, scale, taus,  \
                                                                          ntau, out_f, out_F);                      \
  else                                                                                                             \
    softmin_points_kernel<DD, SM_MAXTAU + 1, 1><<<grid, 256, sm, stream>>>(X, C, n, k, sx, sc, b, g, gt, scale,     \
                                                                           taus, ntau, out_f, out_F)
  if (d == 16) OTG_SOFTMIN_POINTS(16);
  else if (d == 8) OTG_SOFTMIN_POINTS(8);
  else if (d == 3) OTG_SOFTMIN_POINTS(3);
  else if (d == 2) OTG_SOFTMIN_POINTS(2);
  else return OTG_ERR_UNSUPPORTED;
#undef OTG_SOFTMIN_POINTS
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_softmin_features(const float* M, const int64_t* m_off, const int32_t* rows, const int32_t* cols,
                         const int32_t* ldm, const int64_t* r_off, const int64_t* c_off, const float* b,
                         const float* scale, const float* taus, int32_t ntau, int32_t nprob, int32_t max_rows,
                         const float* g, float* out, cudaStream_t stream) {
  if (!M || !m_off || !rows || !cols || !ldm || !r_off || !c_off || !b || !scale || !taus || !out) return OTG_ERR_ARG;
  if (ntau < 1 || ntau > SM_MAXTAU || nprob < 1 || nprob > 65535 || max_rows < 1) return OTG_ERR_ARG;
  dim3 grid((unsigned)((max_rows + 7) / 8), (unsigned)nprob);
  softmin_features_kernel<<<grid, 256, 0, stream>>>(M, m_off, rows, cols, ldm, r_off, c_off, b, scale, taus, ntau,
                                                    nprob, g, out);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_lazy_loss(int dtype, const void* X, const void* Y, int64_t n, int64_t m, int32_t d, const void* f,
                  const void* g, double reg, double* out, cudaStream_t stream) {
  if (!X || !Y || !f || !g || !out || n < 1 || m < 1 || d < 1 || !(reg > 0)) return OTG_ERR_ARG;
  const size_t esz = dtype == OTG_F64 ? 8 : 4;
  const size_t smem = esz * (size_t)LL_ROWS * (size_t)(d + 1);
  if (smem > 96 * 1024) return OTG_ERR_UNSUPPORTED;
  if (cudaMemsetAsync(out, 0, sizeof(double), stream) != cudaSuccess) return OTG_ERR_CUDA;
  const unsigned blocks = (unsigned)((n + LL_ROWS - 1) / LL_ROWS);
  const double c = -OTG_LOG2E / reg;
  if (dtype == OTG_F64) {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(lazy_loss_kernel<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return OTG_ERR_CUDA;
    lazy_loss_kernel<double><<<blocks, 256, smem, stream>>>((const double*)X, (const double*)Y, n, m, d,
                                                            (const double*)f, (const double*)g, c, out);
  } else if (dtype == OTG_F32) {
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(lazy_loss_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
      return OTG_ERR_CUDA;
    lazy_loss_kernel<float><<<blocks, 256, smem, stream>>>((const float*)X, (const float*)Y, n, m, d,
                                                           (const float*)f, (const float*)g, (float)c, out);
  } else {
    return OTG_ERR_DTYPE;
  }
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_transpose_batched(int dtype, const void* src, int64_t batch, int64_t n, int64_t m, int64_t ld_src,
                          int64_t bs_src, void* dst, int64_t ld_dst, int64_t bs_dst, cudaStream_t stream) {
  if (!src || !dst || batch < 1 || n < 1 || m < 1 || ld_src < m || ld_dst < n || bs_src < n * ld_src ||
      bs_dst < m * ld_dst || batch > 65535)
    return OTG_ERR_ARG;
  const dim3 grid((unsigned)((m + 31) / 32), (unsigned)((ld_dst + 31) / 32), (unsigned)batch);
  if (dtype == OTG_F64)
    transpose_batched_kernel<double><<<grid, 256, 0, stream>>>((const double*)src, n, m, ld_src, bs_src, (double*)dst,
                                                               ld_dst, bs_dst);
  else if (dtype == OTG_F32)
    transpose_batched_kernel<float><<<grid, 256, 0, stream>>>((const float*)src, n, m, ld_src, bs_src, (float*)dst,
                                                              ld_dst, bs_dst);
  else
    return OTG_ERR_DTYPE;
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

}  // extern "C"
