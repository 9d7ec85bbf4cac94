// Greenkhorn: greedy coordinate Sinkhorn on one dense problem
// (ot/bregman/_sinkhorn.py:921-1102, `greenkhorn`, reached through
// ot.sinkhorn(method='greenkhorn'), :192-204).
//
// Each step rescales the ONE row or column whose marginal is furthest from
// its target, so the method is a chain of small dependent steps: a step reads
// one row of K (a column comes from a transposed copy, so it is a contiguous
// read too), updates one violation vector, and ends with an argmax over both
// vectors.  The chain runs in one persistent CTA of GK_THREADS threads, with
// u, v and both violation vectors in shared memory when they fit (global
// memory otherwise): no grid-wide barrier and no host round trip per step;
// the host reads the step count once at the end.
//
// GB300 issues FP64 at a few lanes per clock per SM, and FP64 issue bounds
// the chain, so it keeps FP64 work per entry to three operations: the dot
// product of the rescaled line (one fused multiply-add) and the violation
// update (a rounded product, then a fused multiply-add; the reference rounds
// both products, a difference in the last place, as is the order of its BLAS
// dot products).  The argmax runs on integer keys (the bit pattern of |x|
// orders non-negative floats, and NaN patterns sit above +inf, as numpy's
// argmax ranks NaN first), as do the row/column choice and the stop test;
// each sum is one partial per thread folded by a single warp; the division
// of a rescaling is done once, by one thread, and broadcast.
//
// Reductions run in a fixed order (per-thread sequential partial, then warp 0
// folds the partials in slot order and by xor butterfly), so two runs are
// bit-identical.  Argmax ties go to the lowest index.
#include <algorithm>
#include <climits>
#include <cstdint>

#include "common.cuh"
#include "pot_gb300.h"

namespace {

using otg::warp_sum;

constexpr int GK_THREADS = 256;
constexpr int GK_WARPS = GK_THREADS / 32;
// u, v, viol, viol_2 go to shared memory up to this many bytes
constexpr size_t GK_SMEM_MAX = 192 * 1024;

__device__ __forceinline__ float mul_rn(float x, float y) { return __fmul_rn(x, y); }
__device__ __forceinline__ double mul_rn(double x, double y) { return __dmul_rn(x, y); }
__device__ __forceinline__ float add_rn(float x, float y) { return __fadd_rn(x, y); }
__device__ __forceinline__ double add_rn(double x, double y) { return __dadd_rn(x, y); }
__device__ __forceinline__ float sub_rn(float x, float y) { return __fsub_rn(x, y); }
__device__ __forceinline__ double sub_rn(double x, double y) { return __dsub_rn(x, y); }

// Order key of |x|: unsigned comparison of keys is numpy's argmax order on
// |x| (every NaN maps to one key above +inf's).
template <typename T>
struct GkKey;
template <>
struct GkKey<double> {
  static constexpr unsigned long long kInf = 0x7ff0000000000000ull;
  static __device__ __forceinline__ unsigned long long of(double x) {
    const unsigned long long k = (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffull;
    return k > kInf ? 0x7ff8000000000000ull : k;
  }
};
template <>
struct GkKey<float> {
  static constexpr unsigned long long kInf = 0x7f800000ull;
  static __device__ __forceinline__ unsigned long long of(float x) {
    const unsigned k = __float_as_uint(x) & 0x7fffffffu;
    return k > 0x7f800000u ? 0x7fc00000ull : (unsigned long long)k;
  }
};

struct GkArg {
  unsigned long long k;  // order key of |violation|
  int i;                 // its index; INT_MAX with key 0 for "no entry" (any entry wins the tie)
};

__device__ __forceinline__ GkArg gk_none() { return GkArg{0ull, INT_MAX}; }

__device__ __forceinline__ void gk_take(GkArg& best, unsigned long long k, int i) {
  if (k > best.k || (k == best.k && i < best.i)) {
    best.k = k;
    best.i = i;
  }
}

__device__ __forceinline__ void gk_warp_argmax(GkArg& x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, x.k, o);
    const int oi = __shfl_xor_sync(0xffffffffu, x.i, o);
    gk_take(x, ok, oi);
  }
}

template <typename T>
__device__ __forceinline__ GkArg gk_scan(const T* viol, int len) {
  GkArg best = gk_none();
  for (int i = threadIdx.x; i < len; i += GK_THREADS) gk_take(best, GkKey<T>::of(viol[i]), i);
  return best;
}

// Block state.  The argmax slots are double-buffered: block argmax k writes
// buffer k & 1; a thread reads argmax k-2's slots before it reaches the next
// barrier, which every thread passes before argmax k writes them again.
template <typename T>
struct GkShared {
  T part[GK_THREADS];  // one sum partial per thread
  T bc[4];             // values broadcast by thread 0
  unsigned long long k1[2][GK_WARPS], k2[2][GK_WARPS];
  int i1[2][GK_WARPS], i2[2][GK_WARPS];
};

// Fixed-order sum of the threads' partials into warp 0 (every lane of warp 0
// returns it; the other warps return 0 and must not use it).  The caller
// follows it with a barrier after warp 0 has published what it needs; that
// barrier also orders this fold's reads of `part` before the next fold's
// writes.
template <typename T>
__device__ __forceinline__ T gk_fold(GkShared<T>& sh, T x) {
  sh.part[threadIdx.x] = x;
  __syncthreads();
  T s = 0;
  if (threadIdx.x < 32) {
    s = sh.part[threadIdx.x];
#pragma unroll
    for (int k = 1; k < GK_WARPS; ++k) s += sh.part[threadIdx.x + 32 * k];
    s = warp_sum(s);
  }
  return s;
}

template <typename T>
__device__ __forceinline__ void gk_block_argmax(GkShared<T>& sh, GkArg& r1, GkArg& r2, int& buf) {
  gk_warp_argmax(r1);
  gk_warp_argmax(r2);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) {
    sh.k1[buf][w] = r1.k;
    sh.i1[buf][w] = r1.i;
    sh.k2[buf][w] = r2.k;
    sh.i2[buf][w] = r2.i;
  }
  __syncthreads();
  r1 = l < GK_WARPS ? GkArg{sh.k1[buf][l], sh.i1[buf][l]} : gk_none();
  r2 = l < GK_WARPS ? GkArg{sh.k2[buf][l], sh.i2[buf][l]} : gk_none();
  buf ^= 1;
  gk_warp_argmax(r1);
  gk_warp_argmax(r2);
}

// K = exp(-M / reg) (the reference's `nx.exp(-M / reg)`, :1042) and its
// transpose, through 32 x 32 shared-memory tiles so both writes coalesce.
template <typename T>
__global__ void __launch_bounds__(256) gk_gibbs_kernel(const T* __restrict__ M, int64_t n, int64_t m, int64_t ldm,
                                                       T reg, T* __restrict__ K, T* __restrict__ KT) {
  __shared__ T tile[32][33];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int64_t tm = (m + 31) / 32, tiles = ((n + 31) / 32) * tm;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    const int64_t i0 = (t / tm) * 32, j0 = (t % tm) * 32;
    for (int r = ty; r < 32; r += 8) {
      const int64_t i = i0 + r, j = j0 + tx;
      if (i < n && j < m) {
        const T k = exp(-M[i * ldm + j] / reg);
        K[i * m + j] = k;
        tile[r][tx] = k;
      }
    }
    __syncthreads();
    for (int r = ty; r < 32; r += 8) {
      const int64_t j = j0 + r, i = i0 + tx;
      if (i < n && j < m) KT[j * n + i] = tile[tx][r];
    }
    __syncthreads();
  }
}

// u, v = 1/n, 1/m, or exp of the warm-start potentials (:1044-1048).
template <typename T>
__global__ void gk_start_kernel(int64_t n, int64_t m, const T* __restrict__ wu, const T* __restrict__ wv,
                                T u0, T v0, T* __restrict__ u, T* __restrict__ v) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n + m; k += (int64_t)gridDim.x * blockDim.x) {
    if (k < n)
      u[k] = wu ? exp(wu[k]) : u0;
    else
      v[k - n] = wv ? exp(wv[k - n]) : v0;
  }
}

// viol = G 1 - a, viol_2 = G^T 1 - b with G_ij = (u_i K_ij) v_j (:1049-1052);
// one warp per row of K (lines 0 .. n-1) or of K^T (lines n .. n+m-1).
template <typename T>
__global__ void gk_viol_kernel(const T* __restrict__ K, const T* __restrict__ KT, int64_t n, int64_t m,
                               const T* __restrict__ a, const T* __restrict__ b, const T* __restrict__ u,
                               const T* __restrict__ v, T* __restrict__ viol, T* __restrict__ viol2) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t line = blockIdx.x * (int64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); line < n + m; line += warps) {
    T s = 0;
    if (line < n) {
      const T* row = K + line * m;
      const T ui = u[line];
      for (int64_t j = lane; j < m; j += 32) s = add_rn(s, mul_rn(mul_rn(ui, row[j]), v[j]));
      s = warp_sum(s);
      if (lane == 0) viol[line] = sub_rn(s, a[line]);
    } else {
      const int64_t j = line - n;
      const T* col = KT + j * n;
      const T vj = v[j];
      for (int64_t i = lane; i < n; i += 32) s = add_rn(s, mul_rn(mul_rn(u[i], col[i]), vj));
      s = warp_sum(s);
      if (lane == 0) viol2[j] = sub_rn(s, b[j]);
    }
  }
}

// The step chain (:1058-1090), one CTA.  With `staged`, u, v, viol and viol_2
// live in dynamic shared memory for the whole chain (copied in at the start,
// u and v copied back at the end); otherwise the kernel works on them in
// global memory.
template <typename T>
__global__ void __launch_bounds__(GK_THREADS, 1)
    gk_steps_kernel(const T* __restrict__ K, const T* __restrict__ KT, int n, int m, const T* __restrict__ a,
                    const T* __restrict__ b, T* gu, T* gv, T* gviol, T* gviol2, int staged, int32_t num_iter_max,
                    double stop_thr, int32_t* info) {
  __shared__ GkShared<T> sh;
  extern __shared__ __align__(16) unsigned char gk_dyn[];
  const int tid = threadIdx.x;
  T *u = gu, *v = gv, *viol = gviol, *viol2 = gviol2;
  if (staged) {
    u = (T*)gk_dyn;
    v = u + n;
    viol = v + m;
    viol2 = viol + n;
    for (int i = tid; i < n; i += GK_THREADS) {
      u[i] = gu[i];
      viol[i] = gviol[i];
    }
    for (int j = tid; j < m; j += GK_THREADS) {
      v[j] = gv[j];
      viol2[j] = gviol2[j];
    }
    __syncthreads();
  }
  int buf = 0;
  GkArg own1 = gk_scan(viol, n), own2 = gk_scan(viol2, m);
  GkArg g1 = own1, g2 = own2;
  gk_block_argmax(sh, g1, g2, buf);
  int32_t last = -1, status = OTG_STATUS_MAXITER;
  // the stop test on keys: |x| <= thr for non-negative thr (a negative or NaN
  // threshold never stops, as in the reference)
  const T thr = (T)stop_thr;
  const bool thr_ok = thr >= T(0);
  const unsigned long long thr_key = thr_ok ? GkKey<T>::of(thr) : 0ull;
  for (int32_t ii = 0; ii < num_iter_max; ++ii) {
    last = ii;
    const bool nan1 = g1.k > GkKey<T>::kInf, nan2 = g2.k > GkKey<T>::kInf;
    // nx.maximum propagates NaN, and NaN <= stopThr is false (:1063, :1085);
    // on non-NaN keys, key order is value order
    const bool stop = !nan1 && !nan2 && thr_ok && (g1.k > g2.k ? g1.k : g2.k) <= thr_key;
    if (!nan1 && !nan2 && g1.k > g2.k) {
      // rescale row r (:1066-1073)
      const int r = g1.i;
      const T* Kr = K + (int64_t)r * m;
      T p = 0;
#pragma unroll 4
      for (int j = tid; j < m; j += GK_THREADS) p += Kr[j] * v[j];
      const T dot1 = gk_fold(sh, p);
      if (tid == 0) {
        const T old_u = u[r];
        const T new_u = a[r] / dot1;
        sh.bc[0] = sub_rn(new_u, old_u);
        u[r] = new_u;  // nothing else reads u[r] in a row step
        // the row's own violation, new_u (K_r . v) - a_r: the reference forms
        // (new_u K_r) . v - a_r (:1070); both are rounding noise around zero
        viol[r] = sub_rn(mul_rn(new_u, dot1), a[r]);
      }
      __syncthreads();
      const T du = sh.bc[0];
      own2 = gk_none();
#pragma unroll 4
      for (int j = tid; j < m; j += GK_THREADS) {
        const T nv = fma(mul_rn(Kr[j], du), v[j], viol2[j]);
        viol2[j] = nv;
        gk_take(own2, GkKey<T>::of(nv), j);
      }
      if (r % GK_THREADS == tid) own1 = gk_scan(viol, n);
    } else {
      // rescale column c (:1074-1083)
      const int c = g2.i;
      const T* Kc = KT + (int64_t)c * n;
      T p = 0;
#pragma unroll 4
      for (int i = tid; i < n; i += GK_THREADS) p += Kc[i] * u[i];
      const T dot1 = gk_fold(sh, p);
      if (tid == 0) {
        const T old_v = v[c];
        const T new_v = b[c] / dot1;
        sh.bc[0] = add_rn(-old_v, new_v);
        viol2[c] = sub_rn(mul_rn(new_v, dot1), b[c]);
        v[c] = new_v;  // nothing else reads v in a column step
      }
      __syncthreads();
      const T dv = sh.bc[0];
      own1 = gk_none();
#pragma unroll 4
      for (int i = tid; i < n; i += GK_THREADS) {
        const T nv = fma(mul_rn(dv, Kc[i]), u[i], viol[i]);
        viol[i] = nv;
        gk_take(own1, GkKey<T>::of(nv), i);
      }
      if (c % GK_THREADS == tid) own2 = gk_scan(viol2, m);
    }
    g1 = own1;
    g2 = own2;
    gk_block_argmax(sh, g1, g2, buf);
    if (stop) {  // the reference tests the maximum it chose from, after the step (:1085-1086)
      status = OTG_STATUS_CONVERGED;
      break;
    }
  }
  if (staged) {
    __syncthreads();
    for (int i = tid; i < n; i += GK_THREADS) gu[i] = u[i];
    for (int j = tid; j < m; j += GK_THREADS) gv[j] = v[j];
  }
  if (tid == 0) {
    info[0] = last;
    info[1] = status;
  }
}

// G_ij = (u_i K_ij) v_j: the reference keeps G up to date row by row and
// column by column (:1068, :1077), and every entry's last write used the
// final u_i and v_j, so the plan is this product of the final scalings.
template <typename T>
__global__ void gk_plan_kernel(const T* __restrict__ K, int64_t n, int64_t m, const T* __restrict__ u,
                               const T* __restrict__ v, T* __restrict__ G, int64_t ldg) {
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    const T ui = u[i];
    for (int64_t j = threadIdx.x; j < m; j += blockDim.x) G[i * ldg + j] = mul_rn(mul_rn(ui, K[i * m + j]), v[j]);
  }
}

inline size_t gk_align(size_t x) { return (x + 255) & ~size_t(255); }

template <typename T>
size_t gk_bytes(int64_t n, int64_t m) {
  return 2 * gk_align((size_t)n * m * sizeof(T)) + gk_align(n * sizeof(T)) + gk_align(m * sizeof(T));
}

template <typename T>
int gk_run(const void* M, int64_t n, int64_t m, int64_t ldm, const void* a, const void* b, double reg,
           const void* warm_u, const void* warm_v, int32_t num_iter_max, double stop_thr, void* G, int64_t ldg,
           void* u, void* v, int32_t* info, void* workspace, cudaStream_t stream) {
  char* w = (char*)workspace;
  T* K = (T*)w;
  w += gk_align((size_t)n * m * sizeof(T));
  T* KT = (T*)w;
  w += gk_align((size_t)n * m * sizeof(T));
  T* viol = (T*)w;
  w += gk_align(n * sizeof(T));
  T* viol2 = (T*)w;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tiles = ((n + 31) / 32) * ((m + 31) / 32);
  gk_gibbs_kernel<T><<<(unsigned)std::min<int64_t>(tiles, (int64_t)sms * 8), 256, 0, stream>>>(
      (const T*)M, n, m, ldm, (T)reg, K, KT);
  gk_start_kernel<T><<<(unsigned)std::min<int64_t>((n + m + 255) / 256, (int64_t)sms * 4), 256, 0, stream>>>(
      n, m, (const T*)warm_u, (const T*)warm_v, (T)(1.0 / (double)n), (T)(1.0 / (double)m), (T*)u, (T*)v);
  gk_viol_kernel<T><<<(unsigned)std::min<int64_t>((n + m + 7) / 8, (int64_t)sms * 8), 256, 0, stream>>>(
      K, KT, n, m, (const T*)a, (const T*)b, (const T*)u, (const T*)v, viol, viol2);
  const size_t smem = 2 * (size_t)(n + m) * sizeof(T);
  const int staged = smem <= GK_SMEM_MAX;
  if (staged &&
      cudaFuncSetAttribute(gk_steps_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GK_SMEM_MAX) !=
          cudaSuccess)
    return OTG_ERR_CUDA;
  gk_steps_kernel<T><<<1, GK_THREADS, staged ? smem : 0, stream>>>(K, KT, (int)n, (int)m, (const T*)a, (const T*)b,
                                                                  (T*)u, (T*)v, viol, viol2, staged, num_iter_max,
                                                                  stop_thr, info);
  if (G)
    gk_plan_kernel<T><<<(unsigned)std::min<int64_t>(n, (int64_t)sms * 8), 256, 0, stream>>>(
        K, n, m, (const T*)u, (const T*)v, (T*)G, ldg);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

}  // namespace

extern "C" {

size_t otg_greenkhorn_workspace_bytes(int dtype, int64_t n, int64_t m) {
  if (n < 1 || m < 1) return 0;
  return dtype == OTG_F64 ? gk_bytes<double>(n, m) : gk_bytes<float>(n, m);
}

int otg_greenkhorn(int dtype, const void* M, int64_t n, int64_t m, int64_t ldm, const void* a, const void* b,
                   double reg, const void* warm_u, const void* warm_v, int32_t num_iter_max, double stop_thr,
                   void* G, int64_t ldg, void* u, void* v, int32_t* info, void* workspace, size_t workspace_bytes,
                   cudaStream_t stream) {
  if (!M || !a || !b || !u || !v || !info || n < 1 || m < 1 || n > (1 << 30) || m > (1 << 30) || ldm < m ||
      (G && ldg < m) || num_iter_max < 0 || (!warm_u) != (!warm_v))
    return OTG_ERR_ARG;
  if (dtype != OTG_F32 && dtype != OTG_F64) return OTG_ERR_DTYPE;
  if (!workspace || workspace_bytes < otg_greenkhorn_workspace_bytes(dtype, n, m)) return OTG_ERR_WORKSPACE;
  if (dtype == OTG_F64)
    return gk_run<double>(M, n, m, ldm, a, b, reg, warm_u, warm_v, num_iter_max, stop_thr, G, ldg, u, v, info,
                          workspace, stream);
  return gk_run<float>(M, n, m, ldm, a, b, reg, warm_u, warm_v, num_iter_max, stop_thr, G, ldg, u, v, info,
                       workspace, stream);
}

}  // extern "C"
