// Shared device helpers for the entropic-OT kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <math.h>

#define OTG_LOG2E 1.4426950408889634
#define OTG_LN2 0.6931471805599453

namespace otg {

// ---------------------------------------------------------------------------
// exp2 / log2 in the working precision.  fp32 uses the MUFU ex2 instruction
// (PTX ex2.approx.ftz.f32, relative error about 2^-22); fp64 calls the CUDA
// library exp2.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ double ex2(double x) { return exp2(x); }
__device__ __forceinline__ float lg2(float x) { return log2f(x); }
__device__ __forceinline__ double lg2(double x) { return log2(x); }

// Packed fp32x2 arithmetic (sm_100 family): one instruction for a pair of
// floats in a 64-bit register, each lane rounded as the scalar operation.
__device__ __forceinline__ uint64_t pack2(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ uint64_t pack2u(uint32_t lo, uint32_t hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(lo), "r"(hi));
  return r;
}
__device__ __forceinline__ void unpack2(uint64_t p, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(p));
}
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
// max of three floats in one instruction (NaN inputs handled as by fmaxf)
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

template <typename T> struct Vec;
template <> struct Vec<float> { using type = float4; static constexpr int N = 4; };
template <> struct Vec<double> { using type = double2; static constexpr int N = 2; };

__device__ __forceinline__ void unpack(const float4& q, float* o) { o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.w; }
__device__ __forceinline__ void unpack(const double2& q, double* o) { o[0] = q.x; o[1] = q.y; }

// Streaming 128-bit load that does not allocate in L1 (the cost matrix is
// read once per pass).
__device__ __forceinline__ float4 ld_stream(const float4* p) {
  float4 r;
  asm volatile("ld.global.nc.L1::no_allocate.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w) : "l"(p));
  return r;
}
__device__ __forceinline__ double2 ld_stream(const double2* p) {
  double2 r;
  asm volatile("ld.global.nc.L1::no_allocate.v2.f64 {%0,%1}, [%2];"
               : "=d"(r.x), "=d"(r.y) : "l"(p));
  return r;
}

// ---------------------------------------------------------------------------
// (max, sum) pairs of a base-2 log-sum-exp: the value is  mx + log2(s).
// An empty pair is (-inf, 0).  Merging is associative and commutative, so
// partial pairs from any split of a row or column combine in any order.
// ---------------------------------------------------------------------------
// A NaN maximum is dropped by fmax but poisons the sum through ex2(NaN), so
// NaN inputs still give a NaN result, as they do in the reference.
template <typename T>
__device__ __forceinline__ void lse_merge(T& mx, T& s, T mx2, T s2) {
  T nm = fmax(mx, mx2);
  if (nm == -INFINITY) return;  // both empty
  s = s * ex2(mx - nm) + s2 * ex2(mx2 - nm);
  mx = nm;
}

template <typename T>
__device__ __forceinline__ T lse_value(T mx, T s) {
  if (mx == -INFINITY) return -INFINITY;
  return mx + lg2(s);
}

// Merge `cnt` (max, sum) pairs stored as consecutive (mx, s) values at
// p, p + stride, p + 2 stride, ...  (L2-coherent loads, eight independent
// loads in flight before the dependent merges).
template <typename T>
__device__ __forceinline__ void lse_merge_strided(T& mx, T& s, const T* p, int64_t stride, int cnt) {
  int r = 0;
  for (; r + 8 <= cnt; r += 8) {
    T m8[8], s8[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) { m8[k] = __ldcg(p + (r + k) * stride); s8[k] = __ldcg(p + (r + k) * stride + 1); }
#pragma unroll
    for (int k = 0; k < 8; ++k) lse_merge(mx, s, m8[k], s8[k]);
  }
  for (; r < cnt; ++r) lse_merge(mx, s, __ldcg(p + r * stride), __ldcg(p + r * stride + 1));
}

template <typename T>
__device__ __forceinline__ T sum_strided(const T* p, int64_t stride, int cnt) {
  T acc = 0;
  int r = 0;
  for (; r + 8 <= cnt; r += 8) {
    T v8[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v8[k] = __ldcg(p + (r + k) * stride + 1);
#pragma unroll
    for (int k = 0; k < 8; ++k) acc += v8[k];
  }
  for (; r < cnt; ++r) acc += __ldcg(p + r * stride + 1);
  return acc;
}

template <typename T>
__device__ __forceinline__ void warp_lse(T& mx, T& s) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    T m2 = __shfl_xor_sync(0xffffffffu, mx, o);
    T s2 = __shfl_xor_sync(0xffffffffu, s, o);
    lse_merge(mx, s, m2, s2);
  }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

template <typename T>
__device__ __forceinline__ T warp_max(T x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x = fmax(x, __shfl_xor_sync(0xffffffffu, x, o));
  return x;
}

__device__ __forceinline__ int warp_or(int x) { return __any_sync(0xffffffffu, x) ? 1 : 0; }

// ---------------------------------------------------------------------------
// Reductions in a fixed order.  Floating-point addition is not associative,
// so a sum whose terms arrive through atomics changes from run to run in its
// last bits; a stopping test on such a sum can then stop at a different
// iteration.  Every error that feeds a stop decision is therefore summed in
// an order fixed by the data layout alone: partials are stored in fixed
// slots and summed by these helpers.
//
// warp_sum's xor butterfly combines partner values commutatively at every
// step, so all lanes hold the same, order-fixed value.
// ---------------------------------------------------------------------------
// Block sum of one double per thread; every thread gets the result.  All
// threads of the block call it.
__device__ __forceinline__ double block_sum_fixed(double x) {
  __shared__ double red[33];
  x = warp_sum(x);
  __syncthreads();  // red may still be read by a previous call
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
    red[32] = t;
  }
  __syncthreads();
  return red[32];
}

// Sum of p[0 .. cnt) by one block (thread t folds t, t + blockDim, ... in
// increasing order); every thread gets the result.
__device__ __forceinline__ double block_sum_slots(const double* p, int64_t cnt) {
  double x = 0.0;
  for (int64_t i = threadIdx.x; i < cnt; i += blockDim.x) x += __ldcg(p + i);
  return block_sum_fixed(x);
}

// *out = sum of slots[0 .. cnt) in a fixed order; launch with ONE block of
// BS threads.  (A template, so that every translation unit may include it.)
template <int BS>
__global__ void __launch_bounds__(BS) slot_sum_kernel(const double* __restrict__ slots, int64_t cnt, double* out) {
  const double t = block_sum_slots(slots, cnt);
  if (threadIdx.x == 0) *out = t;
}

// ---------------------------------------------------------------------------
// Bounded grid barrier for cooperative (co-resident) launches.
// bar[0] counts arrivals, bar[1] is the generation.  A block that waits
// longer than `timeout_ns` (globaltimer) sets *abort and leaves; callers check
// *abort after every barrier and return, so no wait is unbounded.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire_i(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ bool grid_barrier(unsigned* bar, unsigned nblocks, int* abort_flag,
                                             uint64_t timeout_ns) {
  __syncthreads();
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    unsigned gen = ld_acquire(bar + 1);
    __threadfence();
    unsigned arrived = atomicAdd(bar, 1u);
    if (arrived == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      uint64_t t0 = globaltimer();
      unsigned spins = 0;
      while (ld_acquire(bar + 1) == gen) {
        if (++spins > 64) __nanosleep(64);
        if ((spins & 255u) == 0) {
          if (ld_acquire_i(abort_flag)) { ok = 0; break; }
          if (globaltimer() - t0 > timeout_ns) { atomicExch(abort_flag, 1); ok = 0; break; }
        }
      }
    }
    __threadfence();
    if (ld_acquire_i(abort_flag)) ok = 0;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace otg
