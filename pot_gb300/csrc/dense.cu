// Dense-cost Sinkhorn (scaling and log-domain forms) as ONE persistent
// cooperative kernel per solve, plus the plan / loss kernel.
//
// Reference behaviour restated here: PythonOT/POT ot/bregman/_sinkhorn.py
//   sinkhorn_knopp  :487-687  (v = b / K^T u ; u = 1 / (diag(1/a) K v), NaN/zero
//                              revert :633-645, L2 column-marginal check every
//                              10th iteration :646-658)
//   sinkhorn_log    :690-918  (v = log b - LSE_i(Mr + u) ; u = log a - LSE_j(Mr + v),
//                              same check :884-899)
//   sinkhorn_stabilized :1105-1368 (scalings over absorbed potentials; see
//                              "Stabilised form" below)
// and ot/unbalanced/_sinkhorn.py
//   sinkhorn_knopp_unbalanced :565-818 (u first: u = (a / K v)^fi1,
//                              v = (b / K^T u)^fi2 with K = exp(-M/reg) c and
//                              c = alpha beta^T; revert on a zero K^T u or a
//                              non-finite scaling; the relative sup-norm change
//                              of (u, v) checked EVERY iteration)
//
// One iteration is one COLUMN pass and one ROW pass over M:
//   column pass  : partial column reductions over row chunks      -> barrier
//   column merge : combine partials, v update, and the marginal error of the
//                  PREVIOUS iteration when it was a check iteration  -> barrier
//   row pass     : row reductions with the new v, u update fused    -> barrier
// The column marginal of exp(Mr + u + v) after iteration k equals
// exp(v_j + LSE_i(Mr + u)_j), and LSE_i(Mr + u) is exactly what iteration
// k+1's column pass computes, so the stopping test costs no extra pass over M:
// the solve stops one column pass later with (u, v) of iteration k, which is
// what the reference returns.
//
// Log-domain arithmetic runs in base 2: x = M * c with c = -log2(e)/reg,
// potentials are kept as log2 values, and exp is the MUFU ex2 instruction.
//
// Stabilised form.  The reference keeps scalings u = exp(F - alpha/reg),
// v = exp(G - beta/reg) over absorbed potentials and, whenever max u or max v
// exceeds tau, moves them into alpha, beta and resets u = 1/n, v = 1/m
// (:1282-1296).  In exact arithmetic F + G follows the log-domain v-first
// iteration started from F0 = alpha0/reg - log n; an absorption only shifts
// the gauge: F by -log n and G by -log m at the absorbing iteration, after
// which G carries +log n per absorption.  The kernel therefore runs the log
// iteration on (F, G) in that standard gauge and tracks, per row and column,
// the reference point SA, SB of the last absorption, so that
// u = exp(F - SA), v = exp(G - SB) exactly as the reference sees them:
//   start          SA = alpha0/reg, SB = beta0/reg
//   absorption     SA = F + log n,  SB = G - log n
// The absorption test max(F - SA) > log tau, max(G - SB) > log tau is a
// grid-wide max folded into the column merge and the row pass.  A check
// iteration that absorbed measures the plan of the shifted gauge, i.e. the
// column sums divided by n m (:1298-1306).  The host turns (F, G), the
// absorption count and the last-iteration flag back into the reference's
// logu, logv, alpha, beta.
#include <cuda.h>
#include <algorithm>
#include <cmath>
#include <mutex>
#include "common.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

template <typename T> struct Pair { T mx, s; };

template <typename T>
__device__ __forceinline__ Pair<T> ldcg_pair(const Pair<T>* p) {
  const T* q = reinterpret_cast<const T*>(p);
  return Pair<T>{__ldcg(q), __ldcg(q + 1)};
}

template <typename T>
struct DenseArgs {
  const T* M; int64_t n, m, ldm;
  const T* a; const T* b;
  const T* warm_u; const T* warm_v;     // natural-log warm start or null
  T c;                                  // -log2(e) / reg
  int max_iter;
  double stop_thr;
  T *u0, *u1, *v0, *v1, *loga2, *logb2;
  Pair<T>* pcol;                        // [Sr][m]
  Pair<T>* prow;                        // [Sc][n]
  int Sr, Sc;
  int64_t rchunk, cchunk;
  T *out_u, *out_v;                     // natural units
  double* hist; int hist_cap;
  int* info;                            // status, niter, nchecks, abort, numflag
  unsigned* bar;
  uint64_t timeout_ns;
  // stabilised form only
  T *sa, *sb;                           // absorption reference points (base 2)
  T log2n, log2m, log2tau;
  int period;                           // iterations between marginal checks
  unsigned long long* mslot;            // STAB: [2] max(F - SA), [2] max(G - SB); UNB: [2][6] maxima
  // unbalanced form only (sa, sb then hold alpha*u and beta*v)
  T fi1, fi2;
  const T* alw; const T* bew;           // c = alw bew^T (null: ones)
  unsigned* slab_cnt;                   // [nslabs] column-pass units done per slab
  double* eslab;                        // [nslabs] squared marginal error of each slab (check passes)
};

// Per-thread maxima carried out of a pass (stabilised: d0; unbalanced:
// |u_new - u_old|, |u_new|, |u_old|).
struct Track {
  double d0 = -INFINITY, d1 = -INFINITY, d2 = -INFINITY;
};

template <int METHOD> struct LogDomain {
  static constexpr bool value = METHOD == OTG_METHOD_LOG || METHOD == OTG_METHOD_STAB;
};

// Internal variant of the scaling form whose matrix operand is the Gibbs
// kernel K = ex2(M * c) itself (OtgDenseProblem::K), not the cost.
constexpr int OTG_METHOD_KNOPP_K = 16;

// Gibbs factor of one loaded entry: the entry itself when it is K, else the
// exponential of the cost entry (the same ex2(M * c) either way).
template <typename T, int METHOD>
__device__ __forceinline__ T gibbs(T x, T c) {
  if (METHOD == OTG_METHOD_KNOPP_K) return x;
  return ex2(x * c);
}

// K = ex2(M * c) entry by entry (c = -log2(e)/reg, the factor of the
// solver's passes), one row per CTA iteration.
template <typename T>
__global__ void gibbs_kernel(const T* __restrict__ M, int64_t n, int64_t m, int64_t ldm, T c, T* __restrict__ K,
                             int64_t ldk) {
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x)
    for (int64_t j = threadIdx.x; j < m; j += blockDim.x) K[i * ldk + j] = gibbs<T, OTG_METHOD_KNOPP>(M[i * ldm + j], c);
}

// Order-preserving map of doubles to unsigned keys (atomicMax on keys = max
// on values; key 0 is below every value).
__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double key_value(unsigned long long k) {
  return (k >> 63) ? __longlong_as_double((long long)(k & 0x7fffffffffffffffull)) : __longlong_as_double((long long)~k);
}

// Block-wide max of one value per thread, then one atomicMax per CTA.  All
// threads of the block call it.
__device__ void block_max_atomic(double x, unsigned long long* slot) {
  __shared__ double red[32];
  x = warp_max(x);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = -INFINITY;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmax(t, red[k]);
    if (t != -INFINITY) atomicMax(slot, order_key(t));
  }
  __syncthreads();
}

constexpr int RW = 4;     // rows per warp in the row pass
constexpr int GCOL = 4;   // rows folded per max update in the column pass

// ---------------------------------------------------------------------------
// Column pass: one CTA-unit = (row chunk r, slab of 32*VW columns).  The 8
// warps split the chunk's rows, each lane folds its VW columns, and the 8
// warp results are merged in shared memory, so each column has one partial
// pair per row chunk (few chunks: a short merge).
// ---------------------------------------------------------------------------
template <typename T, int METHOD>
__device__ __forceinline__ void merge_col(const DenseArgs<T>& A, int64_t j, const T* __restrict__ vcur,
                                          T* __restrict__ vnxt, bool check, bool update, T err_shift, double& e2,
                                          Track& tr);

// Column merge folded into the column pass: the CTA that completes the last
// row chunk of a slab merges that slab's columns (per-thread error and
// tracking accumulators), so the pass needs no grid barrier before the merge.
template <typename T> struct ColFuse {
  const T* vcur; T* vnxt;
  bool check, update;
  T shift;
  Track tr;
};

template <typename T, int METHOD, bool VEC>
__device__ void col_pass(const DenseArgs<T>& A, const T* __restrict__ u, int lane, ColFuse<T>* fuse = nullptr) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  __shared__ T s_mx[8][32 * Vec<T>::N], s_s[8][32 * Vec<T>::N];
  const int warp = threadIdx.x >> 5;
  const int64_t n = A.n, m = A.m;
  const int64_t slab_w = 32 * VW;
  const int64_t nslabs = (m + slab_w - 1) / slab_w;
  const int64_t units = nslabs * A.Sr;
  for (int64_t unit = blockIdx.x; unit < units; unit += gridDim.x) {
    const int64_t slab = unit % nslabs, r = unit / nslabs;
    const int64_t c0 = r * A.rchunk, c1 = min(n, c0 + A.rchunk);
    const int64_t sub = (c1 - c0 + 7) / 8;
    const int64_t i0 = min(c1, c0 + warp * sub), i1 = min(c1, i0 + sub);
    const int64_t j0 = slab * slab_w + lane * VW;
    T mx[VW], s[VW];
#pragma unroll
    for (int k = 0; k < VW; ++k) { mx[k] = -INFINITY; s[k] = 0; }
    if (j0 < m) {
      for (int64_t i = i0; i < i1; i += GCOL) {
        T x[GCOL][VW];
        T ur[GCOL];
#pragma unroll
        for (int g = 0; g < GCOL; ++g) {
          const int64_t row = i + g;
          if (row < i1) {
            const T* Mrow = A.M + row * A.ldm + j0;
            if (VEC) {
              V q = ld_stream(reinterpret_cast<const V*>(Mrow));
              unpack(q, x[g]);
            } else {
#pragma unroll
              for (int k = 0; k < VW; ++k) x[g][k] = (j0 + k < m) ? Mrow[k] : T(0);
            }
            ur[g] = __ldcg(u + row);
          } else {
#pragma unroll
            for (int k = 0; k < VW; ++k) x[g][k] = T(0);
            ur[g] = LogDomain<METHOD>::value ? T(-INFINITY) : T(0);
          }
        }
        if (LogDomain<METHOD>::value) {
#pragma unroll
          for (int k = 0; k < VW; ++k) {
            T t[GCOL];
            T gm = -INFINITY;
#pragma unroll
            for (int g = 0; g < GCOL; ++g) { t[g] = fma(x[g][k], A.c, ur[g]); gm = fmax(gm, t[g]); }
            T nm = fmax(mx[k], gm);
            if (nm != -INFINITY) {
              T acc = s[k] * ex2(mx[k] - nm);
#pragma unroll
              for (int g = 0; g < GCOL; ++g) acc += ex2(t[g] - nm);
              s[k] = acc;
              mx[k] = nm;
            }
          }
        } else {
#pragma unroll
          for (int k = 0; k < VW; ++k) {
#pragma unroll
            for (int g = 0; g < GCOL; ++g) s[k] = fma(gibbs<T, METHOD>(x[g][k], A.c), ur[g], s[k]);
          }
        }
      }
    }
#pragma unroll
    for (int k = 0; k < VW; ++k) { s_mx[warp][lane * VW + k] = mx[k]; s_s[warp][lane * VW + k] = s[k]; }
    __syncthreads();
    // threads 0..32*VW-1 merge the 8 warp results of one column each
    for (int c = threadIdx.x; c < 32 * VW; c += blockDim.x) {
      const int64_t j = slab * slab_w + c;
      if (j < m) {
        T M0 = -INFINITY, S0 = 0;
        for (int w = 0; w < 8; ++w) {
          if (LogDomain<METHOD>::value) lse_merge(M0, S0, s_mx[w][c], s_s[w][c]);
          else S0 += s_s[w][c];
        }
        A.pcol[r * m + j] = Pair<T>{M0, S0};
      }
    }
    if (fuse) {
      __shared__ int s_last;
      __threadfence();  // this unit's partials, before its arrival is counted
      __syncthreads();
      if (threadIdx.x == 0) {
        const unsigned prev = atomicAdd(A.slab_cnt + slab, 1u);
        s_last = prev == (unsigned)(A.Sr - 1);
        if (s_last) atomicExch(A.slab_cnt + slab, 0u);  // every chunk has arrived: ready for the next pass
      }
      __syncthreads();
      if (s_last) {
        __threadfence();
        double e2 = 0.0;
        for (int c = threadIdx.x; c < slab_w; c += blockDim.x) {
          const int64_t j = slab * slab_w + c;
          if (j < m)
            merge_col<T, METHOD>(A, j, fuse->vcur, fuse->vnxt, fuse->check, fuse->update, fuse->shift, e2, fuse->tr);
        }
        // the slab's error in its own slot (which CTA merges a slab varies
        // from run to run; the slot and the order within it do not)
        if (fuse->check) {
          e2 = block_sum_fixed(e2);
          if (threadIdx.x == 0) A.eslab[slab] = e2;
        }
      }
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// Row pass: one CTA-unit = (group of RW rows, column chunk cc); the 8 warps
// split the chunk's columns and merge in shared memory.  With one column
// chunk the potential update is applied directly; otherwise the partial pairs
// are merged after a barrier by row_merge.
// ---------------------------------------------------------------------------
template <typename T, int METHOD>
__device__ __forceinline__ T row_finalize(const DenseArgs<T>& A, int64_t i, T mx, T s, int* numflag) {
  if (LogDomain<METHOD>::value) {
    const T unew = __ldcg(A.loga2 + i) - lse_value(mx, s);
    if (METHOD == OTG_METHOD_STAB && isnan(unew)) atomicExch(numflag, 1);
    return unew;
  } else if (METHOD == OTG_METHOD_UNB) {
    const T al = A.alw ? A.alw[i] : T(1);
    const T unew = pow(A.a[i] / (al * s), A.fi1);
    if (!isfinite(unew)) atomicExch(numflag, 1);
    return unew;
  } else {
    T unew = T(1) / ((T(1) / A.a[i]) * s);
    if (!isfinite(unew)) atomicExch(numflag, 1);
    return unew;
  }
}

// Bookkeeping after a row update: the stabilised form's absorption test, the
// unbalanced form's alpha*u and change maxima.
template <typename T, int METHOD>
__device__ __forceinline__ void row_after(const DenseArgs<T>& A, int64_t i, T un, const T* __restrict__ uold,
                                          Track& tr) {
  if (METHOD == OTG_METHOD_STAB) tr.d0 = fmax(tr.d0, (double)(un - __ldcg(A.sa + i)));
  if (METHOD == OTG_METHOD_UNB) {
    A.sa[i] = (A.alw ? A.alw[i] : T(1)) * un;
    const T uo = __ldcg(uold + i);
    tr.d0 = fmax(tr.d0, (double)fabs(un - uo));
    tr.d1 = fmax(tr.d1, (double)fabs(un));
    tr.d2 = fmax(tr.d2, (double)fabs(uo));
  }
}

template <typename T, int METHOD, bool VEC>
__device__ void row_pass(const DenseArgs<T>& A, const T* __restrict__ v, T* __restrict__ unew, int lane,
                         const T* __restrict__ uold, Track& tr) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  __shared__ T r_mx[8][RW], r_s[8][RW];
  const int warp = threadIdx.x >> 5;
  const int64_t n = A.n, m = A.m;
  const int64_t ngroups = (n + RW - 1) / RW;
  const int64_t units = ngroups * A.Sc;
  for (int64_t unit = blockIdx.x; unit < units; unit += gridDim.x) {
    const int64_t grp = unit % ngroups, cc = unit / ngroups;
    const int64_t r0 = grp * RW;
    const int64_t c0 = cc * A.cchunk, c1 = min(m, c0 + A.cchunk);
    T mx[RW], s[RW];
#pragma unroll
    for (int r = 0; r < RW; ++r) { mx[r] = -INFINITY; s[r] = 0; }
    for (int64_t j = c0 + (warp * 32 + lane) * VW; j < c1; j += 256 * VW) {
      T vv[VW];
      if (VEC) {
        unpack(__ldcg(reinterpret_cast<const V*>(v + j)), vv);
      } else {
#pragma unroll
        for (int k = 0; k < VW; ++k) vv[k] = (j + k < c1) ? __ldcg(v + j + k) : (LogDomain<METHOD>::value ? T(-INFINITY) : T(0));
      }
      T x[RW][VW];
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        const int64_t row = r0 + r;
        const T* Mrow = A.M + (row < n ? row : n - 1) * A.ldm + j;
        if (VEC) {
          V q = ld_stream(reinterpret_cast<const V*>(Mrow));
          unpack(q, x[r]);
        } else {
#pragma unroll
          for (int k = 0; k < VW; ++k) x[r][k] = (j + k < c1) ? Mrow[k] : T(0);
        }
      }
#pragma unroll
      for (int r = 0; r < RW; ++r) {
        if (LogDomain<METHOD>::value) {
          T t[VW];
          T gm = -INFINITY;
#pragma unroll
          for (int k = 0; k < VW; ++k) { t[k] = fma(x[r][k], A.c, vv[k]); gm = fmax(gm, t[k]); }
          T nm = fmax(mx[r], gm);
          if (nm != -INFINITY) {
            T acc = s[r] * ex2(mx[r] - nm);
#pragma unroll
            for (int k = 0; k < VW; ++k) acc += ex2(t[k] - nm);
            s[r] = acc;
            mx[r] = nm;
          }
        } else {
#pragma unroll
          for (int k = 0; k < VW; ++k) s[r] = fma(gibbs<T, METHOD>(x[r][k], A.c), vv[k], s[r]);
        }
      }
    }
#pragma unroll
    for (int r = 0; r < RW; ++r) {
      if (LogDomain<METHOD>::value) warp_lse(mx[r], s[r]);
      else s[r] = warp_sum(s[r]);
    }
    if (lane == 0) {
#pragma unroll
      for (int r = 0; r < RW; ++r) { r_mx[warp][r] = mx[r]; r_s[warp][r] = s[r]; }
    }
    __syncthreads();
    if (threadIdx.x < RW) {
      const int r = threadIdx.x;
      const int64_t row = r0 + r;
      if (row < n) {
        T M0 = -INFINITY, S0 = 0;
        for (int w = 0; w < 8; ++w) {
          if (LogDomain<METHOD>::value) lse_merge(M0, S0, r_mx[w][r], r_s[w][r]);
          else S0 += r_s[w][r];
        }
        if (A.Sc == 1) {
          const T un = row_finalize<T, METHOD>(A, row, M0, S0, A.info + 4);
          unew[row] = un;
          row_after<T, METHOD>(A, row, un, uold, tr);
        } else {
          A.prow[cc * n + row] = Pair<T>{M0, S0};
        }
      }
    }
    __syncthreads();
  }
}

template <typename T, int METHOD>
__device__ void row_merge(const DenseArgs<T>& A, T* __restrict__ unew, long gtid, long nthreads,
                          const T* __restrict__ uold, Track& tr) {
  for (int64_t i = gtid; i < A.n; i += nthreads) {
    T mx = -INFINITY, s = 0;
    const T* base = reinterpret_cast<const T*>(A.prow + i);
    if (LogDomain<METHOD>::value) lse_merge_strided(mx, s, base, 2 * A.n, A.Sc);
    else s = sum_strided(base, 2 * A.n, A.Sc);
    const T un = row_finalize<T, METHOD>(A, i, mx, s, A.info + 4);
    unew[i] = un;
    row_after<T, METHOD>(A, i, un, uold, tr);
  }
}

// Column merge: combine the Sr partials of column j, update v, and add the
// squared column-marginal violation of (u_cur, v_cur) when `check` (with the
// plan scaled by 2^err_shift).  The stabilised form also returns the
// thread's max of v_new - SB.
template <typename T, int METHOD>
__device__ __forceinline__ void merge_col(const DenseArgs<T>& A, int64_t j, const T* __restrict__ vcur,
                                          T* __restrict__ vnxt, bool check, bool update, T err_shift, double& e2,
                                          Track& tr) {
  {
    T mx = -INFINITY, s = 0;
    const T* base = reinterpret_cast<const T*>(A.pcol + j);
    if (LogDomain<METHOD>::value) lse_merge_strided(mx, s, base, 2 * A.m, A.Sr);
    else s = sum_strided(base, 2 * A.m, A.Sr);
    const T bj = A.b[j];
    if (LogDomain<METHOD>::value) {
      const T L = lse_value(mx, s);
      if (check) {
        double cs = (double)ex2(__ldcg(vcur + j) + L + err_shift);
        e2 += (cs - (double)bj) * (cs - (double)bj);
      }
      if (update) {
        const T vn = __ldcg(A.logb2 + j) - L;
        vnxt[j] = vn;
        if (METHOD == OTG_METHOD_STAB) {
          if (isnan(vn)) atomicExch(A.info + 4, 1);
          tr.d0 = fmax(tr.d0, (double)(vn - __ldcg(A.sb + j)));
        }
      }
    } else {
      if (check) {
        double cs = (double)(__ldcg(vcur + j) * s);
        e2 += (cs - (double)bj) * (cs - (double)bj);
      }
      if (update && METHOD == OTG_METHOD_UNB) {
        const T be = A.bew ? A.bew[j] : T(1);
        const T vn = pow(bj / (be * s), A.fi2);
        if (s == T(0) || !isfinite(vn)) atomicExch(A.info + 4, 1);
        vnxt[j] = vn;
        A.sb[j] = be * vn;
        const T vo = __ldcg(vcur + j);
        tr.d0 = fmax(tr.d0, (double)fabs(vn - vo));
        tr.d1 = fmax(tr.d1, (double)fabs(vn));
        tr.d2 = fmax(tr.d2, (double)fabs(vo));
      } else if (update) {
        T vn = bj / s;
        if (s == T(0) || !isfinite(vn)) atomicExch(A.info + 4, 1);
        vnxt[j] = vn;
      }
    }
  }
}

// Column merge after a separate column pass (unbalanced form: no error).
template <typename T, int METHOD>
__device__ void col_merge(const DenseArgs<T>& A, const T* __restrict__ vcur, T* __restrict__ vnxt, bool update,
                          long gtid, long nthreads, Track& tr) {
  double e2 = 0.0;
  for (int64_t j = gtid; j < A.m; j += nthreads) merge_col<T, METHOD>(A, j, vcur, vnxt, false, update, T(0), e2, tr);
}

template <typename T> struct BlocksPerSM { static constexpr int value = sizeof(T) == 4 ? 4 : 2; };

template <typename T, int METHOD, bool VEC>
__global__ void __launch_bounds__(256, BlocksPerSM<T>::value) dense_sinkhorn_kernel(DenseArgs<T> A) {
  const int lane = threadIdx.x & 31;
  const long gtid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nthreads = (long)gridDim.x * blockDim.x;
  int* abort_flag = A.info + 3;
  const T L2E = T(OTG_LOG2E);

  // Phase 0: initial state.
  for (int64_t i = gtid; i < A.n; i += nthreads) {
    if (METHOD == OTG_METHOD_UNB) {
      A.u0[i] = A.warm_u ? exp(A.warm_u[i]) : T(1);
    } else if (METHOD == OTG_METHOD_STAB) {
      const T s0 = A.warm_u ? A.warm_u[i] * L2E : T(0);
      A.sa[i] = s0;
      A.u0[i] = s0 - A.log2n;
      A.loga2[i] = lg2(A.a[i]);
    } else if (LogDomain<METHOD>::value) {
      A.u0[i] = A.warm_u ? A.warm_u[i] * L2E : T(0);
      A.loga2[i] = lg2(A.a[i]);
    } else {
      A.u0[i] = A.warm_u ? exp(A.warm_u[i]) : T(1) / T(A.n);
    }
  }
  for (int64_t j = gtid; j < A.m; j += nthreads) {
    if (METHOD == OTG_METHOD_UNB) {
      const T v0 = A.warm_v ? exp(A.warm_v[j]) : T(1);
      A.v0[j] = v0;
      A.sb[j] = (A.bew ? A.bew[j] : T(1)) * v0;
    } else if (METHOD == OTG_METHOD_STAB) {
      const T s0 = A.warm_v ? A.warm_v[j] * L2E : T(0);
      A.sb[j] = s0;
      A.v0[j] = s0 - A.log2m;
      A.logb2[j] = lg2(A.b[j]);
    } else if (LogDomain<METHOD>::value) {
      A.v0[j] = A.warm_v ? A.warm_v[j] * L2E : T(0);
      A.logb2[j] = lg2(A.b[j]);
    } else {
      A.v0[j] = A.warm_v ? exp(A.warm_v[j]) : T(1) / T(A.m);
    }
  }
  if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;

  T *ucur = A.u0, *unxt = A.u1, *vcur = A.v0, *vnxt = A.v1;
  bool prev_check = false;
  bool absorbed = false;  // stabilised form: the last completed iteration absorbed
  int nabs = 0;
  int nchk = 0;
  int status = OTG_STATUS_MAXITER, niter = A.max_iter - 1;
  if (METHOD == OTG_METHOD_UNB) {
    // u first; the relative change of (u, v) is the error of every iteration
    for (int ii = 0; ii < A.max_iter; ++ii) {
      unsigned long long* sl = A.mslot + 6 * (ii & 1);
      Track ut;
      row_pass<T, METHOD, VEC>(A, A.sb, unxt, lane, ucur, ut);
      if (A.Sc == 1) {
        block_max_atomic(ut.d0, sl); block_max_atomic(ut.d1, sl + 1); block_max_atomic(ut.d2, sl + 2);
      }
      if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      if (A.Sc > 1) {
        row_merge<T, METHOD>(A, unxt, gtid, nthreads, ucur, ut);
        block_max_atomic(ut.d0, sl); block_max_atomic(ut.d1, sl + 1); block_max_atomic(ut.d2, sl + 2);
        if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      }
      col_pass<T, METHOD, VEC>(A, A.sa, lane);
      if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      Track vt;
      col_merge<T, METHOD>(A, vcur, vnxt, true, gtid, nthreads, vt);
      block_max_atomic(vt.d0, sl + 3); block_max_atomic(vt.d1, sl + 4); block_max_atomic(vt.d2, sl + 5);
      if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      if (ld_acquire_i(A.info + 4)) { status = OTG_STATUS_NUMERICAL; niter = ii; break; }  // previous pair kept
      double mk[6];
      for (int q = 0; q < 6; ++q) mk[q] = key_value(__ldcg(sl + q));
      const double err = 0.5 * (mk[0] / fmax(fmax(mk[1], mk[2]), 1.0) + mk[3] / fmax(fmax(mk[4], mk[5]), 1.0));
      if (gtid == 0) {
        if (ii < A.hist_cap) A.hist[ii] = err;
        unsigned long long* other = A.mslot + 6 * ((ii + 1) & 1);
        for (int q = 0; q < 6; ++q) other[q] = 0ull;
      }
      nchk = ii + 1;
      T* t;
      t = ucur; ucur = unxt; unxt = t;
      t = vcur; vcur = vnxt; vnxt = t;
      if (err < A.stop_thr) { status = OTG_STATUS_CONVERGED; niter = ii; break; }
    }
  }
  for (int ii = 0; METHOD != OTG_METHOD_UNB; ++ii) {
    const bool update = ii < A.max_iter;
    double* slot = A.hist + (nchk < A.hist_cap ? nchk : A.hist_cap - 1);
    const T shift = (METHOD == OTG_METHOD_STAB && absorbed) ? -(A.log2n + A.log2m) : T(0);
    ColFuse<T> cf{vcur, vnxt, prev_check, update, shift, Track{}};
    col_pass<T, METHOD, VEC>(A, ucur, lane, &cf);
    if (METHOD == OTG_METHOD_STAB && update) block_max_atomic(cf.tr.d0, A.mslot + 2 + (ii & 1));
    if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
    if (prev_check) {
      // the slabs' errors summed in slab order: the same value in every CTA
      // and in every run
      const double e2 = block_sum_slots(A.eslab, (A.m + 32 * Vec<T>::N - 1) / (32 * Vec<T>::N));
      if (gtid == 0) *slot = e2;
      ++nchk;
      const bool stop = METHOD == OTG_METHOD_STAB ? sqrt(e2) <= A.stop_thr : sqrt(e2) < A.stop_thr;
      if (stop) { status = OTG_STATUS_CONVERGED; niter = ii - 1; break; }
    }
    if (!update) { status = OTG_STATUS_MAXITER; niter = A.max_iter - 1; break; }
    if (!LogDomain<METHOD>::value && ld_acquire_i(A.info + 4)) {
      // zero column sum or non-finite v: revert to the previous pair
      status = OTG_STATUS_NUMERICAL; niter = ii; break;
    }
    Track ut;
    row_pass<T, METHOD, VEC>(A, vnxt, unxt, lane, ucur, ut);
    if (METHOD == OTG_METHOD_STAB && A.Sc == 1) block_max_atomic(ut.d0, A.mslot + (ii & 1));
    if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
    if (A.Sc > 1) {
      row_merge<T, METHOD>(A, unxt, gtid, nthreads, ucur, ut);
      if (METHOD == OTG_METHOD_STAB) block_max_atomic(ut.d0, A.mslot + (ii & 1));
      if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
    }
    if (METHOD != OTG_METHOD_LOG && ld_acquire_i(A.info + 4)) {
      status = OTG_STATUS_NUMERICAL; niter = ii; break;
    }
    if (METHOD == OTG_METHOD_STAB) {
      // absorption test on u = 2^(F - SA), v = 2^(G - SB) of this iteration;
      // the slots of the other parity were last read one iteration ago
      const double mu = key_value(__ldcg(A.mslot + (ii & 1)));
      const double mv = key_value(__ldcg(A.mslot + 2 + (ii & 1)));
      absorbed = mu > (double)A.log2tau || mv > (double)A.log2tau;
      if (absorbed) {
        ++nabs;
        for (int64_t i = gtid; i < A.n; i += nthreads) A.sa[i] = __ldcg(unxt + i) + A.log2n;
        for (int64_t j = gtid; j < A.m; j += nthreads) A.sb[j] = __ldcg(vnxt + j) - A.log2n;
      }
      if (gtid == 0) { A.mslot[(ii + 1) & 1] = 0ull; A.mslot[2 + ((ii + 1) & 1)] = 0ull; }
    }
    T* t;
    t = ucur; ucur = unxt; unxt = t;
    t = vcur; vcur = vnxt; vnxt = t;
    prev_check = (ii % A.period == 0);
  }

  // Final state in natural units.
  const T LN2 = T(OTG_LN2);
  for (int64_t i = gtid; i < A.n; i += nthreads)
    A.out_u[i] = LogDomain<METHOD>::value ? __ldcg(ucur + i) * LN2 : __ldcg(ucur + i);
  for (int64_t j = gtid; j < A.m; j += nthreads)
    A.out_v[j] = LogDomain<METHOD>::value ? __ldcg(vcur + j) * LN2 : __ldcg(vcur + j);
  if (gtid == 0) {
    A.info[0] = status;
    A.info[1] = niter;
    A.info[2] = nchk;
    A.info[5] = nabs;
    A.info[6] = absorbed ? 1 : 0;
  }
}

// ---------------------------------------------------------------------------
// Plan and loss: P_ij = exp(-M_ij/reg + u_i + v_j) (log form, natural-log
// potentials) or u_i exp(-M_ij/reg) v_j (scaling form); loss = sum M * P in
// fp64.  Either output may be null.
// ---------------------------------------------------------------------------
template <typename T, int METHOD>
__global__ void __launch_bounds__(256) dense_plan_kernel(const T* __restrict__ M, int64_t n, int64_t m, int64_t ldm,
                                                         const T* __restrict__ u, const T* __restrict__ v, T c,
                                                         T* __restrict__ P, int64_t ldp, double* loss) {
  const T L2E = T(OTG_LOG2E);
  double acc = 0.0;
  for (int64_t i = blockIdx.x; i < n; i += gridDim.x) {
    const T ui = u[i];
    const T* Mrow = M + i * ldm;
    T racc = 0;  // this thread's share of the row in the working type, fp64 across rows
    for (int64_t j = threadIdx.x; j < m; j += blockDim.x) {
      const T x = Mrow[j];
      T p;
      if (LogDomain<METHOD>::value) p = ex2(fma(x, c, (ui + v[j]) * L2E));
      else p = ui * ex2(x * c) * v[j];
      if (P) P[i * ldp + j] = p;
      racc = fma(x, p, racc);
    }
    if (loss) acc += (double)racc;
  }
  if (loss) {
    acc = warp_sum(acc);
    __shared__ double red[32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) red[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
      atomicAdd(loss, t);
    }
  }
}

// ---------------------------------------------------------------------------
// Marginals of the plan exp(-M_ij/reg + u_i + v_j) (natural-log potentials),
// accumulated in fp64 in a fixed order: one warp per row for the row sums;
// for the column sums a CTA owns 32 columns, its 8 warps take every 8th row
// (lane = column) and their partials are added in warp order.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256) dense_rowsum_kernel(const T* __restrict__ M, int64_t n, int64_t m, int64_t ldm,
                                                           const T* __restrict__ u, const T* __restrict__ v, T c,
                                                           double* __restrict__ rows) {
  const T L2E = T(OTG_LOG2E);
  const int64_t i = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  const T ui = u[i] * L2E;
  double acc = 0.0;
  for (int64_t j = lane; j < m; j += 32) acc += (double)ex2(fma(M[i * ldm + j], c, ui + v[j] * L2E));
  acc = warp_sum(acc);
  if (lane == 0) rows[i] = acc;
}

template <typename T>
__global__ void __launch_bounds__(256) dense_colsum_kernel(const T* __restrict__ M, int64_t n, int64_t m, int64_t ldm,
                                                           const T* __restrict__ u, const T* __restrict__ v, T c,
                                                           double* __restrict__ cols) {
  __shared__ double part[8][32];
  const T L2E = T(OTG_LOG2E);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t j = (int64_t)blockIdx.x * 32 + lane;
  double acc = 0.0;
  if (j < m) {
    const T vj = v[j] * L2E;
    for (int64_t i = warp; i < n; i += 8) acc += (double)ex2(fma(M[i * ldm + j], c, u[i] * L2E + vj));
  }
  part[warp][lane] = acc;
  __syncthreads();
  if (warp == 0 && j < m) {
    double t = 0.0;
    for (int w = 0; w < 8; ++w) t += part[w][lane];
    cols[j] = t;
  }
}

}  // namespace otg

using namespace otg;

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
namespace {

struct Layout {
  int grid, Sr, Sc;
  int64_t rchunk, cchunk;
  size_t off_state, off_pcol, off_prow, off_hist, off_ctrl, off_cnt, off_eslab, total;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Default grid: every SM holds BLOCKS_PER_SM<T> CTAs of 256 threads (the
// kernels are compiled with matching __launch_bounds__), so the layout does
// not depend on which template variant runs.
template <typename T>
int default_grid() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms * BlocksPerSM<T>::value;
}

template <typename T>
int resolve_grid(int requested) {
  const int g = default_grid<T>();
  return (requested > 0 && requested < g) ? requested : g;
}

template <typename T>
Layout make_layout(int64_t n, int64_t m, int hist_cap, int grid) {
  constexpr int VW = Vec<T>::N;
  Layout L{};
  L.grid = grid;
  // column pass: CTA units (slab, row chunk), about two per CTA, each warp
  // at least 4 rows; row pass: CTA units (RW rows, column chunk), a column
  // split only when there are fewer row groups than CTAs
  const int64_t nslabs = (m + 32 * VW - 1) / (32 * VW);
  int64_t Sr = (2 * (int64_t)grid + nslabs - 1) / nslabs;
  Sr = std::max<int64_t>(1, std::min<int64_t>(Sr, (n + 31) / 32));
  L.rchunk = (n + Sr - 1) / Sr;
  L.Sr = (int)((n + L.rchunk - 1) / L.rchunk);
  const int64_t ngroups = (n + RW - 1) / RW;
  int64_t Sc = ngroups >= grid ? 1 : (grid + ngroups - 1) / ngroups;
  Sc = std::max<int64_t>(1, std::min<int64_t>(Sc, (m + 256 * VW - 1) / (256 * VW)));
  int64_t cch = (m + Sc - 1) / Sc;
  cch = (cch + 256 * VW - 1) / (256 * VW) * (256 * VW);
  L.cchunk = cch;
  L.Sc = (int)((m + cch - 1) / cch);
  size_t off = 0;
  L.off_state = off; off = align_up(off + sizeof(T) * (4 * ((size_t)n + 4) + 4 * ((size_t)m + 4)), 256);
  L.off_pcol = off; off = align_up(off + sizeof(Pair<T>) * (size_t)L.Sr * m, 256);
  L.off_prow = off; off = align_up(off + sizeof(Pair<T>) * (size_t)(L.Sc > 1 ? L.Sc : 0) * n, 256);
  L.off_hist = off; off = align_up(off + sizeof(double) * (size_t)hist_cap, 256);
  L.off_ctrl = off; off = align_up(off + 256, 256);
  L.off_cnt = off; off = align_up(off + sizeof(unsigned) * (size_t)nslabs, 256);
  L.off_eslab = off; off = align_up(off + sizeof(double) * (size_t)nslabs, 256);
  L.total = off;
  return L;
}

template <typename T, int METHOD, bool VEC>
int launch_dense(const OtgDenseProblem* p, void* ws, cudaStream_t st) {
  const int grid = resolve_grid<T>(p->grid);
  {
    int per = 0, dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, dense_sinkhorn_kernel<T, METHOD, VEC>, 256, 0);
    if ((int64_t)per * sms < grid) return OTG_ERR_UNSUPPORTED;  // co-residency not possible
  }
  Layout L = make_layout<T>(p->n, p->m, p->hist_cap, grid);
  if (p->workspace_bytes < L.total) return OTG_ERR_WORKSPACE;
  char* base = static_cast<char*>(ws);
  DenseArgs<T> A{};
  A.M = static_cast<const T*>(p->M); A.n = p->n; A.m = p->m; A.ldm = p->ldm;
  A.a = static_cast<const T*>(p->a); A.b = static_cast<const T*>(p->b);
  A.warm_u = static_cast<const T*>(p->warm_u); A.warm_v = static_cast<const T*>(p->warm_v);
  A.c = (T)(-OTG_LOG2E / p->reg);
  A.max_iter = p->max_iter; A.stop_thr = p->stop_thr;
  T* st_ = reinterpret_cast<T*>(base + L.off_state);
  const int64_t n = p->n, m = p->m;
  // vectors are 16-byte aligned inside the state block
  auto al = [](int64_t k) { return (k + 3) / 4 * 4; };
  int64_t o = 0;
  A.u0 = st_ + o; o += al(n); A.u1 = st_ + o; o += al(n); A.loga2 = st_ + o; o += al(n);
  A.v0 = st_ + o; o += al(m); A.v1 = st_ + o; o += al(m); A.logb2 = st_ + o; o += al(m);
  A.sa = st_ + o; o += al(n); A.sb = st_ + o; o += al(m);
  A.pcol = reinterpret_cast<Pair<T>*>(base + L.off_pcol);
  A.prow = reinterpret_cast<Pair<T>*>(base + L.off_prow);
  A.Sr = L.Sr; A.Sc = L.Sc; A.rchunk = L.rchunk; A.cchunk = L.cchunk;
  A.out_u = static_cast<T*>(p->out_u); A.out_v = static_cast<T*>(p->out_v);
  A.hist = reinterpret_cast<double*>(base + L.off_hist); A.hist_cap = p->hist_cap;
  A.info = reinterpret_cast<int*>(base + L.off_ctrl);
  A.bar = reinterpret_cast<unsigned*>(base + L.off_ctrl + 32);
  A.timeout_ns = p->timeout_ms > 0 ? (uint64_t)p->timeout_ms * 1000000ull : 4000000000ull;
  A.log2n = (T)std::log2((double)n);
  A.log2m = (T)std::log2((double)m);
  A.log2tau = (T)(METHOD == OTG_METHOD_STAB ? std::log2(p->tau) : 0.0);
  A.period = METHOD == OTG_METHOD_STAB ? p->check_period : 10;
  A.mslot = reinterpret_cast<unsigned long long*>(base + L.off_ctrl + 64);
  A.slab_cnt = reinterpret_cast<unsigned*>(base + L.off_cnt);
  A.eslab = reinterpret_cast<double*>(base + L.off_eslab);
  if (METHOD == OTG_METHOD_UNB) {
    A.fi1 = (T)(std::isinf(p->reg_m1) ? 1.0 : p->reg_m1 / (p->reg_m1 + p->reg));
    A.fi2 = (T)(std::isinf(p->reg_m2) ? 1.0 : p->reg_m2 / (p->reg_m2 + p->reg));
    A.alw = p->c_ones ? nullptr : static_cast<const T*>(p->a);
    A.bew = p->c_ones ? nullptr : static_cast<const T*>(p->b);
  }
  cudaError_t e = cudaMemsetAsync(base + L.off_hist, 0, L.total - L.off_hist, st);
  if (e != cudaSuccess) return OTG_ERR_CUDA;
  void* args[] = {&A};
  e = cudaLaunchCooperativeKernel((const void*)dense_sinkhorn_kernel<T, METHOD, VEC>, dim3(grid), dim3(256), args, 0, st);
  if (e != cudaSuccess) return OTG_ERR_CUDA;
  return OTG_OK;
}

template <typename T>
int dispatch_dense(const OtgDenseProblem* p, void* ws, cudaStream_t st) {
  constexpr int VW = Vec<T>::N;
  if (p->method == OTG_METHOD_KNOPP && p->K) {
    // the passes read K in place of M
    OtgDenseProblem q = *p;
    q.M = p->K;
    q.ldm = p->ldk;
    const bool vk = (q.m % VW == 0) && (q.ldm % VW == 0) && ((uintptr_t)q.M % 16 == 0);
    return vk ? launch_dense<T, OTG_METHOD_KNOPP_K, true>(&q, ws, st)
              : launch_dense<T, OTG_METHOD_KNOPP_K, false>(&q, ws, st);
  }
  const bool vec = (p->m % VW == 0) && (p->ldm % VW == 0) && ((uintptr_t)p->M % 16 == 0);
  if (p->method == OTG_METHOD_LOG)
    return vec ? launch_dense<T, OTG_METHOD_LOG, true>(p, ws, st) : launch_dense<T, OTG_METHOD_LOG, false>(p, ws, st);
  if (p->method == OTG_METHOD_STAB)
    return vec ? launch_dense<T, OTG_METHOD_STAB, true>(p, ws, st) : launch_dense<T, OTG_METHOD_STAB, false>(p, ws, st);
  if (p->method == OTG_METHOD_UNB)
    return vec ? launch_dense<T, OTG_METHOD_UNB, true>(p, ws, st) : launch_dense<T, OTG_METHOD_UNB, false>(p, ws, st);
  return vec ? launch_dense<T, OTG_METHOD_KNOPP, true>(p, ws, st) : launch_dense<T, OTG_METHOD_KNOPP, false>(p, ws, st);
}

int check_problem(const OtgDenseProblem* p) {
  if (!p || !p->M || !p->a || !p->b || !p->out_u || !p->out_v) return OTG_ERR_ARG;
  if (p->n < 1 || p->m < 1 || p->ldm < p->m || p->hist_cap < 1) return OTG_ERR_ARG;
  if (p->K && p->ldk < p->m) return OTG_ERR_ARG;
  if (p->dtype != OTG_F32 && p->dtype != OTG_F64) return OTG_ERR_DTYPE;
  if (p->method != OTG_METHOD_LOG && p->method != OTG_METHOD_KNOPP && p->method != OTG_METHOD_STAB &&
      p->method != OTG_METHOD_UNB)
    return OTG_ERR_ARG;
  if (p->method == OTG_METHOD_UNB && (!(p->reg_m1 > 0) || !(p->reg_m2 > 0) || p->hist_cap < p->max_iter))
    return OTG_ERR_ARG;
  if (p->method == OTG_METHOD_STAB && (p->check_period < 1 || !(p->tau > 0))) return OTG_ERR_ARG;
  if (p->max_iter < 0) return OTG_ERR_ARG;
  return OTG_OK;
}

}  // namespace

extern "C" {

size_t otg_dense_workspace_bytes(int dtype, int64_t n, int64_t m, int hist_cap, int grid) {
  if (dtype == OTG_F64) return make_layout<double>(n, m, hist_cap, resolve_grid<double>(grid)).total;
  return make_layout<float>(n, m, hist_cap, resolve_grid<float>(grid)).total;
}

size_t otg_dense_info_offset(int dtype, int64_t n, int64_t m, int hist_cap, int grid) {
  if (dtype == OTG_F64) return make_layout<double>(n, m, hist_cap, resolve_grid<double>(grid)).off_hist;
  return make_layout<float>(n, m, hist_cap, resolve_grid<float>(grid)).off_hist;
}

int otg_sinkhorn_dense(const OtgDenseProblem* p, void* workspace, cudaStream_t stream) {
  int rc = check_problem(p);
  if (rc != OTG_OK) return rc;
  if (!workspace) return OTG_ERR_WORKSPACE;
  if (p->dtype == OTG_F64) return dispatch_dense<double>(p, workspace, stream);
  return dispatch_dense<float>(p, workspace, stream);
}

int otg_dense_plan(int dtype, int method, const void* M, int64_t n, int64_t m, int64_t ldm,
                   const void* u, const void* v, double reg, void* P, int64_t ldp, double* loss,
                   cudaStream_t stream) {
  if (!M || !u || !v || n < 1 || m < 1 || ldm < m || (P && ldp < m)) return OTG_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int64_t blocks = std::min<int64_t>(n, (int64_t)sms * 8);
  if (loss) cudaMemsetAsync(loss, 0, sizeof(double), stream);
  const double c = -OTG_LOG2E / reg;
  if (method == OTG_METHOD_STAB) method = OTG_METHOD_LOG;  // plan of natural-log potentials
  if (method == OTG_METHOD_UNB) method = OTG_METHOD_KNOPP; // plan of scalings (alpha u, beta v)
  if (dtype == OTG_F64) {
    if (method == OTG_METHOD_LOG)
      dense_plan_kernel<double, OTG_METHOD_LOG><<<blocks, 256, 0, stream>>>((const double*)M, n, m, ldm, (const double*)u, (const double*)v, c, (double*)P, ldp, loss);
    else
      dense_plan_kernel<double, OTG_METHOD_KNOPP><<<blocks, 256, 0, stream>>>((const double*)M, n, m, ldm, (const double*)u, (const double*)v, c, (double*)P, ldp, loss);
  } else if (dtype == OTG_F32) {
    if (method == OTG_METHOD_LOG)
      dense_plan_kernel<float, OTG_METHOD_LOG><<<blocks, 256, 0, stream>>>((const float*)M, n, m, ldm, (const float*)u, (const float*)v, (float)c, (float*)P, ldp, loss);
    else
      dense_plan_kernel<float, OTG_METHOD_KNOPP><<<blocks, 256, 0, stream>>>((const float*)M, n, m, ldm, (const float*)u, (const float*)v, (float)c, (float*)P, ldp, loss);
  } else {
    return OTG_ERR_DTYPE;
  }
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_gibbs_kernel(int dtype, const void* M, int64_t n, int64_t m, int64_t ldm, double reg, void* K,
                     int64_t ldk, cudaStream_t stream) {
  // any reg: the factor c = -log2(e)/reg is the solver's (reg = 0 gives its non-finite K)
  if (!M || !K || n < 1 || m < 1 || ldm < m || ldk < m) return OTG_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t blocks = std::min<int64_t>(n, (int64_t)sms * 16);
  if (dtype == OTG_F64)
    gibbs_kernel<double><<<blocks, 256, 0, stream>>>((const double*)M, n, m, ldm, (double)(-OTG_LOG2E / reg),
                                                     (double*)K, ldk);
  else if (dtype == OTG_F32)
    gibbs_kernel<float><<<blocks, 256, 0, stream>>>((const float*)M, n, m, ldm, (float)(-OTG_LOG2E / reg),
                                                    (float*)K, ldk);
  else
    return OTG_ERR_DTYPE;
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_dense_marginals(int dtype, const void* M, int64_t n, int64_t m, int64_t ldm, const void* u, const void* v,
                        double reg, double* rowsum, double* colsum, cudaStream_t stream) {
  if (!M || !u || !v || !rowsum || !colsum || n < 1 || m < 1 || ldm < m || !(reg > 0)) return OTG_ERR_ARG;
  const double c = -OTG_LOG2E / reg;
  const dim3 rg((unsigned)((n + 7) / 8)), cg((unsigned)((m + 31) / 32));
  if (dtype == OTG_F64) {
    dense_rowsum_kernel<double><<<rg, 256, 0, stream>>>((const double*)M, n, m, ldm, (const double*)u, (const double*)v, c, rowsum);
    dense_colsum_kernel<double><<<cg, 256, 0, stream>>>((const double*)M, n, m, ldm, (const double*)u, (const double*)v, c, colsum);
  } else if (dtype == OTG_F32) {
    dense_rowsum_kernel<float><<<rg, 256, 0, stream>>>((const float*)M, n, m, ldm, (const float*)u, (const float*)v, (float)c, rowsum);
    dense_colsum_kernel<float><<<cg, 256, 0, stream>>>((const float*)M, n, m, ldm, (const float*)u, (const float*)v, (float)c, colsum);
  } else {
    return OTG_ERR_DTYPE;
  }
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free entry point.
//
// Some callers cannot allocate device memory at solve time: a host program
// whose own allocator owns the whole device pool and hands out no extra
// buffers, or a latency-bound loop (a control or serving loop) that must not
// pay cudaMalloc / cudaFree, which can synchronise the device.  For them the
// solver's scratch lives in one file-scope device array of fixed size that
// every GPU loading this library keeps until the process exits.
//
// All calls share the array: it keeps the last call's contents (the launch
// clears the error history and control words that must start at zero), and
// calls whose kernels overlap on the GPU race on it, so callers serialise
// them (one stream, or their own ordering).
// ---------------------------------------------------------------------------
namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[OTG_NOALLOC_SCRATCH_BYTES];

// Host code cannot use g_noalloc_scratch as a device address (on the host
// it names a stand-in object), so its device address is looked up with
// cudaGetSymbolAddress, with the device current, the first time a context
// calls, and cached.  The cache is keyed by the CUDA context's unique ID
// (cuCtxGetId), not by the device ordinal: after cudaDeviceReset, or in a
// context other than the primary one (cuCtxCreate, green contexts), the
// module and its array live at another address, and a context gets a new
// ID when it is created again.  A mutex guards the cache against host
// threads making their first calls at the same time.
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);

struct NoallocCache {
  std::mutex mu;
  CtxGetCurrentFn get_current = nullptr;
  CtxGetIdFn get_id = nullptr;
  bool resolved = false;
  static constexpr int kSlots = 64;
  unsigned long long ids[kSlots] = {};
  void* ptrs[kSlots] = {};
  int used = 0;
};
NoallocCache g_noalloc;

int noalloc_scratch(void** out) {
  std::lock_guard<std::mutex> lock(g_noalloc.mu);
  if (!g_noalloc.resolved) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_noalloc.get_current = reinterpret_cast<CtxGetCurrentFn>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_noalloc.get_id = reinterpret_cast<CtxGetIdFn>(f);
    g_noalloc.resolved = true;
  }
  if (!g_noalloc.get_current || !g_noalloc.get_id) return OTG_ERR_CUDA;
  CUcontext ctx = nullptr;
  if (g_noalloc.get_current(&ctx) != CUDA_SUCCESS) return OTG_ERR_CUDA;
  if (!ctx) {
    // no context on this thread yet: the runtime makes the current device's
    // primary context current on its first call that needs one
    void* probe = nullptr;
    if (cudaGetSymbolAddress(&probe, g_noalloc_scratch) != cudaSuccess) return OTG_ERR_CUDA;
    if (g_noalloc.get_current(&ctx) != CUDA_SUCCESS || !ctx) return OTG_ERR_CUDA;
  }
  unsigned long long id = 0;
  if (g_noalloc.get_id(ctx, &id) != CUDA_SUCCESS) return OTG_ERR_CUDA;
  for (int k = 0; k < g_noalloc.used; ++k)
    if (g_noalloc.ids[k] == id) { *out = g_noalloc.ptrs[k]; return OTG_OK; }
  void* ptr = nullptr;
  if (cudaGetSymbolAddress(&ptr, g_noalloc_scratch) != cudaSuccess || !ptr) return OTG_ERR_CUDA;
  // a full table still works, the lookup is just repeated for later contexts
  if (g_noalloc.used < NoallocCache::kSlots) {
    g_noalloc.ids[g_noalloc.used] = id;
    g_noalloc.ptrs[g_noalloc.used] = ptr;
    ++g_noalloc.used;
  }
  *out = ptr;
  return OTG_OK;
}

template <typename T>
int noalloc_solve(const OtgDenseProblem* p, double* err_hist, int32_t* info, cudaStream_t st) {
  const Layout L = make_layout<T>(p->n, p->m, p->hist_cap, resolve_grid<T>(p->grid));
  if (L.total > (size_t)OTG_NOALLOC_SCRATCH_BYTES) return OTG_ERR_NOALLOC_TOO_LARGE;
  void* scratch = nullptr;
  int rc = noalloc_scratch(&scratch);
  if (rc != OTG_OK) return rc;
  OtgDenseProblem q = *p;
  q.workspace_bytes = OTG_NOALLOC_SCRATCH_BYTES;
  rc = dispatch_dense<T>(&q, scratch, st);
  if (rc != OTG_OK) return rc;
  char* base = static_cast<char*>(scratch);
  if (cudaMemcpyAsync(err_hist, base + L.off_hist, sizeof(double) * (size_t)p->hist_cap,
                      cudaMemcpyDeviceToDevice, st) != cudaSuccess) return OTG_ERR_CUDA;
  if (cudaMemcpyAsync(info, base + L.off_ctrl, 8 * sizeof(int32_t), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
    return OTG_ERR_CUDA;
  return OTG_OK;
}

}  // namespace

extern "C" int otg_sinkhorn_dense_noalloc(const OtgDenseProblem* p, double* err_hist, int32_t* info,
                                          cudaStream_t stream) {
  int rc = check_problem(p);
  if (rc != OTG_OK) return rc;
  if (!err_hist || !info) return OTG_ERR_ARG;
  if (p->dtype == OTG_F64) return noalloc_solve<double>(p, err_hist, info, stream);
  return noalloc_solve<float>(p, err_hist, info, stream);
}
