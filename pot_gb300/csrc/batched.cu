// Batched Sinkhorn over many independent dense problems of uneven size, in
// ONE persistent launch.
//
// Reference behaviour restated here (PythonOT/POT):
//   ot/batch/_utils.py:165-290  bregman_log_projection_batch: u first, then v;
//                               row-marginal L2 check every 10th iteration
//   ot/batch/_utils.py:46-162   bregman_projection_batch (scaling form), same order
//   ot/bregman/_sinkhorn.py:690-918  sinkhorn_log: v first, then u; column check
// Differences by design: every problem stops on its own error (a per-problem
// convergence flag on the device) instead of the reference's max over the
// batch; uneven sizes are native (a problem table) instead of zero-weight
// padding.
//
// Execution: one CTA per problem at a time; CTAs pull problem indices from a
// device counter in the host-given order (largest work first).  Warp 8 is a
// producer that streams the problem's cost rows through a shared-memory ring
// with 1-D bulk copies (cp.async.bulk, mbarrier completion); warps 0-7
// consume.  Both half-steps read M in row order:
//   row half-step (A): warp per row, lanes split the columns, LSE over j;
//   column half-step (B): thread per VW columns, folding rows into running
//                         (max, sum) pairs kept in registers.
// The potentials stay in shared memory for the whole solve.  As in the dense
// kernel, the marginal error of a check iteration is formed from the next
// half-step's LSE, so checking costs no extra pass; the producer waits for the
// stop decision only at those points.
#include <algorithm>
#include "common.cuh"
#include "tma.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

constexpr int BT_CONSUMERS = 256;           // 8 consumer warps
constexpr int BT_THREADS = BT_CONSUMERS + 32;
constexpr int BT_STAGES = 5;
constexpr uint32_t BT_STAGE_BYTES = 32768;
constexpr int BT_GCOL = 4;                  // rows folded per max update (B pass)

template <typename T> struct BtLimits;
template <> struct BtLimits<float> { static constexpr int NMAX = 4096; static constexpr int G = 4; };
template <> struct BtLimits<double> { static constexpr int NMAX = 2048; static constexpr int G = 4; };

template <typename T>
struct BatchArgs {
  const T* M;
  const int64_t* m_off;      // element offset of problem p's cost block
  const int32_t* rows;       // n_p
  const int32_t* cols;       // m_p
  const int32_t* ldm;        // row stride (elements), multiple of 16 bytes
  const int64_t* r_off;      // offset of a_p / u_p in the packed row vectors
  const int64_t* c_off;      // offset of b_p / v_p in the packed column vectors
  const T* a; const T* b;
  const T* warm_u; const T* warm_v;  // natural-log warm start or null
  const double* reg;         // per problem
  const int32_t* order;      // processing order
  int32_t nprob;
  int32_t max_iter;
  double stop_thr;
  int32_t u_first;           // 1: batch order (u, v, row error); 0: sinkhorn_log order
  T* out_u; T* out_v;        // natural-log potentials (log) or scalings (knopp)
  int32_t* status; int32_t* niter; double* err;
  int32_t* queue;            // [0] problem counter, [1] abort flag
  uint64_t timeout_ns;
};

template <typename T>
struct BtShared {
  T* ring;
  uint64_t* full;
  uint64_t* empty;
  T* ua; T* ub; T* v;
  double* red;
  int* ctl;                  // [0] problem, [1] stop decision
};

template <typename T>
__device__ __forceinline__ BtShared<T> bt_carve(unsigned char* base) {
  BtShared<T> S;
  S.ring = reinterpret_cast<T*>(base);
  size_t off = (size_t)BT_STAGES * BT_STAGE_BYTES;
  S.full = reinterpret_cast<uint64_t*>(base + off); off += 8 * BT_STAGES;
  S.empty = reinterpret_cast<uint64_t*>(base + off); off += 8 * BT_STAGES;
  S.red = reinterpret_cast<double*>(base + off); off += 8 * 16;
  S.ctl = reinterpret_cast<int*>(base + off); off += 16 * 4;
  off = (off + 15) / 16 * 16;
  S.ua = reinterpret_cast<T*>(base + off); off += sizeof(T) * BtLimits<T>::NMAX;
  S.ub = reinterpret_cast<T*>(base + off); off += sizeof(T) * BtLimits<T>::NMAX;
  S.v = reinterpret_cast<T*>(base + off); off += sizeof(T) * BtLimits<T>::NMAX;
  return S;
}

template <typename T>
constexpr size_t bt_smem_bytes() {
  return (size_t)BT_STAGES * BT_STAGE_BYTES + 16 * BT_STAGES + 8 * 16 + 16 * 4 + 16 + 3 * sizeof(T) * BtLimits<T>::NMAX;
}

// Rows of one problem that fit in a stage.
__device__ __forceinline__ int bt_chunk_rows(int n, int ldm, int esize) {
  int r = (int)(BT_STAGE_BYTES / ((uint32_t)ldm * esize));
  return r < n ? r : n;
}

// ----------------------------- producer ------------------------------------
template <typename T>
__device__ __forceinline__ bool bt_produce_pass(const BtShared<T>& S, const T* Mp, int n, int ldm,
                                                uint32_t& gchunk, int* abort_flag, uint64_t tmo) {
  const int R = bt_chunk_rows(n, ldm, sizeof(T));
  for (int r0 = 0; r0 < n; r0 += R) {
    const int rows = min(R, n - r0);
    const uint32_t stage = gchunk % BT_STAGES;
    const uint32_t round = gchunk / BT_STAGES;
    if (!mbar_wait(S.empty + stage, (round & 1u) ^ 1u, abort_flag, tmo)) return false;
    const uint32_t bytes = (uint32_t)rows * (uint32_t)ldm * sizeof(T);
    mbar_arrive_expect_tx(S.full + stage, bytes);
    bulk_g2s(reinterpret_cast<unsigned char*>(S.ring) + (size_t)stage * BT_STAGE_BYTES,
             Mp + (int64_t)r0 * ldm, bytes, S.full + stage);
    ++gchunk;
  }
  return true;
}

// ----------------------------- consumers -----------------------------------
// Row half-step: u_dst[i] = f(a_i, LSE_j / sum_j) for every row; with
// `check`, accumulates the squared row-marginal violation of (u_cur, v).
template <typename T, int METHOD>
__device__ __forceinline__ bool bt_row_pass(const BtShared<T>& S, const T* __restrict__ a, int n, int m, int ldm, T c,
                                            const T* u_cur, T* u_dst, bool check, double& e2,
                                            uint32_t& gchunk, int* abort_flag, uint64_t tmo) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int R = bt_chunk_rows(n, ldm, sizeof(T));
  for (int r0 = 0; r0 < n; r0 += R) {
    const int rows = min(R, n - r0);
    const uint32_t stage = gchunk % BT_STAGES;
    if (!mbar_wait(S.full + stage, (gchunk / BT_STAGES) & 1u, abort_flag, tmo)) return false;
    const T* base = S.ring + (size_t)stage * (BT_STAGE_BYTES / sizeof(T));
    for (int rr = warp; rr < rows; rr += BT_CONSUMERS / 32) {
      const T* row = base + (size_t)rr * ldm;
      T mx = -INFINITY, s = 0;
      for (int j = lane * VW; j < m; j += 32 * VW) {
        T x[VW], vv[VW];
        unpack(*reinterpret_cast<const V*>(row + j), x);
        unpack(*reinterpret_cast<const V*>(S.v + j), vv);
        if (METHOD == OTG_METHOD_LOG) {
          T t[VW];
          T gm = -INFINITY;
#pragma unroll
          for (int k = 0; k < VW; ++k) { t[k] = fma(x[k], c, vv[k]); gm = fmax(gm, t[k]); }
          T nm = fmax(mx, gm);
          if (nm != -INFINITY) {
            T acc = s * ex2(mx - nm);
#pragma unroll
            for (int k = 0; k < VW; ++k) acc += ex2(t[k] - nm);
            s = acc;
            mx = nm;
          }
        } else {
#pragma unroll
          for (int k = 0; k < VW; ++k) s = fma(ex2(x[k] * c), vv[k], s);
        }
      }
      if (METHOD == OTG_METHOD_LOG) warp_lse(mx, s);
      else s = warp_sum(s);
      if (lane == 0) {
        const int i = r0 + rr;
        const T ai = a[i];
        if (METHOD == OTG_METHOD_LOG) {
          const T L = lse_value(mx, s);
          if (check) { double rs = (double)ex2(u_cur[i] + L) - (double)ai; e2 += rs * rs; }
          u_dst[i] = lg2(ai) - L;
        } else {
          if (check) { double rs = (double)(u_cur[i] * s) - (double)ai; e2 += rs * rs; }
          u_dst[i] = ai / s;
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(S.empty + stage);
    ++gchunk;
  }
  return true;
}

// Column half-step: column reductions folded over all rows into registers.
// Returns the per-column results in L[g][k] (log: base-2 LSE; knopp: sum).
template <typename T, int METHOD, int G>
__device__ __forceinline__ bool bt_col_pass(const BtShared<T>& S, int n, int m, int ldm, T c, const T* u,
                                            T (&L)[G][Vec<T>::N], uint32_t& gchunk, int* abort_flag, uint64_t tmo) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  const int tid = threadIdx.x, lane = tid & 31;
  T mx[G][VW], s[G][VW];
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int k = 0; k < VW; ++k) { mx[g][k] = -INFINITY; s[g][k] = 0; }
  const int R = bt_chunk_rows(n, ldm, sizeof(T));
  for (int r0 = 0; r0 < n; r0 += R) {
    const int rows = min(R, n - r0);
    const uint32_t stage = gchunk % BT_STAGES;
    if (!mbar_wait(S.full + stage, (gchunk / BT_STAGES) & 1u, abort_flag, tmo)) return false;
    const T* base = S.ring + (size_t)stage * (BT_STAGE_BYTES / sizeof(T));
#pragma unroll
    for (int g = 0; g < G; ++g) {
      const int j = (g * BT_CONSUMERS + tid) * VW;
      if (j < m) {
        for (int rr = 0; rr < rows; rr += BT_GCOL) {
          T x[BT_GCOL][VW], ur[BT_GCOL];
#pragma unroll
          for (int q = 0; q < BT_GCOL; ++q) {
            if (rr + q < rows) {
              unpack(*reinterpret_cast<const V*>(base + (size_t)(rr + q) * ldm + j), x[q]);
              ur[q] = u[r0 + rr + q];
            } else {
#pragma unroll
              for (int k = 0; k < VW; ++k) x[q][k] = 0;
              ur[q] = METHOD == OTG_METHOD_LOG ? T(-INFINITY) : T(0);
            }
          }
          if (METHOD == OTG_METHOD_LOG) {
#pragma unroll
            for (int k = 0; k < VW; ++k) {
              T t[BT_GCOL];
              T gm = -INFINITY;
#pragma unroll
              for (int q = 0; q < BT_GCOL; ++q) { t[q] = fma(x[q][k], c, ur[q]); gm = fmax(gm, t[q]); }
              T nm = fmax(mx[g][k], gm);
              if (nm != -INFINITY) {
                T acc = s[g][k] * ex2(mx[g][k] - nm);
#pragma unroll
                for (int q = 0; q < BT_GCOL; ++q) acc += ex2(t[q] - nm);
                s[g][k] = acc;
                mx[g][k] = nm;
              }
            }
          } else {
#pragma unroll
            for (int k = 0; k < VW; ++k)
#pragma unroll
              for (int q = 0; q < BT_GCOL; ++q) s[g][k] = fma(ex2(x[q][k] * c), ur[q], s[g][k]);
          }
        }
      }
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(S.empty + stage);
    ++gchunk;
  }
#pragma unroll
  for (int g = 0; g < G; ++g)
#pragma unroll
    for (int k = 0; k < VW; ++k) L[g][k] = METHOD == OTG_METHOD_LOG ? lse_value(mx[g][k], s[g][k]) : s[g][k];
  return true;
}

// Block reduction of e2 over the consumer warps (named barrier 3).
template <typename T>
__device__ __forceinline__ double bt_reduce(const BtShared<T>& S, double e2) {
  e2 = warp_sum(e2);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) S.red[warp] = e2;
  named_bar(3, BT_CONSUMERS);
  double t = 0;
#pragma unroll
  for (int w = 0; w < BT_CONSUMERS / 32; ++w) t += S.red[w];
  named_bar(3, BT_CONSUMERS);
  return t;
}

template <typename T, int METHOD, int G>
__device__ void bt_consume_problem(const BatchArgs<T>& A, const BtShared<T>& S, int p, uint32_t& gchunk) {
  constexpr int VW = Vec<T>::N;
  const int tid = threadIdx.x;
  const int n = A.rows[p], m = A.cols[p], ldm = A.ldm[p];
  const T* a = A.a + A.r_off[p];
  const T* b = A.b + A.c_off[p];
  const T c = (T)(-OTG_LOG2E / A.reg[p]);
  const T L2E = T(OTG_LOG2E);
  int* abort_flag = A.queue + 1;
  const uint64_t tmo = A.timeout_ns;
  // initial potentials (base-2 logs for the log form; scalings for knopp)
  for (int i = tid; i < n; i += BT_CONSUMERS) {
    if (METHOD == OTG_METHOD_LOG) S.ua[i] = A.warm_u ? A.warm_u[A.r_off[p] + i] * L2E : T(0);
    else S.ua[i] = A.warm_u ? exp(A.warm_u[A.r_off[p] + i]) : T(1);
  }
  for (int j = tid; j < ldm; j += BT_CONSUMERS) {
    T v0 = METHOD == OTG_METHOD_LOG ? T(0) : T(1);
    if (j < m && A.warm_v) v0 = METHOD == OTG_METHOD_LOG ? A.warm_v[A.c_off[p] + j] * L2E : exp(A.warm_v[A.c_off[p] + j]);
    if (j >= m) v0 = METHOD == OTG_METHOD_LOG ? T(-INFINITY) : T(0);  // padded columns contribute nothing
    S.v[j] = v0;
  }
  named_bar(3, BT_CONSUMERS);
  T* ucur = S.ua;
  T* ualt = S.ub;
  bool prev_check = false;
  int status = OTG_STATUS_MAXITER, niter = A.max_iter - 1;
  double last_err = -1.0;
  for (int ii = 0;; ++ii) {
    if (ii == A.max_iter && !prev_check) break;
    const bool decide = prev_check || ii == A.max_iter;
    double e2 = 0.0;
    T L[G][VW];
    // ---- first half-step (its result is committed only after the decision)
    if (A.u_first) {
      bt_row_pass<T, METHOD>(S, a, n, m, ldm, c, ucur, ualt, prev_check, e2, gchunk, abort_flag, tmo);
    } else {
      bt_col_pass<T, METHOD, G>(S, n, m, ldm, c, ucur, L, gchunk, abort_flag, tmo);
      if (prev_check) {
#pragma unroll
        for (int g = 0; g < G; ++g)
#pragma unroll
          for (int k = 0; k < VW; ++k) {
            const int j = (g * BT_CONSUMERS + tid) * VW + k;
            if (j < m) {
              double cs = METHOD == OTG_METHOD_LOG ? (double)ex2(S.v[j] + L[g][k]) : (double)(S.v[j] * L[g][k]);
              cs -= (double)b[j];
              e2 += cs * cs;
            }
          }
      }
    }
    named_bar(3, BT_CONSUMERS);
    if (decide) {
      const double tot = bt_reduce(S, e2);
      if (tid == 0) {
        int stop = 0;
        if (prev_check) {
          last_err = sqrt(tot);
          if (last_err < A.stop_thr) { stop = 1; status = OTG_STATUS_CONVERGED; niter = ii - 1; }
        }
        if (!stop && ii == A.max_iter) { stop = 1; status = OTG_STATUS_MAXITER; niter = A.max_iter - 1; }
        if (*(volatile int*)abort_flag) { stop = 1; status = OTG_STATUS_ABORTED; }
        S.ctl[1] = stop;
      }
      named_bar(2, BT_THREADS);  // hands the decision to the producer as well
      if (S.ctl[1]) break;       // state of iteration ii-1 is intact
    }
    // ---- commit the first half-step, run the second
    if (A.u_first) {
      T* t = ucur; ucur = ualt; ualt = t;
      bt_col_pass<T, METHOD, G>(S, n, m, ldm, c, ucur, L, gchunk, abort_flag, tmo);
      named_bar(3, BT_CONSUMERS);
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int k = 0; k < VW; ++k) {
          const int j = (g * BT_CONSUMERS + tid) * VW + k;
          if (j < m) S.v[j] = METHOD == OTG_METHOD_LOG ? lg2(b[j]) - L[g][k] : b[j] / L[g][k];
        }
      named_bar(3, BT_CONSUMERS);
    } else {
#pragma unroll
      for (int g = 0; g < G; ++g)
#pragma unroll
        for (int k = 0; k < VW; ++k) {
          const int j = (g * BT_CONSUMERS + tid) * VW + k;
          if (j < m) S.v[j] = METHOD == OTG_METHOD_LOG ? lg2(b[j]) - L[g][k] : b[j] / L[g][k];
        }
      named_bar(3, BT_CONSUMERS);
      double dummy = 0.0;
      bt_row_pass<T, METHOD>(S, a, n, m, ldm, c, ucur, ucur, false, dummy, gchunk, abort_flag, tmo);
      named_bar(3, BT_CONSUMERS);
    }
    prev_check = (ii % 10 == 0);
  }
  // results in natural units
  const T LN2 = T(OTG_LN2);
  for (int i = tid; i < n; i += BT_CONSUMERS)
    A.out_u[A.r_off[p] + i] = METHOD == OTG_METHOD_LOG ? ucur[i] * LN2 : ucur[i];
  for (int j = tid; j < m; j += BT_CONSUMERS)
    A.out_v[A.c_off[p] + j] = METHOD == OTG_METHOD_LOG ? S.v[j] * LN2 : S.v[j];
  if (tid == 0) { A.status[p] = status; A.niter[p] = niter; A.err[p] = last_err; }
}

// Producer warp: the whole warp follows the consumers' pass and decision
// schedule (so named barriers are reached by all its lanes); lane 0 issues.
template <typename T>
__device__ void bt_produce_problem(const BatchArgs<T>& A, const BtShared<T>& S, int p, uint32_t& gchunk, bool& pok) {
  const int lane = threadIdx.x & 31;
  const int n = A.rows[p], ldm = A.ldm[p];
  const T* Mp = A.M + A.m_off[p];
  int* abort_flag = A.queue + 1;
  bool prev_check = false;
  for (int ii = 0;; ++ii) {
    if (ii == A.max_iter && !prev_check) break;
    const bool decide = prev_check || ii == A.max_iter;
    if (lane == 0 && pok) pok = bt_produce_pass<T>(S, Mp, n, ldm, gchunk, abort_flag, A.timeout_ns);
    __syncwarp();
    if (decide) {
      named_bar(2, BT_THREADS);
      if (S.ctl[1]) break;
    }
    if (lane == 0 && pok) pok = bt_produce_pass<T>(S, Mp, n, ldm, gchunk, abort_flag, A.timeout_ns);
    __syncwarp();
    prev_check = (ii % 10 == 0);
  }
}

template <typename T, int METHOD>
__global__ void __launch_bounds__(BT_THREADS, 1) batched_sinkhorn_kernel(BatchArgs<T> A) {
  extern __shared__ __align__(128) unsigned char smem[];
  const BtShared<T> S = bt_carve<T>(smem);
  const int tid = threadIdx.x;
  int* abort_flag = A.queue + 1;
  if (tid == 0) {
    for (int s = 0; s < BT_STAGES; ++s) { mbar_init(S.full + s, 1); mbar_init(S.empty + s, BT_CONSUMERS / 32); }
    fence_mbar_init();
  }
  __syncthreads();
  uint32_t gchunk = 0;  // chunks issued (producer lane 0) / consumed (consumers)
  bool pok = true;
  while (true) {
    if (tid == 0) S.ctl[0] = *(volatile int*)abort_flag ? A.nprob : atomicAdd(A.queue, 1);
    named_bar(1, BT_THREADS);
    const int k = S.ctl[0];
    named_bar(1, BT_THREADS);  // everyone has read the index before it can change
    if (k >= A.nprob) break;
    const int p = A.order[k];
    if (tid >= BT_CONSUMERS) {
      bt_produce_problem<T>(A, S, p, gchunk, pok);
    } else {
      const int m = A.cols[p];
      const int G = (m + BT_CONSUMERS * Vec<T>::N - 1) / (BT_CONSUMERS * Vec<T>::N);
      if (G <= 1) bt_consume_problem<T, METHOD, 1>(A, S, p, gchunk);
      else if (G <= 2) bt_consume_problem<T, METHOD, 2>(A, S, p, gchunk);
      else bt_consume_problem<T, METHOD, 4>(A, S, p, gchunk);
    }
  }
  // After an abort, wait (bounded) for this CTA's copies still in flight
  // before its shared memory is released.
  if (tid == BT_CONSUMERS && *(volatile int*)abort_flag) {
    const uint32_t lo = gchunk > (uint32_t)BT_STAGES ? gchunk - BT_STAGES : 0u;
    for (uint32_t q = lo; q < gchunk; ++q) {
      const uint64_t t0 = globaltimer();
      while (!mbar_try_wait(S.full + q % BT_STAGES, (q / BT_STAGES) & 1u))
        if (globaltimer() - t0 > A.timeout_ns) break;
    }
  }
}

}  // namespace otg

using namespace otg;

namespace {

template <typename T, int METHOD>
int launch_batched(const OtgBatchProblem* q, cudaStream_t st) {
  BatchArgs<T> A{};
  A.M = static_cast<const T*>(q->M);
  A.m_off = q->m_off; A.rows = q->rows; A.cols = q->cols; A.ldm = q->ldm;
  A.r_off = q->r_off; A.c_off = q->c_off;
  A.a = static_cast<const T*>(q->a); A.b = static_cast<const T*>(q->b);
  A.warm_u = static_cast<const T*>(q->warm_u); A.warm_v = static_cast<const T*>(q->warm_v);
  A.reg = q->reg; A.order = q->order; A.nprob = q->nprob;
  A.max_iter = q->max_iter; A.stop_thr = q->stop_thr; A.u_first = q->u_first;
  A.out_u = static_cast<T*>(q->out_u); A.out_v = static_cast<T*>(q->out_v);
  A.status = q->status; A.niter = q->niter; A.err = q->err; A.queue = q->queue;
  A.timeout_ns = q->timeout_ms > 0 ? (uint64_t)q->timeout_ms * 1000000ull : 4000000000ull;
  const size_t smem = bt_smem_bytes<T>();
  auto kern = batched_sinkhorn_kernel<T, METHOD>;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return OTG_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  int grid = std::min(sms, q->nprob);
  if (q->grid > 0 && q->grid < grid) grid = q->grid;
  if (cudaMemsetAsync(q->queue, 0, 2 * sizeof(int32_t), st) != cudaSuccess) return OTG_ERR_CUDA;
  kern<<<grid, BT_THREADS, smem, st>>>(A);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

}  // namespace

extern "C" {

int otg_batch_limits(int dtype, int32_t* max_rows, int32_t* max_cols, int32_t* row_bytes_max) {
  if (dtype == OTG_F64) {
    *max_rows = BtLimits<double>::NMAX;
    *max_cols = std::min(BtLimits<double>::NMAX, BT_CONSUMERS * 2 * BtLimits<double>::G);
  } else {
    *max_rows = BtLimits<float>::NMAX;
    *max_cols = std::min(BtLimits<float>::NMAX, BT_CONSUMERS * 4 * BtLimits<float>::G);
  }
  *row_bytes_max = (int32_t)BT_STAGE_BYTES;
  return OTG_OK;
}

int otg_sinkhorn_batched(const OtgBatchProblem* q, cudaStream_t stream) {
  if (!q || !q->M || !q->m_off || !q->rows || !q->cols || !q->ldm || !q->r_off || !q->c_off || !q->a || !q->b ||
      !q->reg || !q->order || !q->out_u || !q->out_v || !q->status || !q->niter || !q->err || !q->queue)
    return OTG_ERR_ARG;
  if (q->nprob < 1 || q->max_iter < 0) return OTG_ERR_ARG;
  if (q->method != OTG_METHOD_LOG && q->method != OTG_METHOD_KNOPP) return OTG_ERR_ARG;
  if (q->dtype == OTG_F64)
    return q->method == OTG_METHOD_LOG ? launch_batched<double, OTG_METHOD_LOG>(q, stream)
                                       : launch_batched<double, OTG_METHOD_KNOPP>(q, stream);
  if (q->dtype == OTG_F32)
    return q->method == OTG_METHOD_LOG ? launch_batched<float, OTG_METHOD_LOG>(q, stream)
                                       : launch_batched<float, OTG_METHOD_KNOPP>(q, stream);
  return OTG_ERR_DTYPE;
}

}  // extern "C"
