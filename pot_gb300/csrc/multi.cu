// Work-balanced batched log-domain Sinkhorn: every SM works on every active
// problem in every half-step, so the time follows the batch's total work and
// a slow problem is spread over the whole GPU instead of one CTA.
//
// Reference behaviour (PythonOT/POT): per problem, the order and stopping test
// of ot/bregman/_sinkhorn.py:880-899 (sinkhorn_log: v first, then u; L2
// column-marginal error every 10th iteration); problems stop individually.
// With `joint` the whole batch stops together at the first check whose
// LARGEST error is below the threshold (ot/batch/_utils.py:273-278 and
// :152-157).  The scaling form (LOGF = false) runs the same passes with sums
// of K_ij = exp(-M_ij/reg) products instead of log-sum-exps (the scaling
// iteration of ot/batch/_utils.py:146-151 on the transposed problem).
//
// The squared marginal error of each column is stored in its own slot and
// summed per problem in a fixed order, so a problem's error, and with it
// its stop index, is the same in every run.
//
// Anderson mixing (no reference counterpart; the warm-start refinement).
// The map F(v) = colT(rowT(v)) (a row update followed by a column update)
// has the Sinkhorn potentials as fixed points.  With and_depth = D > 0 the v
// of the next row pass is  sum_k alpha_k F(v_k)  over the last D iterates,
// alpha minimising |sum_k alpha_k (F(v_k) - v_k)|_2 with sum alpha = 1
// (normal equations of the residual Gram matrix with a Tikhonov term
// 1e-10 trace / D; a non-finite or wildly extrapolating solution restarts
// the history with the plain step).  u is always the exact row update of the
// v in use, so the stop test measures exactly what it measures for plain
// sinkhorn_log: the column marginal of (u, v) with u = rowT(v).
//
// One persistent cooperative launch.  Each iteration:
//   column pass : units (problem, row chunk, slab of 32*VW columns) over all
//                 active problems -> partial (max, sum) per column  | barrier
//   column merge: per column of every active problem: combine partials, new
//                 v into the spare buffer, squared marginal error of the
//                 previous check iteration per problem               | barrier
//   decision    : (check iterations) converged problems are written out and
//                 leave the active list                              | barrier
//   row pass    : units (problem, group of RW rows, column chunk) -> u   | barrier
// All active problems share the iteration index, so the v buffers swap
// globally.  Work units map to problems through prefix sums over the active
// list (binary search).
//
// Tail.  Once few problems are left, an iteration costs the latency of its
// grid barriers and dependent loads (~19 us, whatever the grid size), so a
// batch whose last problems are slow to converge spends most of its time
// there.  When at most tail_max problems remain and each fits (about) the
// shared memory of one thread-block cluster, the batch kernel stops at the
// decision point and multi_tail_kernel (launched behind it on the same
// stream) finishes them: one cluster per problem, its cost block resident in
// the CTAs' shared memory (rows beyond a CTA's tile, up to as many again,
// read from the block each pass), column partials merged through
// distributed shared memory and two hardware cluster barriers per
// iteration.  The iteration, the stop test and the outputs are those of the
// batch kernel.
#include <algorithm>
#include <cooperative_groups.h>
#include "common.cuh"
#include "anderson.cuh"
#include "../../include/pot_gb300.h"

namespace cg = cooperative_groups;

namespace otg {

// 256 threads at no more than 64 registers, four CTAs per SM (float): the
// loads in flight come from the 32 resident warps (measured: 0.79 of the copy peak
// against 0.71 for two CTAs of 118 registers with loads software-pipelined
// one group ahead, on 512 cost blocks of 2048 x 2048).
constexpr int MT_THREADS = 256;
// CTAs per SM: float at 64 registers; double keeps 128 registers (no spills)
template <typename T> struct MtBlocks { static constexpr int value = sizeof(T) == 4 ? 4 : 2; };
constexpr int MT_RW = 4;       // rows per warp in the row pass
constexpr int MT_GCOL = 4;     // rows folded per max update (column pass)

template <typename T> struct MPair { T mx, s; };

template <typename T>
struct MultiArgs {
  const T* M; const int64_t* m_off; const int32_t* rows; const int32_t* cols; const int32_t* ldm;
  const int64_t* r_off; const int64_t* c_off;
  const T* a; const T* b; const T* warm_u;
  const double* reg;
  int32_t nprob, max_iter;
  double stop_thr;
  // per-problem decomposition: partial buffers sized for nsr_max row chunks;
  // the split in use (nsr, rchunk) is chosen at every rebuild of the active
  // list from the amount of work left
  const int32_t* nsr_max;
  int32_t* nsr;             // row chunks (column pass), device-chosen
  int32_t* rchunk;          // rows per chunk, device-chosen
  const int64_t* pc_off;    // offset of problem's partials [nsr_max][m]
  // state
  T* u; T* v0; T* v1;       // base-2 potentials, packed like a / b
  MPair<T>* pcol;
  double* err2;             // per problem: squared error of the last check (joint stop)
  double* e2col;            // per column: squared marginal error (check passes), packed like b
  bool joint;               // whole-batch stop on the largest error
  // Anderson mixing of the v update (depth 0: off): history slots of F(v)
  // and of the residual F(v) - v, [depth][total_cols] each (slot-major,
  // packed like b), residual Gram matrices [nprob][depth][depth] and the
  // number of iterates taken so far per problem
  int and_depth;
  int64_t total_cols;
  T* and_F; T* and_R;
  double* and_G;
  int32_t* and_cnt;
  int32_t* active;          // active problem ids [nprob]
  int64_t* ucol_pre;        // prefix of column-pass units over the active list [nprob+1]
  int64_t* urow_pre;        // prefix of row-pass units
  int64_t* colpre;          // prefix of columns (merge) over the active list
  int32_t* ctl;             // [0] n active, [1] abort
  int32_t* leave_cnt;       // [2] problems leaving at a decision (alternate decisions)
  unsigned* bar;
  // outputs
  T* out_u; T* out_v;
  int32_t* status; int32_t* niter; double* err;
  uint64_t timeout_ns;
  T omega;                  // over-relaxation (1: plain)
  bool relax;
  int period;               // iterations between stop tests
  int upw, cap_fill, cap_tail;  // schedule: units per warp, row-split caps
  // tail handoff: most problems handed over (0: never), CTAs per cluster,
  // shared-memory bytes for one CTA's rows of a cost block
  int tail_max, tail_cl;
  int64_t tail_tile;
};

// Tail kernel limits: columns, rows per CTA
constexpr int TL_MAXM = 2048;
constexpr int TL_MAXR = 1024;
constexpr int TL_THREADS = 256;

// Index of the active slot whose prefix range holds `unit` (pre[k] <= unit < pre[k+1]).
__device__ __forceinline__ int mt_find(const int64_t* pre, int n, int64_t unit) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldcg(pre + mid) <= unit) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Slot cursor over a prefix array: pre[k] <= item < pre[k+1].  Items visited
// in increasing order mostly stay in the slot or move to the next one, so the
// binary search (a chain of dependent L2 loads) runs about once per problem.
struct MtSlot {
  int k = -1;
  int64_t lo = 0, hi = 0;
  __device__ __forceinline__ bool seek(const int64_t* pre, int n, int64_t item) {
    if (k >= 0 && item >= lo && item < hi) return false;
    if (k >= 0 && item >= hi && k + 1 < n && __ldcg(pre + k + 2) > item) ++k;
    else k = mt_find(pre, n, item);
    lo = __ldcg(pre + k);
    hi = __ldcg(pre + k + 1);
    return true;
  }
};

// Contiguous share [beg, end) of `total` items for worker w of nw.
__device__ __forceinline__ void mt_share(int64_t total, long w, long nw, int64_t& beg, int64_t& end) {
  beg = total * w / nw;
  end = total * (w + 1) / nw;
}

template <typename T, bool LOGF>
__device__ void mt_col_pass(const MultiArgs<T>& A, int nact, long gwarp, long nwarps, int lane) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  const int64_t total = __ldcg(A.ucol_pre + nact);
  int64_t ubeg, uend;
  mt_share(total, gwarp, nwarps, ubeg, uend);
  MtSlot sl;
  int p = 0, n = 0, m = 0, ldm = 0, rc = 1;
  int64_t nslabs = 1;
  const T* Mp = nullptr;
  const T* up = nullptr;
  T c = 0;
  for (int64_t unit = ubeg; unit < uend; ++unit) {
    if (sl.seek(A.ucol_pre, nact, unit)) {
      p = __ldcg(A.active + sl.k);
      n = A.rows[p]; m = A.cols[p]; ldm = A.ldm[p];
      nslabs = (m + 32 * VW - 1) / (32 * VW);
      rc = __ldcg(A.rchunk + p);
      Mp = A.M + A.m_off[p];
      up = A.u + A.r_off[p];
      c = (T)(-OTG_LOG2E / A.reg[p]);
    }
    const int64_t local = unit - sl.lo;
    const int64_t slab = local % nslabs, r = local / nslabs;  // r < nsr[p]
    const int i0 = (int)(r * rc), i1 = min(n, i0 + rc);
    const int j0 = (int)(slab * 32 * VW) + lane * VW;
    T mx[VW], s[VW];
#pragma unroll
    for (int q = 0; q < VW; ++q) { mx[q] = -INFINITY; s[q] = 0; }
    if (j0 < m) {
      auto load_group = [&](int i, T (&x)[MT_GCOL][VW], T (&ur)[MT_GCOL]) {
#pragma unroll
        for (int g = 0; g < MT_GCOL; ++g) {
          if (i + g < i1) {
            unpack(ld_stream(reinterpret_cast<const V*>(Mp + (int64_t)(i + g) * ldm + j0)), x[g]);
            ur[g] = __ldcg(up + i + g);
          } else {
#pragma unroll
            for (int q = 0; q < VW; ++q) x[g][q] = 0;
            ur[g] = LOGF ? T(-INFINITY) : T(0);
          }
        }
      };
      for (int i = i0; i < i1; i += MT_GCOL) {
        T x[MT_GCOL][VW], ur[MT_GCOL];
        load_group(i, x, ur);
        if constexpr (!LOGF) {
          // scaling form: s_j += K_ij u_i with K_ij = 2^(M_ij c)
#pragma unroll
          for (int q = 0; q < VW; ++q)
#pragma unroll
            for (int g = 0; g < MT_GCOL; ++g) s[q] = fma(ex2(x[g][q] * c), ur[g], s[q]);
        } else {
#pragma unroll
        for (int q = 0; q < VW; ++q) {
          T t[MT_GCOL];
          T gm = -INFINITY;
#pragma unroll
          for (int g = 0; g < MT_GCOL; ++g) { t[g] = fma(x[g][q], c, ur[g]); gm = fmax(gm, t[g]); }
          const T nm = fmax(mx[q], gm);
          if (nm != -INFINITY) {
            T acc = s[q] * ex2(mx[q] - nm);
#pragma unroll
            for (int g = 0; g < MT_GCOL; ++g) acc += ex2(t[g] - nm);
            s[q] = acc;
            mx[q] = nm;
          }
        }
        }
      }
      MPair<T>* pc = A.pcol + A.pc_off[p] + r * m;
#pragma unroll
      for (int q = 0; q < VW; ++q)
        if (j0 + q < m) pc[j0 + q] = MPair<T>{mx[q], s[q]};
    }
  }
}

// Column merge over every column of every active problem; per problem the
// squared marginal error of (u_cur, v_cur) is accumulated when `check`.
template <typename T, bool LOGF>
__device__ void mt_col_merge(const MultiArgs<T>& A, int nact, const T* vcur, T* vnxt, bool check, bool update,
                             long gtid, long nthreads, bool relax_v) {
  const int64_t total = __ldcg(A.colpre + nact);
  // each warp takes a contiguous range of columns, its lanes adjacent ones
  const long w = gtid >> 5, nw = nthreads >> 5;
  const int lane = (int)(gtid & 31);
  const int64_t groups = (total + 31) / 32;
  int64_t gbeg, gend;
  mt_share(groups, w, nw, gbeg, gend);
  MtSlot sl;
  int p = 0, m = 0, nsr = 1;
  const MPair<T>* pc = nullptr;
  for (int64_t e = gbeg * 32 + lane; e < min(gend * 32, total); e += 32) {
    if (sl.seek(A.colpre, nact, e)) {
      p = __ldcg(A.active + sl.k);
      m = A.cols[p];
      pc = A.pcol + A.pc_off[p];
      nsr = __ldcg(A.nsr + p);
    }
    const int j = (int)(e - sl.lo);
    T mx = -INFINITY, s = 0;
    if (LOGF) lse_merge_strided(mx, s, reinterpret_cast<const T*>(pc + j), 2 * (int64_t)m, nsr);
    else s = sum_strided(reinterpret_cast<const T*>(pc + j), 2 * (int64_t)m, nsr);
    const T L = LOGF ? lse_value(mx, s) : s;
    const int64_t cj = A.c_off[p] + j;
    const T bj = A.b[cj];
    if (check) {
      // column marginal of the iterate (u_cur, v_cur), in the column's own slot
      const double cs = (LOGF ? (double)ex2(__ldcg(vcur + cj) + L) : (double)(__ldcg(vcur + cj) * L)) - (double)bj;
      A.e2col[cj] = cs * cs;
    }
    if (update) {
      const T vn = LOGF ? lg2(bj) - L : bj / L;
      vnxt[cj] = relax_v ? fma(A.omega, vn - __ldcg(vcur + cj), __ldcg(vcur + cj)) : vn;
    }
  }
}

template <typename T, bool LOGF>
__device__ void mt_row_pass(const MultiArgs<T>& A, int nact, const T* v, long gwarp, long nwarps, int lane) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  const int64_t total = __ldcg(A.urow_pre + nact);
  int64_t ubeg, uend;
  mt_share(total, gwarp, nwarps, ubeg, uend);
  MtSlot sl;
  int p = 0, n = 0, m = 0, ldm = 0;
  const T* Mp = nullptr;
  const T* vp = nullptr;
  T c = 0;
  for (int64_t unit = ubeg; unit < uend; ++unit) {
    if (sl.seek(A.urow_pre, nact, unit)) {
      p = __ldcg(A.active + sl.k);
      n = A.rows[p]; m = A.cols[p]; ldm = A.ldm[p];
      Mp = A.M + A.m_off[p];
      vp = v + A.c_off[p];
      c = (T)(-OTG_LOG2E / A.reg[p]);
    }
    const int64_t grp = unit - sl.lo;
    const int r0 = (int)grp * MT_RW;
    T mx[MT_RW], s[MT_RW];
#pragma unroll
    for (int r = 0; r < MT_RW; ++r) { mx[r] = -INFINITY; s[r] = 0; }
    auto load_step = [&](int j, T (&x)[MT_RW][VW], T (&vv)[VW]) {
      // v beyond m (padding up to ldm) is masked out (-inf, or 0 for scalings)
#pragma unroll
      for (int q = 0; q < VW; ++q) vv[q] = (j + q < m) ? __ldcg(vp + j + q) : (LOGF ? T(-INFINITY) : T(0));
#pragma unroll
      for (int r = 0; r < MT_RW; ++r) {
        const int row = min(r0 + r, n - 1);
        unpack(ld_stream(reinterpret_cast<const V*>(Mp + (int64_t)row * ldm + j)), x[r]);
      }
    };
    for (int j = lane * VW; j < m; j += 32 * VW) {
      T vv[VW];
      T x[MT_RW][VW];
      load_step(j, x, vv);
      if constexpr (!LOGF) {
#pragma unroll
        for (int r = 0; r < MT_RW; ++r)
#pragma unroll
          for (int q = 0; q < VW; ++q) s[r] = fma(ex2(x[r][q] * c), vv[q], s[r]);
      } else {
#pragma unroll
      for (int r = 0; r < MT_RW; ++r) {
        T t[VW];
        T gm = -INFINITY;
#pragma unroll
        for (int q = 0; q < VW; ++q) { t[q] = fma(x[r][q], c, vv[q]); gm = fmax(gm, t[q]); }
        const T nm = fmax(mx[r], gm);
        if (nm != -INFINITY) {
          T acc = s[r] * ex2(mx[r] - nm);
#pragma unroll
          for (int q = 0; q < VW; ++q) acc += ex2(t[q] - nm);
          s[r] = acc;
          mx[r] = nm;
        }
      }
      }
    }
#pragma unroll
    for (int r = 0; r < MT_RW; ++r) {
      if (LOGF) warp_lse(mx[r], s[r]);
      else s[r] = warp_sum(s[r]);
    }
#pragma unroll
    for (int r = 0; r < MT_RW; ++r) {
      if (lane == r && r0 + r < n) {
        const int64_t ri = A.r_off[p] + r0 + r;
        const T un = LOGF ? lg2(A.a[ri]) - lse_value(mx[r], s[r]) : A.a[ri] / s[r];
        A.u[ri] = A.relax ? fma(A.omega, un - __ldcg(A.u + ri), __ldcg(A.u + ri)) : un;
      }
    }
  }
}

// Rebuild the active list and its prefix sums (one CTA, block-wide scan).
// Problems whose flag is set leave the list.
template <typename T>
__device__ void mt_rebuild(const MultiArgs<T>& A, int nact, const int32_t* leaving, int* s_scan, int64_t nwarps) {
  // serial in chunks of blockDim: scan of keep flags
  __shared__ int s_base;
  __shared__ int64_t s_ucol, s_urow, s_col;
  constexpr int VW = Vec<T>::N;
  if (threadIdx.x == 0) { s_base = 0; s_ucol = 0; s_urow = 0; s_col = 0; }
  __syncthreads();
  for (int c0 = 0; c0 < nact; c0 += blockDim.x) {
    const int k = c0 + threadIdx.x;
    int p = -1, keep = 0;
    if (k < nact) { p = __ldcg(A.active + k); keep = leaving[p] ? 0 : 1; }
    s_scan[threadIdx.x] = keep;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
      const int add = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
      __syncthreads();
      s_scan[threadIdx.x] += add;
      __syncthreads();
    }
    const int pos = s_base + s_scan[threadIdx.x] - keep;
    if (keep) A.active[pos] = p;  // compaction never overtakes the reads of this chunk
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) s_base += s_scan[threadIdx.x];
    __syncthreads();
  }
  // split factor: about upw (default 8) column-pass units per warp over the
  // remaining work
  __shared__ int64_t s_slabs;
  if (threadIdx.x == 0) s_slabs = 0;
  __syncthreads();
  {
    int64_t part = 0;
    for (int k = threadIdx.x; k < s_base; k += blockDim.x) {
      const int m = A.cols[__ldcg(A.active + k)];
      part += (m + 32 * VW - 1) / (32 * VW);
    }
    atomicAdd(reinterpret_cast<unsigned long long*>(&s_slabs), (unsigned long long)part);
  }
  __syncthreads();
  // capped at cap_fill (16) chunks while the batch fills the GPU (more
  // splits only lengthen the merge); a few remaining problems split up to
  // cap_tail (64) ways, since then the time per pass is that of one unit
  int64_t S = s_slabs > 0 ? ((int64_t)A.upw * nwarps + s_slabs - 1) / s_slabs : 1;
  const int64_t cap = s_slabs * A.cap_fill >= nwarps ? A.cap_fill : A.cap_tail;
  S = S > cap ? cap : S;
  for (int k = threadIdx.x; k < s_base; k += blockDim.x) {
    const int p = A.active[k];
    const int n = A.rows[p];
    const int ns = (int)(S < (int64_t)A.nsr_max[p] ? S : (int64_t)A.nsr_max[p]);
    const int rc = (n + ns - 1) / ns;
    A.rchunk[p] = rc;
    A.nsr[p] = (n + rc - 1) / rc;
  }
  __syncthreads();
  // prefix sums of units and columns over the new list: block-wide scans
  // (warp shuffles, then the warp totals), chunk by chunk with running bases
  __shared__ int64_t s_wt[3][MT_THREADS / 32];
  __shared__ int64_t s_run[3];
  if (threadIdx.x == 0) { s_run[0] = 0; s_run[1] = 0; s_run[2] = 0; }
  __syncthreads();
  const int na = s_base;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwb = blockDim.x >> 5;
  for (int c0 = 0; c0 < na; c0 += blockDim.x) {
    const int k = c0 + threadIdx.x;
    int64_t own[3] = {0, 0, 0};
    if (k < na) {
      const int p = A.active[k];
      const int m = A.cols[p];
      own[0] = (int64_t)((m + 32 * VW - 1) / (32 * VW)) * A.nsr[p];
      own[1] = (A.rows[p] + MT_RW - 1) / MT_RW;
      own[2] = m;
    }
    int64_t inc[3] = {own[0], own[1], own[2]};
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int64_t up = __shfl_up_sync(0xffffffffu, inc[q], o);
        if (lane >= o) inc[q] += up;
      }
    }
    if (lane == 31) { s_wt[0][wid] = inc[0]; s_wt[1][wid] = inc[1]; s_wt[2][wid] = inc[2]; }
    __syncthreads();
    int64_t before[3] = {s_run[0], s_run[1], s_run[2]};
    for (int w = 0; w < wid; ++w) { before[0] += s_wt[0][w]; before[1] += s_wt[1][w]; before[2] += s_wt[2][w]; }
    if (k < na) {
      A.ucol_pre[k] = before[0] + inc[0] - own[0];
      A.urow_pre[k] = before[1] + inc[1] - own[1];
      A.colpre[k] = before[2] + inc[2] - own[2];
    }
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < nwb; ++w) { s_run[0] += s_wt[0][w]; s_run[1] += s_wt[1][w]; s_run[2] += s_wt[2][w]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    A.ucol_pre[na] = s_run[0]; A.urow_pre[na] = s_run[1]; A.colpre[na] = s_run[2];
    // hand the rest to the tail kernel when every remaining block fits a cluster
    int tail = A.tail_max > 0 && na > 0 && na <= A.tail_max;
    for (int k = 0; tail && k < na; ++k) {
      const int p = A.active[k];
      const int64_t rcap = (A.rows[p] + A.tail_cl - 1) / A.tail_cl;
      // rows beyond the shared tile are streamed: up to twice the tile per CTA
      if (A.cols[p] > TL_MAXM || rcap > TL_MAXR || rcap * A.ldm[p] * (int64_t)sizeof(T) > 2 * A.tail_tile) tail = 0;
    }
    A.ctl[2] = tail;
    A.ctl[0] = na;
    __threadfence();
  }
  __syncthreads();
}

// Anderson step (one CTA per active problem, anderson.cuh): the new v of
// every active problem is mixed over its history.  Kept out of line, like
// the joint decision: it must not weigh on the registers of the passes.
template <typename T>
__device__ __noinline__ void mt_anderson(const MultiArgs<T>& A, int nact, const T* vcur, T* vnxt) {
  for (int k = blockIdx.x; k < nact; k += gridDim.x) {
    const int p = __ldcg(A.active + k);
    anderson_step<T>(A.and_depth, A.cols[p], A.c_off[p], A.total_cols, vcur, vnxt, A.and_F, A.and_R,
                     A.and_G + (int64_t)p * A.and_depth * A.and_depth, A.and_cnt + p);
  }
}

// Whole-batch stop decision (joint mode): every problem's error into
// err2[p] (its column slots summed in a fixed order), then the largest over
// the batch (a max: the same in any order).  Returns 1 when the batch stops,
// 0 when it goes on, -1 when a grid barrier gave up.  Kept out of line: it
// runs once per check and its registers must not weigh on the passes.
template <typename T>
__device__ __noinline__ int mt_joint_decision(const MultiArgs<T>& A, int nact) {
  for (int k = blockIdx.x; k < nact; k += gridDim.x) {
    const int p = __ldcg(A.active + k);
    const double e2 = block_sum_slots(A.e2col + A.c_off[p], A.cols[p]);
    if (threadIdx.x == 0) A.err2[p] = e2;
  }
  if (!grid_barrier(A.bar, gridDim.x, A.ctl + 1, A.timeout_ns)) return -1;
  __shared__ double s_mx[MT_THREADS / 32];
  double mx = 0.0;
  for (int k = threadIdx.x; k < nact; k += blockDim.x) {
    const double e2 = __ldcg(A.err2 + __ldcg(A.active + k));
    mx = isnan(e2) ? (double)INFINITY : fmax(mx, e2);  // a NaN error never meets the test
  }
  mx = warp_max(mx);
  if ((threadIdx.x & 31) == 0) s_mx[threadIdx.x >> 5] = mx;
  __syncthreads();
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) mx = fmax(mx, s_mx[w]);
  __syncthreads();
  return sqrt(mx) < A.stop_thr ? 1 : 0;
}

template <typename T, bool LOGF>
__global__ void __launch_bounds__(MT_THREADS, MtBlocks<T>::value) multi_sinkhorn_kernel(MultiArgs<T> A, int32_t* leaving) {
  __shared__ int s_scan[MT_THREADS];
  const int lane = threadIdx.x & 31;
  const long nwb = blockDim.x >> 5;
  const long gwarp = blockIdx.x * nwb + (threadIdx.x >> 5);
  const long nwarps = gridDim.x * nwb;
  const long gtid = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long nthreads = (long)gridDim.x * blockDim.x;
  int* abort_flag = A.ctl + 1;
  const T L2E = T(OTG_LOG2E);
  // outputs: natural-log potentials (log form) or the scalings themselves
  const T OUTF = LOGF ? T(OTG_LN2) : T(1);
  // initial state: u from the warm start (natural log) or zero log / unit scaling
  for (int p = blockIdx.x; p < A.nprob; p += gridDim.x) {
    const int n = A.rows[p], m = A.cols[p];
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const int64_t ri = A.r_off[p] + i;
      if (LOGF) A.u[ri] = A.warm_u ? A.warm_u[ri] * L2E : T(0);
      else A.u[ri] = A.warm_u ? exp(A.warm_u[ri]) : T(1);
    }
    for (int j = threadIdx.x; j < m; j += blockDim.x) A.v0[A.c_off[p] + j] = LOGF ? T(0) : T(1);
    if (threadIdx.x == 0) {
      leaving[p] = 0;
      A.err2[p] = 0.0;
      if (A.and_depth > 0) A.and_cnt[p] = 0;
    }
  }
  if (blockIdx.x == 0) {
    for (int k = threadIdx.x; k < A.nprob; k += blockDim.x) A.active[k] = k;
  }
  if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
  if (blockIdx.x == 0) mt_rebuild<T>(A, A.nprob, leaving, s_scan, nwarps);
  if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;

  T* vcur = A.v0;
  T* vnxt = A.v1;
  bool prev_check = false;
  int ndec = 0;  // decisions taken (the same count in every CTA)
  for (int ii = 0;; ++ii) {
    const int nact = ld_acquire_i(A.ctl);
    if (nact == 0) break;
    const bool decide = prev_check || ii == A.max_iter;
    if (ii == A.max_iter && !prev_check) {
      // every active problem ends without a final check (state of ii-1)
      for (int k = blockIdx.x; k < nact; k += gridDim.x) {
        const int p = __ldcg(A.active + k);
        for (int i = threadIdx.x; i < A.rows[p]; i += blockDim.x) A.out_u[A.r_off[p] + i] = __ldcg(A.u + A.r_off[p] + i) * OUTF;
        for (int j = threadIdx.x; j < A.cols[p]; j += blockDim.x) A.out_v[A.c_off[p] + j] = __ldcg(vcur + A.c_off[p] + j) * OUTF;
        if (threadIdx.x == 0) { A.status[p] = OTG_STATUS_MAXITER; A.niter[p] = A.max_iter - 1; A.err[p] = -1.0; }
      }
      break;
    }
    mt_col_pass<T, LOGF>(A, nact, gwarp, nwarps, lane);
    if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
    // the first v comes from u alone (v0 is not an iterate): relaxed from the second on
    mt_col_merge<T, LOGF>(A, nact, vcur, vnxt, prev_check, ii < A.max_iter, gtid, nthreads, A.relax && ii > 0);
    if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
    if (decide) {
      // per-problem errors: the problem's column slots summed in a fixed order
      bool joint_conv = false;
      if (A.joint && prev_check) {
        const int jc = mt_joint_decision<T>(A, nact);
        if (jc < 0) return;
        joint_conv = jc == 1;
      }
      // decide per problem, write out the leaving ones (state of iteration ii-1)
      int nleave = 0;
      for (int k = blockIdx.x; k < nact; k += gridDim.x) {
        const int p = __ldcg(A.active + k);
        double e = -1.0;
        if (prev_check) e = sqrt(A.joint ? __ldcg(A.err2 + p) : block_sum_slots(A.e2col + A.c_off[p], A.cols[p]));
        const bool conv = prev_check && (A.joint ? joint_conv : e < A.stop_thr);
        const bool leave = conv || ii == A.max_iter;
        if (leave) {
          for (int i = threadIdx.x; i < A.rows[p]; i += blockDim.x) A.out_u[A.r_off[p] + i] = __ldcg(A.u + A.r_off[p] + i) * OUTF;
          for (int j = threadIdx.x; j < A.cols[p]; j += blockDim.x) A.out_v[A.c_off[p] + j] = __ldcg(vcur + A.c_off[p] + j) * OUTF;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
          if (leave) {
            A.status[p] = conv ? OTG_STATUS_CONVERGED : OTG_STATUS_MAXITER;
            A.niter[p] = conv ? ii - 1 : A.max_iter - 1;
            A.err[p] = e;
          }
          leaving[p] = leave ? 1 : 0;
          nleave += leave ? 1 : 0;
        }
      }
      if (threadIdx.x == 0 && nleave) atomicAdd(A.leave_cnt + (ndec & 1), nleave);
      if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      // the active list and its prefix sums change only when a problem left
      const bool changed = ld_acquire_i(A.leave_cnt + (ndec & 1)) != 0;
      // the other counter was last read a decision ago: ready for the next one
      if (blockIdx.x == 0 && threadIdx.x == 0) A.leave_cnt[(ndec + 1) & 1] = 0;
      ++ndec;
      if (changed) {
        if (blockIdx.x == 0) mt_rebuild<T>(A, nact, leaving, s_scan, nwarps);
        if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      }
      if (ld_acquire_i(A.ctl) == 0) break;
      if (ld_acquire_i(A.ctl + 2)) {
        // handoff: v of iteration ii is in vnxt, u of ii-1 in A.u; the tail
        // kernel continues with this iteration's row pass
        if (blockIdx.x == 0 && threadIdx.x == 0) {
          A.ctl[3] = ii;
          A.ctl[4] = vnxt == A.v1 ? 1 : 0;
          __threadfence();
          A.ctl[5] = 1;
        }
        break;
      }
    }
    if constexpr (LOGF) {
      // Anderson mixing of the new v (from the second iteration on: the first
      // v comes from u alone and is not an iterate of the map)
      if (A.and_depth > 0 && ii >= 1) {
        mt_anderson<T>(A, ld_acquire_i(A.ctl), vcur, vnxt);
        if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
      }
    }
    { T* t = vcur; vcur = vnxt; vnxt = t; }
    const int nact2 = ld_acquire_i(A.ctl);
    mt_row_pass<T, LOGF>(A, nact2, vcur, gwarp, nwarps, lane);
    if (!grid_barrier(A.bar, gridDim.x, abort_flag, A.timeout_ns)) return;
    prev_check = (ii % A.period == 0);
  }
}

// Shared-memory layout of one tail CTA: its rows of the cost block (tile),
// then column partials, row-group scratch, the full v, its share of the new
// v, its rows' u and log2(a), and its squared-error partial.
template <typename T>
struct TailSmem {
  static constexpr int VW = Vec<T>::N;
  static constexpr size_t part = sizeof(MPair<T>) * TL_MAXM;
  static constexpr size_t scratch = sizeof(MPair<T>) * 16 * 32 * VW;
  static constexpr size_t vec = sizeof(T) * TL_MAXM;
  static constexpr size_t rows = sizeof(T) * TL_MAXR;
  static constexpr size_t aux = part + scratch + 2 * vec + 2 * rows + 16;
};

// One handed-over problem (slot q of the active list), solved by the calling
// cluster to its end; every CTA of the cluster calls it.
template <typename T>
__device__ void tail_solve(const MultiArgs<T>& A, int q, cg::cluster_group& cl) {
  constexpr int VW = Vec<T>::N;
  using V = typename Vec<T>::type;
  using SM = TailSmem<T>;
  extern __shared__ __align__(16) unsigned char tl_smem[];
  const int CL = (int)cl.num_blocks();
  const int rank = (int)cl.block_rank();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, tid = threadIdx.x;
  const int p = __ldcg(A.active + q);
  const int n = A.rows[p], m = A.cols[p], ldm = A.ldm[p];
  const int rcap = (n + CL - 1) / CL;
  const int i0 = min(n, rank * rcap), i1 = min(n, i0 + rcap), nr = i1 - i0;
  const int jb = (int)((int64_t)m * rank / CL), je = (int)((int64_t)m * (rank + 1) / CL);
  const T c = (T)(-OTG_LOG2E / A.reg[p]);
  const T L2E = T(OTG_LOG2E), LN2 = T(OTG_LN2);
  const int64_t ro = A.r_off[p], co = A.c_off[p];
  const size_t tile_bytes = (size_t)A.tail_tile;
  T* tile = reinterpret_cast<T*>(tl_smem);
  MPair<T>* part = reinterpret_cast<MPair<T>*>(tl_smem + tile_bytes);
  MPair<T>* scr = reinterpret_cast<MPair<T>*>(tl_smem + tile_bytes + SM::part);
  T* vfull = reinterpret_cast<T*>(tl_smem + tile_bytes + SM::part + SM::scratch);
  T* vshare = vfull + TL_MAXM;
  T* us = vshare + TL_MAXM;
  T* las = us + TL_MAXR;
  double* errp = reinterpret_cast<double*>(las + TL_MAXR);
  __shared__ double s_red[TL_THREADS / 32];
  // the first nres rows live in the tile, the rest are read from the cost block
  const T* gM = A.M + A.m_off[p] + (int64_t)i0 * ldm;
  const int nres = min(nr, (int)(tile_bytes / ((size_t)ldm * sizeof(T))));
  auto ldrow = [&](int i, int j) -> V {
    if (i < nres) return *reinterpret_cast<const V*>(tile + (int64_t)i * ldm + j);
    return ld_stream(reinterpret_cast<const V*>(gM + (int64_t)i * ldm + j));
  };
  (void)L2E;

  // load this CTA's rows of the cost block, its u, log2(a), and v of the handoff
  {
    const V* src = reinterpret_cast<const V*>(gM);
    V* dst = reinterpret_cast<V*>(tile);
    const int64_t nv = (int64_t)nres * ldm / VW;
    for (int64_t k = tid; k < nv; k += TL_THREADS) dst[k] = ld_stream(src + k);
    for (int i = tid; i < nr; i += TL_THREADS) {
      us[i] = __ldcg(A.u + ro + i0 + i);
      las[i] = lg2(A.a[ro + i0 + i]);
    }
    const T* vh = (__ldcg(A.ctl + 4) ? A.v1 : A.v0) + co;
    for (int j = tid; j < m; j += TL_THREADS) vfull[j] = __ldcg(vh + j);
  }
  cl.sync();

  // row pass over this CTA's rows with vfull; u relaxed like the batch kernel
  auto row_pass = [&]() {
    const int groups = (nr + MT_RW - 1) / MT_RW;
    for (int grp = warp; grp < groups; grp += TL_THREADS / 32) {
      const int r0 = grp * MT_RW;
      T mx[MT_RW], s[MT_RW];
#pragma unroll
      for (int r = 0; r < MT_RW; ++r) { mx[r] = -INFINITY; s[r] = 0; }
      for (int j = lane * VW; j < m; j += 32 * VW) {
        T vv[VW];
#pragma unroll
        for (int k = 0; k < VW; ++k) vv[k] = (j + k < m) ? vfull[j + k] : T(-INFINITY);
#pragma unroll
        for (int r = 0; r < MT_RW; ++r) {
          const int row = min(r0 + r, nr - 1);
          T x[VW];
          unpack(ldrow(row, j), x);
          T t[VW];
          T gm = -INFINITY;
#pragma unroll
          for (int k = 0; k < VW; ++k) { t[k] = fma(x[k], c, vv[k]); gm = fmax(gm, t[k]); }
          const T nm = fmax(mx[r], gm);
          if (nm != -INFINITY) {
            T acc = s[r] * ex2(mx[r] - nm);
#pragma unroll
            for (int k = 0; k < VW; ++k) acc += ex2(t[k] - nm);
            s[r] = acc;
            mx[r] = nm;
          }
        }
      }
#pragma unroll
      for (int r = 0; r < MT_RW; ++r) warp_lse(mx[r], s[r]);
#pragma unroll
      for (int r = 0; r < MT_RW; ++r) {
        if (lane == r && r0 + r < nr) {
          const T un = las[r0 + r] - lse_value(mx[r], s[r]);
          us[r0 + r] = A.relax ? fma(A.omega, un - us[r0 + r], us[r0 + r]) : un;
        }
      }
    }
    __syncthreads();
  };

  // column pass: partial (max, sum) per column over this CTA's rows -> part
  auto col_pass = [&]() {
    const int nslabs = (m + 32 * VW - 1) / (32 * VW);
    const int RG = nslabs >= 8 ? 1 : (8 + nslabs - 1) / nslabs;
    for (int unit = warp; unit < nslabs * RG; unit += TL_THREADS / 32) {
      const int slab = unit % nslabs, g = unit / nslabs;
      const int ra = nr * g / RG, rb = nr * (g + 1) / RG;
      const int j0 = slab * 32 * VW + lane * VW;
      T mx[VW], s[VW];
#pragma unroll
      for (int k = 0; k < VW; ++k) { mx[k] = -INFINITY; s[k] = 0; }
      if (j0 < m) {
        for (int i = ra; i < rb; i += MT_GCOL) {
          T x[MT_GCOL][VW], ur[MT_GCOL];
#pragma unroll
          for (int gg = 0; gg < MT_GCOL; ++gg) {
            if (i + gg < rb) {
              unpack(ldrow(i + gg, j0), x[gg]);
              ur[gg] = us[i + gg];
            } else {
#pragma unroll
              for (int k = 0; k < VW; ++k) x[gg][k] = 0;
              ur[gg] = -INFINITY;
            }
          }
#pragma unroll
          for (int k = 0; k < VW; ++k) {
            T t[MT_GCOL];
            T gm = -INFINITY;
#pragma unroll
            for (int gg = 0; gg < MT_GCOL; ++gg) { t[gg] = fma(x[gg][k], c, ur[gg]); gm = fmax(gm, t[gg]); }
            const T nm = fmax(mx[k], gm);
            if (nm != -INFINITY) {
              T acc = s[k] * ex2(mx[k] - nm);
#pragma unroll
              for (int gg = 0; gg < MT_GCOL; ++gg) acc += ex2(t[gg] - nm);
              s[k] = acc;
              mx[k] = nm;
            }
          }
        }
        MPair<T>* dst = RG == 1 ? part : scr + (int64_t)g * m;
#pragma unroll
        for (int k = 0; k < VW; ++k)
          if (j0 + k < m) dst[j0 + k] = MPair<T>{mx[k], s[k]};
      }
    }
    __syncthreads();
    if (RG > 1) {
      for (int j = tid; j < m; j += TL_THREADS) {
        T mx = -INFINITY, s = 0;
        for (int g = 0; g < RG; ++g) lse_merge(mx, s, scr[(int64_t)g * m + j].mx, scr[(int64_t)g * m + j].s);
        part[j] = MPair<T>{mx, s};
      }
      __syncthreads();
    }
  };

  auto write_out = [&](int status, int niter, double e) {
    for (int i = tid; i < nr; i += TL_THREADS) A.out_u[ro + i0 + i] = us[i] * LN2;
    if (rank == 0) {
      for (int j = tid; j < m; j += TL_THREADS) A.out_v[co + j] = vfull[j] * LN2;
      if (tid == 0) { A.status[p] = status; A.niter[p] = niter; A.err[p] = e; }
    }
  };

  const int ii0 = __ldcg(A.ctl + 3);
  row_pass();
  bool prev_check = (ii0 % A.period == 0);
  for (int it = ii0 + 1;; ++it) {
    if (it == A.max_iter && !prev_check) {
      cl.sync();  // no CTA leaves while another may still read its shared memory
      write_out(OTG_STATUS_MAXITER, A.max_iter - 1, -1.0);
      return;
    }
    col_pass();
    cl.sync();
    // merge this CTA's share of the columns; new v into vshare
    double e2 = 0.0;
    const bool update = it < A.max_iter;
    for (int j = jb + tid; j < je; j += TL_THREADS) {
      T mx = -INFINITY, s = 0;
      for (int r2 = 0; r2 < CL; ++r2) {
        const MPair<T> pr = cl.map_shared_rank(part, r2)[j];
        lse_merge(mx, s, pr.mx, pr.s);
      }
      const T L = lse_value(mx, s);
      const T bj = A.b[co + j];
      if (prev_check) {
        const double cs = (double)ex2(vfull[j] + L) - (double)bj;
        e2 += cs * cs;
      }
      if (update) {
        const T vn = lg2(bj) - L;
        vshare[j] = A.relax ? fma(A.omega, vn - vfull[j], vfull[j]) : vn;
      }
    }
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    if (lane == 0) s_red[warp] = e2;
    __syncthreads();
    if (tid == 0) {
      double t = 0.0;
      for (int w = 0; w < TL_THREADS / 32; ++w) t += s_red[w];
      *errp = t;
    }
    cl.sync();
    if (prev_check || it == A.max_iter) {
      double t = 0.0;
      for (int r2 = 0; r2 < CL; ++r2) t += *cl.map_shared_rank(errp, r2);
      const double e = prev_check ? sqrt(t) : -1.0;
      const bool conv = prev_check && e < A.stop_thr;
      if (conv || it == A.max_iter) {
        cl.sync();
        write_out(conv ? OTG_STATUS_CONVERGED : OTG_STATUS_MAXITER, conv ? it - 1 : A.max_iter - 1, e);
        return;
      }
    }
    // gather the new v from the owners of its shares
    for (int j = tid; j < m; j += TL_THREADS) {
      const int owner = (int)(((int64_t)(j + 1) * CL + m - 1) / m) - 1;
      vfull[j] = cl.map_shared_rank(vshare, owner)[j];
    }
    __syncthreads();
    row_pass();
    prev_check = (it % A.period == 0);
  }
}

// Tail workers: each cluster takes handed-over problems from a queue (slot
// counter in the control block) until none is left, so more problems than
// resident clusters can be handed over.
template <typename T>
__global__ void __launch_bounds__(TL_THREADS) multi_tail_kernel(MultiArgs<T> A) {
  cg::cluster_group cl = cg::this_cluster();
  // uniform over the grid: written by the batch kernel before it ended
  if (__ldcg(A.ctl + 5) == 0 || __ldcg(A.ctl + 1) != 0) return;
  const int nact = __ldcg(A.ctl);
  __shared__ int s_q;
  for (;;) {
    if (cl.block_rank() == 0 && threadIdx.x == 0) s_q = atomicAdd(A.ctl + 6, 1);
    cl.sync();
    const int q = *cl.map_shared_rank(&s_q, 0);
    cl.sync();  // every CTA has read rank 0's slot before rank 0 moves on or leaves
    if (q >= nact) return;
    tail_solve<T>(A, q, cl);
  }
}

}  // namespace otg

using namespace otg;

namespace {
// Cluster shape of the tail kernel on this device: 16 CTAs per cluster when
// the device schedules such clusters at full shared memory, else 8 (the
// portable size); max = clusters resident at once (the tail workers).
// Queried once per device and type.
struct TailCfg { int cl = 0, max = 0; size_t smem = 0; int64_t tile = 0; int err = 0; };

template <typename T>
TailCfg tail_config() {
  static TailCfg cache[16];
  static bool known[16] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= 16) return TailCfg{};
  if (known[dev]) return cache[dev];
  TailCfg tc;
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t smem = optin > 1024 ? (size_t)optin - 1024 : 0;  // room for the static shared arrays
  cudaError_t e0 = smem > TailSmem<T>::aux + 16 * 1024
                       ? cudaFuncSetAttribute(multi_tail_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                       : cudaErrorInvalidValue;
  tc.err = (int)e0;
  if (e0 == cudaSuccess) {
    cudaFuncSetAttribute(multi_tail_kernel<T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    for (int cl : {16, 8}) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3((unsigned)cl);
      cfg.blockDim = dim3(TL_THREADS);
      cfg.dynamicSmemBytes = smem;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = (unsigned)cl;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      cfg.attrs = at;
      cfg.numAttrs = 1;
      int ncl = 0;
      const cudaError_t eq = cudaOccupancyMaxActiveClusters(&ncl, multi_tail_kernel<T>, &cfg);
      tc.err = (int)eq;
      if (eq == cudaSuccess && ncl >= 1) {
        tc.cl = cl;
        tc.max = ncl;
        tc.smem = smem;
        tc.tile = (int64_t)((smem - TailSmem<T>::aux) / 16 * 16);
        break;
      }
    }
  }
  cudaGetLastError();  // a refused attribute or query leaves no error behind
  cache[dev] = tc;
  known[dev] = true;
  return tc;
}

// Device bytes of the Anderson history: F and residual slots, Gram matrices, counts.
size_t anderson_ws_bytes(size_t es, int64_t nprob, int64_t cols, int depth) {
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  return 2 * r(es * (size_t)depth * (size_t)cols) + r(8 * (size_t)nprob * depth * depth) + r(4 * (size_t)nprob);
}

template <typename T, bool LOGF>
int launch_multi(const OtgMultiProblem* q, cudaStream_t st) {
  MultiArgs<T> A{};
  A.M = static_cast<const T*>(q->M); A.m_off = q->m_off; A.rows = q->rows; A.cols = q->cols; A.ldm = q->ldm;
  A.r_off = q->r_off; A.c_off = q->c_off;
  A.a = static_cast<const T*>(q->a); A.b = static_cast<const T*>(q->b); A.warm_u = static_cast<const T*>(q->warm_u);
  A.reg = q->reg; A.nprob = q->nprob; A.max_iter = q->max_iter; A.stop_thr = q->stop_thr;
  A.nsr_max = q->nsr_max; A.pc_off = q->pc_off;
  A.out_u = static_cast<T*>(q->out_u); A.out_v = static_cast<T*>(q->out_v);
  A.status = q->status; A.niter = q->niter; A.err = q->err;
  A.timeout_ns = q->timeout_ms > 0 ? (uint64_t)q->timeout_ms * 1000000ull : 4000000000ull;
  A.and_depth = LOGF ? q->anderson_depth : 0;
  A.total_cols = q->total_cols;
  A.relax = LOGF && A.and_depth == 0 && q->omega != 0.0 && q->omega != 1.0;
  A.joint = q->joint_stop != 0;
  A.omega = (T)q->omega;
  A.period = q->check_period > 0 ? q->check_period : 10;
  A.upw = q->units_per_warp > 0 ? std::min(q->units_per_warp, 1024) : 8;
  A.cap_fill = q->split_cap_fill > 0 ? std::min(q->split_cap_fill, 64) : 16;
  A.cap_tail = q->split_cap_tail > 0 ? std::min(q->split_cap_tail, 64) : 64;
  const TailCfg tc = tail_config<T>();
  A.tail_cl = tc.cl;
  A.tail_tile = tc.tile;
  // float64 passes are bound by FP64 throughput, which every SM of the batch
  // kernel supplies and one cluster per problem does not: no default handoff
  const int def_tail = sizeof(T) == 8 ? 0 : 3 * tc.max;
  A.tail_max = q->tail_problems < 0 || tc.cl == 0 ? 0 : (q->tail_problems > 0 ? q->tail_problems : def_tail);
  // the whole-batch stop keeps every problem to the end; the tail kernel runs
  // the plain or over-relaxed log form only
  if (A.joint || !LOGF || A.and_depth > 0) A.tail_max = 0;
  // carve the workspace
  char* w = static_cast<char*>(q->workspace);
  size_t off = 0;
  auto take = [&](size_t bytes) { char* p = w + off; off += (bytes + 255) / 256 * 256; return p; };
  A.u = reinterpret_cast<T*>(take(sizeof(T) * q->total_rows));
  A.v0 = reinterpret_cast<T*>(take(sizeof(T) * q->total_cols));
  A.v1 = reinterpret_cast<T*>(take(sizeof(T) * q->total_cols));
  A.pcol = reinterpret_cast<MPair<T>*>(take(sizeof(MPair<T>) * q->total_partials));
  A.err2 = reinterpret_cast<double*>(take(sizeof(double) * q->nprob));
  A.e2col = reinterpret_cast<double*>(take(sizeof(double) * q->total_cols));
  A.active = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * q->nprob));
  A.ucol_pre = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (q->nprob + 1)));
  A.urow_pre = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (q->nprob + 1)));
  A.colpre = reinterpret_cast<int64_t*>(take(sizeof(int64_t) * (q->nprob + 1)));
  int32_t* leaving = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * q->nprob));
  A.nsr = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * q->nprob));
  A.rchunk = reinterpret_cast<int32_t*>(take(sizeof(int32_t) * q->nprob));
  char* ctlp = take(64);
  A.ctl = reinterpret_cast<int32_t*>(ctlp);
  A.bar = reinterpret_cast<unsigned*>(ctlp + 32);
  A.leave_cnt = reinterpret_cast<int32_t*>(ctlp + 48);
  if (off > q->workspace_bytes) return OTG_ERR_WORKSPACE;
  if (A.and_depth > 0) {
    if (!q->anderson_ws || q->anderson_ws_bytes < anderson_ws_bytes(sizeof(T), q->nprob, q->total_cols, A.and_depth))
      return OTG_ERR_WORKSPACE;
    char* aw = static_cast<char*>(q->anderson_ws);
    size_t ao = 0;
    auto atake = [&](size_t bytes) { char* p = aw + ao; ao += (bytes + 255) / 256 * 256; return p; };
    A.and_F = reinterpret_cast<T*>(atake(sizeof(T) * (size_t)A.and_depth * (size_t)q->total_cols));
    A.and_R = reinterpret_cast<T*>(atake(sizeof(T) * (size_t)A.and_depth * (size_t)q->total_cols));
    A.and_G = reinterpret_cast<double*>(atake(sizeof(double) * (size_t)q->nprob * A.and_depth * A.and_depth));
    A.and_cnt = reinterpret_cast<int32_t*>(atake(sizeof(int32_t) * (size_t)q->nprob));
  }
  if (cudaMemsetAsync(ctlp, 0, 64, st) != cudaSuccess) return OTG_ERR_CUDA;
  int dev = 0, sms = 0, per = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, multi_sinkhorn_kernel<T, LOGF>, MT_THREADS, 0);
  int grid = sms * std::min(per, MtBlocks<T>::value);
  if (q->grid > 0 && q->grid < grid) grid = q->grid;
  if (grid < 1) return OTG_ERR_UNSUPPORTED;
  void* args[] = {&A, &leaving};
  cudaError_t e = cudaLaunchCooperativeKernel((const void*)multi_sinkhorn_kernel<T, LOGF>, dim3(grid), dim3(MT_THREADS),
                                              args, 0, st);
  if (e != cudaSuccess) return OTG_ERR_CUDA;
  if (A.tail_max > 0) {
    // behind the batch kernel on the stream; returns at once unless it was handed problems
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(std::min(A.tail_max, tc.max) * A.tail_cl));  // resident workers
    cfg.blockDim = dim3(TL_THREADS);
    cfg.dynamicSmemBytes = tc.smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)A.tail_cl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, multi_tail_kernel<T>, A);
    if (e != cudaSuccess) return OTG_ERR_CUDA;
  }
  return OTG_OK;
}

size_t multi_ws(int dtype, int64_t nprob, int64_t rows, int64_t cols, int64_t partials) {
  const size_t es = dtype == OTG_F64 ? 8 : 4;
  auto r = [](size_t b) { return (b + 255) / 256 * 256; };
  return r(es * rows) + 2 * r(es * cols) + r(2 * es * partials) + r(8 * nprob) + r(8 * cols) + r(4 * nprob) +
         3 * r(8 * (nprob + 1)) + 3 * r(4 * nprob) + r(64);
}
}  // namespace

extern "C" {

size_t otg_multi_workspace_bytes(int dtype, int32_t nprob, int64_t total_rows, int64_t total_cols,
                                 int64_t total_partials) {
  return multi_ws(dtype, nprob, total_rows, total_cols, total_partials);
}

size_t otg_multi_anderson_bytes(int dtype, int32_t nprob, int64_t total_cols, int32_t depth) {
  if (depth <= 0) return 0;
  return anderson_ws_bytes(dtype == OTG_F64 ? 8 : 4, nprob, total_cols, depth);
}

int otg_multi_tail_config(int dtype, int32_t* cluster_ctas, int32_t* max_clusters, int64_t* tile_bytes,
                          int32_t* cuda_error) {
  if (!cluster_ctas || !max_clusters || !tile_bytes || !cuda_error) return OTG_ERR_ARG;
  TailCfg tc;
  if (dtype == OTG_F64) tc = tail_config<double>();
  else if (dtype == OTG_F32) tc = tail_config<float>();
  else return OTG_ERR_DTYPE;
  *cluster_ctas = tc.cl;
  *max_clusters = tc.max;
  *tile_bytes = tc.tile;
  *cuda_error = tc.err;
  return OTG_OK;
}

int otg_sinkhorn_multi(const OtgMultiProblem* q, cudaStream_t stream) {
  if (!q || !q->M || !q->m_off || !q->rows || !q->cols || !q->ldm || !q->r_off || !q->c_off || !q->a || !q->b ||
      !q->reg || !q->nsr_max || !q->pc_off || !q->out_u || !q->out_v || !q->status || !q->niter ||
      !q->err || !q->workspace)
    return OTG_ERR_ARG;
  if (q->nprob < 1 || q->max_iter < 1) return OTG_ERR_ARG;
  if (q->anderson_depth < 0 || q->anderson_depth > OTG_ANDERSON_MAX_DEPTH) return OTG_ERR_ARG;
  if (q->anderson_depth > 0 && q->scaling != 0) return OTG_ERR_UNSUPPORTED;
  const bool logf = q->scaling == 0;
  if (q->dtype == OTG_F64) return logf ? launch_multi<double, true>(q, stream) : launch_multi<double, false>(q, stream);
  if (q->dtype == OTG_F32) return logf ? launch_multi<float, true>(q, stream) : launch_multi<float, false>(q, stream);
  return OTG_ERR_DTYPE;
}

}  // extern "C"
