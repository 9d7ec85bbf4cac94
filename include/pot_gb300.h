/* pot_gb300 — C ABI of the GB300 entropic-OT kernels.
 *
 * Plain pointers and sizes only.  Every array argument is DEVICE memory of
 * the current CUDA device unless stated otherwise; every call is
 * asynchronous on `stream` and returns an OTG_* status code for argument or
 * launch errors.  Results that the reference reports through its Python log
 * dict (iteration index, marginal errors, warnings) are written to a small
 * device "info" block that the caller reads after synchronising.
 *
 * The reference (PythonOT/POT) has no C interface for this path: its entry
 * points are Python functions.  Each declaration names the reference
 * function whose arithmetic it replaces.
 */
#ifndef POT_GB300_H
#define POT_GB300_H

#include <stddef.h>
#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

/* element types */
#define OTG_F32 0
#define OTG_F64 1

/* Sinkhorn forms */
#define OTG_METHOD_KNOPP 0 /* scaling form,  ot/bregman/_sinkhorn.py:487 sinkhorn_knopp */
#define OTG_METHOD_LOG 1   /* log form,      ot/bregman/_sinkhorn.py:690 sinkhorn_log   */
#define OTG_METHOD_STAB 2  /* log-stabilised scaling form with absorption,
                              ot/bregman/_sinkhorn.py:1105 sinkhorn_stabilized       */
#define OTG_METHOD_UNB 3   /* unbalanced scaling form with KL marginal penalties,
                              ot/unbalanced/_sinkhorn.py:565 sinkhorn_knopp_unbalanced */

/* return codes */
#define OTG_OK 0
#define OTG_ERR_ARG -1
#define OTG_ERR_DTYPE -2
#define OTG_ERR_WORKSPACE -3
#define OTG_ERR_CUDA -4
#define OTG_ERR_UNSUPPORTED -5
#define OTG_ERR_NOALLOC_TOO_LARGE -6 /* needs more scratch than OTG_NOALLOC_SCRATCH_BYTES */

/* solve status written to info[0] */
#define OTG_STATUS_CONVERGED 0 /* error below stopThr at a check iteration      */
#define OTG_STATUS_MAXITER 1   /* numItermax reached ("did not converge")      */
#define OTG_STATUS_NUMERICAL 2 /* zero / NaN / Inf scaling: reverted (knopp)     */
#define OTG_STATUS_ABORTED 3   /* a bounded device wait ran out                 */

/* ------------------------------------------------------------------------
 * Dense-cost Sinkhorn, one problem, the whole iteration loop in one
 * persistent cooperative launch.
 * Replaces the loops of ot/bregman/_sinkhorn.py:626-663 (sinkhorn_knopp),
 * :880-899 (sinkhorn_log) and :1273-1327 (sinkhorn_stabilized) behind
 * ot.sinkhorn / ot.sinkhorn2 (ot/bregman/_sinkhorn.py:21, :237).
 *
 * OTG_METHOD_STAB runs the log iteration on F = alpha/reg + log u,
 * G = beta/reg + log v in the gauge of a run without absorptions, started
 * from F0 = alpha0/reg - log n, and reproduces the reference's absorption
 * decisions (max u or max v above tau) and the check-iteration errors they
 * affect.  out_u, out_v receive F, G in that gauge; info[5] counts the
 * absorptions up to the returned iteration and info[6] says whether that
 * iteration absorbed.  The reference's own values are then
 *   logu = F - k log n,  logv = G + k log n                (info[6] == 0)
 *   logu = F - k log n,  logv = G + (k-1) log n - log m    (info[6] == 1)
 * with k = info[5]; alpha = reg logu, beta = reg logv.
 *
 * OTG_METHOD_UNB iterates u first, u = (a / K v)^fi1, v = (b / K^T u)^fi2
 * with fi = reg_m / (reg_m + reg) and K = exp(-M/reg) c, and logs the
 * relative sup-norm change of (u, v) at EVERY iteration (hist_cap >=
 * max_iter; the history holds the errors themselves, not their squares);
 * out_u, out_v receive the scalings u, v; a zero K^T u or a non-finite
 * scaling keeps the previous pair (status OTG_STATUS_NUMERICAL).
 * ---------------------------------------------------------------------- */
typedef struct OtgDenseProblem {
  int32_t dtype;      /* OTG_F32 or OTG_F64: type of M, a, b, warm_*, out_* */
  int32_t method;     /* OTG_METHOD_KNOPP, OTG_METHOD_LOG or OTG_METHOD_STAB */
  const void* M;      /* n x m cost, row-major, leading dimension ldm        */
  int64_t n, m, ldm;
  const void* a;      /* source weights (n)                                  */
  const void* b;      /* target weights (m)                                  */
  const void* warm_u; /* optional natural-log warm start (n) or NULL; STAB:  */
  const void* warm_v; /* alpha0/reg and beta0/reg                           */
  double reg;         /* entropic regularisation (> 0)                       */
  int32_t max_iter;   /* numItermax                                          */
  int32_t hist_cap;   /* capacity of the error history (>= max_iter/10 + 2)  */
  double stop_thr;    /* stopThr on the L2 column-marginal violation         */
  void* out_u;        /* knopp: scaling u; log: log_u (natural log)  (n)     */
  void* out_v;        /* knopp: scaling v; log: log_v                (m)     */
  size_t workspace_bytes;
  int32_t grid;       /* CTAs (0 = all co-resident CTAs); tuning knob        */
  int32_t timeout_ms; /* bound on any single device wait (0 = 4000 ms)       */
  double tau;         /* STAB: absorption threshold on the scalings (> 0)    */
  int32_t check_period; /* STAB: iterations between marginal checks (>= 1) */
  int32_t reserved;
  double reg_m1, reg_m2; /* UNB: marginal penalties (INFINITY = hard constraint) */
  int32_t c_ones;     /* UNB: 0 -> c = a b^T (reg_type 'kl'), 1 -> c = ones    */
  int32_t reserved2;
  /* KNOPP: optional Gibbs kernel K = exp(-M/reg) from otg_gibbs_kernel (same
   * dtype, n x m, row stride ldk, 16-byte aligned rows for the vector path),
   * or NULL.  The passes then read K instead of taking an exponential of
   * every cost entry each iteration, as the reference does (K of
   * ot/bregman/_sinkhorn.py:621); the iterates are bit-identical either way.
   * Pays where exponentials bound the solve (float64). */
  const void* K;
  int64_t ldk;
} OtgDenseProblem;

/* Workspace size for otg_sinkhorn_dense (device bytes, 256-byte aligned). */
size_t otg_dense_workspace_bytes(int dtype, int64_t n, int64_t m, int hist_cap, int grid);
/* Byte offset inside the workspace of the result block:
 *   double err_hist[hist_cap]; then int32 info[8] 256-byte aligned after it
 *   (info[0] status, info[1] niter = last loop index, info[2] number of
 *   logged errors, info[3] abort flag, info[5] and info[6] the absorption
 *   count and last-iteration flag of OTG_METHOD_STAB). */
size_t otg_dense_info_offset(int dtype, int64_t n, int64_t m, int hist_cap, int grid);
int otg_sinkhorn_dense(const OtgDenseProblem* p, void* workspace, cudaStream_t stream);

/* Plan and/or loss from potentials: P = exp(-M/reg + u + v) (log form) or
 * diag(u) exp(-M/reg) diag(v) (scaling form); *loss = sum(M * P) in fp64.
 * P or loss may be NULL; OTG_METHOD_STAB takes natural-log potentials like
 * the log form.  Replaces the returns of ot/bregman/_sinkhorn.py:681-687,
 * :915-918 and :1340-1368 and the loss of sinkhorn2 :435-438. */
int otg_dense_plan(int dtype, int method, const void* M, int64_t n, int64_t m, int64_t ldm,
                   const void* u, const void* v, double reg, void* P, int64_t ldp, double* loss,
                   cudaStream_t stream);

/* K = exp(-M/reg) (n x m, row stride ldk), computed exactly as the scaling
 * form of otg_sinkhorn_dense computes it on the fly: the Gibbs kernel of
 * ot/bregman/_sinkhorn.py:621. */
int otg_gibbs_kernel(int dtype, const void* M, int64_t n, int64_t m, int64_t ldm, double reg, void* K,
                     int64_t ldk, cudaStream_t stream);

/* Row and column sums of P = exp(-M/reg + u + v) (natural-log potentials),
 * accumulated in fp64 (rowsum: n, colsum: m).  The marginal error of the
 * epsilon-scaling loop, ot/bregman/_sinkhorn.py:1534-1542. */
int otg_dense_marginals(int dtype, const void* M, int64_t n, int64_t m, int64_t ldm, const void* u, const void* v,
                        double reg, double* rowsum, double* colsum, cudaStream_t stream);

/* Greenkhorn, the greedy coordinate Sinkhorn, on one dense problem.
 * Replaces ot/bregman/_sinkhorn.py:1034-1102 (greenkhorn, reached through
 * ot.sinkhorn(method='greenkhorn'), :192-204).  K = exp(-M/reg) and its
 * transpose are built in the workspace; u, v start at 1/n, 1/m, or at
 * exp(warm_u), exp(warm_v) (both or neither); each of at most num_iter_max
 * steps rescales the row or column with the largest |marginal violation|,
 * the whole chain in one CTA.  Outputs: the scalings u (n) and v (m), the
 * plan G_ij = u_i K_ij v_j when G is not NULL (leading dimension ldg), and
 * info[0] = last step index (the reference's log["n_iter"]; -1 when
 * num_iter_max is 0), info[1] = OTG_STATUS_CONVERGED or OTG_STATUS_MAXITER.
 * All pointers are device pointers of the dtype; info is device int32[2]. */
size_t otg_greenkhorn_workspace_bytes(int dtype, int64_t n, int64_t m);
int otg_greenkhorn(int dtype, const void* M, int64_t n, int64_t m, int64_t ldm, const void* a, const void* b,
                   double reg, const void* warm_u, const void* warm_v, int32_t num_iter_max, double stop_thr,
                   void* G, int64_t ldg, void* u, void* v, int32_t* info, void* workspace, size_t workspace_bytes,
                   cudaStream_t stream);

/* Loss of a lazy plan, sum_ij C_ij exp(f_i + g_j - C_ij/reg) with
 * C_ij = |x_i - y_j|^2 (X: n x d, Y: m x d row-major; f, g natural-log
 * potentials), fp64 accumulation.  Replaces the block loop of
 * ot/bregman/_empirical.py:470-478 (empirical_sinkhorn2, isLazy=True). */
int otg_lazy_loss(int dtype, const void* X, const void* Y, int64_t n, int64_t m, int32_t d, const void* f,
                  const void* g, double reg, double* out, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Entropic Wasserstein barycenter of n_hists histograms on one support of
 * size dim (cost M: dim x dim), the iteration loop driven natively with one
 * host synchronisation per error check.  Replaces
 * ot/bregman/_barycenter.py:141-259 (barycenter_sinkhorn, OTG_METHOD_KNOPP)
 * and :403-473 (_barycenter_sinkhorn_log, OTG_METHOD_LOG) behind
 * ot.bregman.barycenter (:23).
 * ---------------------------------------------------------------------- */
typedef struct OtgBaryProblem {
  int32_t dtype, method;   /* OTG_F32/OTG_F64; OTG_METHOD_KNOPP or OTG_METHOD_LOG */
  const void* M;           /* dim x dim cost, leading dimension ldm               */
  int64_t dim, ldm;
  const void* A;           /* dim x n_hists histograms, row-major                 */
  int32_t n_hists;
  int32_t max_iter;        /* numItermax (>= 1)                                   */
  const void* weights;     /* n_hists barycentric weights                         */
  double reg, stop_thr;
  void* out_bar;           /* dim: the barycenter                                 */
  double* err_hist;        /* HOST: errors of the check iterations (ii % 10 == 1) */
  int32_t hist_cap;
  int32_t* info;           /* HOST int32[3]: status, niter (last loop index), checks */
  void* workspace; size_t workspace_bytes;
} OtgBaryProblem;

size_t otg_barycenter_workspace_bytes(int dtype, int method, int64_t dim, int32_t n_hists);
int otg_barycenter(const OtgBaryProblem* p, cudaStream_t stream);

/* Batched transpose: dst[b] (m x ld_dst, batch stride bs_dst) = src[b]^T
 * (src[b]: n x m, leading dimension ld_src, batch stride bs_src), with +inf
 * in the padding columns [n, ld_dst).  The batch order of ot.batch
 * (u first, row-marginal check; ot/batch/_utils.py:268-278) is the
 * sinkhorn_log order of the transposed problem, which the work-balanced
 * kernel (otg_sinkhorn_multi) then solves. */
int otg_transpose_batched(int dtype, const void* src, int64_t batch, int64_t n, int64_t m, int64_t ld_src,
                          int64_t bs_src, void* dst, int64_t ld_dst, int64_t bs_dst, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Batched dense Sinkhorn: many independent problems of uneven size in ONE
 * persistent launch, one CTA per problem at a time, each problem stopping on
 * its own marginal error.  Replaces the loops of ot/batch/_utils.py:268-278
 * (bregman_log_projection_batch, u_first = 1), :141-149
 * (bregman_projection_batch, knopp, u_first = 1) and, with u_first = 0, runs
 * the per-problem order of ot/bregman/_sinkhorn.py:880-899 (sinkhorn_log).
 * Problem p's cost block is M + m_off[p], rows[p] x cols[p] with row stride
 * ldm[p] (elements; ldm*elem a multiple of 16 bytes, m_off*elem 16-byte
 * aligned; padded columns must hold a finite value or +inf).  a/u use
 * r_off[p], b/v use c_off[p] into the packed vectors.  All table arrays are
 * device memory.  Limits come from otg_batch_limits.
 * ---------------------------------------------------------------------- */
typedef struct OtgBatchProblem {
  int32_t dtype, method;
  const void* M;
  const int64_t* m_off;
  const int32_t* rows;
  const int32_t* cols;
  const int32_t* ldm;
  const int64_t* r_off;
  const int64_t* c_off;
  const void* a;
  const void* b;
  const void* warm_u;   /* natural-log warm start (packed like a) or NULL */
  const void* warm_v;
  const double* reg;    /* per problem */
  const int32_t* order; /* processing order, a permutation of 0..nprob-1 */
  int32_t nprob;
  int32_t max_iter;
  double stop_thr;
  int32_t u_first;
  int32_t grid;         /* CTAs (0 = one per SM) */
  void* out_u;          /* log: natural-log potentials; knopp: scalings */
  void* out_v;
  int32_t* status;      /* per problem, OTG_STATUS_* */
  int32_t* niter;       /* per problem, last loop index */
  double* err;          /* per problem, last logged marginal error (-1 if none) */
  int32_t* queue;       /* 2 int32 of device scratch (work counter, abort flag) */
  int32_t timeout_ms;
} OtgBatchProblem;

int otg_batch_limits(int dtype, int32_t* max_rows, int32_t* max_cols, int32_t* row_bytes_max);
int otg_sinkhorn_batched(const OtgBatchProblem* q, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Work-balanced batched log-domain Sinkhorn: all SMs work on every active
 * problem in every half-step (one persistent cooperative launch); problems
 * leave the active set as they converge.  Per problem the order and stop
 * test of ot/bregman/_sinkhorn.py:880-899 (sinkhorn_log).  Same packed
 * layout as otg_sinkhorn_batched; nsr_max[p] (>= 1) bounds the row split of
 * problem p's column reductions and pc_off[p] places its nsr_max[p] x cols[p]
 * partial pairs (total_partials in all).  The workspace size comes from
 * otg_multi_workspace_bytes.
 * ---------------------------------------------------------------------- */
typedef struct OtgMultiProblem {
  int32_t dtype;
  int32_t nprob;
  const void* M;
  const int64_t* m_off;
  const int32_t* rows;
  const int32_t* cols;
  const int32_t* ldm;
  const int64_t* r_off;
  const int64_t* c_off;
  const void* a;
  const void* b;
  const void* warm_u;   /* natural-log source warm start or NULL */
  const double* reg;
  int32_t max_iter;
  int32_t grid;
  double stop_thr;
  const int32_t* nsr_max;
  const int64_t* pc_off;
  int64_t total_rows, total_cols, total_partials;
  void* out_u;
  void* out_v;
  int32_t* status;
  int32_t* niter;
  double* err;
  void* workspace;
  size_t workspace_bytes;
  int32_t timeout_ms;
  /* over-relaxation of the potential updates, f <- (1 - omega) f + omega f_new
   * (1 or 0: plain Sinkhorn, the reference's iteration).  No reference
   * counterpart: used by the warm-start refinement; the stop test is still the
   * exact column-marginal error of the iterate. */
  double omega;
  /* iterations between stop tests: 0 or 10 is the reference's schedule
   * (sinkhorn_log tests at ii % 10 == 0); 1 tests every iteration with the
   * same criterion (no reference counterpart). */
  int32_t check_period;
  /* schedule (0: default): column-pass units aimed at per warp (8), the
   * row-split cap while the batch fills the GPU (16) and once few problems
   * remain (64; at most 64).  CTAs per SM are set through `grid`.  Changes
   * how work is divided, not the iteration; chosen per workload by the
   * autotuner of pot_gb300/tune.py. */
  int32_t units_per_warp;
  int32_t split_cap_fill;
  int32_t split_cap_tail;
  /* tail handoff: once at most this many problems remain and each fits the
   * shared memory of one thread-block cluster, a cluster per problem
   * finishes them (same iteration and stop test, cluster barriers instead of
   * grid barriers; clusters take the problems from a queue).  0: default
   * (three times the clusters the device holds at once in float32; never in
   * float64, whose passes are bound by FP64 throughput); negative: never. */
  int32_t tail_problems;
  /* whole-batch stop (ot.batch's rule, ot/batch/_utils.py:152-157, :273-278):
   * 0: every problem stops on its own error; 1: all problems stop together
   * at the first check whose LARGEST error is below stop_thr (each reports
   * that stop index and its own error; no tail handoff). */
  int32_t joint_stop;
  /* 0: log form (potentials are natural logs); 1: scaling form with
   * K = exp(-M/reg) (ot/batch/_utils.py:141-151 on the transposed problem;
   * outputs are the scalings themselves; no omega, no tail handoff). */
  int32_t scaling;
  /* Anderson mixing of the v update over the last anderson_depth iterates
   * (0: off; at most OTG_ANDERSON_MAX_DEPTH; log form only, replaces omega).
   * No reference counterpart: the stop test is unchanged, and u is always
   * the exact row update of the v in use, so the returned pair has an exact
   * row marginal and a checked column marginal, as in sinkhorn_log.  Needs
   * otg_multi_anderson_bytes() of device memory in anderson_ws. */
  int32_t anderson_depth;
  int32_t reserved;
  void* anderson_ws;
  size_t anderson_ws_bytes;
} OtgMultiProblem;
#define OTG_ANDERSON_MAX_DEPTH 8
size_t otg_multi_workspace_bytes(int dtype, int32_t nprob, int64_t total_rows, int64_t total_cols,
                                 int64_t total_partials);
int otg_sinkhorn_multi(const OtgMultiProblem* q, cudaStream_t stream);
/* Device bytes of the Anderson history (anderson_ws) for a batch. */
size_t otg_multi_anderson_bytes(int dtype, int32_t nprob, int64_t total_cols, int32_t depth);
/* The tail handoff's cluster shape on the current device: CTAs per cluster
 * (0: no tail handoff), clusters resident at once, shared-memory bytes of
 * cost block per CTA, and the CUDA error code of the last configuration
 * query (0 when it succeeded). */
int otg_multi_tail_config(int dtype, int32_t* cluster_ctas, int32_t* max_clusters, int64_t* tile_bytes,
                          int32_t* cuda_error);

/* ------------------------------------------------------------------------
 * Batched point-cloud solves on the tensor cores: P pairs of clouds X_p
 * (n x d) and Y_p (m x d), fp32, the same n, m, d for every pair, packed
 * pair after pair, squared-Euclidean cost that is never stored: every pass
 * rebuilds the cost tiles from the points (tcgen05, fp16 hi/lo x3, as
 * otg_sinkhorn_online) and folds them into per-row log-sum-exps, so a pass
 * reads points instead of a cost block (16 MiB per 2048 x 2048 pair).  Per
 * pair the iteration, stop test and outputs are those of otg_sinkhorn_multi
 * on the stored cost: sinkhorn_log order (ot/bregman/_sinkhorn.py:880-899,
 * v first), column-marginal L2 error every check_period iterations (0: 10),
 * each pair stopping on its own, optional Anderson mixing of the v update
 * (anderson_depth, at most OTG_ANDERSON_MAX_DEPTH).  reg: one absolute value
 * per pair (otg_pairs_max_cost gives each pair's largest cost, to set it
 * relative to that).  a, b: P x n, P x m weights; warm_u: P x n natural-log
 * source potentials or NULL; out_u, out_v: P x n, P x m natural-log
 * potentials; status, niter, err per pair as otg_sinkhorn_multi.  No
 * reference counterpart for the batching; replaces the stored-cost passes of
 * the pair solver of the warm-start workload.
 * ---------------------------------------------------------------------- */
typedef struct OtgPairsProblem {
  const float* X;
  const float* Y;
  int32_t npairs;
  int32_t d;
  int64_t n, m;
  const float* a;
  const float* b;
  const double* reg;
  const float* warm_u;
  int32_t max_iter;
  int32_t check_period;
  double stop_thr;
  int32_t anderson_depth;
  int32_t timeout_ms;
  float* out_u;
  float* out_v;
  int32_t* status;
  int32_t* niter;
  double* err;
  void* workspace;
  size_t workspace_bytes;
  float sum_window_log2;  /* as in OtgOnlineProblem (0: default) */
} OtgPairsProblem;
size_t otg_pairs_workspace_bytes(int32_t npairs, int64_t n, int64_t m, int32_t d, int32_t anderson_depth);
/* Each pair's largest squared distance max_ij |x_i - y_j|^2 (device, P
 * doubles), from one max-only pass on the tensor cores. */
int otg_pairs_max_cost(const OtgPairsProblem* q, double* maxc, cudaStream_t stream);
int otg_sinkhorn_pairs(const OtgPairsProblem* q, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Online ("lazy") log-domain Sinkhorn on point clouds with squared-Euclidean
 * cost that is never stored: cost tiles |x|^2 + |y|^2 - 2 x.y come from
 * tcgen05 MMAs on high/low half planes of the points (prescaled by the
 * powers of two scale_x, scale_y), folded into per-row running LSE pairs.
 * Replaces the blockwise loop of ot/bregman/_empirical.py:205-248
 * (empirical_sinkhorn, isLazy=True): f first, then g; the L1 row-marginal
 * error after iterations with (i+1) % 10 == 0, compared with <=.  The host
 * loop runs inside the call (one synchronisation per check), so the call
 * returns with the results; info[0] status, info[1] niter, info[2] number
 * of logged errors, info[3] row blocks recomputed by fix-up passes (rows
 * whose shifted sums left their range; info is HOST memory, 4 int32;
 * err_hist is HOST memory, hist_cap doubles).  X: n x d,
 * Y: m x d fp32 row-major, d <= 128; a, b weights; warm_f, warm_g optional
 * natural-log potentials.
 * ---------------------------------------------------------------------- */
typedef struct OtgOnlineProblem {
  const float* X; const float* Y;
  int64_t n, m;
  int32_t d;
  int32_t max_iter;
  const float* a; const float* b;
  const float* warm_f; const float* warm_g;
  double reg;
  double stop_thr;
  float scale_x, scale_y;
  float* out_f; float* out_g;
  double* err_hist; int32_t hist_cap;
  int32_t* info;         /* HOST, 4 ints */
  void* workspace; size_t workspace_bytes;
  int32_t timeout_ms;
  /* shifted-sum acceptance window of the folded passes, in log2 units: a
   * row's sum outside [2^-w, 2^w] is recomputed by the fix-up pass.  0: the
   * default [2^-70, 2^100]; a narrow window sends most rows through the
   * fix-up (a test of that path; the results are the same). */
  float sum_window_log2;
} OtgOnlineProblem;
size_t otg_online_workspace_bytes(int64_t n, int64_t m, int32_t d);
int otg_sinkhorn_online(const OtgOnlineProblem* p, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Squared-Euclidean cost blocks for a table of point-cloud pairs:
 * M_p[i, j] = sum_k (X_p[i, k] - Y_p[j, k])^2 for j < cols[p]; padded
 * columns [cols[p], ldm[p]) are set to +inf.  max_out (optional, one value
 * per problem) receives max_ij M_p.  Replaces ot/utils.py:400 dist
 * (sqeuclidean) and ot/batch/_linear.py:178 dist_batch for the batched path.
 * ---------------------------------------------------------------------- */
typedef struct OtgCostTable {
  int32_t dtype;
  int32_t nprob;
  const void* X; const void* Y;
  const int64_t* x_off;  /* element offset of X_p (row-major rows[p] x dim[p]) */
  const int64_t* y_off;
  const int32_t* rows; const int32_t* cols; const int32_t* dim;
  int32_t max_dim;
  void* M;
  const int64_t* m_off;
  const int32_t* ldm;
  void* max_out;
  int32_t fixed_dim;  /* 0, or the dimension every problem shares when it is 2, 3, 8 or 16
                         (float32: register-tiled kernel with 16-byte stores; must equal
                         max_dim, and every m_off[p] and ldm[p] must be a multiple of 4;
                         for 8 and 16 also 16-byte loads of the points: X and Y 16-byte
                         aligned, every x_off[p], y_off[p] a multiple of 4, else the
                         generic kernel runs) */
} OtgCostTable;
int otg_batched_sqdist(const OtgCostTable* t, int32_t max_rows, cudaStream_t stream);

/* Plans and values of a batch from its potentials (log: natural-log
 * potentials; knopp: scalings).  out_vals[3p] = sum M*T, out_vals[3p+1] =
 * sum T log(T + 1e-16) (kl = 0) or sum T log(T/(a b^T) + 1e-16) (kl = 1),
 * out_vals[3p+2] = sum T, all fp64.  P may be NULL (values only); it uses
 * M's layout.  Replaces ot/batch/_linear.py:326-345 and _utils.py:4-21. */
typedef struct OtgPlanTable {
  int32_t dtype, method, nprob, kl;
  const void* M;
  const int64_t* m_off;
  const int32_t* rows; const int32_t* cols; const int32_t* ldm;
  const int64_t* r_off; const int64_t* c_off;
  const void* u; const void* v; const void* a; const void* b;
  const double* reg;
  void* P;
  double* out_vals;
} OtgPlanTable;
int otg_batched_plan(const OtgPlanTable* t, int32_t max_rows, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Learned warm start: kernels of the point-cloud network's forward, backward
 * and AdamW step.  No counterpart in the reference (the network feeds the
 * warmstart argument of ot/bregman/_sinkhorn.py:864-868).  All fp32.
 * ---------------------------------------------------------------------- */
/* Voronoi cell masses for the learned warm start's coarse problem: w[p*k + c] = fraction of
 * the n points of X_p (row-major n x d, problem stride sx elements) whose nearest of the k
 * centres C_p (k x d, stride sc) is centre c.  d in {2, 3, 8, 16}. */
int otg_nearest_mass(const float* X, const float* C, int32_t nprob, int32_t n, int32_t k, int32_t d, int64_t sx,
                     int64_t sc, float* w, cudaStream_t stream);
/* Soft-min distances of every source point of every problem to its target
 * measure, at ntau (<= 8) temperatures relative to scale[p]:
 * out[(r_off[p]+i)*ntau + k] = -tau_k ln sum_j b_j exp(g_j - M_ij / (scale[p] tau_k)).
 * g (natural-log target potentials packed like b) may be NULL (zero
 * potential).  f32 problem table as for otg_sinkhorn_batched. */
/* Soft-mins of the n points of each cloud of X (P x n x d, pair stride sx)
 * over the k weighted atoms C of the pair (P x k x d, stride sc; weights b,
 * P x k), squared distances computed on the fly: out_f (P x n, optional) =
 * the c-transform -g_tau log sum_k b_k exp(g_k - |x - y_k|^2 / (scale g_tau)),
 * out_F (P x n x ntau) = the same with g = 0 at each taus[t]; units of
 * scale[p].  d in {2, 3, 8, 16}; OTG_ERR_UNSUPPORTED otherwise.  (Learned
 * warm start: the multiscale prior and the network's distance features.) */
int otg_softmin_points(const float* X, const float* C, int32_t nprob, int32_t n, int32_t k, int32_t d, int64_t sx,
                       int64_t sc, const float* b, const float* g, float g_tau, const float* scale,
                       const float* taus, int32_t ntau, float* out_f, float* out_F, cudaStream_t stream);
int otg_softmin_features(const float* M, const int64_t* m_off, const int32_t* rows, const int32_t* cols,
                         const int32_t* ldm, const int64_t* r_off, const int64_t* c_off, const float* b,
                         const float* scale, const float* taus, int32_t ntau, int32_t nprob, int32_t max_rows,
                         const float* g, float* out, cudaStream_t stream);
/* C = alpha op(A) op(B) + beta C (+ bias[N]) (ReLU if relu); op(A) M x K
 * stored [M,K] (ta=0) or [K,M] (ta=1); op(B) K x N stored [K,N] or [N,K]. */
int otg_gemm_f32(int ta, int tb, int64_t M, int64_t N, int64_t K, float alpha, const float* A, int64_t lda,
                 const float* B, int64_t ldb, float beta, float* C, int64_t ldc, const float* bias, int relu,
                 cudaStream_t stream);
int otg_mlp_relu_bwd(float* dY, const float* Y, int64_t n, cudaStream_t stream);
int otg_mlp_colsum(const float* X, int64_t R, int64_t C, float* out, cudaStream_t stream);
/* Fused inference of the warm-start network (shipped sizes d = 16, widths
 * 32/32, head input 22 + 2 x 32, head width 64; OTG_ERR_UNSUPPORTED for
 * others): encoder + mean pooling of P clouds of n points into s (P x h2),
 * and the head over the per-point inputs Z (P x n x dz) with the pooled
 * summaries sX, sY -> f (P x n). */
int otg_mlp_encode_pool(const float* X, int64_t P, int64_t n, int32_t d, int32_t h1, int32_t h2, const float* W1,
                        const float* b1, const float* W2, const float* b2, float* s, cudaStream_t stream);
int otg_mlp_head(const float* Z, int64_t P, int64_t n, int32_t dz, int32_t h2, int32_t h3, const float* sX,
                 const float* sY, const float* W3, const float* b3, const float* W4, const float* b4, const float* W5,
                 const float* b5, float* f, cudaStream_t stream);
int otg_mlp_segment_mean(const float* X, int64_t P, int64_t n, int64_t C, float* out, cudaStream_t stream);
int otg_mlp_segment_mean_bwd(const float* dS, int64_t P, int64_t n, int64_t C, float* dX, int accumulate,
                             cudaStream_t stream);
int otg_mlp_concat3(const float* x, const float* sx, const float* sy, int64_t P, int64_t n, int64_t d, int64_t H,
                    float* z, cudaStream_t stream);
int otg_mlp_concat3_bwd(const float* dz, int64_t P, int64_t n, int64_t d, int64_t H, float* dsx, float* dsy,
                        cudaStream_t stream);
/* loss (fp64, device) = mean over P segments of sum_r ((f - mean f) - t)^2 / n;
 * df = its gradient. */
int otg_mlp_centered_mse(const float* f, const float* t, int64_t P, int64_t n, double* loss, float* df,
                         cudaStream_t stream);
int otg_mlp_adamw(float* w, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2, float eps,
                  float wd, int step, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Entropic Gromov-Wasserstein tensor product on the tensor cores.
 * Replaces the two GEMMs of ot/gromov/_utils.py:244-280 (tensor_product)
 * used by gwggrad (:323-354) inside entropic_gromov_wasserstein
 * (ot/gromov/_bregman.py:198-242).
 *
 * otg_split_half: half-precision high/low planes hi + lo = scale * X (or
 * scale * X^T), X rows x cols fp32; out planes have ld_out columns.
 * otg_gemm_split3: C = A B^T for operands given as high/low half planes
 * (A: a_rows x lda, B: b_rows x ldb, both K-major, rows and leading dims
 * multiples of 128, zero-padded beyond the data; K = k_alloc, a multiple of
 * 64), three tcgen05 MMAs per k-step (Ah Bh + Ah Bl + Al Bh), fp32 TMEM
 * accumulation.  mode 0 writes scale * C as high/low planes (a_rows x ld_h,
 * ld_h >= b_rows); mode 1 writes out_ij = s_acc C_ij + s_vec (rowv_i +
 * colv_j) for i < M, j < N (fp32, ld_o).  abort_flag: one device int32,
 * zero on entry; set if a bounded wait runs out.
 * ---------------------------------------------------------------------- */
typedef struct OtgSplitGemm {
  const void* a_hi; const void* a_lo; int64_t a_rows, lda;
  const void* b_hi; const void* b_lo; int64_t b_rows, ldb;
  int64_t k_alloc;
  int32_t mode;
  float scale, s_acc, s_vec;
  void* out_hi; void* out_lo; int64_t ld_h;
  float* out; int64_t ld_o;
  int64_t M, N;
  const float* rowv; const float* colv;
  int32_t* abort_flag;
  int32_t timeout_ms;
  /* mode 1, optional: out += s_add * addend (M x N, leading dimension
   * ld_add; may alias out) -- the (1 - alpha) M term of fused GW,
   * ot/gromov/_bregman.py:1184-1190 */
  const float* addend; int64_t ld_add; float s_add;
  /* batched form (batch > 1; 0 or 1: one product): `batch` independent
   * products of equal shape, one per grid z-slice.  The planes stack the
   * problems' padded planes (A: batch * a_rows rows, B: batch * b_rows
   * rows); problem z reads rows z*a_rows.. of A and z*b_rows.. of B and
   * writes mode-0 planes from row z*a_rows.  Mode 1: problem z writes
   * out + z*o_bstride, reads rowv + z*rowv_bstride, colv + z*colv_bstride
   * and addend + z*addend_bstride (element strides).  Replaces the batched
   * einsum chains of ot/batch/_quadratic.py:535-572 (tensor_product_batch). */
  int64_t batch;
  int64_t o_bstride, rowv_bstride, colv_bstride, addend_bstride;
} OtgSplitGemm;
int otg_split_half(const float* X, int64_t rows, int64_t cols, int64_t ldx, float scale, int transpose, void* hi,
                   void* lo, int64_t ld_out, cudaStream_t stream);
int otg_gemm_split3(const OtgSplitGemm* g, cudaStream_t stream);
/* otg_split_half over `batch` problems: problem z reads X + z*sx and writes
 * its planes at hi/lo + z*so (element strides). */
int otg_split_half_batched(const float* X, int64_t rows, int64_t cols, int64_t ldx, int64_t sx, float scale,
                           int transpose, void* hi, void* lo, int64_t ld_out, int64_t so, int64_t batch,
                           cudaStream_t stream);
/* Batched tiled GEMM (CUDA cores), C_z = alpha op(A_z) op(B_z) + beta C_z for z < batch with
 * element strides sA, sB, sC between batch members; replaces the einsum chains of
 * ot/batch/_quadratic.py:535-572 (tensor_product_batch). */
int otg_gemm_batched(int dtype, int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const void* A,
                     int64_t lda, int64_t sA, const void* B, int64_t ldb, int64_t sB, double beta, void* C,
                     int64_t ldc, int64_t sC, int64_t batch, cudaStream_t stream);
/* fp64 tiled GEMM (CUDA cores) for the float64 path: C = alpha op(A) op(B) + beta C. */
int otg_gemm_f64(int ta, int tb, int64_t M, int64_t N, int64_t K, double alpha, const double* A, int64_t lda,
                 const double* B, int64_t ldb, double beta, double* C, int64_t ldc, cudaStream_t stream);

/* ------------------------------------------------------------------------
 * Allocation-free variant of otg_sinkhorn_dense.  No counterpart in the
 * reference: it exists for callers that cannot allocate device memory
 * when they solve, e.g. a host whose own allocator owns the device pool, or
 * a latency-bound loop that must not pay cudaMalloc/cudaFree (which can
 * synchronise the device).  The solver's scratch is one static device array
 * of OTG_NOALLOC_SCRATCH_BYTES inside this library, held by every GPU that
 * loads it until the process exits; p->workspace_bytes is ignored.
 *
 * The caller still passes all inputs and outputs, plus the result block:
 * err_hist (device, hist_cap doubles: the squared L2 column-marginal
 * violation of each check, the same values as the allocating entry point's
 * history) and info (device, 8 int32, same meaning as there).
 *
 * Problems whose scratch exceeds the maximum are rejected with
 * OTG_ERR_NOALLOC_TOO_LARGE (about n = m = 16384 in float32 with the
 * default grid fits; a smaller p->grid lowers the need).  The first call in
 * a CUDA context looks up the array's device address in that context and
 * caches it by the context's unique ID (a context created again after
 * cudaDeviceReset, or a non-primary context on the same device, looks it up
 * afresh); make that first call before any stream capture.  Every call in
 * a context shares the array and it keeps the
 * last call's contents: the call clears what must start at zero, and calls
 * whose kernels overlap on the GPU race, so serialise them.
 * ---------------------------------------------------------------------- */
#define OTG_NOALLOC_SCRATCH_BYTES (16u << 20)
int otg_sinkhorn_dense_noalloc(const OtgDenseProblem* p, double* err_hist, int32_t* info,
                               cudaStream_t stream);

/* ------------------------------------------------------------------------
 * ABI self-description (host only, no GPU needed).  For the struct named
 * `name` (e.g. "OtgDenseProblem") writes sizeof to out[0] and the offset of
 * each field, in declaration order, to out[1..]; returns the count written
 * (1 + fields), or OTG_ERR_ARG for an unknown name or a too small `cap`.
 * Bindings (ctypes, cgo, JNI) check their struct mirrors with it.
 * ---------------------------------------------------------------------- */
int otg_abi_layout(const char* name, int64_t* out, int32_t cap);

#ifdef __cplusplus
}
#endif
#endif /* POT_GB300_H */
