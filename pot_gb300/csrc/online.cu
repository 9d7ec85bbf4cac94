// Online ("lazy") log-domain Sinkhorn on point clouds: the squared-Euclidean
// cost is never stored.  Reference behaviour (PythonOT/POT):
// ot/bregman/_empirical.py:190-263 (empirical_sinkhorn, isLazy=True):
//   f = log a - LSE_j(g - C/reg), then g = log b - LSE_i(f - C/reg);
//   at iterations with (i+1) % 10 == 0 the L1 violation of the ROW marginal is
//   compared with stopThr using <=.
//
// One half-step = one launch of online_pass_kernel.  A CTA owns 128 "row"
// points (X for the f update, Y for the g update), kept resident in shared
// memory as high/low half planes; it streams the other cloud in tiles of 128
// points through a TMA ring.  For every tile, one thread issues 3 tcgen05 MMAs
// per 16-wide k-step (Ah Bh + Ah Bl + Al Bh: the dot products x.y with about
// 22 significant bits) into one of four TMEM buffers (the MMAs run up to three
// tiles ahead of the epilogue); sixteen epilogue warps (four per TMEM lane
// quarter, each taking 32 of the 128 columns) read the tile and fold
// t_ij = alpha * acc_ij + h_j  into a running base-2 (max, sum) per row, where
//   alpha = 2 log2(e) / (reg sx sy)     (acc carries the operand prescales)
//   h_j   = g2_j - log2(e) |y_j|^2 / reg  (-inf for padding)
//   and the row term -log2(e) |x_i|^2 / reg is added after the reduction.
// The pass writes the new potential and the h vector the next pass needs,
// and, on check passes, the L1 row-marginal violation of the previous
// potentials (the LSE it computes is the one the marginal needs).
#include <cuda.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <mutex>
#include "common.cuh"
#include "tma.cuh"
#include "tc.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

constexpr int OL_M = 128, OL_N = 128, OL_K = 64, OL_STAGES = 4;
constexpr uint32_t OL_TILE = OL_M * OL_K * 2;          // one half plane tile (16 KiB)
constexpr uint32_t OL_HVEC = OL_N * 4;                 // h slice of a tile (512 B)
constexpr uint32_t OL_STAGE = 2 * OL_TILE;             // streamed hi, lo (1024-aligned tiles)
constexpr int OL_MAXKT = 2;                            // d <= 128
constexpr int OL_EPI = 16;                             // epilogue warps (4 per TMEM lane quarter)
constexpr int OL_NBUF = 4;                             // TMEM accumulator buffers of 128 columns
constexpr int OL_THREADS = OL_EPI * 32 + 64;           // + producer + MMA

struct OnlinePass {
  int n_rows;          // valid rows of the resident side
  int col_tiles;       // tiles of the streamed side
  int k_tiles;
  float alpha;         // 2 log2(e) / (reg sx sy)
  const float* h;      // streamed side, padded to col_tiles*128 (bulk-copied per tile)
  const float* rterm;  // resident side: -log2(e) |x_i|^2 / reg
  const float* logw2;  // resident side: log2 of the weights
  const float* pot2;   // resident side current potential (base 2), for the check
  const float* w;      // resident side weights, for the check
  float* pot_out2;     // new potential (base 2)
  const float* other_norm2;  // resident side: log2(e)|x|^2/reg, to form the next pass's h
  float* h_out;        // h for the next pass: pot_new2 - other_norm2 (-inf beyond n_rows)
  double* err;         // check passes: per-row |marginal violation| slots, else null
  int* abort_flag;
  uint64_t timeout_ns;
  // column split: CTA (b, s) streams tiles [s T / S, (s + 1) T / S) and, with
  // S > 1, leaves its per-row (max, sum) in part[s][2][rows_pad] for
  // online_finalize_kernel
  int split;
  int rows_pad;
  float* part;
  // batch of pairs (active == null: one problem).  CTA blockIdx.x takes row
  // block blockIdx.x % nrb of the pair in active slot blockIdx.x / nrb; slots
  // at or beyond *count have left the batch and their CTAs return at once.
  // Planes and per-row vectors hold pair p's rows from p * rows_per_pair
  // (resident side) and p * cols_per_pair (streamed side); alpha_p is the
  // pair's alpha.  err_sq: the check error of a row is the squared violation
  // (the L2 test of sinkhorn_log) instead of the absolute one (L1).
  const int* active;
  const int* count;
  int nrb;
  int64_t rows_per_pair, cols_per_pair;
  const float* alpha_p;
  int err_sq;
};

// MAXP: instead of the log-sum-exp, each row's max of t (the max cost of a
// pair batch, which sets its regularisation): no exponentials.
template <bool MAXP>
__global__ void __launch_bounds__(OL_THREADS, 1)
online_pass_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                   const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, OnlinePass P) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* resident = smem;                                   // [kt][hi, lo] tiles
  unsigned char* ring = smem + OL_MAXKT * 2 * OL_TILE;              // [stage][hi, lo] of one k-tile
  float* hbuf = reinterpret_cast<float*>(ring + OL_STAGES * OL_STAGE);  // [stage][128] h slices
  uint64_t* bars = reinterpret_cast<uint64_t*>(hbuf + OL_STAGES * OL_N);
  uint64_t* res_full = bars;            // resident operand landed
  uint64_t* full = bars + 1;            // [OL_STAGES]
  uint64_t* empty = full + OL_STAGES;   // [OL_STAGES]
  uint64_t* accf = empty + OL_STAGES;   // [OL_NBUF]
  uint64_t* acce = accf + OL_NBUF;      // [OL_NBUF]
  uint32_t* tslot = reinterpret_cast<uint32_t*>(acce + OL_NBUF);
  float* red = reinterpret_cast<float*>(tslot + 4);                 // [3][2][128] (mx, s) of column groups 1-3
  unsigned* relcnt = reinterpret_cast<unsigned*>(red + 6 * OL_M);   // [OL_STAGES] epilogue warps done
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int pair = 0, rblk = blockIdx.x;
  if (P.active) {
    const int slot = blockIdx.x / P.nrb;
    if (slot >= __ldcg(P.count)) return;  // the whole CTA, before any barrier or TMEM allocation
    pair = __ldcg(P.active + slot);
    rblk = blockIdx.x % P.nrb;
  }
  const int64_t rbase = (int64_t)pair * P.rows_per_pair, cbase = (int64_t)pair * P.cols_per_pair;
  const int r0 = rblk * OL_M;
  const int cs = blockIdx.y;
  const int t0 = (int)((int64_t)cs * P.col_tiles / P.split), t1 = (int)((int64_t)(cs + 1) * P.col_tiles / P.split);
  const int ntl = t1 - t0;                     // this CTA's streamed tiles
  const int nsteps = ntl * P.k_tiles;          // streamed (tile, k-tile) steps

  if (threadIdx.x == 0) {
    mbar_init(res_full, 1);
    for (int s = 0; s < OL_STAGES; ++s) { mbar_init(full + s, 1); mbar_init(empty + s, 1); }
    for (int b = 0; b < OL_NBUF; ++b) { mbar_init(accf + b, 1); mbar_init(acce + b, OL_EPI); }
    for (int s2 = 0; s2 < OL_STAGES; ++s2) relcnt[s2] = 0u;
    fence_mbar_init();
    prefetch_tmap(&tAh); prefetch_tmap(&tAl); prefetch_tmap(&tBh); prefetch_tmap(&tBl);
  }
  if (warp == OL_EPI + 1) tmem_alloc(tslot, OL_NBUF * OL_N);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == OL_EPI) {
    // producer
    if (lane == 0) {
      mbar_arrive_expect_tx(res_full, 2 * OL_TILE * P.k_tiles);
      for (int kt = 0; kt < P.k_tiles; ++kt) {
        tma_load_2d(resident + (2 * kt) * OL_TILE, &tAh, kt * OL_K, (int)(rbase + r0), res_full);
        tma_load_2d(resident + (2 * kt + 1) * OL_TILE, &tAl, kt * OL_K, (int)(rbase + r0), res_full);
      }
      int issued = 0;
      for (int q = 0; q < nsteps; ++q) {
        const int s = q % OL_STAGES;
        if (!mbar_wait(empty + s, ((q / OL_STAGES) & 1u) ^ 1u, P.abort_flag, P.timeout_ns)) break;
        const int tile = t0 + q / P.k_tiles, kt = q % P.k_tiles;
        unsigned char* st = ring + s * OL_STAGE;
        mbar_arrive_expect_tx(full + s, 2 * OL_TILE + OL_HVEC);
        tma_load_2d(st, &tBh, kt * OL_K, (int)(cbase + tile * OL_N), full + s);
        tma_load_2d(st + OL_TILE, &tBl, kt * OL_K, (int)(cbase + tile * OL_N), full + s);
        bulk_g2s(hbuf + s * OL_N, P.h + cbase + (int64_t)tile * OL_N, OL_HVEC, full + s);
        ++issued;
      }
      const int lo = issued > OL_STAGES ? issued - OL_STAGES : 0;
      for (int q = lo; q < issued; ++q) {
        const uint64_t t0 = globaltimer();
        while (!mbar_try_wait(full + q % OL_STAGES, (q / OL_STAGES) & 1u))
          if (globaltimer() - t0 > P.timeout_ns) break;
      }
      const uint64_t t0 = globaltimer();
      while (!mbar_try_wait(res_full, 0)) if (globaltimer() - t0 > P.timeout_ns) break;
    }
  } else if (warp == OL_EPI + 1) {
    // MMA issuer: one accumulator tile per streamed tile, TMEM buffers in turn
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_f16(OL_M, OL_N, false);
      bool ok = mbar_wait(res_full, 0, P.abort_flag, P.timeout_ns);
      int q = 0, committed = 0;
      for (int tile = 0; tile < ntl && ok; ++tile) {
        const int b = tile % OL_NBUF;
        if (!mbar_wait(acce + b, ((tile / OL_NBUF) & 1) ^ 1, P.abort_flag, P.timeout_ns)) break;
        tc_fence_after();
        const uint32_t dst = tmem + (uint32_t)(b * OL_N);
        uint32_t acc = 0;
        for (int kt = 0; kt < P.k_tiles; ++kt, ++q) {
          const int s = q % OL_STAGES;
          if (!mbar_wait(full + s, (q / OL_STAGES) & 1u, P.abort_flag, P.timeout_ns)) { ok = false; break; }
          tc_fence_after();
          unsigned char* st = ring + s * OL_STAGE;
          const uint64_t ah = umma_desc_k128(resident + (2 * kt) * OL_TILE);
          const uint64_t al = umma_desc_k128(resident + (2 * kt + 1) * OL_TILE);
          const uint64_t bh = umma_desc_k128(st), bl = umma_desc_k128(st + OL_TILE);
#pragma unroll
          for (int kk = 0; kk < OL_K / 16; ++kk) {
            const uint64_t o = (uint64_t)(kk * 32) >> 4;
            umma_f16(dst, ah + o, bh + o, idesc, acc);
            acc = 1;
            umma_f16(dst, ah + o, bl + o, idesc, 1);
            umma_f16(dst, al + o, bh + o, idesc, 1);
          }
          // the stage's h slice is read by the epilogue: release the stage only
          // after the epilogue is done with this tile (see below), except for
          // stages of earlier k-tiles of the same tile, which only the MMAs read
          if (kt + 1 < P.k_tiles) umma_commit(empty + s);
        }
        if (!ok) break;
        umma_commit(accf + b);
        committed = tile + 1;
      }
      if (committed > 0) {
        const int c = committed - 1;
        const uint64_t t0 = globaltimer();
        while (!mbar_try_wait(accf + (c % OL_NBUF), (c / OL_NBUF) & 1)) if (globaltimer() - t0 > P.timeout_ns) break;
      }
    }
  } else {
    // epilogue: warp w reads TMEM lane quarter w % 4 (rows 32 (w % 4) + lane)
    // and columns 32 (w / 4) .. +31 of each tile
    const int quarter = warp & 3, cgrp = warp >> 2;
    const int row_local = quarter * 32 + lane;
    // running (max, sum) per row; the sum is Kahan-compensated (sc) and each
    // tile adds one partial sum of 32 terms, so rounding does not grow with
    // the number of streamed points
    float mx = -INFINITY, sm = 0.f, sc = 0.f;
    int ok = 1;
    for (int tile = 0; tile < ntl && ok; ++tile) {
      const int b = tile % OL_NBUF;
      if (lane == 0) ok = (mbar_wait(accf + b, (tile / OL_NBUF) & 1, P.abort_flag, P.timeout_ns) &&
                           !*(volatile int*)P.abort_flag) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
      if (!ok) break;
      tc_fence_after();
      // the last k-step's stage holds this tile's h slice
      const int qlast = tile * P.k_tiles + P.k_tiles - 1;
      const float* h = hbuf + (qlast % OL_STAGES) * OL_N;
      {
        // packed fp32x2 arithmetic (one instruction per column pair, each
        // lane rounded as the scalar op) and three-input max: the epilogue
        // is bound by instruction issue, and the partial sums group the
        // terms exactly as four scalar accumulators would
        uint32_t v[32];
        const int col = cgrp * 32;
        tmem_ld32u(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * OL_N + col), v);
        const ulonglong2* hv = reinterpret_cast<const ulonglong2*>(h + col);
        const float alpha = P.alpha_p ? __ldg(P.alpha_p + pair) : P.alpha;
        const uint64_t a2 = pack2(alpha, alpha);
        uint64_t t2[16];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const ulonglong2 hh = hv[i];
          t2[2 * i] = fma2(pack2u(v[4 * i], v[4 * i + 1]), a2, hh.x);
          t2[2 * i + 1] = fma2(pack2u(v[4 * i + 2], v[4 * i + 3]), a2, hh.y);
        }
        float t[32];
#pragma unroll
        for (int i = 0; i < 16; ++i) unpack2(t2[i], t[2 * i], t[2 * i + 1]);
        float m1[11];
#pragma unroll
        for (int i = 0; i < 10; ++i) m1[i] = fmax3(t[3 * i], t[3 * i + 1], t[3 * i + 2]);
        m1[10] = fmaxf(t[30], t[31]);
        const float n0 = fmax3(m1[0], m1[1], m1[2]), n1 = fmax3(m1[3], m1[4], m1[5]);
        const float n2 = fmax3(m1[6], m1[7], m1[8]), n3 = fmaxf(m1[9], m1[10]);
        const float nm = fmax3(mx, fmax3(n0, n1, n2), n3);
        if (MAXP) {
          mx = nm;
        } else if (nm != -INFINITY) {
          const float r = ex2(mx - nm);
          sm *= r;
          sc *= r;
          const uint64_t nm2 = pack2(nm, nm);
          uint64_t acc0 = 0ull, acc1 = 0ull;  // columns 4k, 4k+1 and 4k+2, 4k+3
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            float x0, x1;
            unpack2(sub2(t2[i], nm2), x0, x1);
            const uint64_t e2 = pack2(ex2(x0), ex2(x1));
            if (i & 1) acc1 = add2(acc1, e2);
            else acc0 = add2(acc0, e2);
          }
          float p0, p1, p2, p3;
          unpack2(acc0, p0, p1);
          unpack2(acc1, p2, p3);
          const float part = (p0 + p1) + (p2 + p3);
          const float y = part - sc;
          const float tt = sm + y;
          sc = (tt - sm) - y;
          sm = tt;
          mx = nm;
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) {
        mbar_arrive(acce + b);
        // the tile's last stage (its h slice) is released once all
        // epilogue warps have read it
        const int s = qlast % OL_STAGES;
        if (atomicAdd(relcnt + s, 1u) == (unsigned)(OL_EPI - 1)) { atomicExch(relcnt + s, 0u); mbar_arrive(empty + s); }
      }
    }
    // merge the four column groups of each row
    if (cgrp > 0) { red[(cgrp - 1) * 2 * OL_M + row_local] = mx; red[(cgrp - 1) * 2 * OL_M + OL_M + row_local] = sm; }
    named_bar(1, OL_EPI * 32);
    if (cgrp == 0 && ok) {
      for (int g = 0; g < 3; ++g) lse_merge(mx, sm, red[g * 2 * OL_M + row_local], red[g * 2 * OL_M + OL_M + row_local]);
      const int row = r0 + row_local;
      const int64_t ri = rbase + row;  // the row in the packed vectors
      if (MAXP) {
        if (row < P.n_rows) P.pot_out2[ri] = mx + P.rterm[ri];
      } else if (P.split > 1) {
        P.part[((size_t)cs * 2) * P.rows_pad + row] = mx;
        P.part[((size_t)cs * 2 + 1) * P.rows_pad + row] = sm;
      } else if (row < P.n_rows) {
        const float L = lse_value(mx, sm) + P.rterm[ri];  // base-2 LSE_j(g2_j - C_ij log2e/reg)
        const float pnew = P.logw2[ri] - L;
        if (P.err) {
          const double e = (double)ex2(P.pot2[ri] + L) - (double)P.w[ri];
          P.err[ri] = P.err_sq ? e * e : fabs(e);
        }
        P.pot_out2[ri] = pnew;
        P.h_out[ri] = pnew - P.other_norm2[ri];
      } else {
        P.h_out[ri] = -INFINITY;  // padding rows of the resident side
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == OL_EPI + 1) {
    tc_fence_after();
    tmem_dealloc(tmem, OL_NBUF * OL_N);
  }
}

// Column-split passes: merge the S partial (max, sum) pairs of each row and
// apply the potential update of the pass's epilogue (check passes: the row's
// error into its slot).
__global__ void __launch_bounds__(256) online_finalize_kernel(OnlinePass P) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row < P.rows_pad) {
    if (row < P.n_rows) {
      float mx = -INFINITY, sm = 0.f;
      for (int c = 0; c < P.split; ++c)
        lse_merge(mx, sm, P.part[((size_t)c * 2) * P.rows_pad + row], P.part[((size_t)c * 2 + 1) * P.rows_pad + row]);
      const float L = lse_value(mx, sm) + P.rterm[row];
      const float pnew = P.logw2[row] - L;
      if (P.err) P.err[row] = fabs((double)ex2(P.pot2[row] + L) - (double)P.w[row]);
      P.pot_out2[row] = pnew;
      P.h_out[row] = pnew - P.other_norm2[row];
    } else {
      P.h_out[row] = -INFINITY;
    }
  }
}


__global__ void prep_points_kernel(const float* __restrict__ X, int64_t n, int d, float scale, __half* hi, __half* lo,
                                   int64_t ld, float k2, float* norm2) {
  // one warp per point: half planes of scale*x and log2(e)|x|^2/reg (k2 = log2(e)/reg)
  const int64_t i = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (i >= n) return;
  float s = 0.f;
  for (int k = lane; k < d; k += 32) {
    const float x = X[i * d + k];
    s = fmaf(x, x, s);
    const float xs = x * scale;
    const __half h = __float2half_rn(xs);
    hi[i * ld + k] = h;
    lo[i * ld + k] = __float2half_rn(xs - __half2float(h));
  }
  s = warp_sum(s);
  if (lane == 0) norm2[i] = s * k2;
}

__global__ void init_h_kernel(const float* pot2, const float* norm2, int64_t n, int64_t npad, float* h) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x)
    h[i] = i < n ? pot2[i] - norm2[i] : -INFINITY;
}

__global__ void log2w_kernel(const float* w, int64_t n, float* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = lg2(w[i]);
}

__global__ void scale_kernel(const float* x, int64_t n, float s, float* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = x[i] * s;
}

__global__ void neg_kernel(const float* x, int64_t n, float* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = -x[i];
}

}  // namespace otg

using namespace otg;

namespace {

typedef CUresult (*EncodeTiledFn2)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn2 ol_encode_fn() {
  static EncodeTiledFn2 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn2>(p);
  });
  return fn;
}

bool ol_plane_map(CUtensorMap* m, const void* base, int64_t rows, int64_t ld) {
  EncodeTiledFn2 fn = ol_encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {OL_K, OL_M};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

constexpr size_t OL_SMEM = (size_t)OL_MAXKT * 2 * OL_TILE + (size_t)OL_STAGES * OL_STAGE + OL_STAGES * OL_HVEC +
                           1024 /*align*/ + 256 /*barriers*/ + 6 * OL_M * 4 /*red*/ + 64 /*counters*/;

size_t a16(size_t x) { return (x + 255) / 256 * 256; }

constexpr int OL_MAX_SPLIT = 8;

// Column split for a pass of `nb` row blocks over `tiles` streamed tiles:
// the S in 1..8 whose grid (nb x S CTAs, one per SM at a time) loses the
// least to its last partial wave, keeping at least 32 tiles per CTA (fewer
// lose more to the pipeline's fill and drain than the wave gains; measured).
int choose_split(int nb, int tiles, int sms) {
  int best = 1;
  double best_eff = 0.0;
  for (int S = 1; S <= OL_MAX_SPLIT; ++S) {
    if (S > 1 && tiles / S < 32) break;
    const double waves = (double)nb * S / sms;
    const double eff = waves / std::ceil(waves);
    if (eff > best_eff + 0.02) { best_eff = eff; best = S; }
  }
  return best;
}

}  // namespace

extern "C" {

size_t otg_online_workspace_bytes(int64_t n, int64_t m, int32_t d) {
  const int64_t np = (n + 127) / 128 * 128, mp = (m + 127) / 128 * 128;
  const int64_t dp = (d + 63) / 64 * 64;
  size_t b = 0;
  b += 2 * a16(2 * np * dp) + 2 * a16(2 * mp * dp);          // half planes
  b += 5 * a16(4 * np) + 4 * a16(4 * mp);                    // norms, log2 w, potentials, h
  b += a16(8 * 64);                                          // err slots, flag
  b += a16(8 * (size_t)std::max(np, mp));                    // per-row errors of a check pass
  b += a16(4 * np) + a16(4 * mp);                            // negated norms
  b += a16(4 * 2 * (size_t)OL_MAX_SPLIT * (size_t)std::max(np, mp));  // column-split partials
  return b;
}

int otg_sinkhorn_online(const OtgOnlineProblem* p, cudaStream_t st) {
  if (!p || !p->X || !p->Y || !p->a || !p->b || !p->out_f || !p->out_g || !p->workspace || !p->info || !p->err_hist)
    return OTG_ERR_ARG;
  if (p->n < 1 || p->m < 1 || p->d < 1 || p->d > 64 * OL_MAXKT || !(p->reg > 0)) return OTG_ERR_ARG;
  if (p->workspace_bytes < otg_online_workspace_bytes(p->n, p->m, p->d)) return OTG_ERR_WORKSPACE;
  const int64_t n = p->n, m = p->m;
  const int64_t np = (n + 127) / 128 * 128, mp = (m + 127) / 128 * 128;
  const int dp = (p->d + 63) / 64 * 64;
  char* w = static_cast<char*>(p->workspace);
  size_t off = 0;
  auto take = [&](size_t bytes) { char* q = w + off; off += a16(bytes); return q; };
  __half* xh = reinterpret_cast<__half*>(take(2 * np * dp));
  __half* xl = reinterpret_cast<__half*>(take(2 * np * dp));
  __half* yh = reinterpret_cast<__half*>(take(2 * mp * dp));
  __half* yl = reinterpret_cast<__half*>(take(2 * mp * dp));
  float* xn2 = reinterpret_cast<float*>(take(4 * np));
  float* la2 = reinterpret_cast<float*>(take(4 * np));
  float* f2[2] = {reinterpret_cast<float*>(take(4 * np)), reinterpret_cast<float*>(take(4 * np))};
  float* yn2 = reinterpret_cast<float*>(take(4 * mp));
  float* lb2 = reinterpret_cast<float*>(take(4 * mp));
  float* g2 = reinterpret_cast<float*>(take(4 * mp));
  float* hy = reinterpret_cast<float*>(take(4 * mp));
  float* hx = reinterpret_cast<float*>(take(4 * np));
  double* errs = reinterpret_cast<double*>(take(8 * 64));
  int* flag = reinterpret_cast<int*>(errs + 62);
  double* erow = reinterpret_cast<double*>(take(8 * (size_t)std::max(np, mp)));
  const float k2 = (float)(OTG_LOG2E / p->reg);
  const float sx = p->scale_x, sy = p->scale_y;
  // planes are zero beyond the data; norms, weights and potentials set below
  if (cudaMemsetAsync(w, 0, off, st) != cudaSuccess) return OTG_ERR_CUDA;
  prep_points_kernel<<<(unsigned)((n + 7) / 8), 256, 0, st>>>(p->X, n, p->d, sx, xh, xl, dp, k2, xn2);
  prep_points_kernel<<<(unsigned)((m + 7) / 8), 256, 0, st>>>(p->Y, m, p->d, sy, yh, yl, dp, k2, yn2);
  log2w_kernel<<<256, 256, 0, st>>>(p->a, n, la2);
  log2w_kernel<<<256, 256, 0, st>>>(p->b, m, lb2);
  // initial potentials (natural log in, base 2 inside)
  if (p->warm_f) scale_kernel<<<256, 256, 0, st>>>(p->warm_f, n, (float)OTG_LOG2E, f2[0]);
  if (p->warm_g) scale_kernel<<<256, 256, 0, st>>>(p->warm_g, m, (float)OTG_LOG2E, g2);
  init_h_kernel<<<256, 256, 0, st>>>(g2, yn2, m, mp, hy);
  if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
  CUtensorMap mxh, mxl, myh, myl;
  if (!ol_plane_map(&mxh, xh, np, dp) || !ol_plane_map(&mxl, xl, np, dp) || !ol_plane_map(&myh, yh, mp, dp) ||
      !ol_plane_map(&myl, yl, mp, dp))
    return OTG_ERR_CUDA;
  static bool attr = false;
  if (!attr) {
    if (cudaFuncSetAttribute(online_pass_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)OL_SMEM) !=
        cudaSuccess)
      return OTG_ERR_CUDA;
    attr = true;
  }
  // row terms as separate buffers: -xn2, -yn2
  float* nx = reinterpret_cast<float*>(take(4 * np));
  float* ny = reinterpret_cast<float*>(take(4 * mp));
  float* part = reinterpret_cast<float*>(take(4 * 2 * (size_t)OL_MAX_SPLIT * (size_t)std::max(np, mp)));
  if (off > p->workspace_bytes) return OTG_ERR_WORKSPACE;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int split_f = choose_split((int)(np / OL_M), (int)(mp / OL_N), sms);
  const int split_g = choose_split((int)(mp / OL_M), (int)(np / OL_N), sms);
  // one pass: the pass kernel over (row blocks x column split), then, when
  // split, the merge of the partials
  // (check passes: the per-row errors go to erow, their sum to `eslot`)
  auto pass = [&](OnlinePass& P, const CUtensorMap& ah, const CUtensorMap& al, const CUtensorMap& bh,
                  const CUtensorMap& bl, int64_t rows_pad, int split, double* eslot_of_pass) {
    P.split = split; P.rows_pad = (int)rows_pad; P.part = part;
    online_pass_kernel<false><<<dim3((unsigned)(rows_pad / OL_M), (unsigned)split), OL_THREADS, OL_SMEM, st>>>(ah, al, bh,
                                                                                                       bl, P);
    if (split > 1) online_finalize_kernel<<<(unsigned)((rows_pad + 255) / 256), 256, 0, st>>>(P);
    // the L1 error: the row slots summed in a fixed order (the same value in every run)
    if (P.err) slot_sum_kernel<1024><<<1, 1024, 0, st>>>(P.err, P.n_rows, eslot_of_pass);
  };
  neg_kernel<<<256, 256, 0, st>>>(xn2, n, nx);
  neg_kernel<<<256, 256, 0, st>>>(yn2, m, ny);
  const float alpha = (float)(2.0 * OTG_LOG2E / (p->reg * (double)sx * (double)sy));
  const uint64_t tmo = p->timeout_ms > 0 ? (uint64_t)p->timeout_ms * 1000000ull : 4000000000ull;
  int cur = 0, nchk = 0, status = OTG_STATUS_MAXITER, niter = p->max_iter - 1;
  for (int it = 0; it < p->max_iter; ++it) {
    const bool check = (it > 0) && (it % 10 == 0);  // error of iteration it-1 ((it-1)+1) % 10 == 0
    double* eslot = errs + (nchk % 60);
    // f pass: rows = X, streamed = Y (h = g2 - |y|^2 k2)
    OnlinePass A{};
    A.n_rows = (int)n; A.col_tiles = (int)(mp / OL_N); A.k_tiles = dp / OL_K; A.alpha = alpha;
    A.h = hy; A.rterm = nx; A.logw2 = la2; A.pot2 = f2[cur]; A.w = p->a; A.pot_out2 = f2[cur ^ 1];
    A.other_norm2 = xn2; A.h_out = hx; A.err = check ? erow : nullptr; A.abort_flag = flag; A.timeout_ns = tmo;
    pass(A, mxh, mxl, myh, myl, np, split_f, eslot);
    if (check) {
      double e = 0;
      if (cudaMemcpyAsync(&e, eslot, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
      if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
      if (nchk < p->hist_cap) p->err_hist[nchk] = e;
      ++nchk;
      if (e <= p->stop_thr) { status = OTG_STATUS_CONVERGED; niter = it - 1; break; }
    }
    cur ^= 1;
    // g pass: rows = Y, streamed = X (h = f2 - |x|^2 k2)
    OnlinePass B{};
    B.n_rows = (int)m; B.col_tiles = (int)(np / OL_N); B.k_tiles = dp / OL_K; B.alpha = alpha;
    B.h = hx; B.rterm = ny; B.logw2 = lb2; B.pot2 = g2; B.w = p->b; B.pot_out2 = g2;
    B.other_norm2 = yn2; B.h_out = hy; B.err = nullptr; B.abort_flag = flag; B.timeout_ns = tmo;
    pass(B, myh, myl, mxh, mxl, mp, split_g, nullptr);
    if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
  }
  // a last check at max_iter when (max_iter) % 10 == 0 is done by the next f pass
  if (status == OTG_STATUS_MAXITER && p->max_iter > 0 && p->max_iter % 10 == 0) {
    double* eslot = errs + (nchk % 60);
    OnlinePass A{};
    A.n_rows = (int)n; A.col_tiles = (int)(mp / OL_N); A.k_tiles = dp / OL_K; A.alpha = alpha;
    A.h = hy; A.rterm = nx; A.logw2 = la2; A.pot2 = f2[cur]; A.w = p->a; A.pot_out2 = f2[cur ^ 1];
    A.other_norm2 = xn2; A.h_out = hx; A.err = erow; A.abort_flag = flag; A.timeout_ns = tmo;
    pass(A, mxh, mxl, myh, myl, np, split_f, eslot);
    double e = 0;
    cudaMemcpyAsync(&e, eslot, 8, cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    if (nchk < p->hist_cap) p->err_hist[nchk] = e;
    ++nchk;
    if (e <= p->stop_thr) status = OTG_STATUS_CONVERGED;
  }
  // outputs in natural units
  scale_kernel<<<256, 256, 0, st>>>(f2[cur], n, (float)OTG_LN2, p->out_f);
  scale_kernel<<<256, 256, 0, st>>>(g2, m, (float)OTG_LN2, p->out_g);
  int hflag = 0;
  cudaMemcpyAsync(&hflag, flag, 4, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
  p->info[0] = hflag ? OTG_STATUS_ABORTED : status;
  p->info[1] = niter;
  p->info[2] = nchk;
  return OTG_OK;
}

}  // extern "C"
