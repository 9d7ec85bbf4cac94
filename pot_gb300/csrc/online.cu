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
//
// Folded passes (d <= 64, one K-tile): the planes carry sqrt(alpha) on both
// sides, and one more MMA per tile reads 16 extension columns of each side
// (exact three-piece fp16 encodings of h_j and of the row's shift s_i, the
// row's LSE of the previous pass in the same direction), so the accumulator
// already holds t_ij - s_i: the epilogue only exponentiates and sums (no
// running max, no per-tile rescaling, no h slices in the stages).  A row
// whose shifted sum leaves [2^-70, 2^100] writes nothing and its row block
// is recomputed with the running max by the pass's fix-up launch (the first
// pass of each side, which has no shift yet, and column-split passes keep
// the running max throughout).
#include <cuda.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include "common.cuh"
#include "tma.cuh"
#include "tc.cuh"
#include "anderson.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

constexpr int OL_M = 128, OL_N = 128, OL_K = 64, OL_STAGES = 4;
constexpr uint32_t OL_TILE = OL_M * OL_K * 2;          // one half plane tile (16 KiB)
constexpr uint32_t OL_TILE_NARROW = OL_M * 16 * 2;     // a narrow (16-wide) plane tile (4 KiB)
constexpr uint32_t OL_HVEC = OL_N * 4;                 // h slice of a tile (512 B)
constexpr uint32_t OL_EXT = OL_M * 16 * 2;             // an extension tile: 128 points x 16 halves (4 KiB)
constexpr uint32_t OL_EXTRA = 8192;                    // h slices / the last stage's extension tiles
constexpr uint32_t OL_STAGE = 2 * OL_TILE;             // streamed hi, lo (1024-aligned tiles)
// narrow planes: stages of 16 KiB (dot hi, lo; folded: extension hi, lo;
// 4 KiB each), eight of them in the ring (the deeper ring hides the L2
// latency of the short narrow tiles)
constexpr int OL_NS_NARROW = 8;
constexpr uint32_t OL_STAGE_NARROW = 16384;
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
  // narrow planes (d <= 16): one K-tile of 16 values, 32-byte rows written by
  // TMA with the 32-byte swizzle, one k-step (three MMAs) per streamed tile;
  // the tiles keep their 16 KiB shared-memory slots (only 4 KiB are used)
  int narrow;
  // folded passes (OL_FMAX, OL_FSUM; one K-tile): the resident side's new
  // extension columns (row form with the new shift, str form with the new
  // h) and shift; the shift read (s_i, base 2, without the row term);
  // per-row failure marks, the failed units of the pass and its fix-up's
  // counters.  fixup: this launch recomputes the marked rows of the listed
  // units (units_enc: active holds the units) and clears the marks.
  __half* ext_row; __half* ext_str;
  const float* shift; float* shift_out;
  unsigned char* fail;
  int* fail_list; int* fail_cnt; unsigned* done_cnt;
  int fixup, units_enc;
  float sum_lo, sum_hi;  // acceptance range of the shifted sums
};

// Epilogue modes of a pass.
//   OL_LSE : t = alpha acc + h_j (h slice from the stage): running base-2
//            max and sum per row.
//   OL_MAXP: the running max of t only (the max cost of a pair).
//   OL_FMAX: folded: alpha is in the planes and the extension columns add
//            h_j - s_i, so the accumulator holds t - s_i itself (s_i: the
//            row's shift, its LSE of the previous pass in this direction);
//            running max and sum of it.
//   OL_FSUM: folded, the plain sum of 2^(t - s_i): no running max, no
//            rescaling.  A row whose sum leaves [2^-70, 2^100] writes nothing
//            and is recomputed in OL_FMAX by the pass's fix-up launch.
enum { OL_LSE = 0, OL_MAXP = 1, OL_FMAX = 2, OL_FSUM = 3 };

// Extension columns of a point: 16 halves (the last 10 zero) in one plane,
// read by one MMA (no low plane).  A value v is carried as
// 256 a + b + c with a = fp16(v / 256), r = v - 256 a (exact in fp32),
// b = fp16(r), c = fp16(r - b): about 33 significant bits for |v| up to
// 1.6e7 (larger magnitudes are clamped; -inf marks padding and becomes
// -1.6e7, whose exponential is 0; NaN stays NaN).
//   row form (the point resident):  [256, 1, 1, a(-s), b(-s), c(-s)]
//   str form (the point streamed):  [a(h), b(h), c(h), 256, 1, 1]
// so the extension MMA adds 256 a(h) + b(h) + c(h) + 256 a(-s) + b(-s) +
// c(-s) = h_j - s_i (every product exact).
__device__ __forceinline__ void ext_put(__half* ext, int64_t row, float v, bool str) {
  float cl = fminf(fmaxf(v, -1.6e7f), 1.6e7f);
  if (isnan(v)) cl = v;
  const __half a = __float2half_rn(cl * 0.00390625f);
  const float r = cl - __half2float(a) * 256.f;
  const __half b = __float2half_rn(r);
  const __half c = __float2half_rn(r - __half2float(b));
  const __half z = __float2half_rn(0.f), c256 = __float2half_rn(256.f), one = __float2half_rn(1.f);
  __align__(16) __half H[8] = {z, z, z, z, z, z, z, z};
  if (str) { H[0] = a; H[1] = b; H[2] = c; H[3] = c256; H[4] = one; H[5] = one; }
  else { H[0] = c256; H[1] = one; H[2] = one; H[3] = a; H[4] = b; H[5] = c; }
  uint4* ph = reinterpret_cast<uint4*>(ext + row * 16);
  ph[0] = *reinterpret_cast<const uint4*>(H);
  ph[1] = make_uint4(0u, 0u, 0u, 0u);
}

// Shifted-sum arithmetic of one warp's 32 columns (accumulator values t - s
// already in registers): the exponentials summed as packed pairs (columns
// 4k, 4k+1 and 4k+2, 4k+3), one Kahan-compensated partial per tile.
__device__ __forceinline__ void ol_fsum_acc(const uint32_t* v, float& sm, float& sc) {
  uint64_t acc0 = 0ull, acc1 = 0ull;
#pragma unroll
  for (int i = 0; i < 16; ++i) {
    const uint64_t e2 = pack2(ex2(__uint_as_float(v[2 * i])), ex2(__uint_as_float(v[2 * i + 1])));
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
}

// One tile of the epilogue for one warp: its 32 columns of the tile's
// accumulator (TMEM address taddr) fold into the running base-2 (max, sum)
// (OL_FSUM: sum) of the warp's rows.  The TMEM buffer (acce_b) is handed
// back as soon as its contents are in registers, and in the unfolded modes,
// from the last epilogue warp, the stage holding the h slice (empty_s,
// counted in relcnt_s).
template <int MODE>
__device__ __forceinline__ void ol_epi_tile(uint32_t taddr, const float* hcol, uint64_t a2, uint64_t* acce_b,
                                            unsigned* relcnt_s, uint64_t* empty_s, int lane, float& mx, float& sm,
                                            float& sc) {
  uint32_t v[32];
  tmem_ld32u(taddr, v);
  if constexpr (MODE == OL_FSUM) {
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(acce_b);
    ol_fsum_acc(v, sm, sc);
    return;
  }
  // packed fp32x2 arithmetic (one instruction per column pair, each lane
  // rounded as the scalar op) and three-input max: fewer instructions for
  // the same arithmetic, and the partial sums group the terms exactly as
  // four scalar accumulators would
  uint64_t t2[16];
  if constexpr (MODE == OL_FMAX) {
#pragma unroll
    for (int i = 0; i < 16; ++i) t2[i] = pack2u(v[2 * i], v[2 * i + 1]);
    tc_fence_before();
    __syncwarp();
    if (lane == 0) mbar_arrive(acce_b);
  } else {
    const ulonglong2* hv = reinterpret_cast<const ulonglong2*>(hcol);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const ulonglong2 hh = hv[i];
      t2[2 * i] = fma2(pack2u(v[4 * i], v[4 * i + 1]), a2, hh.x);
      t2[2 * i + 1] = fma2(pack2u(v[4 * i + 2], v[4 * i + 3]), a2, hh.y);
    }
    // the accumulator and the h slice are in registers now: hand the TMEM
    // buffer back to the MMA warp and the stage to the producer before the
    // arithmetic
    tc_fence_before();
    __syncwarp();
    if (lane == 0) {
      mbar_arrive(acce_b);
      // the stage is released once all epilogue warps have read its h slice
      if (atomicAdd(relcnt_s, 1u) == (unsigned)(OL_EPI - 1)) { atomicExch(relcnt_s, 0u); mbar_arrive(empty_s); }
    }
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
  if (MODE == OL_MAXP) {
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
    // each tile adds one Kahan-compensated partial sum of 32 terms, so
    // rounding does not grow with the number of streamed points
    const float part = (p0 + p1) + (p2 + p3);
    const float y = part - sc;
    const float tt = sm + y;
    sc = (tt - sm) - y;
    sm = tt;
    mx = nm;
  }
}

// The MMAs of one streamed (tile, k-tile) step into TMEM column dst; FOLD:
// then the extension MMA (rext: the resident rows' row form, sext: the
// streamed points' str form), which adds h_j - s_i.
template <bool FOLD>
__device__ __forceinline__ void ol_mma_step(const OnlinePass& P, uint32_t dst, const unsigned char* resident,
                                            const unsigned char* st, const unsigned char* st_lo, int kt,
                                            uint32_t idesc, const unsigned char* rext, const unsigned char* sext) {
  if (P.narrow) {
    // one 16-wide k-step: 32-byte swizzled rows
    const uint64_t ah = umma_desc_k32(resident), al = umma_desc_k32(resident + OL_TILE);
    const uint64_t bh = umma_desc_k32(st), bl = umma_desc_k32(st_lo);
    umma_f16(dst, ah, bh, idesc, 0);
    umma_f16(dst, ah, bl, idesc, 1);
    umma_f16(dst, al, bh, idesc, 1);
  } else {
    const uint64_t ah = umma_desc_k128(resident + (2 * kt) * OL_TILE);
    const uint64_t al = umma_desc_k128(resident + (2 * kt + 1) * OL_TILE);
    const uint64_t bh = umma_desc_k128(st), bl = umma_desc_k128(st_lo);
#pragma unroll
    for (int kk = 0; kk < OL_K / 16; ++kk) {
      const uint64_t o = (uint64_t)(kk * 32) >> 4;
      umma_f16(dst, ah + o, bh + o, idesc, (kt | kk) ? 1u : 0u);
      umma_f16(dst, ah + o, bl + o, idesc, 1);
      umma_f16(dst, al + o, bh + o, idesc, 1);
    }
  }
  if constexpr (FOLD) umma_f16(dst, umma_desc_k32(rext), umma_desc_k32(sext), idesc, 1);
}

// The rows' results after the last tile: column groups 1-3 hand their
// (max, sum) to group 0 through `red` (the caller's named barrier sits
// between the two halves), group 0 merges and writes the row outputs.
// Returns false for a row that failed (OL_FSUM: its sum left the range; it
// writes nothing and is marked for the fix-up).  A fix-up launch
// (P.fixup) writes only the rows marked, and clears the marks.
// A row's inputs for its finish, loaded by the finishing thread when the
// unit starts (their memory latency then hides behind the unit's tiles).
struct OlRowIn { float shift, rterm, logw2, onorm, pot2, w; };

template <int MODE>
__device__ __forceinline__ OlRowIn ol_row_in(const OnlinePass& P, int64_t ri, bool valid) {
  OlRowIn v{0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (!valid) return v;
  v.rterm = P.rterm[ri];
  if (MODE == OL_MAXP) return v;
  if (MODE == OL_FMAX || MODE == OL_FSUM) v.shift = P.shift[ri];
  v.logw2 = P.logw2[ri];
  v.onorm = P.other_norm2[ri];
  if (P.err) { v.pot2 = P.pot2[ri]; v.w = P.w[ri]; }
  return v;
}

template <int MODE>
__device__ __forceinline__ bool ol_rows_out(const OnlinePass& P, const float* red, int row_local, float mx, float sm,
                                            int r0, int64_t rbase, int cs, const OlRowIn& in) {
  constexpr bool FOLD = MODE == OL_FMAX || MODE == OL_FSUM;
  if constexpr (MODE == OL_FSUM) {
    for (int g = 0; g < 3; ++g) sm += red[g * 2 * OL_M + OL_M + row_local];
  } else {
    for (int g = 0; g < 3; ++g) lse_merge(mx, sm, red[g * 2 * OL_M + row_local], red[g * 2 * OL_M + OL_M + row_local]);
  }
  const int row = r0 + row_local;
  const int64_t ri = rbase + row;  // the row in the packed vectors
  if constexpr (MODE == OL_MAXP) {
    if (row < P.n_rows) P.pot_out2[ri] = mx + in.rterm;
    return true;
  }
  if (MODE != OL_FSUM && P.split > 1) {
    P.part[((size_t)cs * 2) * P.rows_pad + row] = mx;
    P.part[((size_t)cs * 2 + 1) * P.rows_pad + row] = sm;
    return true;
  }
  if (row >= P.n_rows) {
    if constexpr (!FOLD) P.h_out[ri] = -INFINITY;  // padding rows of the resident side
    return true;                                     // (folded: the str form keeps its padding values)
  }
  if (P.fixup && !P.fail[ri]) return true;
  float lse_t;  // base-2 LSE_j(t_ij), without the row term
  if constexpr (MODE == OL_FSUM) {
    if (!(sm >= P.sum_lo && sm <= P.sum_hi)) {
      P.fail[ri] = 1;
      return false;
    }
    lse_t = in.shift + lg2(sm);
  } else if constexpr (MODE == OL_FMAX) {
    lse_t = in.shift + lse_value(mx, sm);
  } else {
    lse_t = lse_value(mx, sm);
  }
  const float L = lse_t + in.rterm;  // base-2 LSE_j(g2_j - C_ij log2e/reg)
  const float pnew = in.logw2 - L;
  if (P.err) {
    const double e = (double)ex2(in.pot2 + L) - (double)in.w;
    P.err[ri] = P.err_sq ? e * e : fabs(e);
  }
  P.pot_out2[ri] = pnew;
  const float hn = pnew - in.onorm;
  if constexpr (FOLD) {
    ext_put(P.ext_str, ri, hn, true);
    ext_put(P.ext_row, ri, -lse_t, false);
    P.shift_out[ri] = lse_t;
    if (P.fixup) P.fail[ri] = 0;
  } else {
    P.h_out[ri] = hn;
  }
  return true;
}

// Shared-memory carve-up of both pass kernels:
//   [resident 64 KiB][ring 128 KiB][extra 8 KiB][barriers, red, counters]
// The ring holds OL_STAGES stages of 32 KiB, or with narrow planes
// OL_NS_NARROW stages of 16 KiB (dot hi at 0, lo at 4 KiB, folded: the
// extension tile at 8 KiB).
// Unfolded passes: up to two resident k-tiles (hi, lo), the h slices in the
// extra region.  Folded passes (one k-tile): the resident dot tile at 0 (hi)
// and 16 KiB (lo), its extension tile at 32 KiB, the streamed extension
// tiles of stages 0-3 at 36, 40, 44 and 48 KiB (narrow planes: inside the
// stage, at 8 KiB).
struct OlSmem {
  unsigned char* resident; unsigned char* ring; unsigned char* extra; float* hbuf;
  uint64_t *res_full, *full, *empty, *accf, *acce, *res_empty;
  uint32_t* tslot; float* red; unsigned* relcnt; int* uflag;
};
static_assert(OL_STAGES == 4, "extension slot map assumes four stages");
static_assert(2 * OL_TILE + OL_EXT * (1 + OL_STAGES) <= OL_MAXKT * 2 * OL_TILE, "extension tiles fit the resident region");
__device__ __forceinline__ OlSmem ol_carve(unsigned char* smem_raw) {
  OlSmem S;
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  S.resident = smem;
  S.ring = smem + OL_MAXKT * 2 * OL_TILE;
  S.extra = S.ring + OL_STAGES * OL_STAGE;
  S.hbuf = reinterpret_cast<float*>(S.extra);  // [stage][128] h slices
  uint64_t* bars = reinterpret_cast<uint64_t*>(S.extra + OL_EXTRA);
  S.res_full = bars;                     // resident operand landed
  S.full = bars + 1;                     // [OL_NS_NARROW]
  S.empty = S.full + OL_NS_NARROW;       // [OL_NS_NARROW]
  S.accf = S.empty + OL_NS_NARROW;       // [OL_NBUF]
  S.acce = S.accf + OL_NBUF;             // [OL_NBUF]
  S.res_empty = S.acce + OL_NBUF;        // resident operand no longer read (batch kernel)
  S.tslot = reinterpret_cast<uint32_t*>(S.res_empty + 1);
  S.red = reinterpret_cast<float*>(S.tslot + 4);              // [3][2][128] (mx, s) of column groups 1-3
  S.relcnt = reinterpret_cast<unsigned*>(S.red + 6 * OL_M);   // [OL_NS_NARROW] epilogue warps done
  S.uflag = reinterpret_cast<int*>(S.relcnt + OL_NS_NARROW);  // a row of the unit failed
  return S;
}
__device__ __forceinline__ unsigned char* ol_res_ext(const OlSmem& S) { return S.resident + 2 * OL_TILE; }
__device__ __forceinline__ unsigned char* ol_ext_slot(const OlSmem& S, int s) {
  return S.resident + 2 * OL_TILE + OL_EXT * (1 + s);
}
// Ring geometry of a pass: stage count, stage bytes, offset of the lo tile.
// Stage s = q & mask, its phase (q >> shift) & 1 (both counts powers of two).
struct OlRing {
  int ns, mask, shift; uint32_t sb, lo;
  __device__ __forceinline__ explicit OlRing(bool narrow)
      : ns(narrow ? OL_NS_NARROW : OL_STAGES), mask(ns - 1), shift(narrow ? 3 : 2),
        sb(narrow ? OL_STAGE_NARROW : OL_STAGE), lo(narrow ? OL_TILE_NARROW : OL_TILE) {}
};
static_assert(OL_STAGES == 4 && OL_NS_NARROW == 8, "ring masks and shifts");
__device__ __forceinline__ unsigned char* ol_stage_ext(const OlSmem& S, const OlRing& R, bool narrow, int s) {
  return narrow ? S.ring + s * R.sb + 2 * OL_TILE_NARROW : ol_ext_slot(S, s);
}

__device__ __forceinline__ void ol_setup(const OlSmem& S, const CUtensorMap* tAh, const CUtensorMap* tAl,
                                         const CUtensorMap* tBh, const CUtensorMap* tBl) {
  if (threadIdx.x == 0) {
    mbar_init(S.res_full, 1);
    mbar_init(S.res_empty, 1);
    for (int s = 0; s < OL_NS_NARROW; ++s) { mbar_init(S.full + s, 1); mbar_init(S.empty + s, 1); }
    for (int b = 0; b < OL_NBUF; ++b) { mbar_init(S.accf + b, 1); mbar_init(S.acce + b, OL_EPI); }
    for (int s2 = 0; s2 < OL_NS_NARROW; ++s2) S.relcnt[s2] = 0u;
    *S.uflag = 0;
    fence_mbar_init();
    prefetch_tmap(tAh); prefetch_tmap(tAl); prefetch_tmap(tBh); prefetch_tmap(tBl);
  }
  if ((threadIdx.x >> 5) == OL_EPI + 1) tmem_alloc(S.tslot, OL_NBUF * OL_N);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
}

// A unit (pair, row block) whose rows failed goes to the pass's fix-up list
// (encoded as pair * nrb + row block).  Called by one epilogue thread after
// the epilogue's named barrier.
__device__ __forceinline__ void ol_note_unit(const OnlinePass& P, int* uflag, int pair, int r0) {
  if (*uflag) {
    *uflag = 0;
    P.fail_list[atomicAdd(P.fail_cnt, 1)] = pair * P.nrb + r0 / OL_M;
    atomicAdd(P.fail_cnt + 2, 1);  // units recomputed over the solve (a statistic)
  }
}

// Fix-up launches: the last CTA to finish empties the list for the next pass.
__device__ __forceinline__ void ol_fixup_done(const OnlinePass& P) {
  __threadfence();
  if (atomicAdd(P.done_cnt, 1u) == gridDim.x - 1) {
    *P.fail_cnt = 0;
    *P.done_cnt = 0u;
    __threadfence();
  }
}

// One problem: CTA (blockIdx.x, blockIdx.y) takes row block blockIdx.x and
// the streamed tiles of column range blockIdx.y, one unit per CTA.
template <int MODE>
__global__ void __launch_bounds__(OL_THREADS, 1)
online_pass_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                   const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl,
                   const __grid_constant__ CUtensorMap tR, const __grid_constant__ CUtensorMap tS, OnlinePass P) {
  constexpr bool FOLD = MODE == OL_FMAX || MODE == OL_FSUM;
  extern __shared__ unsigned char smem_raw[];
  const OlSmem S = ol_carve(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int r0 = blockIdx.x * OL_M;
  const int cs = blockIdx.y;
  const int t0 = (int)((int64_t)cs * P.col_tiles / P.split), t1 = (int)((int64_t)(cs + 1) * P.col_tiles / P.split);
  const int ntl = t1 - t0;                     // this CTA's streamed tiles
  const int nsteps = ntl * P.k_tiles;          // streamed (tile, k-tile) steps
  ol_setup(S, &tAh, &tAl, &tBh, &tBl);
  const uint32_t tmem = *S.tslot;
  const OlRing R(P.narrow != 0);

  if (warp == OL_EPI) {
    // producer
    if (lane == 0) {
      const uint32_t tbytes = P.narrow ? OL_TILE_NARROW : OL_TILE;  // bytes of one plane tile
      mbar_arrive_expect_tx(S.res_full, 2 * tbytes * P.k_tiles + (FOLD ? OL_EXT : 0));
      for (int kt = 0; kt < P.k_tiles; ++kt) {
        tma_load_2d(S.resident + (2 * kt) * OL_TILE, &tAh, kt * OL_K, r0, S.res_full);
        tma_load_2d(S.resident + (2 * kt + 1) * OL_TILE, &tAl, kt * OL_K, r0, S.res_full);
      }
      if (FOLD) {
        tma_load_2d(ol_res_ext(S), &tR, 0, r0, S.res_full);
      }
      int issued = 0;
      for (int q = 0; q < nsteps; ++q) {
        const int s = (q & R.mask);
        if (!mbar_wait(S.empty + s, ((q >> R.shift) & 1u) ^ 1u, P.abort_flag, P.timeout_ns)) break;
        const int tile = t0 + q / P.k_tiles, kt = q % P.k_tiles;
        unsigned char* st = S.ring + s * R.sb;
        if (FOLD) {
          unsigned char* ex = ol_stage_ext(S, R, P.narrow, s);
          mbar_arrive_expect_tx(S.full + s, 2 * tbytes + OL_EXT);
          tma_load_2d(st, &tBh, kt * OL_K, tile * OL_N, S.full + s);
          tma_load_2d(st + R.lo, &tBl, kt * OL_K, tile * OL_N, S.full + s);
          tma_load_2d(ex, &tS, 0, tile * OL_N, S.full + s);
        } else {
          mbar_arrive_expect_tx(S.full + s, 2 * tbytes + OL_HVEC);
          tma_load_2d(st, &tBh, kt * OL_K, tile * OL_N, S.full + s);
          tma_load_2d(st + R.lo, &tBl, kt * OL_K, tile * OL_N, S.full + s);
          bulk_g2s(S.hbuf + s * OL_N, P.h + (int64_t)tile * OL_N, OL_HVEC, S.full + s);
        }
        ++issued;
      }
      // copies still in flight land before the CTA leaves
      const int lo = issued > R.ns ? issued - R.ns : 0;
      for (int q = lo; q < issued; ++q) {
        const uint64_t w0 = globaltimer();
        while (!mbar_try_wait(S.full + (q & R.mask), (q >> R.shift) & 1u))
          if (globaltimer() - w0 > P.timeout_ns) break;
      }
      const uint64_t w0 = globaltimer();
      while (!mbar_try_wait(S.res_full, 0)) if (globaltimer() - w0 > P.timeout_ns) break;
    }
  } else if (warp == OL_EPI + 1) {
    // MMA issuer: one accumulator tile per streamed tile, TMEM buffers in turn
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_f16(OL_M, OL_N, false);
      bool ok = mbar_wait(S.res_full, 0, P.abort_flag, P.timeout_ns);
      int q = 0, committed = 0;
      for (int tile = 0; tile < ntl && ok; ++tile) {
        const int b = tile % OL_NBUF;
        if (!mbar_wait(S.acce + b, ((tile / OL_NBUF) & 1) ^ 1, P.abort_flag, P.timeout_ns)) break;
        tc_fence_after();
        for (int kt = 0; kt < P.k_tiles; ++kt, ++q) {
          const int s = (q & R.mask);
          if (!mbar_wait(S.full + s, (q >> R.shift) & 1u, P.abort_flag, P.timeout_ns)) { ok = false; break; }
          tc_fence_after();
          ol_mma_step<FOLD>(P, tmem + (uint32_t)(b * OL_N), S.resident, S.ring + s * R.sb, S.ring + s * R.sb + R.lo,
                            kt, idesc, ol_res_ext(S), ol_stage_ext(S, R, P.narrow, s));
          // unfolded: the stage's h slice is read by the epilogue, which
          // releases the tile's last stage; other stages only the MMAs read
          if (FOLD || kt + 1 < P.k_tiles) umma_commit(S.empty + s);
        }
        if (!ok) break;
        umma_commit(S.accf + b);
        committed = tile + 1;
      }
      if (committed > 0) {
        const int c = committed - 1;
        const uint64_t w0 = globaltimer();
        while (!mbar_try_wait(S.accf + (c % OL_NBUF), (c / OL_NBUF) & 1)) if (globaltimer() - w0 > P.timeout_ns) break;
      }
    }
  } else {
    // epilogue: warp w reads TMEM lane quarter w % 4 (rows 32 (w % 4) + lane)
    // and columns 32 (w / 4) .. +31 of each tile
    const int quarter = warp & 3, cgrp = warp >> 2;
    const int row_local = quarter * 32 + lane;
    const OlRowIn rin = ol_row_in<MODE>(P, r0 + row_local, cgrp == 0 && r0 + row_local < P.n_rows);
    float mx = -INFINITY, sm = 0.f, sc = 0.f;
    int ok = 1;
    const uint64_t a2 = pack2(P.alpha, P.alpha);
    for (int tile = 0; tile < ntl && ok; ++tile) {
      const int b = tile % OL_NBUF;
      // (mbar_wait itself polls the abort flag while it spins)
      if (lane == 0) ok = mbar_wait(S.accf + b, (tile / OL_NBUF) & 1, P.abort_flag, P.timeout_ns) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);
      __syncwarp();
      if (!ok) break;
      tc_fence_after();
      // the last k-step's stage holds this tile's h slice
      const int s = (tile * P.k_tiles + P.k_tiles - 1) & R.mask;
      ol_epi_tile<MODE>(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * OL_N + cgrp * 32),
                        S.hbuf + s * OL_N + cgrp * 32, a2, S.acce + b, S.relcnt + s, S.empty + s, lane, mx, sm, sc);
    }
    // merge the four column groups of each row
    if (cgrp > 0) { S.red[(cgrp - 1) * 2 * OL_M + row_local] = mx; S.red[(cgrp - 1) * 2 * OL_M + OL_M + row_local] = sm; }
    named_bar(1, OL_EPI * 32);
    if (cgrp == 0 && ok && !ol_rows_out<MODE>(P, S.red, row_local, mx, sm, r0, 0, cs, rin)) *S.uflag = 1;
    if constexpr (MODE == OL_FSUM) {
      named_bar(1, OL_EPI * 32);
      if (warp == 0 && lane == 0) ol_note_unit(P, S.uflag, 0, r0);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == OL_EPI + 1) {
    tc_fence_after();
    tmem_dealloc(tmem, OL_NBUF * OL_N);
  }
}

// A batch of pairs: units (active slot, row block), taken by the CTAs in
// turn (one CTA per SM keeps its TMEM, barriers and pipeline across its
// units; the stage and tile counters run on).  Slot k's pair is active[k],
// k < *count.  With units_enc (fix-up launches) the list holds the units
// themselves, pair * nrb + row block, *count of them.  OL_MAXP: instead of
// the log-sum-exp, each row's max of t (the max cost of a pair, which sets
// its regularisation): no exponentials.
template <int MODE>
__global__ void __launch_bounds__(OL_THREADS, 1)
online_batch_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                    const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl,
                    const __grid_constant__ CUtensorMap tR, const __grid_constant__ CUtensorMap tS, OnlinePass P) {
  constexpr bool FOLD = MODE == OL_FMAX || MODE == OL_FSUM;
  extern __shared__ unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nunits = P.units_enc ? __ldcg(P.count) : __ldcg(P.count) * P.nrb;
  if ((int)blockIdx.x >= nunits) {  // the whole CTA, before any barrier or TMEM allocation
    if (P.fixup && threadIdx.x == 0) ol_fixup_done(P);
    return;
  }
  const OlSmem S = ol_carve(smem_raw);
  const int ntl = P.col_tiles;                 // streamed tiles per unit
  const int nsteps = ntl * P.k_tiles;          // streamed (tile, k-tile) steps per unit
  // unit u -> pair, resident rows (offset of the pair and of the row block)
  auto unit_rows = [&](int u, int& pair, int64_t& rbase, int64_t& cbase, int& r0) {
    if (P.units_enc) {
      const int e = __ldcg(P.active + u);
      pair = e / P.nrb;
      r0 = (e % P.nrb) * OL_M;
    } else {
      pair = __ldcg(P.active + u / P.nrb);
      r0 = (u % P.nrb) * OL_M;
    }
    rbase = (int64_t)pair * P.rows_per_pair;
    cbase = (int64_t)pair * P.cols_per_pair;
  };
  ol_setup(S, &tAh, &tAl, &tBh, &tBl);
  const uint32_t tmem = *S.tslot;
  const OlRing R(P.narrow != 0);

  if (warp == OL_EPI) {
    // producer: per unit the resident tile (once the previous unit's MMAs
    // are done with it), then the streamed stages; the stage counter q runs
    // on across units
    if (lane == 0) {
      const uint32_t tbytes = P.narrow ? OL_TILE_NARROW : OL_TILE;  // bytes of one plane tile
      int q = 0, lu = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x, ++lu) {
        int pair, r0;
        int64_t rbase, cbase;
        unit_rows(u, pair, rbase, cbase, r0);
        if (lu > 0 && !mbar_wait(S.res_empty, (lu - 1) & 1, P.abort_flag, P.timeout_ns)) break;
        mbar_arrive_expect_tx(S.res_full, 2 * tbytes * P.k_tiles + (FOLD ? OL_EXT : 0));
        for (int kt = 0; kt < P.k_tiles; ++kt) {
          tma_load_2d(S.resident + (2 * kt) * OL_TILE, &tAh, kt * OL_K, (int)(rbase + r0), S.res_full);
          tma_load_2d(S.resident + (2 * kt + 1) * OL_TILE, &tAl, kt * OL_K, (int)(rbase + r0), S.res_full);
        }
        if (FOLD) {
          tma_load_2d(ol_res_ext(S), &tR, 0, (int)(rbase + r0), S.res_full);
        }
        for (int qs = 0; qs < nsteps; ++qs, ++q) {
          const int s = (q & R.mask);
          if (!mbar_wait(S.empty + s, ((q >> R.shift) & 1u) ^ 1u, P.abort_flag, P.timeout_ns)) { ok = false; break; }
          const int tile = qs / P.k_tiles, kt = qs % P.k_tiles;
          unsigned char* st = S.ring + s * R.sb;
          const int crow = (int)(cbase + tile * OL_N);
          if (FOLD) {
            unsigned char* ex = ol_stage_ext(S, R, P.narrow, s);
            mbar_arrive_expect_tx(S.full + s, 2 * tbytes + OL_EXT);
            tma_load_2d(st, &tBh, kt * OL_K, crow, S.full + s);
            tma_load_2d(st + R.lo, &tBl, kt * OL_K, crow, S.full + s);
            tma_load_2d(ex, &tS, 0, crow, S.full + s);
          } else {
            mbar_arrive_expect_tx(S.full + s, 2 * tbytes + OL_HVEC);
            tma_load_2d(st, &tBh, kt * OL_K, crow, S.full + s);
            tma_load_2d(st + R.lo, &tBl, kt * OL_K, crow, S.full + s);
            bulk_g2s(S.hbuf + s * OL_N, P.h + cbase + (int64_t)tile * OL_N, OL_HVEC, S.full + s);
          }
        }
      }
      // copies still in flight land before the CTA leaves
      const int lo = q > R.ns ? q - R.ns : 0;
      for (int qq = lo; qq < q; ++qq) {
        const uint64_t w0 = globaltimer();
        while (!mbar_try_wait(S.full + (qq & R.mask), (qq >> R.shift) & 1u))
          if (globaltimer() - w0 > P.timeout_ns) break;
      }
      if (lu > 0) {
        const uint64_t w0 = globaltimer();
        while (!mbar_try_wait(S.res_full, (lu - 1) & 1)) if (globaltimer() - w0 > P.timeout_ns) break;
      }
    }
  } else if (warp == OL_EPI + 1) {
    // MMA issuer: the tile counter T and the stage counter q run on across units
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_f16(OL_M, OL_N, false);
      int q = 0, T = 0, committed = 0, lu = 0;
      bool ok = true;
      for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x, ++lu) {
        if (!mbar_wait(S.res_full, lu & 1, P.abort_flag, P.timeout_ns)) break;
        tc_fence_after();
        for (int tile = 0; tile < ntl && ok; ++tile, ++T) {
          const int b = T % OL_NBUF;
          if (!mbar_wait(S.acce + b, ((T / OL_NBUF) & 1) ^ 1, P.abort_flag, P.timeout_ns)) { ok = false; break; }
          tc_fence_after();
          for (int kt = 0; kt < P.k_tiles; ++kt, ++q) {
            const int s = (q & R.mask);
            if (!mbar_wait(S.full + s, (q >> R.shift) & 1u, P.abort_flag, P.timeout_ns)) { ok = false; break; }
            tc_fence_after();
            ol_mma_step<FOLD>(P, tmem + (uint32_t)(b * OL_N), S.resident, S.ring + s * R.sb,
                              S.ring + s * R.sb + R.lo, kt, idesc, ol_res_ext(S), ol_stage_ext(S, R, P.narrow, s));
            if (FOLD || kt + 1 < P.k_tiles) umma_commit(S.empty + s);
          }
          if (!ok) break;
          umma_commit(S.accf + b);
          committed = T + 1;
        }
        // the resident tile is free once this unit's MMAs have completed
        if (ok) umma_commit(S.res_empty);
      }
      if (committed > 0) {
        const int c = committed - 1;
        const uint64_t w0 = globaltimer();
        while (!mbar_try_wait(S.accf + (c % OL_NBUF), (c / OL_NBUF) & 1)) if (globaltimer() - w0 > P.timeout_ns) break;
      }
    }
  } else {
    // epilogue: warp w reads TMEM lane quarter w % 4 (rows 32 (w % 4) + lane)
    // and columns 32 (w / 4) .. +31 of each tile
    const int quarter = warp & 3, cgrp = warp >> 2;
    const int row_local = quarter * 32 + lane;
    int ok = 1, T = 0;
    for (int u = blockIdx.x; u < nunits && ok; u += gridDim.x) {
      int pair, r0;
      int64_t rbase, cbase;
      unit_rows(u, pair, rbase, cbase, r0);
      const OlRowIn rin = ol_row_in<MODE>(P, rbase + r0 + row_local, cgrp == 0 && r0 + row_local < P.n_rows);
      float mx = -INFINITY, sm = 0.f, sc = 0.f;
      const float alpha = P.alpha_p ? __ldg(P.alpha_p + pair) : P.alpha;
      const uint64_t a2 = pack2(alpha, alpha);
      for (int tile = 0; tile < ntl; ++tile, ++T) {
        const int b = T % OL_NBUF;
        if (lane == 0) ok = mbar_wait(S.accf + b, (T / OL_NBUF) & 1, P.abort_flag, P.timeout_ns) ? 1 : 0;
        ok = __shfl_sync(0xffffffffu, ok, 0);
        __syncwarp();
        if (!ok) break;
        tc_fence_after();
        const int s = (T * P.k_tiles + P.k_tiles - 1) & R.mask;
        ol_epi_tile<MODE>(tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(b * OL_N + cgrp * 32),
                          S.hbuf + s * OL_N + cgrp * 32, a2, S.acce + b, S.relcnt + s, S.empty + s, lane, mx, sm,
                          sc);
      }
      if (cgrp > 0) { S.red[(cgrp - 1) * 2 * OL_M + row_local] = mx; S.red[(cgrp - 1) * 2 * OL_M + OL_M + row_local] = sm; }
      named_bar(1, OL_EPI * 32);
      if (cgrp == 0 && ok && !ol_rows_out<MODE>(P, S.red, row_local, mx, sm, r0, rbase, 0, rin)) *S.uflag = 1;
      // the partials are read (and the unit's failures marked) before the
      // next unit writes them again
      named_bar(1, OL_EPI * 32);
      if (MODE == OL_FSUM && warp == 0 && lane == 0) ol_note_unit(P, S.uflag, pair, r0);
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == OL_EPI + 1) {
    tc_fence_after();
    tmem_dealloc(tmem, OL_NBUF * OL_N);
  }
  if (P.fixup && threadIdx.x == 0) ol_fixup_done(P);
}

// Column-split passes: merge the S partial (max, sum) pairs of each row and
// apply the potential update of the pass's epilogue (check passes: the row's
// error into its slot).
__global__ void __launch_bounds__(256) online_finalize_kernel(OnlinePass P) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  const bool fold = P.ext_str != nullptr;  // partials of t - s_i (OL_FMAX)
  if (row < P.rows_pad) {
    if (row < P.n_rows) {
      float mx = -INFINITY, sm = 0.f;
      for (int c = 0; c < P.split; ++c)
        lse_merge(mx, sm, P.part[((size_t)c * 2) * P.rows_pad + row], P.part[((size_t)c * 2 + 1) * P.rows_pad + row]);
      const float lse_t = lse_value(mx, sm) + (fold ? P.shift[row] : 0.f);
      const float L = lse_t + P.rterm[row];
      const float pnew = P.logw2[row] - L;
      if (P.err) P.err[row] = fabs((double)ex2(P.pot2[row] + L) - (double)P.w[row]);
      P.pot_out2[row] = pnew;
      if (fold) {
        ext_put(P.ext_str, row, pnew - P.other_norm2[row], true);
        ext_put(P.ext_row, row, -lse_t, false);
        P.shift_out[row] = lse_t;
      } else {
        P.h_out[row] = pnew - P.other_norm2[row];
      }
    } else if (!fold) {
      P.h_out[row] = -INFINITY;
    }
  }
}

// Extension columns of one side at the start of a solve: str form from the
// starting h = pot2 - norm2 (-inf on padding rows), row form and shift 0.
__global__ void ext_init_kernel(const float* __restrict__ pot2, const float* __restrict__ norm2, int64_t n,
                                int64_t npad, __half* se, __half* re, float* shift) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npad; i += (int64_t)gridDim.x * blockDim.x) {
    ext_put(se, i, i < n ? pot2[i] - norm2[i] : -INFINITY, true);
    ext_put(re, i, 0.f, false);
    shift[i] = 0.f;
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

// ---------------------------------------------------------------------------
// Batched pair solves (otg_sinkhorn_pairs): the cost of every pass rebuilt
// from the points by online_pass_kernel over the active pairs.
// ---------------------------------------------------------------------------
struct PairsState {
  int P;
  int n, m;                   // valid rows per pair (X side, Y side)
  int64_t n_pad, m_pad;       // padded rows per pair
  const float* a; const float* b;     // caller's weights, P x n, P x m
  float* u2;                  // X side potential, base 2, P x n_pad
  float* v2[2];               // Y side potential, base 2, double-buffered
  float* xk; float* yk;       // |x|^2 log2(e)/reg_p, |y|^2 log2(e)/reg_p
  float* hx; float* hy;       // streamed-side vectors of the next pass
  __half* ye_s;                       // folded: the Y side's str-form extension columns
  double* erow;               // per-row squared column-marginal violations (Y side)
  const int* act; const int* cnt;     // active pair list in use and its length
  int* act_next; int* cnt_next;       // the list after a decision
  int* flag;                  // per active slot: leaves at this decision
  float* out_u; float* out_v;
  int32_t* status; int32_t* niter; double* err;
  double stop_thr;
  // Anderson history
  int depth;
  float* aF; float* aR; double* aG; int32_t* acnt;
};

// One warp per point: fp16 high/low planes of scale * x (pair p's rows from
// p * ld_rows; alpha_p: times sqrt(alpha_p[p])) and the raw squared norm |x|^2.
__global__ void prep_pairs_kernel(const float* __restrict__ X, int P, int n, int d, int64_t n_pad, float scale0,
                                  const float* __restrict__ alpha_p, __half* hi, __half* lo, int64_t ld, float* norm) {
  const int64_t g = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (g >= (int64_t)P * n) return;
  const int64_t p = g / n, i = g % n, row = p * n_pad + i;
  // folded passes: the pair's sqrt(alpha) in both sides' planes
  const float scale = alpha_p ? scale0 * sqrtf(alpha_p[p]) : scale0;
  float s = 0.f;
  for (int k = lane; k < d; k += 32) {
    const float x = X[g * d + k];
    s = fmaf(x, x, s);
    const float xs = x * scale;
    const __half h = __float2half_rn(xs);
    hi[row * ld + k] = h;
    lo[row * ld + k] = __float2half_rn(xs - __half2float(h));
  }
  s = warp_sum(s);
  if (lane == 0) norm[row] = s;
}

// max-only pass inputs: h = |y|^2 (-inf on padding rows)
__global__ void pairs_hmax_kernel(const float* __restrict__ yn, int P, int m, int64_t m_pad, float* h) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)P * m_pad;
       e += (int64_t)gridDim.x * blockDim.x)
    h[e] = (e % m_pad) < m ? yn[e] : -INFINITY;
}

// Per pair: the largest row max (one CTA per pair).
__global__ void pairs_max_finish_kernel(const float* __restrict__ rowmax, int n, int64_t n_pad, double* maxc) {
  __shared__ float red[32];
  float x = -INFINITY;
  for (int i = threadIdx.x; i < n; i += blockDim.x) x = fmaxf(x, rowmax[(int64_t)blockIdx.x * n_pad + i]);
  x = warp_max(x);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = -INFINITY;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t = fmaxf(t, red[k]);
    maxc[blockIdx.x] = (double)t;
  }
}

// Per pair: k2 = log2(e) / reg and the pass factor alpha = 2 k2 / (sx sy).
__global__ void pairs_scale_kernel(const double* __restrict__ reg, int P, double sxy, float* k2, float* alpha) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
    const double k = OTG_LOG2E / reg[p];
    k2[p] = (float)k;
    alpha[p] = (float)(2.0 * k / sxy);
  }
}

// The extension-column arrays of one side (null: unfolded passes).
struct ExtPtrs { __half* row; __half* str; };

// One side's per-row vectors: scaled norms nk = |x|^2 k2 and -nk, log2 of
// the weights, the starting potential (base 2; warm: natural log) and the h
// of the first pass that streams this side (pot - nk; -inf on padding rows);
// folded passes: the extension columns (str form from that h, row form and
// shift 0).
__global__ void pairs_side_kernel(const float* __restrict__ norm, const float* __restrict__ k2, const float* w,
                                  const float* warm, int P, int n, int64_t n_pad, float* nk, float* neg_nk,
                                  float* logw2, float* pot2, float* h, ExtPtrs ext, float* shift) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < (int64_t)P * n_pad;
       e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = e / n_pad, i = e % n_pad;
    if (i < n) {
      const float v = norm[e] * k2[p];
      nk[e] = v;
      neg_nk[e] = -v;
      logw2[e] = lg2(w[p * n + i]);
      const float u0 = warm ? warm[p * n + i] * (float)OTG_LOG2E : 0.f;
      if (pot2) pot2[e] = u0;
      if (h) h[e] = u0 - v;
      if (ext.row) ext_put(ext.str, e, u0 - v, true);
    } else {
      nk[e] = 0.f;
      neg_nk[e] = 0.f;
      logw2[e] = -INFINITY;
      if (pot2) pot2[e] = 0.f;
      if (h) h[e] = -INFINITY;
      if (ext.row) ext_put(ext.str, e, -INFINITY, true);
    }
    if (ext.row) {  // folded passes: row form with shift 0
      ext_put(ext.row, e, 0.f, false);
      shift[e] = 0.f;
    }
  }
}

// Decision at a check (one CTA per active slot): the pair's error (its row
// slots summed in a fixed order), convergence, and for a leaving pair its
// outputs (the pair (u, v_old) in natural logs).  check = 0: no error was
// measured (the pairs leave only at max_iter).
__global__ void pairs_decide_kernel(PairsState S, const float* __restrict__ vold, int ii, int check, int at_max) {
  const int slot = blockIdx.x;
  if (slot >= __ldcg(S.cnt)) return;
  const int p = __ldcg(S.act + slot);
  double e = -1.0;
  bool conv = false;
  if (check) {
    e = sqrt(block_sum_slots(S.erow + (int64_t)p * S.m_pad, S.m));
    conv = e < S.stop_thr;
  }
  const bool leave = conv || at_max;
  if (leave) {
    const float LN2 = (float)OTG_LN2;
    for (int i = threadIdx.x; i < S.n; i += blockDim.x) S.out_u[(int64_t)p * S.n + i] = S.u2[(int64_t)p * S.n_pad + i] * LN2;
    for (int j = threadIdx.x; j < S.m; j += blockDim.x) S.out_v[(int64_t)p * S.m + j] = vold[(int64_t)p * S.m_pad + j] * LN2;
    if (threadIdx.x == 0) {
      S.status[p] = conv ? OTG_STATUS_CONVERGED : OTG_STATUS_MAXITER;
      S.niter[p] = ii - 1;
      S.err[p] = e;
    }
  }
  if (threadIdx.x == 0) S.flag[slot] = leave ? 1 : 0;
}

// The active list without the leaving pairs (one CTA, block-wide scan).
__global__ void __launch_bounds__(1024) pairs_compact_kernel(PairsState S) {
  __shared__ int s_warp[32];
  __shared__ int s_base;
  const int n = __ldcg(S.cnt);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_base = 0;
  __syncthreads();
  for (int c0 = 0; c0 < n; c0 += blockDim.x) {
    const int k = c0 + threadIdx.x;
    const int keep = k < n && !__ldcg(S.flag + k);
    int inc = keep;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int up = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += up;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    int before = s_base;
    for (int w = 0; w < wid; ++w) before += s_warp[w];
    if (keep) S.act_next[before + inc - 1] = __ldcg(S.act + k);
    __syncthreads();
    if (threadIdx.x == 0)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s_base += s_warp[w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *S.cnt_next = s_base;
}

// Anderson mixing of the new v of every active pair, then the h of the next
// pass (which streams the Y side) from the mixed v (folded passes: its
// str-form extension columns).
__global__ void pairs_anderson_kernel(PairsState S, const float* __restrict__ vold, float* vnew) {
  const int slot = blockIdx.x;
  if (slot >= __ldcg(S.cnt)) return;
  const int p = __ldcg(S.act + slot);
  const int64_t co = (int64_t)p * S.m_pad;
  anderson_step<float>(S.depth, S.m, co, (int64_t)S.P * S.m_pad, vold, vnew, S.aF, S.aR,
                       S.aG + (int64_t)p * S.depth * S.depth, S.acnt + p);
  for (int64_t j = threadIdx.x; j < S.m_pad; j += blockDim.x) {
    const float h = j < S.m ? vnew[co + j] - S.yk[co + j] : -INFINITY;
    if (S.ye_s) ext_put(S.ye_s, co + j, h, true);
    else S.hy[co + j] = h;
  }
}

__global__ void fill_int_kernel(int* x, int n, int v) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] = v < 0 ? i : v;
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

// Plane tensor map: ld = 16 (narrow planes, d <= 16): 16 x 128 boxes with
// the 32-byte swizzle; otherwise 64 x 128 boxes with the 128-byte swizzle.
bool ol_plane_map(CUtensorMap* m, const void* base, int64_t rows, int64_t ld) {
  EncodeTiledFn2 fn = ol_encode_fn();
  if (!fn) return false;
  const bool narrow = ld == 16;
  cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {narrow ? 16u : (cuuint32_t)OL_K, OL_M};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, narrow ? CU_TENSOR_MAP_SWIZZLE_32B : CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Width of the planes of d-dimensional points: 16 for d <= 16 (narrow),
// else a multiple of 64.
int ol_plane_width(int d) { return d <= 16 ? 16 : (d + 63) / 64 * 64; }

constexpr size_t OL_SMEM = (size_t)OL_MAXKT * 2 * OL_TILE + (size_t)OL_STAGES * OL_STAGE + OL_EXTRA +
                           1024 /*align*/ + 256 /*barriers*/ + 6 * OL_M * 4 /*red*/ + 64 /*counters*/;
static_assert(OL_SMEM <= 232448, "shared memory of the pass kernels");
static_assert(OL_NS_NARROW * OL_HVEC <= OL_EXTRA, "h slices fit the extra region");
static_assert(OL_NS_NARROW * OL_STAGE_NARROW == OL_STAGES * OL_STAGE, "both rings fill the ring region");

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

// Acceptance range of the shifted sums: [2^-w, 2^w] for a window w > 0,
// else [2^-70, 2^100] (terms below 2^-126 flush to zero, so a sum of at
// least 2^-70 loses at most 2^-40 of itself to them; at most 2^100 leaves no
// term near the float range's end).
void ol_sum_window(float w, float& lo, float& hi) {
  if (w > 0.f) {
    lo = std::exp2(-std::min(w, 70.f));
    hi = std::exp2(std::min(w, 100.f));
  } else {
    lo = 0x1p-70f;
    hi = 0x1p100f;
  }
}

// Dynamic shared memory of every pass kernel instantiation (once).
bool online_attr() {
  static std::once_flag once;
  static bool ok = false;
  std::call_once(once, [] {
    const int sm = (int)OL_SMEM;
    ok = cudaFuncSetAttribute(online_pass_kernel<OL_LSE>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess &&
         cudaFuncSetAttribute(online_pass_kernel<OL_FMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess &&
         cudaFuncSetAttribute(online_pass_kernel<OL_FSUM>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess &&
         cudaFuncSetAttribute(online_batch_kernel<OL_LSE>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess &&
         cudaFuncSetAttribute(online_batch_kernel<OL_MAXP>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess &&
         cudaFuncSetAttribute(online_batch_kernel<OL_FMAX>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess &&
         cudaFuncSetAttribute(online_batch_kernel<OL_FSUM>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm) == cudaSuccess;
  });
  return ok;
}

}  // namespace

extern "C" {

size_t otg_online_workspace_bytes(int64_t n, int64_t m, int32_t d) {
  const int64_t np = (n + 127) / 128 * 128, mp = (m + 127) / 128 * 128;
  const int64_t dp = ol_plane_width(d);
  size_t b = 0;
  b += 2 * a16(2 * np * dp) + 2 * a16(2 * mp * dp);          // half planes
  b += 5 * a16(4 * np) + 4 * a16(4 * mp);                    // norms, log2 w, potentials, h
  b += a16(8 * 64);                                          // err slots, flag
  b += a16(8 * (size_t)std::max(np, mp));                    // per-row errors of a check pass
  b += a16(4 * np) + a16(4 * mp);                            // negated norms
  b += a16(4 * 2 * (size_t)OL_MAX_SPLIT * (size_t)std::max(np, mp));  // column-split partials
  b += 2 * a16(32 * np) + 2 * a16(32 * mp);                  // extension columns (row, str form)
  b += a16(4 * np) + a16(4 * mp) + a16(np) + a16(mp);        // shifts, failure marks
  b += a16(4 * (size_t)std::max(np, mp) / OL_M + 64);        // failed units, fix-up counters
  return b;
}

int otg_sinkhorn_online(const OtgOnlineProblem* p, cudaStream_t st) {
  if (!p || !p->X || !p->Y || !p->a || !p->b || !p->out_f || !p->out_g || !p->workspace || !p->info || !p->err_hist)
    return OTG_ERR_ARG;
  if (p->n < 1 || p->m < 1 || p->d < 1 || p->d > 64 * OL_MAXKT || !(p->reg > 0)) return OTG_ERR_ARG;
  if (p->workspace_bytes < otg_online_workspace_bytes(p->n, p->m, p->d)) return OTG_ERR_WORKSPACE;
  const int64_t n = p->n, m = p->m;
  const int64_t np = (n + 127) / 128 * 128, mp = (m + 127) / 128 * 128;
  const int dp = ol_plane_width(p->d);
  const int nkt = dp == 16 ? 1 : dp / OL_K;  // K-tiles per streamed tile
  // folded passes (one K-tile): alpha in the planes, h and the row shift in
  // the extension columns, so the epilogue only exponentiates and sums
  const bool fold = nkt == 1;
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
  float* nx = reinterpret_cast<float*>(take(4 * np));
  float* ny = reinterpret_cast<float*>(take(4 * mp));
  float* part = reinterpret_cast<float*>(take(4 * 2 * (size_t)OL_MAX_SPLIT * (size_t)std::max(np, mp)));
  // extension columns [row form, str form] of each side
  __half* xe[2];
  __half* ye[2];
  for (int k = 0; k < 2; ++k) xe[k] = reinterpret_cast<__half*>(take(32 * np));
  for (int k = 0; k < 2; ++k) ye[k] = reinterpret_cast<__half*>(take(32 * mp));
  float* shx = reinterpret_cast<float*>(take(4 * np));
  float* shy = reinterpret_cast<float*>(take(4 * mp));
  unsigned char* fax = reinterpret_cast<unsigned char*>(take(np));
  unsigned char* fay = reinterpret_cast<unsigned char*>(take(mp));
  int* flist = reinterpret_cast<int*>(take(4 * (size_t)std::max(np, mp) / OL_M + 64));
  int* fcnt = flist + std::max(np, mp) / OL_M;
  unsigned* fdone = reinterpret_cast<unsigned*>(fcnt + 1);
  if (off > p->workspace_bytes) return OTG_ERR_WORKSPACE;
  const float k2 = (float)(OTG_LOG2E / p->reg);
  const float sx = p->scale_x, sy = p->scale_y;
  const double alpha_d = 2.0 * OTG_LOG2E / (p->reg * (double)sx * (double)sy);
  const float lam = fold ? (float)std::sqrt(alpha_d) : 1.f;  // folded planes: (sx lam x).(sy lam y) = 2 k2 x.y
  // planes are zero beyond the data; norms, weights and potentials set below
  if (cudaMemsetAsync(w, 0, off, st) != cudaSuccess) return OTG_ERR_CUDA;
  prep_points_kernel<<<(unsigned)((n + 7) / 8), 256, 0, st>>>(p->X, n, p->d, sx * lam, xh, xl, dp, k2, xn2);
  prep_points_kernel<<<(unsigned)((m + 7) / 8), 256, 0, st>>>(p->Y, m, p->d, sy * lam, yh, yl, dp, k2, yn2);
  log2w_kernel<<<256, 256, 0, st>>>(p->a, n, la2);
  log2w_kernel<<<256, 256, 0, st>>>(p->b, m, lb2);
  // initial potentials (natural log in, base 2 inside)
  if (p->warm_f) scale_kernel<<<256, 256, 0, st>>>(p->warm_f, n, (float)OTG_LOG2E, f2[0]);
  if (p->warm_g) scale_kernel<<<256, 256, 0, st>>>(p->warm_g, m, (float)OTG_LOG2E, g2);
  init_h_kernel<<<256, 256, 0, st>>>(g2, yn2, m, mp, hy);
  if (fold) {
    ext_init_kernel<<<256, 256, 0, st>>>(f2[0], xn2, n, np, xe[1], xe[0], shx);
    ext_init_kernel<<<256, 256, 0, st>>>(g2, yn2, m, mp, ye[1], ye[0], shy);
  }
  if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
  CUtensorMap mxh, mxl, myh, myl, exr, exs, eyr, eys;
  if (!ol_plane_map(&mxh, xh, np, dp) || !ol_plane_map(&mxl, xl, np, dp) || !ol_plane_map(&myh, yh, mp, dp) ||
      !ol_plane_map(&myl, yl, mp, dp))
    return OTG_ERR_CUDA;
  if (!ol_plane_map(&exr, xe[0], np, 16) || !ol_plane_map(&exs, xe[1], np, 16) || !ol_plane_map(&eyr, ye[0], mp, 16) ||
      !ol_plane_map(&eys, ye[1], mp, 16))
    return OTG_ERR_CUDA;
  if (!online_attr()) return OTG_ERR_CUDA;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int split_f = choose_split((int)(np / OL_M), (int)(mp / OL_N), sms);
  const int split_g = choose_split((int)(mp / OL_M), (int)(np / OL_N), sms);
  // one pass: the pass kernel over (row blocks x column split), then, when
  // split, the merge of the partials; a shifted-sum pass is followed by its
  // fix-up (the running-max pass over the units whose rows failed; empty
  // and at once done when none did)
  // (check passes: the per-row errors go to erow, their sum to `eslot`)
  auto pass = [&](OnlinePass& P, const CUtensorMap& ah, const CUtensorMap& al, const CUtensorMap& bh,
                  const CUtensorMap& bl, const CUtensorMap& rx, const CUtensorMap& sx2, int64_t rows_pad, int split,
                  bool first, double* eslot_of_pass) {
    P.split = split; P.rows_pad = (int)rows_pad; P.part = part;
    const dim3 grid((unsigned)(rows_pad / OL_M), (unsigned)split);
    if (!fold) {
      online_pass_kernel<OL_LSE><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, ah, bh, P);
    } else if (first || split > 1) {
      online_pass_kernel<OL_FMAX><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, rx, sx2, P);
    } else {
      online_pass_kernel<OL_FSUM><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, rx, sx2, P);
      OnlinePass Q = P;
      Q.fixup = 1; Q.units_enc = 1; Q.active = flist; Q.count = fcnt; Q.nrb = (int)(rows_pad / OL_M);
      Q.rows_per_pair = 0; Q.cols_per_pair = 0; Q.alpha_p = nullptr; Q.done_cnt = fdone;
      online_batch_kernel<OL_FMAX><<<(unsigned)std::min<int64_t>(rows_pad / OL_M, sms), OL_THREADS, OL_SMEM, st>>>(
          ah, al, bh, bl, rx, sx2, Q);
    }
    if (split > 1) online_finalize_kernel<<<(unsigned)((rows_pad + 255) / 256), 256, 0, st>>>(P);
    // the L1 error: the row slots summed in a fixed order (the same value in every run)
    if (P.err) slot_sum_kernel<1024><<<1, 1024, 0, st>>>(P.err, P.n_rows, eslot_of_pass);
  };
  neg_kernel<<<256, 256, 0, st>>>(xn2, n, nx);
  neg_kernel<<<256, 256, 0, st>>>(yn2, m, ny);
  const float alpha = (float)alpha_d;
  const uint64_t tmo = p->timeout_ms > 0 ? (uint64_t)p->timeout_ms * 1000000ull : 4000000000ull;
  // f pass: rows = X, streamed = Y (h = g2 - |y|^2 k2)
  auto fpass = [&](OnlinePass& A, int cur, bool check) {
    A = OnlinePass{};
    A.n_rows = (int)n; A.col_tiles = (int)(mp / OL_N); A.k_tiles = nkt; A.narrow = dp == 16; A.alpha = alpha;
    A.h = hy; A.rterm = nx; A.logw2 = la2; A.pot2 = f2[cur]; A.w = p->a; A.pot_out2 = f2[cur ^ 1];
    A.other_norm2 = xn2; A.h_out = hx; A.err = check ? erow : nullptr; A.abort_flag = flag; A.timeout_ns = tmo;
    if (fold) {
      A.ext_row = xe[0]; A.ext_str = xe[1];
      A.shift = shx; A.shift_out = shx; A.fail = fax; A.fail_list = flist; A.fail_cnt = fcnt; A.done_cnt = fdone;
      ol_sum_window(p->sum_window_log2, A.sum_lo, A.sum_hi);
    }
  };
  int cur = 0, nchk = 0, status = OTG_STATUS_MAXITER, niter = p->max_iter - 1;
  for (int it = 0; it < p->max_iter; ++it) {
    const bool check = (it > 0) && (it % 10 == 0);  // error of iteration it-1 ((it-1)+1) % 10 == 0
    double* eslot = errs + (nchk % 60);
    OnlinePass A;
    fpass(A, cur, check);
    pass(A, mxh, mxl, myh, myl, exr, eys, np, split_f, it == 0, eslot);
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
    B.n_rows = (int)m; B.col_tiles = (int)(np / OL_N); B.k_tiles = nkt; B.narrow = dp == 16; B.alpha = alpha;
    B.h = hx; B.rterm = ny; B.logw2 = lb2; B.pot2 = g2; B.w = p->b; B.pot_out2 = g2;
    B.other_norm2 = yn2; B.h_out = hy; B.err = nullptr; B.abort_flag = flag; B.timeout_ns = tmo;
    if (fold) {
      B.ext_row = ye[0]; B.ext_str = ye[1];
      B.shift = shy; B.shift_out = shy; B.fail = fay; B.fail_list = flist; B.fail_cnt = fcnt; B.done_cnt = fdone;
      ol_sum_window(p->sum_window_log2, B.sum_lo, B.sum_hi);
    }
    pass(B, myh, myl, mxh, mxl, eyr, exs, mp, split_g, it == 0, nullptr);
    if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
  }
  // a last check at max_iter when (max_iter) % 10 == 0 is done by the next f pass
  if (status == OTG_STATUS_MAXITER && p->max_iter > 0 && p->max_iter % 10 == 0) {
    double* eslot = errs + (nchk % 60);
    OnlinePass A;
    fpass(A, cur, true);
    pass(A, mxh, mxl, myh, myl, exr, eys, np, split_f, false, eslot);
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
  int hflag = 0, nfix = 0;
  cudaMemcpyAsync(&hflag, flag, 4, cudaMemcpyDeviceToHost, st);
  cudaMemcpyAsync(&nfix, fcnt + 2, 4, cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
  p->info[0] = hflag ? OTG_STATUS_ABORTED : status;
  p->info[1] = niter;
  p->info[2] = nchk;
  p->info[3] = nfix;
  return OTG_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched pair solves: host side
// ---------------------------------------------------------------------------
namespace {

struct PairsLayout {
  int64_t n_pad, m_pad;
  int dp;
  size_t xh, xl, yh, yl, xn, yn, xk, nxk, la2, wa, u2, hx, yk, nyk, lb2, wb, v0, v1, hy, erow, k2, alpha, act0,
      act1, cnt, flag, aF, aR, aG, acnt, xe[2], ye[2], shx, shy, fax, fay, flist, total;
};

PairsLayout pairs_layout(int64_t P, int64_t n, int64_t m, int d, int depth) {
  PairsLayout L{};
  L.n_pad = (n + 127) / 128 * 128;
  L.m_pad = (m + 127) / 128 * 128;
  L.dp = ol_plane_width(d);
  size_t off = 0;
  auto take = [&](size_t bytes) { const size_t o = off; off += a16(bytes); return o; };
  const size_t nx = (size_t)(P * L.n_pad), ny = (size_t)(P * L.m_pad);
  L.xh = take(2 * nx * L.dp); L.xl = take(2 * nx * L.dp);
  L.yh = take(2 * ny * L.dp); L.yl = take(2 * ny * L.dp);
  L.xn = take(4 * nx); L.yn = take(4 * ny);
  L.xk = take(4 * nx); L.nxk = take(4 * nx); L.la2 = take(4 * nx); L.wa = take(4 * nx); L.u2 = take(4 * nx);
  L.hx = take(4 * nx);
  L.yk = take(4 * ny); L.nyk = take(4 * ny); L.lb2 = take(4 * ny); L.wb = take(4 * ny); L.v0 = take(4 * ny);
  L.v1 = take(4 * ny); L.hy = take(4 * ny);
  L.erow = take(8 * ny);
  L.k2 = take(4 * (size_t)P); L.alpha = take(4 * (size_t)P);
  L.act0 = take(4 * (size_t)P); L.act1 = take(4 * (size_t)P); L.cnt = take(64); L.flag = take(4 * (size_t)P);
  if (depth > 0) {
    L.aF = take(4 * (size_t)depth * ny); L.aR = take(4 * (size_t)depth * ny);
    L.aG = take(8 * (size_t)P * depth * depth); L.acnt = take(4 * (size_t)P);
  }
  if (L.dp <= 64) {  // folded passes: extension columns, shifts, failure marks, failed units
    for (int k = 0; k < 2; ++k) L.xe[k] = take(32 * nx);
    for (int k = 0; k < 2; ++k) L.ye[k] = take(32 * ny);
    L.shx = take(4 * nx); L.shy = take(4 * ny); L.fax = take(nx); L.fay = take(ny);
    L.flist = take(4 * (size_t)P * (size_t)(std::max(L.n_pad, L.m_pad) / OL_M));
  }
  L.total = off;
  return L;
}

int pairs_check(const OtgPairsProblem* q) {
  if (!q || !q->X || !q->Y || !q->workspace) return OTG_ERR_ARG;
  if (q->npairs < 1 || q->n < 1 || q->m < 1 || q->d < 1 || q->d > 64 * OL_MAXKT) return OTG_ERR_ARG;
  if ((int64_t)q->npairs * ((q->n + 127) / 128 * 128) > INT32_MAX ||
      (int64_t)q->npairs * ((q->m + 127) / 128 * 128) > INT32_MAX)
    return OTG_ERR_ARG;  // TMA row coordinates are 32-bit
  if (q->anderson_depth < 0 || q->anderson_depth > OTG_ANDERSON_MAX_DEPTH) return OTG_ERR_ARG;
  if (q->workspace_bytes < pairs_layout(q->npairs, q->n, q->m, q->d, q->anderson_depth).total) return OTG_ERR_WORKSPACE;
  return OTG_OK;
}

// CTAs of a batch pass: one per SM (each keeps its TMEM and pipeline across
// the (pair, row block) units it takes), fewer when there are fewer units.
int pairs_grid(int64_t units) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  return (int)std::min<int64_t>(units, sms);
}

// Planes and raw norms of both sides; returns the prescales through sx, sy.
int pairs_prep(const OtgPairsProblem* q, const PairsLayout& L, char* w, float* max_abs_host, const float* alpha_p,
               cudaStream_t st, CUtensorMap* mx_h, CUtensorMap* mx_l, CUtensorMap* my_h, CUtensorMap* my_l) {
  const int P = q->npairs, d = q->d;
  __half* xh = reinterpret_cast<__half*>(w + L.xh);
  __half* xl = reinterpret_cast<__half*>(w + L.xl);
  __half* yh = reinterpret_cast<__half*>(w + L.yh);
  __half* yl = reinterpret_cast<__half*>(w + L.yl);
  // planes are zero beyond the data
  if (cudaMemsetAsync(w + L.xh, 0, L.xn - L.xh, st) != cudaSuccess) return OTG_ERR_CUDA;
  const float sx = max_abs_host[0], sy = max_abs_host[1];
  const int64_t gx = (int64_t)P * q->n, gy = (int64_t)P * q->m;
  prep_pairs_kernel<<<(unsigned)((gx + 7) / 8), 256, 0, st>>>(q->X, P, (int)q->n, d, L.n_pad, sx, alpha_p, xh, xl,
                                                             L.dp, reinterpret_cast<float*>(w + L.xn));
  prep_pairs_kernel<<<(unsigned)((gy + 7) / 8), 256, 0, st>>>(q->Y, P, (int)q->m, d, L.m_pad, sy, alpha_p, yh, yl,
                                                             L.dp, reinterpret_cast<float*>(w + L.yn));
  if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
  if (!ol_plane_map(mx_h, xh, (int64_t)P * L.n_pad, L.dp) || !ol_plane_map(mx_l, xl, (int64_t)P * L.n_pad, L.dp) ||
      !ol_plane_map(my_h, yh, (int64_t)P * L.m_pad, L.dp) || !ol_plane_map(my_l, yl, (int64_t)P * L.m_pad, L.dp))
    return OTG_ERR_CUDA;
  return OTG_OK;
}

// Power-of-two prescale of a cloud set from its largest magnitude (the
// planes' high parts then sit near 2^14).
float pow2_prescale(float max_abs) {
  if (!(max_abs > 0.f)) return 1.f;
  return std::ldexp(1.0f, 14 - (int)std::ceil(std::log2((double)max_abs)));
}

__global__ void absmax_kernel(const float* __restrict__ x, int64_t n, unsigned* out) {
  float m = 0.f;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = fmaxf(m, fabsf(x[i]));
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));  // max of non-negative floats
}

int pairs_scales(const OtgPairsProblem* q, char* w, const PairsLayout& L, cudaStream_t st, float* sxy) {
  unsigned* tmp = reinterpret_cast<unsigned*>(w + L.cnt) + 8;  // two scratch words of the control block
  if (cudaMemsetAsync(tmp, 0, 8, st) != cudaSuccess) return OTG_ERR_CUDA;
  absmax_kernel<<<304, 256, 0, st>>>(q->X, (int64_t)q->npairs * q->n * q->d, tmp);
  absmax_kernel<<<304, 256, 0, st>>>(q->Y, (int64_t)q->npairs * q->m * q->d, tmp + 1);
  unsigned hb[2] = {0u, 0u};
  if (cudaMemcpyAsync(hb, tmp, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
  float fx, fy;
  std::memcpy(&fx, hb, 4);
  std::memcpy(&fy, hb + 1, 4);
  sxy[0] = pow2_prescale(fx);
  sxy[1] = pow2_prescale(fy);
  return OTG_OK;
}

OnlinePass pairs_pass(const PairsLayout& L, char* w, bool x_resident, int n_rows, int tiles, int kt,
                      const int* act, const int* cnt, int* abort_flag, uint64_t tmo) {
  OnlinePass A{};
  A.n_rows = n_rows;
  A.col_tiles = tiles;
  A.k_tiles = kt;
  A.narrow = L.dp == 16;
  A.active = act;
  A.count = cnt;
  A.nrb = (int)((x_resident ? L.n_pad : L.m_pad) / OL_M);
  A.rows_per_pair = x_resident ? L.n_pad : L.m_pad;
  A.cols_per_pair = x_resident ? L.m_pad : L.n_pad;
  A.rows_pad = (int)A.rows_per_pair;
  A.split = 1;
  A.alpha_p = reinterpret_cast<const float*>(w + L.alpha);
  A.abort_flag = abort_flag;
  A.timeout_ns = tmo;
  return A;
}

}  // namespace

extern "C" {

size_t otg_pairs_workspace_bytes(int32_t npairs, int64_t n, int64_t m, int32_t d, int32_t anderson_depth) {
  return pairs_layout(npairs, n, m, d, anderson_depth).total;
}

int otg_pairs_max_cost(const OtgPairsProblem* q, double* maxc, cudaStream_t st) {
  int rc = pairs_check(q);
  if (rc != OTG_OK) return rc;
  if (!maxc) return OTG_ERR_ARG;
  if (!ol_encode_fn() || !online_attr()) return OTG_ERR_CUDA;
  const PairsLayout L = pairs_layout(q->npairs, q->n, q->m, q->d, q->anderson_depth);
  char* w = static_cast<char*>(q->workspace);
  const int P = q->npairs;
  float sxy[2];
  if ((rc = pairs_scales(q, w, L, st, sxy)) != OTG_OK) return rc;
  CUtensorMap mxh, mxl, myh, myl;
  if ((rc = pairs_prep(q, L, w, sxy, nullptr, st, &mxh, &mxl, &myh, &myl)) != OTG_OK) return rc;
  int* cnt = reinterpret_cast<int*>(w + L.cnt);
  int* abort_flag = cnt + 4;
  int* act = reinterpret_cast<int*>(w + L.act0);
  if (cudaMemsetAsync(cnt, 0, 32, st) != cudaSuccess) return OTG_ERR_CUDA;
  fill_int_kernel<<<(P + 255) / 256, 256, 0, st>>>(act, P, -1);
  fill_int_kernel<<<1, 32, 0, st>>>(cnt, 1, P);
  float* h = reinterpret_cast<float*>(w + L.hy);
  pairs_hmax_kernel<<<1024, 256, 0, st>>>(reinterpret_cast<const float*>(w + L.yn), P, (int)q->m, L.m_pad, h);
  // t = |y|^2 - 2 x.y, row max + |x|^2 = max_j |x_i - y_j|^2
  OnlinePass A = pairs_pass(L, w, true, (int)q->n, (int)(L.m_pad / OL_N), L.dp == 16 ? 1 : L.dp / OL_K, act, cnt, abort_flag,
                            q->timeout_ms > 0 ? (uint64_t)q->timeout_ms * 1000000ull : 4000000000ull);
  A.alpha_p = nullptr;
  A.alpha = (float)(-2.0 / ((double)sxy[0] * (double)sxy[1]));
  A.h = h;
  A.rterm = reinterpret_cast<const float*>(w + L.xn);
  float* rowmax = reinterpret_cast<float*>(w + L.u2);
  A.pot_out2 = rowmax;
  online_batch_kernel<OL_MAXP><<<(unsigned)pairs_grid(P * A.nrb), OL_THREADS, OL_SMEM, st>>>(mxh, mxl, myh, myl, mxh,
                                                                                        myh, A);
  pairs_max_finish_kernel<<<P, 256, 0, st>>>(rowmax, (int)q->n, L.n_pad, maxc);
  int hflag = 0;
  if (cudaMemcpyAsync(&hflag, abort_flag, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
  return hflag ? OTG_ERR_CUDA : OTG_OK;
}

int otg_sinkhorn_pairs(const OtgPairsProblem* q, cudaStream_t st) {
  int rc = pairs_check(q);
  if (rc != OTG_OK) return rc;
  if (!q->a || !q->b || !q->reg || !q->out_u || !q->out_v || !q->status || !q->niter || !q->err || q->max_iter < 1)
    return OTG_ERR_ARG;
  if (!ol_encode_fn() || !online_attr()) return OTG_ERR_CUDA;
  const PairsLayout L = pairs_layout(q->npairs, q->n, q->m, q->d, q->anderson_depth);
  char* w = static_cast<char*>(q->workspace);
  const int P = q->npairs, D = q->anderson_depth;
  const int period = q->check_period > 0 ? q->check_period : 10;
  const uint64_t tmo = q->timeout_ms > 0 ? (uint64_t)q->timeout_ms * 1000000ull : 4000000000ull;
  float sxy[2];
  if ((rc = pairs_scales(q, w, L, st, sxy)) != OTG_OK) return rc;
  auto F = [&](size_t off) { return reinterpret_cast<float*>(w + off); };
  // folded passes (one K-tile): the pair's alpha in the planes, h and the
  // row shift in the extension columns
  const bool fold = L.dp <= 64;
  int* cnt = reinterpret_cast<int*>(w + L.cnt);  // [0], [1] list lengths, [4] abort flag, [12], [13] fix-up
  int* abort_flag = cnt + 4;
  int* fcnt = cnt + 12;
  unsigned* fdone = reinterpret_cast<unsigned*>(cnt + 13);
  int* act[2] = {reinterpret_cast<int*>(w + L.act0), reinterpret_cast<int*>(w + L.act1)};
  if (cudaMemsetAsync(cnt, 0, 64, st) != cudaSuccess) return OTG_ERR_CUDA;
  pairs_scale_kernel<<<(P + 255) / 256, 256, 0, st>>>(q->reg, P, (double)sxy[0] * (double)sxy[1], F(L.k2),
                                                     F(L.alpha));
  CUtensorMap mxh, mxl, myh, myl, exr, exs, eyr, eys;
  if ((rc = pairs_prep(q, L, w, sxy, fold ? F(L.alpha) : nullptr, st, &mxh, &mxl, &myh, &myl)) != OTG_OK) return rc;
  __half* xe[2] = {nullptr, nullptr};
  __half* ye[2] = {nullptr, nullptr};
  if (fold) {
    for (int k = 0; k < 2; ++k) {
      xe[k] = reinterpret_cast<__half*>(w + L.xe[k]);
      ye[k] = reinterpret_cast<__half*>(w + L.ye[k]);
    }
    if (!ol_plane_map(&exr, xe[0], (int64_t)P * L.n_pad, 16) || !ol_plane_map(&exs, xe[1], (int64_t)P * L.n_pad, 16) ||
        !ol_plane_map(&eyr, ye[0], (int64_t)P * L.m_pad, 16) || !ol_plane_map(&eys, ye[1], (int64_t)P * L.m_pad, 16))
      return OTG_ERR_CUDA;
  }
  if (fold && (cudaMemsetAsync(w + L.fax, 0, (size_t)P * L.n_pad, st) != cudaSuccess ||
               cudaMemsetAsync(w + L.fay, 0, (size_t)P * L.m_pad, st) != cudaSuccess))
    return OTG_ERR_CUDA;
  pairs_side_kernel<<<1024, 256, 0, st>>>(F(L.xn), F(L.k2), q->a, q->warm_u, P, (int)q->n, L.n_pad, F(L.xk),
                                          F(L.nxk), F(L.la2), F(L.u2), F(L.hx), ExtPtrs{xe[0], xe[1]},
                                          fold ? F(L.shx) : nullptr);
  pairs_side_kernel<<<1024, 256, 0, st>>>(F(L.yn), F(L.k2), q->b, nullptr, P, (int)q->m, L.m_pad, F(L.yk),
                                          F(L.nyk), F(L.lb2), F(L.v0), nullptr, ExtPtrs{ye[0], ye[1]},
                                          fold ? F(L.shy) : nullptr);
  // weights in the padded layout (the check reads them per resident row)
  {
    // logw2 = log2 w on valid rows: w = 2^logw2 exactly enough for the check
    // would round twice; copy the weights themselves instead
    const int64_t ex = (int64_t)P * L.n_pad, ey = (int64_t)P * L.m_pad;
    float* wa = F(L.wa);
    float* wb = F(L.wb);
    if (cudaMemsetAsync(wa, 0, 4 * ex, st) != cudaSuccess || cudaMemsetAsync(wb, 0, 4 * ey, st) != cudaSuccess)
      return OTG_ERR_CUDA;
    if (cudaMemcpy2DAsync(wa, 4 * L.n_pad, q->a, 4 * q->n, 4 * q->n, P, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpy2DAsync(wb, 4 * L.m_pad, q->b, 4 * q->m, 4 * q->m, P, cudaMemcpyDeviceToDevice, st) != cudaSuccess)
      return OTG_ERR_CUDA;
  }
  fill_int_kernel<<<(P + 255) / 256, 256, 0, st>>>(act[0], P, -1);
  fill_int_kernel<<<1, 32, 0, st>>>(cnt, 1, P);
  if (D > 0 && cudaMemsetAsync(w + L.acnt, 0, 4 * (size_t)P, st) != cudaSuccess) return OTG_ERR_CUDA;
  if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;

  PairsState S{};
  S.P = P; S.n = (int)q->n; S.m = (int)q->m; S.n_pad = L.n_pad; S.m_pad = L.m_pad;
  S.a = q->a; S.b = q->b;
  S.u2 = F(L.u2); S.v2[0] = F(L.v0); S.v2[1] = F(L.v1);
  S.xk = F(L.xk); S.yk = F(L.yk); S.hx = F(L.hx); S.hy = F(L.hy);
  if (fold) S.ye_s = ye[1];
  S.erow = reinterpret_cast<double*>(w + L.erow);
  S.flag = reinterpret_cast<int*>(w + L.flag);
  S.out_u = q->out_u; S.out_v = q->out_v; S.status = q->status; S.niter = q->niter; S.err = q->err;
  S.stop_thr = q->stop_thr;
  S.depth = D;
  if (D > 0) {
    S.aF = F(L.aF); S.aR = F(L.aR); S.aG = reinterpret_cast<double*>(w + L.aG);
    S.acnt = reinterpret_cast<int32_t*>(w + L.acnt);
  }
  const int kt = L.dp == 16 ? 1 : L.dp / OL_K;
  const int nrb_x = (int)(L.n_pad / OL_M), nrb_y = (int)(L.m_pad / OL_M);
  // one pass over the active pairs (x_res: X resident); folded: the first
  // pass of each side keeps a running max, later ones sum with the shift and
  // are followed by their fix-up (empty and at once done when no row failed)
  auto run = [&](OnlinePass& A, bool x_res, bool first, int units) {
    const CUtensorMap& ah = x_res ? mxh : myh; const CUtensorMap& al = x_res ? mxl : myl;
    const CUtensorMap& bh = x_res ? myh : mxh; const CUtensorMap& bl = x_res ? myl : mxl;
    const unsigned grid = (unsigned)pairs_grid(units);
    if (!fold) {
      online_batch_kernel<OL_LSE><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, ah, bh, A);
      return;
    }
    __half* const* me = x_res ? xe : ye;
    const CUtensorMap& rx = x_res ? exr : eyr;
    const CUtensorMap& sx2 = x_res ? eys : exs;
    A.ext_row = me[0]; A.ext_str = me[1];
    A.shift = x_res ? F(L.shx) : F(L.shy); A.shift_out = const_cast<float*>(A.shift);
    A.fail = reinterpret_cast<unsigned char*>(w + (x_res ? L.fax : L.fay));
    A.fail_list = reinterpret_cast<int*>(w + L.flist); A.fail_cnt = fcnt; A.done_cnt = fdone;
    ol_sum_window(q->sum_window_log2, A.sum_lo, A.sum_hi);
    if (first) {
      online_batch_kernel<OL_FMAX><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, rx, sx2, A);
      return;
    }
    online_batch_kernel<OL_FSUM><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, rx, sx2, A);
    OnlinePass Q = A;
    Q.fixup = 1; Q.units_enc = 1; Q.active = A.fail_list; Q.count = fcnt;
    online_batch_kernel<OL_FMAX><<<grid, OL_THREADS, OL_SMEM, st>>>(ah, al, bh, bl, rx, sx2, Q);
  };
  int nact = P, sel = 0, cur = 0;
  bool prev_check = false;
  for (int ii = 0;; ++ii) {
    const bool at_max = ii == q->max_iter;
    S.act = act[sel]; S.cnt = cnt + sel; S.act_next = act[sel ^ 1]; S.cnt_next = cnt + (sel ^ 1);
    if (at_max && !prev_check) {
      // every pair left ends without a final check (state of iteration ii-1)
      pairs_decide_kernel<<<nact, 256, 0, st>>>(S, S.v2[cur], ii, 0, 1);
      break;
    }
    // column update (resident Y, streamed X): v_new; on check iterations the
    // squared column-marginal violation of (u, v_old) per row
    OnlinePass G = pairs_pass(L, w, false, (int)q->m, nrb_x, kt, S.act, S.cnt, abort_flag, tmo);
    G.h = S.hx; G.rterm = F(L.nyk); G.logw2 = F(L.lb2); G.pot2 = S.v2[cur]; G.w = F(L.wb);
    G.pot_out2 = S.v2[cur ^ 1]; G.other_norm2 = S.yk; G.h_out = S.hy; G.err = prev_check ? S.erow : nullptr;
    G.err_sq = 1;
    run(G, false, ii == 0, nact * nrb_y);
    if (prev_check || at_max) {
      pairs_decide_kernel<<<nact, 256, 0, st>>>(S, S.v2[cur], ii, prev_check ? 1 : 0, at_max ? 1 : 0);
      pairs_compact_kernel<<<1, 1024, 0, st>>>(S);
      sel ^= 1;
      S.act = act[sel]; S.cnt = cnt + sel; S.act_next = act[sel ^ 1]; S.cnt_next = cnt + (sel ^ 1);
      int hc[8];
      if (cudaMemcpyAsync(hc, cnt, 32, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
      if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
      if (hc[4]) return OTG_ERR_CUDA;  // a bounded device wait ran out
      nact = hc[sel];
      if (nact == 0 || at_max) break;
    }
    if (D > 0 && ii >= 1) pairs_anderson_kernel<<<nact, 256, 0, st>>>(S, S.v2[cur], S.v2[cur ^ 1]);
    // row update (resident X, streamed Y): u, and the h of the next column update
    OnlinePass Fp = pairs_pass(L, w, true, (int)q->n, nrb_y, kt, S.act, S.cnt, abort_flag, tmo);
    Fp.h = S.hy; Fp.rterm = F(L.nxk); Fp.logw2 = F(L.la2); Fp.pot2 = S.u2; Fp.w = F(L.wa);
    Fp.pot_out2 = S.u2; Fp.other_norm2 = S.xk; Fp.h_out = S.hx;
    run(Fp, true, ii == 0, nact * nrb_x);
    if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
    cur ^= 1;
    prev_check = ii % period == 0;
  }
  int hflag = 0;
  if (cudaMemcpyAsync(&hflag, abort_flag, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
  if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
  return hflag ? OTG_ERR_CUDA : OTG_OK;
}

}  // extern "C"
