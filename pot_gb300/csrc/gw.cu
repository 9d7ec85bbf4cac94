// Tensor-core GEMM for the entropic Gromov-Wasserstein tensor product
//   tens = constC - hC1 T hC2^T           (ot/gromov/_utils.py:244-280)
//   gwggrad = 2 tens                      (ot/gromov/_utils.py:323-354)
// with square loss: constC_ij = (C1^2 p)_i + (C2^2 q)_j, hC1 = C1, hC2 = 2 C2
// (ot/gromov/_utils.py:114-126, 233-239).
//
// Each product runs on the 5th-generation tensor cores (tcgen05.mma, kind::f16,
// fp32 accumulation in TMEM) with operands split into half-precision high and
// low parts, X = Xh + Xl, and three MMAs per k-step (Ah Bh + Ah Bl + Al Bh):
// each part carries 11 significant bits, so the products carry about 22 bits,
// close to fp32.  Operands are staged by TMA (128-byte swizzle) through a
// 3-stage shared-memory ring; warp 4 issues the copies, one thread of warp 5
// the MMAs, warps 0-3 read the accumulator tile from TMEM and run the fused
// epilogue:
//   mode 0: write the scaled result again as high/low half planes (the next
//           product's operand);
//   mode 1: out_ij = s_acc * acc_ij + s_vec * (rowv_i + colv_j)
//           [+ s_add * addend_ij]  (the cost of the inner Sinkhorn,
//           2 constC - 2 hC1 T hC2^T, in fp32, optionally weighted and with
//           the linear term of fused GW or the other half of an asymmetric
//           gradient added).
// The tensor-core accumulator is not a round-to-nearest fp32 sum over long K
// (measured error grows like 2^-24 per accumulation step), so every 4
// k-tiles the tile is moved out of TMEM (two buffers, alternating) and added
// into fp32 registers by the epilogue warps, overlapping the next chunk.
// Every wait is bounded; on a timeout the kernel raises an abort flag, drains
// its own copies and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_fp16.h>
#include <algorithm>
#include <mutex>
#include "common.cuh"
#include "tma.cuh"
#include "tc.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

constexpr int GB_M = 128, GB_N = 128, GB_K = 64, GB_STAGES = 3;
constexpr uint32_t GB_TILE_A = GB_M * GB_K * 2;   // 16 KiB
constexpr uint32_t GB_TILE_B = GB_N * GB_K * 2;   // 16 KiB
constexpr uint32_t GB_STAGE = 2 * GB_TILE_A + 2 * GB_TILE_B;
constexpr size_t GB_SMEM = (size_t)GB_STAGES * GB_STAGE + 1024 /*align*/ + 256 /*barriers*/;
constexpr int GB_THREADS = 192;
constexpr int GB_CHUNK = 4;  // k-tiles accumulated in TMEM before promotion to registers

struct GemmEpi {
  int mode;
  int64_t M, N;                 // valid output extent (mode 1 bounds)
  float scale;                  // mode 0
  float s_acc, s_vec;           // mode 1
  __half* out_hi; __half* out_lo; int64_t ld_h;
  float* out; int64_t ld_o;
  const float* rowv; const float* colv;
  const float* addend; int64_t ld_add; float s_add;  // mode 1, optional
  int64_t a_rows, b_rows;       // rows per problem of the stacked planes (batched form)
  int64_t o_bs, rv_bs, cv_bs, add_bs;  // mode 1: element strides between problems
  int k_tiles;
  int* abort_flag;
  uint64_t timeout_ns;
};

__global__ void __launch_bounds__(GB_THREADS, 1)
gemm_split3_kernel(const __grid_constant__ CUtensorMap tAh, const __grid_constant__ CUtensorMap tAl,
                   const __grid_constant__ CUtensorMap tBh, const __grid_constant__ CUtensorMap tBl, GemmEpi ep) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + GB_STAGES * GB_STAGE);
  uint64_t* empty = full + GB_STAGES;
  uint64_t* accf = empty + GB_STAGES;   // [2] chunk accumulated (MMA -> epilogue)
  uint64_t* acce = accf + 2;            // [2] chunk drained (epilogue -> MMA)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(acce + 2);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.y * GB_M, n0 = blockIdx.x * GB_N;
  // problem z of a batch: its rows of the stacked planes start at z a_rows
  // (A, mode-0 output) and z b_rows (B)
  const int z = blockIdx.z;
  const int am0 = (int)(z * ep.a_rows) + m0, bn0 = (int)(z * ep.b_rows) + n0;
  const int nchunks = (ep.k_tiles + GB_CHUNK - 1) / GB_CHUNK;

  if (threadIdx.x == 0) {
    for (int s = 0; s < GB_STAGES; ++s) { mbar_init(full + s, 1); mbar_init(empty + s, 1); }
    for (int b = 0; b < 2; ++b) { mbar_init(accf + b, 1); mbar_init(acce + b, 4); }
    fence_mbar_init();
    prefetch_tmap(&tAh); prefetch_tmap(&tAl); prefetch_tmap(&tBh); prefetch_tmap(&tBl);
  }
  if (warp == 5) tmem_alloc(tslot, 2 * GB_N);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;

  if (warp == 4) {
    if (lane == 0) {
      int issued = 0;
      for (int kt = 0; kt < ep.k_tiles; ++kt) {
        const int s = kt % GB_STAGES;
        const uint32_t round = kt / GB_STAGES;
        if (!mbar_wait(empty + s, (round & 1u) ^ 1u, ep.abort_flag, ep.timeout_ns)) break;
        unsigned char* st = smem + s * GB_STAGE;
        mbar_arrive_expect_tx(full + s, GB_STAGE);
        tma_load_2d(st, &tAh, kt * GB_K, am0, full + s);
        tma_load_2d(st + GB_TILE_A, &tAl, kt * GB_K, am0, full + s);
        tma_load_2d(st + 2 * GB_TILE_A, &tBh, kt * GB_K, bn0, full + s);
        tma_load_2d(st + 2 * GB_TILE_A + GB_TILE_B, &tBl, kt * GB_K, bn0, full + s);
        ++issued;
      }
      // copies still in flight must land before the CTA can leave
      const int lo = issued > GB_STAGES ? issued - GB_STAGES : 0;
      for (int q = lo; q < issued; ++q) {
        const uint64_t t0 = globaltimer();
        while (!mbar_try_wait(full + q % GB_STAGES, (q / GB_STAGES) & 1u))
          if (globaltimer() - t0 > ep.timeout_ns) break;
      }
    }
  } else if (warp == 5) {
    if (lane == 0) {
      const uint32_t idesc = umma_idesc_f16(GB_M, GB_N, false);
      int kt = 0, committed = 0;
      bool ok = true;
      for (int c = 0; c < nchunks && ok; ++c) {
        const int b = c & 1;
        // the epilogue must have drained this buffer (chunk c-2)
        if (!mbar_wait(acce + b, ((c >> 1) & 1) ^ 1, ep.abort_flag, ep.timeout_ns)) break;
        tc_fence_after();
        const uint32_t dst = tmem + (uint32_t)(b * GB_N);
        uint32_t acc = 0;
        const int kend = min(ep.k_tiles, (c + 1) * GB_CHUNK);
        for (; kt < kend; ++kt) {
          const int s = kt % GB_STAGES;
          if (!mbar_wait(full + s, (kt / GB_STAGES) & 1u, ep.abort_flag, ep.timeout_ns)) { ok = false; break; }
          tc_fence_after();
          unsigned char* st = smem + s * GB_STAGE;
          const uint64_t ah = umma_desc_k128(st), al = umma_desc_k128(st + GB_TILE_A);
          const uint64_t bh = umma_desc_k128(st + 2 * GB_TILE_A), bl = umma_desc_k128(st + 2 * GB_TILE_A + GB_TILE_B);
#pragma unroll
          for (int kk = 0; kk < GB_K / 16; ++kk) {
            const uint64_t o = (uint64_t)(kk * 32) >> 4;  // 16 halves = 32 bytes along K
            umma_f16(dst, ah + o, bh + o, idesc, acc);
            acc = 1;
            umma_f16(dst, ah + o, bl + o, idesc, 1);
            umma_f16(dst, al + o, bh + o, idesc, 1);
          }
          umma_commit(empty + s);
        }
        umma_commit(accf + b);
        committed = c + 1;
      }
      // the last chunk's MMAs (and the stages they read) settle before exit
      if (committed > 0) {
        const int c = committed - 1;
        const uint64_t t0 = globaltimer();
        while (!mbar_try_wait(accf + (c & 1), (c >> 1) & 1)) if (globaltimer() - t0 > ep.timeout_ns) break;
      }
    }
  } else {
    // epilogue warps 0-3: lane 32w+l of TMEM holds output row m0 + 32w + l.
    // Every chunk of GB_CHUNK k-tiles is added into fp32 registers with
    // round-to-nearest, so the tensor-core accumulator never sums more than
    // 3 * 4 * GB_CHUNK products.
    float acc[GB_N];
#pragma unroll
    for (int i = 0; i < GB_N; ++i) acc[i] = 0.f;
    int ok = 1;
    for (int c = 0; c < nchunks && ok; ++c) {
      const int b = c & 1;
      if (lane == 0) ok = (mbar_wait(accf + b, (c >> 1) & 1, ep.abort_flag, ep.timeout_ns) &&
                           !*(volatile int*)ep.abort_flag) ? 1 : 0;
      ok = __shfl_sync(0xffffffffu, ok, 0);  // warp-uniform: tcgen05.ld is a whole-warp instruction
      __syncwarp();
      if (!ok) break;
      tc_fence_after();
#pragma unroll
      for (int c0 = 0; c0 < GB_N; c0 += 32) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * GB_N + c0), v);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[c0 + i] += v[i];
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(acce + b);
    }
    if (ok) {
      const int64_t row = m0 + warp * 32 + lane;
#pragma unroll
      for (int c0 = 0; c0 < GB_N; c0 += 32) {
        const int64_t col0 = n0 + c0;
        if (ep.mode == 0) {
          __align__(16) __half h[32], l[32];
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const float x = acc[c0 + i] * ep.scale;
            h[i] = __float2half_rn(x);
            l[i] = __float2half_rn(x - __half2float(h[i]));
          }
          const int64_t prow = z * ep.a_rows + row;  // row of the stacked output planes
          uint4* dh = reinterpret_cast<uint4*>(ep.out_hi + prow * ep.ld_h + col0);
          uint4* dl = reinterpret_cast<uint4*>(ep.out_lo + prow * ep.ld_h + col0);
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            dh[q] = reinterpret_cast<const uint4*>(h)[q];
            dl[q] = reinterpret_cast<const uint4*>(l)[q];
          }
        } else if (row < ep.M) {
          const float rv = ep.rowv[z * ep.rv_bs + row];
          const float* colv = ep.colv + z * ep.cv_bs;
          float* dst = ep.out + z * ep.o_bs + row * ep.ld_o;
          if (ep.addend) {
            const float* add = ep.addend + z * ep.add_bs + row * ep.ld_add;
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const int64_t col = col0 + i;
              if (col < ep.N)
                dst[col] = fmaf(ep.s_add, add[col], ep.s_acc * acc[c0 + i] + ep.s_vec * (rv + colv[col]));
            }
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
              const int64_t col = col0 + i;
              if (col < ep.N) dst[col] = ep.s_acc * acc[c0 + i] + ep.s_vec * (rv + colv[col]);
            }
          }
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 5) {
    tc_fence_after();
    tmem_dealloc(tmem, 2 * GB_N);
  }
}

// hi/lo half planes of scale*X (transpose = 0) or scale*X^T (transpose = 1).
// X is rows x cols (ldx); out has ld_out columns.  32x32 tiles through
// shared memory keep both the read and the write coalesced.  Batched form:
// blockIdx.z selects the problem, sx and so are the element strides between
// problems of X and of the planes.
__global__ void __launch_bounds__(256) split_half_kernel(const float* __restrict__ X, int64_t rows, int64_t cols,
                                                         int64_t ldx, float scale, int transpose,
                                                         __half* __restrict__ hi, __half* __restrict__ lo,
                                                         int64_t ld_out, int64_t sx, int64_t so) {
  __shared__ float tile[32][33];
  X += blockIdx.z * sx;
  hi += blockIdx.z * so;
  lo += blockIdx.z * so;
  const int64_t r0 = (int64_t)blockIdx.y * 32, c0 = (int64_t)blockIdx.x * 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int k = ty; k < 32; k += 8) {
    const int64_t r = r0 + k, c = c0 + tx;
    tile[k][tx] = (r < rows && c < cols) ? X[r * ldx + c] * scale : 0.f;
  }
  __syncthreads();
  for (int k = ty; k < 32; k += 8) {
    int64_t orow, ocol;
    float x;
    if (transpose) { orow = c0 + k; ocol = r0 + tx; x = tile[tx][k]; if (orow >= cols || ocol >= rows) continue; }
    else { orow = r0 + k; ocol = c0 + tx; x = tile[k][tx]; if (orow >= rows || ocol >= cols) continue; }
    const __half h = __float2half_rn(x);
    hi[orow * ld_out + ocol] = h;
    lo[orow * ld_out + ocol] = __float2half_rn(x - __half2float(h));
  }
}

}  // namespace otg

using namespace otg;

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// Half-precision plane of `rows` x `ld` (row-major), boxes of 128 rows x 64
// columns, 128-byte swizzle.
bool make_plane_map(CUtensorMap* m, const void* base, int64_t rows, int64_t ld) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {GB_K, GB_M};
  cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

extern "C" {

int otg_split_half(const float* X, int64_t rows, int64_t cols, int64_t ldx, float scale, int transpose, void* hi,
                   void* lo, int64_t ld_out, cudaStream_t stream) {
  if (!X || !hi || !lo || rows < 1 || cols < 1 || ldx < cols) return OTG_ERR_ARG;
  if (ld_out < (transpose ? rows : cols)) return OTG_ERR_ARG;
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32));
  if (grid.y > 65535) return OTG_ERR_UNSUPPORTED;
  split_half_kernel<<<grid, 256, 0, stream>>>(X, rows, cols, ldx, scale, transpose, static_cast<__half*>(hi),
                                              static_cast<__half*>(lo), ld_out, 0, 0);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_split_half_batched(const float* X, int64_t rows, int64_t cols, int64_t ldx, int64_t sx, float scale,
                           int transpose, void* hi, void* lo, int64_t ld_out, int64_t so, int64_t batch,
                           cudaStream_t stream) {
  if (!X || !hi || !lo || rows < 1 || cols < 1 || ldx < cols || batch < 1) return OTG_ERR_ARG;
  if (ld_out < (transpose ? rows : cols)) return OTG_ERR_ARG;
  if (batch > 1 && (sx < rows * ldx || so < (transpose ? cols : rows) * ld_out)) return OTG_ERR_ARG;
  dim3 grid((unsigned)((cols + 31) / 32), (unsigned)((rows + 31) / 32), (unsigned)batch);
  if (grid.y > 65535 || batch > 65535) return OTG_ERR_UNSUPPORTED;
  split_half_kernel<<<grid, 256, 0, stream>>>(X, rows, cols, ldx, scale, transpose, static_cast<__half*>(hi),
                                              static_cast<__half*>(lo), ld_out, sx, so);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

int otg_gemm_split3(const OtgSplitGemm* g, cudaStream_t stream) {
  if (!g || !g->a_hi || !g->a_lo || !g->b_hi || !g->b_lo || !g->abort_flag) return OTG_ERR_ARG;
  // planes are padded to whole tiles: rows and leading dims multiples of 128
  if (g->a_rows % GB_M || g->b_rows % GB_N || g->lda % 128 || g->ldb % 128 || g->k_alloc % GB_K) return OTG_ERR_ARG;
  if (g->k_alloc > g->lda || g->k_alloc > g->ldb) return OTG_ERR_ARG;
  if ((uintptr_t)g->a_hi % 16 || (uintptr_t)g->a_lo % 16 || (uintptr_t)g->b_hi % 16 || (uintptr_t)g->b_lo % 16)
    return OTG_ERR_ARG;
  GemmEpi ep{};
  ep.mode = g->mode;
  ep.M = g->M; ep.N = g->N;
  ep.scale = g->scale; ep.s_acc = g->s_acc; ep.s_vec = g->s_vec;
  ep.out_hi = static_cast<__half*>(g->out_hi); ep.out_lo = static_cast<__half*>(g->out_lo); ep.ld_h = g->ld_h;
  ep.out = g->out; ep.ld_o = g->ld_o; ep.rowv = g->rowv; ep.colv = g->colv;
  ep.addend = g->addend; ep.ld_add = g->ld_add; ep.s_add = g->s_add;
  const int64_t batch = g->batch > 1 ? g->batch : 1;
  if (batch > 65535) return OTG_ERR_UNSUPPORTED;
  ep.a_rows = batch > 1 ? g->a_rows : 0;
  ep.b_rows = batch > 1 ? g->b_rows : 0;
  ep.o_bs = g->o_bstride; ep.rv_bs = g->rowv_bstride; ep.cv_bs = g->colv_bstride; ep.add_bs = g->addend_bstride;
  if (batch > 1 && (g->a_rows * batch > INT32_MAX || g->b_rows * batch > INT32_MAX)) return OTG_ERR_UNSUPPORTED;
  ep.k_tiles = (int)(g->k_alloc / GB_K);
  ep.abort_flag = g->abort_flag;
  ep.timeout_ns = g->timeout_ms > 0 ? (uint64_t)g->timeout_ms * 1000000ull : 4000000000ull;
  if (g->mode == 0) {
    if (!ep.out_hi || !ep.out_lo || ep.ld_h % 128 || ep.ld_h < g->b_rows || (uintptr_t)ep.out_hi % 16 ||
        (uintptr_t)ep.out_lo % 16)
      return OTG_ERR_ARG;
  } else {
    if (!ep.out || !ep.rowv || !ep.colv || ep.ld_o < ep.N || ep.M > g->a_rows || ep.N > g->b_rows) return OTG_ERR_ARG;
    if (ep.addend && ep.ld_add < ep.N) return OTG_ERR_ARG;
    // problems' outputs and addends must not overlap one another
    if (batch > 1 && (ep.o_bs < ep.M * ep.ld_o || ep.rv_bs < ep.M || ep.cv_bs < ep.N ||
                      (ep.addend && ep.add_bs < ep.M * ep.ld_add)))
      return OTG_ERR_ARG;
  }
  CUtensorMap mah, mal, mbh, mbl;
  const int64_t ar = g->a_rows * batch, br = g->b_rows * batch;  // rows of the stacked planes
  if (!make_plane_map(&mah, g->a_hi, ar, g->lda) || !make_plane_map(&mal, g->a_lo, ar, g->lda) ||
      !make_plane_map(&mbh, g->b_hi, br, g->ldb) || !make_plane_map(&mbl, g->b_lo, br, g->ldb))
    return OTG_ERR_CUDA;
  static bool attr_set = false;
  if (!attr_set) {
    if (cudaFuncSetAttribute(gemm_split3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)GB_SMEM) !=
        cudaSuccess)
      return OTG_ERR_CUDA;
    attr_set = true;
  }
  dim3 grid((unsigned)(g->b_rows / GB_N), (unsigned)(g->a_rows / GB_M), (unsigned)batch);
  if (grid.y > 65535) return OTG_ERR_UNSUPPORTED;
  gemm_split3_kernel<<<grid, GB_THREADS, GB_SMEM, stream>>>(mah, mal, mbh, mbl, ep);
  return cudaGetLastError() == cudaSuccess ? OTG_OK : OTG_ERR_CUDA;
}

}  // extern "C"
