// Entropic Wasserstein barycenters of H histograms on one support, the whole
// iteration loop driven from C++ (one synchronisation per error check).
//
// Reference behaviour (PythonOT/POT ot/bregman/_barycenter.py):
//   barycenter_sinkhorn        :141-259  scaling form with K = exp(-M/reg):
//     UKv = K (A^T / K^T 1)^T ; u = geomMean(UKv) / UKv                 (init)
//     UKv = u * K^T (A / K u) ; u = u * geomBar(w, UKv) / UKv           (loop)
//     at ii % 10 == 1: err = sum_i std_k UKv_ik, stop when < stopThr;
//     returns geomBar(w, UKv) = exp(log(UKv) w)
//   _barycenter_sinkhorn_log   :403-473  log form with Mr = -M/reg:
//     f_k = log(A_k + 1e-16) - LSE_j(Mr_ij + G_jk)   (row pass, all k)
//     logKU_k = LSE_i(Mr_ij + f_ik)                  (column pass, all k)
//     logbar = logKU w ; at ii % 10 == 1: err = sum_i std_k exp(G + logKU);
//     G = logbar - logKU ; returns exp(logbar)
//
// The scaling form's two products per iteration are dense GEMMs (dim x dim
// times dim x H, the tiled GEMM of mlp.cu); the log form's passes are
// log-semiring products: one warp per (row, histogram) for the row LSEs
// (lanes walk the row, so loads coalesce and the 8 warps of a CTA share the
// row in L1), one thread per (column, histogram) for the column LSEs.  The
// per-row updates (geometric barycentre, u, the error) are one fused kernel.
#include <algorithm>
#include <cmath>
#include <vector>
#include "common.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

template <typename T>
__global__ void kmat_kernel(const T* __restrict__ M, int64_t n, int64_t ldm, T c, T* __restrict__ K) {
  const int64_t total = n * n;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = e / n, j = e % n;
    K[e] = ex2(M[i * ldm + j] * c);
  }
}

// X0[i,k] = A[i,k] / colsum_i  (A^T / sum(K, axis=0), transposed back)
template <typename T>
__global__ void bary_scale_kernel(const T* __restrict__ A, const double* __restrict__ colsum, int64_t n, int H,
                                  T* __restrict__ X) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * H; e += (int64_t)gridDim.x * blockDim.x)
    X[e] = A[e] / (T)colsum[e / H];
}

// u[i,k] = geomMean_k(UKv[i,:]) / UKv[i,k]
template <typename T>
__global__ void bary_init_kernel(const T* __restrict__ UKv, int64_t n, int H, T* __restrict__ u) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T s = 0;
    for (int k = 0; k < H; ++k) s += log(UKv[i * H + k]);
    const T gm = exp(s / (T)H);
    for (int k = 0; k < H; ++k) u[i * H + k] = gm / UKv[i * H + k];
  }
}

template <typename T>
__global__ void bary_div_kernel(const T* __restrict__ A, const T* __restrict__ KU, int64_t total, T* __restrict__ X) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    X[e] = A[e] / KU[e];
}

// Population standard deviation of H values (numpy's default ddof = 0).
template <typename T>
__device__ __forceinline__ double row_std(const T* x, int H) {
  double mean = 0;
  for (int k = 0; k < H; ++k) mean += (double)x[k];
  mean /= H;
  double var = 0;
  for (int k = 0; k < H; ++k) { const double d = (double)x[k] - mean; var += d * d; }
  return sqrt(var / H);
}

// Scaling form, per row: UKv = u * KtX ; bar = exp(log(UKv) w) ;
// u = u * bar / UKv ; erow[i] = std_k UKv (check iterations; the rows' slots
// are summed in a fixed order afterwards).
template <typename T>
__global__ void __launch_bounds__(256) bary_update_kernel(T* __restrict__ u, T* __restrict__ KtX,
                                                          const T* __restrict__ w, int64_t n, int H,
                                                          T* __restrict__ bar, double* erow) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    T* ui = u + i * H;
    T* ukv = KtX + i * H;  // overwritten with UKv
    T lb = 0;
    for (int k = 0; k < H; ++k) {
      ukv[k] = ui[k] * ukv[k];
      lb += log(ukv[k]) * w[k];
    }
    const T b = exp(lb);
    bar[i] = b;
    for (int k = 0; k < H; ++k) ui[k] = ui[k] * b / ukv[k];
    if (erow) erow[i] = row_std(ukv, H);
  }
}

// Log form, row pass: out[i,k] = logA[i,k] - LSE_j(c2 M[i,j] + V[j,k] log2e) ln2
// with c2 = -log2(e)/reg.  One warp per (row, histogram).
template <typename T>
__global__ void __launch_bounds__(256) lse_rows_kernel(const T* __restrict__ M, int64_t n, int64_t ldm, T c2,
                                                       const T* __restrict__ V, int H, const T* __restrict__ logA,
                                                       T* __restrict__ out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t i = blockIdx.x;
  const T L2E = T(OTG_LOG2E), LN2 = T(OTG_LN2);
  const T* Mrow = M + i * ldm;
  for (int k = warp; k < H; k += 8) {
    T mx = -INFINITY, s = 0;
    for (int64_t j = lane; j < n; j += 32) {
      const T t = fma(Mrow[j], c2, V[j * H + k] * L2E);
      lse_merge(mx, s, t, T(1));
    }
    warp_lse(mx, s);
    if (lane == 0) out[i * H + k] = logA[i * H + k] - lse_value(mx, s) * LN2;
  }
}

// Log form, column pass: out[j,k] = LSE_i(c2 M[i,j] + V[i,k] log2e) ln2.
// grid = (column tiles of 256, H).
template <typename T>
__global__ void __launch_bounds__(256) lse_cols_kernel(const T* __restrict__ M, int64_t n, int64_t ldm, T c2,
                                                       const T* __restrict__ V, int H, T* __restrict__ out) {
  const int64_t j = (int64_t)blockIdx.x * 256 + threadIdx.x;
  const int k = blockIdx.y;
  if (j >= n) return;
  const T L2E = T(OTG_LOG2E), LN2 = T(OTG_LN2);
  T mx = -INFINITY, s = 0;
  for (int64_t i = 0; i < n; ++i) {
    const T t = fma(M[i * ldm + j], c2, V[i * H + k] * L2E);
    lse_merge(mx, s, t, T(1));
  }
  out[j * H + k] = lse_value(mx, s) * LN2;
}

// Log form, per row: logbar = logKU w ; erow[i] = std_k exp(G + logKU) ;
// G = logbar - logKU.
template <typename T>
__global__ void __launch_bounds__(256) bary_log_update_kernel(T* __restrict__ G, const T* __restrict__ logKU,
                                                              const T* __restrict__ w, int64_t n, int H,
                                                              T* __restrict__ logbar, double* erow) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const T* lk = logKU + i * H;
    T* gi = G + i * H;
    T lb = 0;
    for (int k = 0; k < H; ++k) lb += w[k] * lk[k];
    logbar[i] = lb;
    if (erow) {
      double mean = 0, var = 0;
      for (int k = 0; k < H; ++k) mean += exp((double)gi[k] + (double)lk[k]);
      mean /= H;
      for (int k = 0; k < H; ++k) { const double d = exp((double)gi[k] + (double)lk[k]) - mean; var += d * d; }
      erow[i] = sqrt(var / H);
    }
    for (int k = 0; k < H; ++k) gi[k] = lb - lk[k];
  }
}

template <typename T>
__global__ void log_eps_kernel(const T* __restrict__ A, int64_t total, T* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = log(A[e] + T(1e-16));
}

template <typename T>
__global__ void exp_kernel(const T* __restrict__ x, int64_t total, T* __restrict__ out) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x)
    out[e] = exp(x[e]);
}

}  // namespace otg

using namespace otg;

namespace {

size_t a256(size_t x) { return (x + 255) / 256 * 256; }

unsigned blocks_for(int64_t work) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((work + 255) / 256, 4096)); }

template <typename T>
int gemm(int ta, int tb, int64_t M, int64_t N, int64_t K, const T* A, int64_t lda, const T* B, int64_t ldb, T* C,
         int64_t ldc, cudaStream_t st);
template <>
int gemm<float>(int ta, int tb, int64_t M, int64_t N, int64_t K, const float* A, int64_t lda, const float* B,
                int64_t ldb, float* C, int64_t ldc, cudaStream_t st) {
  return otg_gemm_f32(ta, tb, M, N, K, 1.0f, A, lda, B, ldb, 0.0f, C, ldc, nullptr, 0, st);
}
template <>
int gemm<double>(int ta, int tb, int64_t M, int64_t N, int64_t K, const double* A, int64_t lda, const double* B,
                 int64_t ldb, double* C, int64_t ldc, cudaStream_t st) {
  return otg_gemm_f64(ta, tb, M, N, K, 1.0, A, lda, B, ldb, 0.0, C, ldc, st);
}

template <typename T>
int run_bary(const OtgBaryProblem* p, cudaStream_t st) {
  const int64_t n = p->dim;
  const int H = p->n_hists;
  const T* M = static_cast<const T*>(p->M);
  const T* A = static_cast<const T*>(p->A);
  const T* w = static_cast<const T*>(p->weights);
  T* bar = static_cast<T*>(p->out_bar);
  char* ws = static_cast<char*>(p->workspace);
  size_t off = 0;
  auto take = [&](size_t bytes) { char* q = ws + off; off += a256(bytes); return q; };
  double* err = reinterpret_cast<double*>(take(8 * 2));
  double* erow = reinterpret_cast<double*>(take(8 * (size_t)n));  // per-row errors of a check iteration
  const size_t nh = sizeof(T) * (size_t)n * H;
  T* b1 = reinterpret_cast<T*>(take(nh));
  T* b2 = reinterpret_cast<T*>(take(nh));
  T* b3 = reinterpret_cast<T*>(take(nh));
  const T c2 = (T)(-OTG_LOG2E / p->reg);
  const unsigned gb = blocks_for(n * H);
  int status = OTG_STATUS_MAXITER, niter = p->max_iter - 1, nchk = 0;
  double herr = 0;
  if (p->method == OTG_METHOD_KNOPP) {
    T* K = reinterpret_cast<T*>(take(sizeof(T) * (size_t)n * n));
    double* colsum = reinterpret_cast<double*>(take(8 * (size_t)n));
    double* rowsum = reinterpret_cast<double*>(take(8 * (size_t)n));
    if (off > p->workspace_bytes) return OTG_ERR_WORKSPACE;
    kmat_kernel<T><<<blocks_for(n * n), 256, 0, st>>>(M, n, p->ldm, c2, K);
    // column sums of K: the marginals of exp(-M/reg) with zero potentials
    if (cudaMemsetAsync(b1, 0, sizeof(T) * (size_t)n, st) != cudaSuccess) return OTG_ERR_CUDA;
    int rc = otg_dense_marginals(p->dtype, p->M, n, n, p->ldm, b1, b1, p->reg, rowsum, colsum, st);
    if (rc != OTG_OK) return rc;
    T *u = b1, *KU = b2, *X = b3;
    bary_scale_kernel<T><<<gb, 256, 0, st>>>(A, colsum, n, H, X);
    if ((rc = gemm<T>(0, 0, n, H, n, K, n, X, H, KU, H, st)) != OTG_OK) return rc;
    bary_init_kernel<T><<<blocks_for(n), 256, 0, st>>>(KU, n, H, u);
    for (int ii = 0; ii < p->max_iter; ++ii) {
      if ((rc = gemm<T>(0, 0, n, H, n, K, n, u, H, KU, H, st)) != OTG_OK) return rc;
      bary_div_kernel<T><<<gb, 256, 0, st>>>(A, KU, n * H, X);
      if ((rc = gemm<T>(1, 0, n, H, n, K, n, X, H, KU, H, st)) != OTG_OK) return rc;  // K^T X into KU
      const bool check = ii % 10 == 1;
      bary_update_kernel<T><<<blocks_for(n), 256, 0, st>>>(u, KU, w, n, H, bar, check ? erow : nullptr);
      if (check) {
        slot_sum_kernel<1024><<<1, 1024, 0, st>>>(erow, n, err);  // fixed order: the same error in every run
        if (cudaMemcpyAsync(&herr, err, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
        if (nchk < p->hist_cap) p->err_hist[nchk] = herr;
        ++nchk;
        if (herr < p->stop_thr) { status = OTG_STATUS_CONVERGED; niter = ii; break; }
      }
    }
  } else {
    T* b4 = reinterpret_cast<T*>(take(nh));
    if (off > p->workspace_bytes) return OTG_ERR_WORKSPACE;
    T *logA = b1, *G = b2, *F = b3, *logKU = b4;
    log_eps_kernel<T><<<gb, 256, 0, st>>>(A, n * H, logA);
    if (cudaMemsetAsync(G, 0, nh, st) != cudaSuccess) return OTG_ERR_CUDA;
    const dim3 cgrid((unsigned)((n + 255) / 256), (unsigned)H);
    for (int ii = 0; ii < p->max_iter; ++ii) {
      lse_rows_kernel<T><<<(unsigned)n, 256, 0, st>>>(M, n, p->ldm, c2, G, H, logA, F);
      lse_cols_kernel<T><<<cgrid, 256, 0, st>>>(M, n, p->ldm, c2, F, H, logKU);
      const bool check = ii % 10 == 1;
      // the log barycentre is kept in out_bar and exponentiated at the end
      bary_log_update_kernel<T><<<blocks_for(n), 256, 0, st>>>(G, logKU, w, n, H, bar, check ? erow : nullptr);
      if (check) {
        slot_sum_kernel<1024><<<1, 1024, 0, st>>>(erow, n, err);  // fixed order: the same error in every run
        if (cudaMemcpyAsync(&herr, err, 8, cudaMemcpyDeviceToHost, st) != cudaSuccess) return OTG_ERR_CUDA;
        if (cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
        if (nchk < p->hist_cap) p->err_hist[nchk] = herr;
        ++nchk;
        if (herr < p->stop_thr) { status = OTG_STATUS_CONVERGED; niter = ii; break; }
      }
    }
    exp_kernel<T><<<blocks_for(n), 256, 0, st>>>(bar, n, bar);
  }
  if (cudaGetLastError() != cudaSuccess) return OTG_ERR_CUDA;
  if (status == OTG_STATUS_MAXITER && cudaStreamSynchronize(st) != cudaSuccess) return OTG_ERR_CUDA;
  p->info[0] = status;
  p->info[1] = niter;
  p->info[2] = nchk;
  return OTG_OK;
}

}  // namespace

extern "C" {

size_t otg_barycenter_workspace_bytes(int dtype, int method, int64_t dim, int32_t n_hists) {
  const size_t es = dtype == OTG_F64 ? 8 : 4;
  const size_t nh = a256(es * (size_t)dim * (size_t)n_hists);
  size_t b = a256(16) + a256(8 * (size_t)dim) + 3 * nh;
  if (method == OTG_METHOD_KNOPP) b += a256(es * (size_t)dim * (size_t)dim) + 2 * a256(8 * (size_t)dim);
  else b += nh;
  return b;
}

int otg_barycenter(const OtgBaryProblem* p, cudaStream_t stream) {
  if (!p || !p->M || !p->A || !p->weights || !p->out_bar || !p->workspace || !p->err_hist || !p->info) return OTG_ERR_ARG;
  if (p->dim < 1 || p->n_hists < 1 || p->ldm < p->dim || p->max_iter < 1 || p->hist_cap < 1 || !(p->reg > 0))
    return OTG_ERR_ARG;
  if (p->method != OTG_METHOD_KNOPP && p->method != OTG_METHOD_LOG) return OTG_ERR_ARG;
  if (p->workspace_bytes < otg_barycenter_workspace_bytes(p->dtype, p->method, p->dim, p->n_hists))
    return OTG_ERR_WORKSPACE;
  if (p->dtype == OTG_F64) return run_bary<double>(p, stream);
  if (p->dtype == OTG_F32) return run_bary<float>(p, stream);
  return OTG_ERR_DTYPE;
}

}  // extern "C"
