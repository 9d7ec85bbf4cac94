// Anderson mixing of a Sinkhorn potential update, one CTA per problem.
//
// The map F(v) = colT(rowT(v)) (a row update followed by a column update)
// has the Sinkhorn potentials as fixed points.  With depth D the v of the
// next row update is  sum_k alpha_k F(v_k)  over the last D iterates, alpha
// minimising |sum_k alpha_k (F(v_k) - v_k)|_2 with sum alpha = 1: the normal
// equations of the residual Gram matrix with a Tikhonov term 1e-10 trace / D,
// solved by Gaussian elimination with partial pivoting; a failed solve, or
// one with sum |alpha| >= 1e4, restarts the history and takes the plain step.
// No reference counterpart (the warm-start refinement); the caller's stop
// test is unchanged.
#pragma once
#include "common.cuh"
#include "../../include/pot_gb300.h"

namespace otg {

constexpr double AND_LAMBDA = 1e-10;   // Tikhonov term, relative to trace / D
constexpr double AND_MAX_L1 = 1e4;     // larger sum |alpha|: restart with the plain step

// One problem's step, called by every thread of the CTA.  vold: v_k, vnew:
// F(v_k) on entry and the mixed v on return, both at column offset `co`
// (m columns); F and R: D history slots of stride `stride` (slot-major);
// G: the problem's D x D residual Gram matrix; cnt: iterates taken so far.
template <typename T>
__device__ void anderson_step(int D, int m, int64_t co, int64_t stride, const T* vold, T* vnew, T* F, T* R,
                              double* G, int32_t* cnt_p) {
  constexpr int MD = OTG_ANDERSON_MAX_DEPTH;
  __shared__ double s_dot[MD];
  __shared__ double s_alpha[MD];
  __shared__ int s_keep;
  const int cnt = __ldcg(cnt_p);
  const int s = cnt % D;                       // slot of the new iterate
  const int nh = cnt + 1 < D ? cnt + 1 : D;    // slots in use after the insert
  // insert, and this thread's share of the dots <r_new, R_q>
  double acc[MD];
#pragma unroll
  for (int q = 0; q < MD; ++q) acc[q] = 0.0;
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    const T f = __ldcg(vnew + co + j);
    const T r = f - __ldcg(vold + co + j);
    F[(int64_t)s * stride + co + j] = f;
    R[(int64_t)s * stride + co + j] = r;
#pragma unroll
    for (int q = 0; q < MD; ++q) {
      if (q < nh) {
        const T rq = q == s ? r : __ldcg(R + (int64_t)q * stride + co + j);
        acc[q] += (double)r * (double)rq;
      }
    }
  }
#pragma unroll
  for (int q = 0; q < MD; ++q) {
    if (q < nh) {
      const double d = block_sum_fixed(acc[q]);
      if (threadIdx.x == 0) s_dot[q] = d;
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < nh; ++q) { G[s * D + q] = s_dot[q]; G[q * D + s] = s_dot[q]; }
    // (G + lambda I) w = 1 by Gaussian elimination with partial pivoting
    double Mx[MD][MD + 1];
    double tr = 0.0;
    for (int i = 0; i < nh; ++i) tr += G[i * D + i];
    const double lam = AND_LAMBDA * tr / nh;
    for (int i = 0; i < nh; ++i) {
      for (int j = 0; j < nh; ++j) Mx[i][j] = G[i * D + j] + (i == j ? lam : 0.0);
      Mx[i][nh] = 1.0;
    }
    bool ok = nh > 1 && tr > 0.0;
    for (int c = 0; ok && c < nh; ++c) {
      int piv = c;
      for (int i = c + 1; i < nh; ++i) if (fabs(Mx[i][c]) > fabs(Mx[piv][c])) piv = i;
      if (!(fabs(Mx[piv][c]) > 0.0)) { ok = false; break; }
      if (piv != c) for (int j = c; j <= nh; ++j) { const double t = Mx[c][j]; Mx[c][j] = Mx[piv][j]; Mx[piv][j] = t; }
      for (int i = c + 1; i < nh; ++i) {
        const double f = Mx[i][c] / Mx[c][c];
        for (int j = c; j <= nh; ++j) Mx[i][j] -= f * Mx[c][j];
      }
    }
    double w[MD];
    double sw = 0.0, l1 = 0.0;
    for (int i = nh - 1; ok && i >= 0; --i) {
      double t = Mx[i][nh];
      for (int j = i + 1; j < nh; ++j) t -= Mx[i][j] * w[j];
      w[i] = t / Mx[i][i];
      sw += w[i];
    }
    if (ok) {
      for (int i = 0; i < nh; ++i) { w[i] /= sw; l1 += fabs(w[i]); }
      ok = isfinite(l1) && l1 < AND_MAX_L1;
    }
    for (int i = 0; i < MD; ++i) s_alpha[i] = ok && i < nh ? w[i] : (i == s ? 1.0 : 0.0);
    // a first iterate, or a failed solve: the plain step; after a failure
    // the history restarts with the next iterate
    s_keep = ok;
    *cnt_p = ok || nh == 1 ? cnt + 1 : 0;
  }
  __syncthreads();
  if (s_keep) {
    for (int j = threadIdx.x; j < m; j += blockDim.x) {
      double vm = 0.0;
      for (int q = 0; q < nh; ++q) vm += s_alpha[q] * (double)__ldcg(F + (int64_t)q * stride + co + j);
      vnew[co + j] = (T)vm;
    }
  }
  // after a restart vnew keeps F(v_k): the plain step
  __syncthreads();
}

}  // namespace otg
