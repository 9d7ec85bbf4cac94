// ABI self-description of the public structs of pot_gb300.h: their sizes and
// the offsets of their fields, for bindings (ctypes, cgo, JNI) to check
// their mirrors against the compiled library.  Host code only.
#include <cstddef>
#include <cstring>

#include "../../include/pot_gb300.h"

namespace {
#define OTG_FIELDS_OtgDenseProblem(X) \
  X(dtype) \
  X(method) \
  X(M) \
  X(n) \
  X(m) \
  X(ldm) \
  X(a) \
  X(b) \
  X(warm_u) \
  X(warm_v) \
  X(reg) \
  X(max_iter) \
  X(hist_cap) \
  X(stop_thr) \
  X(out_u) \
  X(out_v) \
  X(workspace_bytes) \
  X(grid) \
  X(timeout_ms) \
  X(tau) \
  X(check_period) \
  X(reserved) \
  X(reg_m1) \
  X(reg_m2) \
  X(c_ones) \
  X(reserved2) \
  X(K) \
  X(ldk)
#define OTG_FIELDS_OtgBaryProblem(X) \
  X(dtype) \
  X(method) \
  X(M) \
  X(dim) \
  X(ldm) \
  X(A) \
  X(n_hists) \
  X(max_iter) \
  X(weights) \
  X(reg) \
  X(stop_thr) \
  X(out_bar) \
  X(err_hist) \
  X(hist_cap) \
  X(info) \
  X(workspace) \
  X(workspace_bytes)
#define OTG_FIELDS_OtgBatchProblem(X) \
  X(dtype) \
  X(method) \
  X(M) \
  X(m_off) \
  X(rows) \
  X(cols) \
  X(ldm) \
  X(r_off) \
  X(c_off) \
  X(a) \
  X(b) \
  X(warm_u) \
  X(warm_v) \
  X(reg) \
  X(order) \
  X(nprob) \
  X(max_iter) \
  X(stop_thr) \
  X(u_first) \
  X(grid) \
  X(out_u) \
  X(out_v) \
  X(status) \
  X(niter) \
  X(err) \
  X(queue) \
  X(timeout_ms)
#define OTG_FIELDS_OtgMultiProblem(X) \
  X(dtype) \
  X(nprob) \
  X(M) \
  X(m_off) \
  X(rows) \
  X(cols) \
  X(ldm) \
  X(r_off) \
  X(c_off) \
  X(a) \
  X(b) \
  X(warm_u) \
  X(reg) \
  X(max_iter) \
  X(grid) \
  X(stop_thr) \
  X(nsr_max) \
  X(pc_off) \
  X(total_rows) \
  X(total_cols) \
  X(total_partials) \
  X(out_u) \
  X(out_v) \
  X(status) \
  X(niter) \
  X(err) \
  X(workspace) \
  X(workspace_bytes) \
  X(timeout_ms) \
  X(omega) \
  X(check_period) \
  X(units_per_warp) \
  X(split_cap_fill) \
  X(split_cap_tail) \
  X(tail_problems) \
  X(joint_stop) \
  X(scaling) \
  X(anderson_depth) \
  X(reserved) \
  X(anderson_ws) \
  X(anderson_ws_bytes)
#define OTG_FIELDS_OtgOnlineProblem(X) \
  X(X) \
  X(Y) \
  X(n) \
  X(m) \
  X(d) \
  X(max_iter) \
  X(a) \
  X(b) \
  X(warm_f) \
  X(warm_g) \
  X(reg) \
  X(stop_thr) \
  X(scale_x) \
  X(scale_y) \
  X(out_f) \
  X(out_g) \
  X(err_hist) \
  X(hist_cap) \
  X(info) \
  X(workspace) \
  X(workspace_bytes) \
  X(timeout_ms) \
  X(sum_window_log2)
#define OTG_FIELDS_OtgCostTable(X) \
  X(dtype) \
  X(nprob) \
  X(X) \
  X(Y) \
  X(x_off) \
  X(y_off) \
  X(rows) \
  X(cols) \
  X(dim) \
  X(max_dim) \
  X(M) \
  X(m_off) \
  X(ldm) \
  X(max_out) \
  X(fixed_dim)
#define OTG_FIELDS_OtgPlanTable(X) \
  X(dtype) \
  X(method) \
  X(nprob) \
  X(kl) \
  X(M) \
  X(m_off) \
  X(rows) \
  X(cols) \
  X(ldm) \
  X(r_off) \
  X(c_off) \
  X(u) \
  X(v) \
  X(a) \
  X(b) \
  X(reg) \
  X(P) \
  X(out_vals)
#define OTG_FIELDS_OtgSplitGemm(X) \
  X(a_hi) \
  X(a_lo) \
  X(a_rows) \
  X(lda) \
  X(b_hi) \
  X(b_lo) \
  X(b_rows) \
  X(ldb) \
  X(k_alloc) \
  X(mode) \
  X(scale) \
  X(s_acc) \
  X(s_vec) \
  X(out_hi) \
  X(out_lo) \
  X(ld_h) \
  X(out) \
  X(ld_o) \
  X(M) \
  X(N) \
  X(rowv) \
  X(colv) \
  X(abort_flag) \
  X(timeout_ms) \
  X(addend) \
  X(ld_add) \
  X(s_add) \
  X(batch) \
  X(o_bstride) \
  X(rowv_bstride) \
  X(colv_bstride) \
  X(addend_bstride)

#define OTG_FIELDS_OtgPairsProblem(X) \
  X(X) \
  X(Y) \
  X(npairs) \
  X(d) \
  X(n) \
  X(m) \
  X(a) \
  X(b) \
  X(reg) \
  X(warm_u) \
  X(max_iter) \
  X(check_period) \
  X(stop_thr) \
  X(anderson_depth) \
  X(timeout_ms) \
  X(out_u) \
  X(out_v) \
  X(status) \
  X(niter) \
  X(err) \
  X(workspace) \
  X(workspace_bytes) \
  X(sum_window_log2)

template <typename S>
int write_layout(int64_t* out, int32_t cap, const size_t* offs, int nf) {
  if (cap < nf + 1) return OTG_ERR_ARG;
  out[0] = (int64_t)sizeof(S);
  for (int k = 0; k < nf; ++k) out[k + 1] = (int64_t)offs[k];
  return nf + 1;
}

}  // namespace

extern "C" int otg_abi_layout(const char* name, int64_t* out, int32_t cap) {
  if (!name || !out) return OTG_ERR_ARG;
  if (std::strcmp(name, "OtgDenseProblem") == 0) {
#define X(fld) offsetof(OtgDenseProblem, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgDenseProblem(X)};
#undef X
    return write_layout<OtgDenseProblem>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgBaryProblem") == 0) {
#define X(fld) offsetof(OtgBaryProblem, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgBaryProblem(X)};
#undef X
    return write_layout<OtgBaryProblem>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgBatchProblem") == 0) {
#define X(fld) offsetof(OtgBatchProblem, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgBatchProblem(X)};
#undef X
    return write_layout<OtgBatchProblem>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgMultiProblem") == 0) {
#define X(fld) offsetof(OtgMultiProblem, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgMultiProblem(X)};
#undef X
    return write_layout<OtgMultiProblem>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgOnlineProblem") == 0) {
#define X(fld) offsetof(OtgOnlineProblem, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgOnlineProblem(X)};
#undef X
    return write_layout<OtgOnlineProblem>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgCostTable") == 0) {
#define X(fld) offsetof(OtgCostTable, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgCostTable(X)};
#undef X
    return write_layout<OtgCostTable>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgPlanTable") == 0) {
#define X(fld) offsetof(OtgPlanTable, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgPlanTable(X)};
#undef X
    return write_layout<OtgPlanTable>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgSplitGemm") == 0) {
#define X(fld) offsetof(OtgSplitGemm, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgSplitGemm(X)};
#undef X
    return write_layout<OtgSplitGemm>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  if (std::strcmp(name, "OtgPairsProblem") == 0) {
#define X(fld) offsetof(OtgPairsProblem, fld),
    static const size_t offs[] = {OTG_FIELDS_OtgPairsProblem(X)};
#undef X
    return write_layout<OtgPairsProblem>(out, cap, offs, (int)(sizeof(offs) / sizeof(offs[0])));
  }
  return OTG_ERR_ARG;
}
