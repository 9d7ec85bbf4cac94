"""ctypes binding of the C ABI declared in ``include/pot_gb300.h``.

The library is the only compute path: importing a solver without it on a GPU
machine raises, there is no CPU fallback.
"""
import ctypes
import os

import torch

from . import _build

OTG_F32, OTG_F64 = 0, 1
OTG_METHOD_KNOPP, OTG_METHOD_LOG, OTG_METHOD_STAB, OTG_METHOD_UNB = 0, 1, 2, 3
STATUS_CONVERGED, STATUS_MAXITER, STATUS_NUMERICAL, STATUS_ABORTED = 0, 1, 2, 3
_ERRORS = {-1: "invalid argument", -2: "unsupported dtype", -3: "workspace too small",
           -4: "CUDA launch error", -5: "unsupported configuration",
           -6: "problem too large for the static scratch of the allocation-free entry point"}

c_i32, c_i64, c_sz, c_dbl, c_vp = ctypes.c_int32, ctypes.c_int64, ctypes.c_size_t, ctypes.c_double, ctypes.c_void_p


class OtgDenseProblem(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("method", c_i32), ("M", c_vp), ("n", c_i64), ("m", c_i64),
                ("ldm", c_i64), ("a", c_vp), ("b", c_vp), ("warm_u", c_vp), ("warm_v", c_vp),
                ("reg", c_dbl), ("max_iter", c_i32), ("hist_cap", c_i32), ("stop_thr", c_dbl),
                ("out_u", c_vp), ("out_v", c_vp), ("workspace_bytes", c_sz), ("grid", c_i32),
                ("timeout_ms", c_i32), ("tau", c_dbl), ("check_period", c_i32), ("reserved", c_i32),
                ("reg_m1", c_dbl), ("reg_m2", c_dbl), ("c_ones", c_i32), ("reserved2", c_i32), ("K", c_vp),
                ("ldk", c_i64)]


class OtgBatchProblem(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("method", c_i32), ("M", c_vp), ("m_off", c_vp), ("rows", c_vp),
                ("cols", c_vp), ("ldm", c_vp), ("r_off", c_vp), ("c_off", c_vp), ("a", c_vp), ("b", c_vp),
                ("warm_u", c_vp), ("warm_v", c_vp), ("reg", c_vp), ("order", c_vp), ("nprob", c_i32),
                ("max_iter", c_i32), ("stop_thr", c_dbl), ("u_first", c_i32), ("grid", c_i32),
                ("out_u", c_vp), ("out_v", c_vp), ("status", c_vp), ("niter", c_vp), ("err", c_vp),
                ("queue", c_vp), ("timeout_ms", c_i32)]


class OtgMultiProblem(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("nprob", c_i32), ("M", c_vp), ("m_off", c_vp), ("rows", c_vp), ("cols", c_vp),
                ("ldm", c_vp), ("r_off", c_vp), ("c_off", c_vp), ("a", c_vp), ("b", c_vp), ("warm_u", c_vp),
                ("reg", c_vp), ("max_iter", c_i32), ("grid", c_i32), ("stop_thr", c_dbl), ("nsr_max", c_vp),
                ("pc_off", c_vp), ("total_rows", c_i64), ("total_cols", c_i64), ("total_partials", c_i64),
                ("out_u", c_vp), ("out_v", c_vp), ("status", c_vp), ("niter", c_vp), ("err", c_vp),
                ("workspace", c_vp), ("workspace_bytes", c_sz), ("timeout_ms", c_i32), ("omega", c_dbl),
                ("check_period", c_i32), ("units_per_warp", c_i32), ("split_cap_fill", c_i32),
                ("split_cap_tail", c_i32), ("tail_problems", c_i32), ("joint_stop", c_i32),
                ("scaling", c_i32), ("anderson_depth", c_i32), ("reserved", c_i32), ("anderson_ws", c_vp),
                ("anderson_ws_bytes", c_sz)]


class OtgPairsProblem(ctypes.Structure):
    _fields_ = [("X", c_vp), ("Y", c_vp), ("npairs", c_i32), ("d", c_i32), ("n", c_i64), ("m", c_i64), ("a", c_vp),
                ("b", c_vp), ("reg", c_vp), ("warm_u", c_vp), ("max_iter", c_i32), ("check_period", c_i32),
                ("stop_thr", c_dbl), ("anderson_depth", c_i32), ("timeout_ms", c_i32), ("out_u", c_vp),
                ("out_v", c_vp), ("status", c_vp), ("niter", c_vp), ("err", c_vp), ("workspace", c_vp),
                ("workspace_bytes", c_sz), ("sum_window_log2", ctypes.c_float)]


class OtgCostTable(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("nprob", c_i32), ("X", c_vp), ("Y", c_vp), ("x_off", c_vp), ("y_off", c_vp),
                ("rows", c_vp), ("cols", c_vp), ("dim", c_vp), ("max_dim", c_i32), ("M", c_vp), ("m_off", c_vp),
                ("ldm", c_vp), ("max_out", c_vp), ("fixed_dim", c_i32)]


class OtgPlanTable(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("method", c_i32), ("nprob", c_i32), ("kl", c_i32), ("M", c_vp),
                ("m_off", c_vp), ("rows", c_vp), ("cols", c_vp), ("ldm", c_vp), ("r_off", c_vp), ("c_off", c_vp),
                ("u", c_vp), ("v", c_vp), ("a", c_vp), ("b", c_vp), ("reg", c_vp), ("P", c_vp), ("out_vals", c_vp)]


class OtgSplitGemm(ctypes.Structure):
    _fields_ = [("a_hi", c_vp), ("a_lo", c_vp), ("a_rows", c_i64), ("lda", c_i64), ("b_hi", c_vp), ("b_lo", c_vp),
                ("b_rows", c_i64), ("ldb", c_i64), ("k_alloc", c_i64), ("mode", c_i32), ("scale", ctypes.c_float),
                ("s_acc", ctypes.c_float), ("s_vec", ctypes.c_float), ("out_hi", c_vp), ("out_lo", c_vp),
                ("ld_h", c_i64), ("out", c_vp), ("ld_o", c_i64), ("M", c_i64), ("N", c_i64), ("rowv", c_vp),
                ("colv", c_vp), ("abort_flag", c_vp), ("timeout_ms", c_i32), ("addend", c_vp), ("ld_add", c_i64),
                ("s_add", ctypes.c_float), ("batch", c_i64), ("o_bstride", c_i64), ("rowv_bstride", c_i64),
                ("colv_bstride", c_i64), ("addend_bstride", c_i64)]


class OtgBaryProblem(ctypes.Structure):
    _fields_ = [("dtype", c_i32), ("method", c_i32), ("M", c_vp), ("dim", c_i64), ("ldm", c_i64), ("A", c_vp),
                ("n_hists", c_i32), ("max_iter", c_i32), ("weights", c_vp), ("reg", c_dbl), ("stop_thr", c_dbl),
                ("out_bar", c_vp), ("err_hist", ctypes.POINTER(c_dbl)), ("hist_cap", c_i32),
                ("info", ctypes.POINTER(c_i32)), ("workspace", c_vp), ("workspace_bytes", c_sz)]


class OtgOnlineProblem(ctypes.Structure):
    _fields_ = [("X", c_vp), ("Y", c_vp), ("n", c_i64), ("m", c_i64), ("d", c_i32), ("max_iter", c_i32),
                ("a", c_vp), ("b", c_vp), ("warm_f", c_vp), ("warm_g", c_vp), ("reg", c_dbl), ("stop_thr", c_dbl),
                ("scale_x", ctypes.c_float), ("scale_y", ctypes.c_float), ("out_f", c_vp), ("out_g", c_vp),
                ("err_hist", ctypes.POINTER(c_dbl)), ("hist_cap", c_i32), ("info", ctypes.POINTER(c_i32)),
                ("workspace", c_vp), ("workspace_bytes", c_sz), ("timeout_ms", c_i32),
                ("sum_window_log2", ctypes.c_float)]


# name -> (restype, argtypes)
SIGNATURES = {
    "otg_abi_layout": (ctypes.c_int, [ctypes.c_char_p, ctypes.POINTER(c_i64), c_i32]),
    "otg_dense_workspace_bytes": (c_sz, [ctypes.c_int, c_i64, c_i64, ctypes.c_int, ctypes.c_int]),
    "otg_dense_info_offset": (c_sz, [ctypes.c_int, c_i64, c_i64, ctypes.c_int, ctypes.c_int]),
    "otg_sinkhorn_dense": (ctypes.c_int, [ctypes.POINTER(OtgDenseProblem), c_vp, c_vp]),
    "otg_dense_plan": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp,
                                      c_dbl, c_vp, c_i64, c_vp, c_vp]),
    "otg_barycenter_workspace_bytes": (c_sz, [ctypes.c_int, ctypes.c_int, c_i64, c_i32]),
    "otg_barycenter": (ctypes.c_int, [ctypes.POINTER(OtgBaryProblem), c_vp]),
    "otg_transpose_batched": (ctypes.c_int, [ctypes.c_int, c_vp, c_i64, c_i64, c_i64, c_i64, c_i64, c_vp, c_i64,
                                             c_i64, c_vp]),
    "otg_lazy_loss": (ctypes.c_int, [ctypes.c_int, c_vp, c_vp, c_i64, c_i64, c_i32, c_vp, c_vp, c_dbl, c_vp, c_vp]),
    "otg_multi_tail_config": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32),
                                              ctypes.POINTER(c_i64), ctypes.POINTER(c_i32)]),
    "otg_gibbs_kernel": (ctypes.c_int, [ctypes.c_int, c_vp, c_i64, c_i64, c_i64, c_dbl, c_vp, c_i64, c_vp]),
    "otg_dense_marginals": (ctypes.c_int, [ctypes.c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_dbl, c_vp, c_vp,
                                           c_vp]),
    "otg_greenkhorn_workspace_bytes": (c_sz, [ctypes.c_int, c_i64, c_i64]),
    "otg_greenkhorn": (ctypes.c_int, [ctypes.c_int, c_vp, c_i64, c_i64, c_i64, c_vp, c_vp, c_dbl, c_vp, c_vp, c_i32,
                                      c_dbl, c_vp, c_i64, c_vp, c_vp, c_vp, c_vp, c_sz, c_vp]),
    "otg_sinkhorn_dense_noalloc":(ctypes.c_int, [ctypes.POINTER(OtgDenseProblem), c_vp, c_vp, c_vp]),
    "otg_batch_limits": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(c_i32), ctypes.POINTER(c_i32),
                                        ctypes.POINTER(c_i32)]),
    "otg_sinkhorn_batched": (ctypes.c_int, [ctypes.POINTER(OtgBatchProblem), c_vp]),
    "otg_multi_workspace_bytes": (c_sz, [ctypes.c_int, c_i32, c_i64, c_i64, c_i64]),
    "otg_sinkhorn_multi": (ctypes.c_int, [ctypes.POINTER(OtgMultiProblem), c_vp]),
    "otg_multi_anderson_bytes": (c_sz, [ctypes.c_int, c_i32, c_i64, c_i32]),
    "otg_pairs_workspace_bytes": (c_sz, [c_i32, c_i64, c_i64, c_i32, c_i32]),
    "otg_pairs_max_cost": (ctypes.c_int, [ctypes.POINTER(OtgPairsProblem), c_vp, c_vp]),
    "otg_sinkhorn_pairs": (ctypes.c_int, [ctypes.POINTER(OtgPairsProblem), c_vp]),
    "otg_online_workspace_bytes": (c_sz, [c_i64, c_i64, c_i32]),
    "otg_sinkhorn_online": (ctypes.c_int, [ctypes.POINTER(OtgOnlineProblem), c_vp]),
    "otg_batched_sqdist": (ctypes.c_int, [ctypes.POINTER(OtgCostTable), c_i32, c_vp]),
    "otg_batched_plan": (ctypes.c_int, [ctypes.POINTER(OtgPlanTable), c_i32, c_vp]),
    "otg_nearest_mass": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_i64, c_i64, c_vp, c_vp]),
    "otg_mlp_encode_pool": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp,
                                            c_vp]),
    "otg_mlp_head": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i32, c_i32, c_i32, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp,
                                     c_vp, c_vp, c_vp]),
    "otg_softmin_points": (ctypes.c_int, [c_vp, c_vp, c_i32, c_i32, c_i32, c_i32, c_i64, c_i64, c_vp, c_vp,
                                           ctypes.c_float, c_vp, c_vp, c_i32, c_vp, c_vp, c_vp]),
    "otg_softmin_features": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_vp, c_i32, c_i32,
                                            c_i32, c_vp, c_vp, c_vp]),
    "otg_gemm_f32": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, ctypes.c_float, c_vp, c_i64,
                                    c_vp, c_i64, ctypes.c_float, c_vp, c_i64, c_vp, ctypes.c_int, c_vp]),
    "otg_gemm_f64": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, c_dbl, c_vp, c_i64, c_vp, c_i64,
                                    c_dbl, c_vp, c_i64, c_vp]),
    "otg_gemm_batched": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_i64, c_i64, c_i64, c_dbl, c_vp,
                                        c_i64, c_i64, c_vp, c_i64, c_i64, c_dbl, c_vp, c_i64, c_i64, c_i64, c_vp]),
    "otg_split_half": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, ctypes.c_float, ctypes.c_int, c_vp, c_vp, c_i64,
                                      c_vp]),
    "otg_gemm_split3": (ctypes.c_int, [ctypes.POINTER(OtgSplitGemm), c_vp]),
    "otg_split_half_batched": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_i64, ctypes.c_float, ctypes.c_int, c_vp,
                                              c_vp, c_i64, c_i64, c_i64, c_vp]),
    "otg_mlp_relu_bwd": (ctypes.c_int, [c_vp, c_vp, c_i64, c_vp]),
    "otg_mlp_colsum": (ctypes.c_int, [c_vp, c_i64, c_i64, c_vp, c_vp]),
    "otg_mlp_segment_mean": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, c_vp]),
    "otg_mlp_segment_mean_bwd": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_vp, ctypes.c_int, c_vp]),
    "otg_mlp_concat3": (ctypes.c_int, [c_vp, c_vp, c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp]),
    "otg_mlp_concat3_bwd": (ctypes.c_int, [c_vp, c_i64, c_i64, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "otg_mlp_centered_mse": (ctypes.c_int, [c_vp, c_vp, c_i64, c_i64, c_vp, c_vp, c_vp]),
    "otg_mlp_adamw": (ctypes.c_int, [c_vp, c_vp, c_vp, c_vp, c_i64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float, ctypes.c_int, c_vp]),
}

_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (and if needed build) the shared library; returns the ctypes handle."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError("pot_gb300 CUDA library not built: %s" % path)
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


LAUNCHES = [0]  # kernel-launching C-ABI calls (plus the tail kernel queued behind each batch solve)


def check(rc, what):
    LAUNCHES[0] += 1
    if rc != 0:
        raise RuntimeError("%s failed: %s (code %d)" % (what, _ERRORS.get(rc, "error"), rc))


def dtype_code(t):
    if t == torch.float32:
        return OTG_F32
    if t == torch.float64:
        return OTG_F64
    raise TypeError("pot_gb300 kernels take float32 or float64 tensors, got %s" % t)


def ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_handle(device=None):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
