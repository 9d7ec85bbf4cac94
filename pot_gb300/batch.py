"""Batched entropic OT on the GPU: drop-ins for ``ot.batch`` and a native
ragged-batch API.

``solve_batch`` / ``solve_sample_batch`` / ``bregman_log_projection_batch``
/ ``bregman_projection_batch`` follow PythonOT/POT ``ot/batch/_linear.py``
(:236-357, :360-435) and ``ot/batch/_utils.py`` (:46-162, :165-290): same
arguments, same returned fields, and the same stop rule: the whole batch
stops at the first check (every 10th iteration) whose LARGEST row-marginal
error is below ``tol`` (``_utils.py:152-157, :273-278``), so every problem
runs to that shared index, as in the reference.  ``per_problem=True`` (no
reference counterpart) lets every problem stop on its own error instead;
problems that converge early are then not iterated further.

``solve_ragged`` / ``solve_sample_ragged`` take problems of uneven sizes
directly (no zero-weight padding) and run them in one persistent launch
(``csrc/batched.cu``).
"""
import ctypes

import numpy as np
import torch

from . import _lib, tune
from ._arrays import Boundary, check_shape, shape_of
from .utils import OTResult


def _vw(dtype):
    return 4 if dtype == torch.float32 else 2


class RaggedLayout:
    """Packed device layout of B problems with uneven sizes.

    Problem p's cost block is rows[p] x ldm[p] elements starting at m_off[p]
    (ldm rounded up to 16 bytes; padded columns hold +inf); a/u slices start
    at r_off[p], b/v slices at c_off[p]."""

    def __init__(self, rows, cols, dtype, device):
        rows = np.asarray(rows, dtype=np.int64)
        cols = np.asarray(cols, dtype=np.int64)
        vw = _vw(dtype)
        ldm = (cols + vw - 1) // vw * vw
        sizes = rows * ldm
        m_off = np.concatenate([[0], np.cumsum(sizes)[:-1]])
        r_off = np.concatenate([[0], np.cumsum(rows)[:-1]])
        c_off = np.concatenate([[0], np.cumsum(cols)[:-1]])
        self.B = len(rows)
        self.rows_np, self.cols_np, self.ldm_np = rows, cols, ldm
        self.m_off_np, self.r_off_np, self.c_off_np = m_off, r_off, c_off
        self.total_m = int(sizes.sum())
        self.total_r = int(rows.sum())
        self.total_c = int(cols.sum())
        self.dtype, self.device = dtype, device
        dev = device
        self.rows = torch.tensor(rows, dtype=torch.int32, device=dev)
        self.cols = torch.tensor(cols, dtype=torch.int32, device=dev)
        self.ldm = torch.tensor(ldm, dtype=torch.int32, device=dev)
        self.m_off = torch.tensor(m_off, dtype=torch.int64, device=dev)
        self.r_off = torch.tensor(r_off, dtype=torch.int64, device=dev)
        self.c_off = torch.tensor(c_off, dtype=torch.int64, device=dev)
        order = np.argsort(-(rows * cols), kind="stable").astype(np.int32)  # largest work first
        self.order = torch.tensor(order, dtype=torch.int32, device=dev)

    def block(self, M_packed, p):
        o = int(self.m_off_np[p])
        n, ld, m = int(self.rows_np[p]), int(self.ldm_np[p]), int(self.cols_np[p])
        return M_packed[o:o + n * ld].view(n, ld)[:, :m]

    def fits_kernel(self):
        lib = _lib.load()
        mr, mc, rb = _lib.c_i32(), _lib.c_i32(), _lib.c_i32()
        lib.otg_batch_limits(_lib.dtype_code(self.dtype), ctypes.byref(mr), ctypes.byref(mc), ctypes.byref(rb))
        es = 4 if self.dtype == torch.float32 else 8
        return (self.rows_np.max() <= mr.value and self.cols_np.max() <= mc.value
                and (self.ldm_np * es).max() <= rb.value)


def pack_dense(layout, Ms):
    """Pack a list of (n_p, m_p) device tensors (or a (B, n, m) tensor) into
    the layout's buffer, padding columns with +inf."""
    buf = torch.empty(layout.total_m, dtype=layout.dtype, device=layout.device)
    for p in range(layout.B):
        n, ld, m = int(layout.rows_np[p]), int(layout.ldm_np[p]), int(layout.cols_np[p])
        blk = buf[int(layout.m_off_np[p]):int(layout.m_off_np[p]) + n * ld].view(n, ld)
        blk[:, :m].copy_(Ms[p])
        if ld > m:
            blk[:, m:].fill_(float("inf"))
    return buf


def run_batched(layout, M_packed, a_packed, b_packed, reg, method, max_iter, tol, u_first,
                warm_u=None, warm_v=None, grid=0, timeout_ms=0):
    """One persistent launch over the whole table.  Returns (u, v, status,
    niter, err) as device tensors (u, v packed like a, b)."""
    lib = _lib.load()
    dev, dt = layout.device, layout.dtype
    B = layout.B
    if not layout.fits_kernel():
        raise ValueError("pot_gb300 batched kernel: a problem exceeds the per-CTA size limits "
                         "(otg_batch_limits); solve it with the dense single-problem path")
    reg_t = torch.as_tensor(reg, dtype=torch.float64, device=dev).reshape(-1)
    if reg_t.numel() == 1:
        reg_t = reg_t.expand(B).contiguous()
    out_u = torch.empty(layout.total_r, dtype=dt, device=dev)
    out_v = torch.empty(layout.total_c, dtype=dt, device=dev)
    status = torch.empty(B, dtype=torch.int32, device=dev)
    niter = torch.empty(B, dtype=torch.int32, device=dev)
    err = torch.empty(B, dtype=torch.float64, device=dev)
    queue = torch.zeros(2, dtype=torch.int32, device=dev)
    q = _lib.OtgBatchProblem(
        dtype=_lib.dtype_code(dt), method=method, M=M_packed.data_ptr(), m_off=layout.m_off.data_ptr(),
        rows=layout.rows.data_ptr(), cols=layout.cols.data_ptr(), ldm=layout.ldm.data_ptr(),
        r_off=layout.r_off.data_ptr(), c_off=layout.c_off.data_ptr(), a=a_packed.data_ptr(),
        b=b_packed.data_ptr(), warm_u=warm_u.data_ptr() if warm_u is not None else None,
        warm_v=warm_v.data_ptr() if warm_v is not None else None, reg=reg_t.data_ptr(),
        order=layout.order.data_ptr(), nprob=B, max_iter=int(max_iter), stop_thr=float(tol),
        u_first=int(u_first), grid=int(grid), out_u=out_u.data_ptr(), out_v=out_v.data_ptr(),
        status=status.data_ptr(), niter=niter.data_ptr(), err=err.data_ptr(), queue=queue.data_ptr(),
        timeout_ms=int(timeout_ms))
    _lib.check(lib.otg_sinkhorn_batched(ctypes.byref(q), _lib.stream_handle(dev)), "otg_sinkhorn_batched")
    return out_u, out_v, status, niter, err, reg_t


def multi_tail_config(dtype=torch.float32):
    """(CTAs per cluster, clusters resident at once, tile bytes per CTA, CUDA
    error of the configuration query) of the batch kernel's tail handoff on
    the current device; 0 CTAs means no handoff."""
    lib = _lib.load()
    cl, mx, err = _lib.c_i32(), _lib.c_i32(), _lib.c_i32()
    tile = _lib.c_i64()
    _lib.check(lib.otg_multi_tail_config(_lib.dtype_code(dtype), ctypes.byref(cl), ctypes.byref(mx),
                                         ctypes.byref(tile), ctypes.byref(err)), "otg_multi_tail_config")
    return cl.value, mx.value, tile.value, err.value


_TAIL_ON = {}


def _tail_enabled(dtype):
    if dtype not in _TAIL_ON:
        _TAIL_ON[dtype] = multi_tail_config(dtype)[0] > 0
    return _TAIL_ON[dtype]


def run_multi(layout, M_packed, a_packed, b_packed, reg, max_iter, tol, warm_u=None, grid=0, timeout_ms=0,
              events=None, omega=1.0, check_period=10, schedule=None, tail_problems=0, info=None, joint=False,
              scaling=False, anderson=0):
    """Work-balanced persistent launch (csrc/multi.cu) in the sinkhorn_log
    order (v first, column-marginal test).  Returns (u, v, status, niter,
    err, reg).  ``joint`` stops the whole batch together on the largest
    error (ot.batch's rule); otherwise every problem stops on its own.
    ``scaling`` runs the scaling form (u, v are then scalings, not natural
    logs).  ``anderson`` > 0 mixes the v updates over that many iterates
    (Anderson acceleration; u stays the exact row update of the v in use).
    ``omega != 1`` over-relaxes the potential updates and
    ``check_period`` other than 10 moves the stop tests (no reference
    counterpart for either; the stop criterion is unchanged).  ``schedule``
    (a ``tune.Schedule``) divides the work; by default the autotuner's cached
    choice for this workload class, else the built-in one.  ``tail_problems``
    bounds the cluster tail handoff (0: default, negative: off); with a dict
    ``info`` the call synchronises and reports the handoff iteration (-1:
    none)."""
    return _run_multi_once(layout, M_packed, a_packed, b_packed, reg, max_iter, tol, warm_u, grid, timeout_ms,
                           events, omega, check_period, schedule, tail_problems, info, joint, scaling, anderson)


def _run_multi_once(layout, M_packed, a_packed, b_packed, reg, max_iter, tol, warm_u=None, grid=0, timeout_ms=0,
                    events=None, omega=1.0, check_period=10, schedule=None, tail_problems=0, info=None,
                    joint=False, scaling=False, anderson=0):
    lib = _lib.load()
    if schedule is None:
        schedule = tune.lookup(layout) or tune.DEFAULT
    if grid == 0 and schedule.ctas_per_sm > 0:
        grid = schedule.ctas_per_sm * torch.cuda.get_device_properties(layout.device).multi_processor_count
    dev, dt = layout.device, layout.dtype
    B = layout.B
    reg_t = torch.as_tensor(reg, dtype=torch.float64, device=dev).reshape(-1)
    if reg_t.numel() == 1:
        reg_t = reg_t.expand(B).contiguous()
    if not hasattr(layout, "pc_off"):
        nsr_max = np.maximum(1, np.minimum(64, (layout.rows_np + 15) // 16)).astype(np.int32)
        sizes = nsr_max.astype(np.int64) * layout.cols_np
        layout.nsr_max_np = nsr_max
        layout.total_partials = int(sizes.sum())
        layout.nsr_max = torch.tensor(nsr_max, dtype=torch.int32, device=dev)
        layout.pc_off = torch.tensor(np.concatenate([[0], np.cumsum(sizes)[:-1]]), dtype=torch.int64, device=dev)
    dcode = _lib.dtype_code(dt)
    wsb = lib.otg_multi_workspace_bytes(dcode, B, layout.total_r, layout.total_c, layout.total_partials)
    ws = torch.empty(wsb, dtype=torch.uint8, device=dev)
    out_u = torch.empty(layout.total_r, dtype=dt, device=dev)
    out_v = torch.empty(layout.total_c, dtype=dt, device=dev)
    status = torch.empty(B, dtype=torch.int32, device=dev)
    niter = torch.empty(B, dtype=torch.int32, device=dev)
    err = torch.empty(B, dtype=torch.float64, device=dev)
    awb = lib.otg_multi_anderson_bytes(dcode, B, layout.total_c, int(anderson)) if anderson else 0
    aws = torch.empty(max(awb, 1), dtype=torch.uint8, device=dev)
    q = _lib.OtgMultiProblem(
        dtype=dcode, nprob=B, M=M_packed.data_ptr(), m_off=layout.m_off.data_ptr(), rows=layout.rows.data_ptr(),
        cols=layout.cols.data_ptr(), ldm=layout.ldm.data_ptr(), r_off=layout.r_off.data_ptr(),
        c_off=layout.c_off.data_ptr(), a=a_packed.data_ptr(), b=b_packed.data_ptr(),
        warm_u=warm_u.data_ptr() if warm_u is not None else None, reg=reg_t.data_ptr(), max_iter=int(max_iter),
        grid=int(grid), stop_thr=float(tol), nsr_max=layout.nsr_max.data_ptr(), pc_off=layout.pc_off.data_ptr(),
        total_rows=layout.total_r, total_cols=layout.total_c, total_partials=layout.total_partials,
        out_u=out_u.data_ptr(), out_v=out_v.data_ptr(), status=status.data_ptr(), niter=niter.data_ptr(),
        err=err.data_ptr(), workspace=ws.data_ptr(), workspace_bytes=wsb, timeout_ms=int(timeout_ms),
        omega=float(omega), check_period=int(check_period), units_per_warp=int(schedule.units_per_warp),
        split_cap_fill=int(schedule.cap_fill), split_cap_tail=int(schedule.cap_tail),
        tail_problems=int(tail_problems), joint_stop=int(bool(joint)), scaling=int(bool(scaling)),
        anderson_depth=int(anderson), anderson_ws=aws.data_ptr() if awb else None, anderson_ws_bytes=awb)
    if events is not None:
        events[0].record()
    _lib.check(lib.otg_sinkhorn_multi(ctypes.byref(q), _lib.stream_handle(dev)), "otg_sinkhorn_multi")
    if (not joint and not scaling and not anderson
            and (tail_problems > 0 or (tail_problems == 0 and dt == torch.float32)) and _tail_enabled(dt)):
        _lib.LAUNCHES[0] += 1  # the tail kernel launched behind the batch kernel
    if events is not None:
        events[1].record()
    if info is not None:
        # control block: the last 256 bytes of the workspace; [3] handoff iteration, [5] handed off
        ctl = ws[wsb - 256:wsb - 256 + 32].cpu().numpy().view(np.int32)
        info["handoff_ii"] = int(ctl[3]) if ctl[5] else -1
        info["handoff_problems"] = int(ctl[0]) if ctl[5] else 0
    return out_u, out_v, status, niter, err, reg_t


def batched_plan(layout, M_packed, u, v, a_packed, b_packed, reg_t, method, kl=False, want_plan=True):
    """Plans (packed like M) and per-problem (value_linear, reg term, mass)."""
    lib = _lib.load()
    dev = layout.device
    P = torch.empty_like(M_packed) if want_plan else None
    vals = torch.empty(3 * layout.B, dtype=torch.float64, device=dev)
    reg_t = reg_t.to(torch.float64).contiguous()  # the plan table reads float64 regularisations
    t = _lib.OtgPlanTable(dtype=_lib.dtype_code(layout.dtype), method=method, nprob=layout.B, kl=int(kl),
                          M=M_packed.data_ptr(), m_off=layout.m_off.data_ptr(), rows=layout.rows.data_ptr(),
                          cols=layout.cols.data_ptr(), ldm=layout.ldm.data_ptr(), r_off=layout.r_off.data_ptr(),
                          c_off=layout.c_off.data_ptr(), u=u.data_ptr(), v=v.data_ptr(), a=a_packed.data_ptr(),
                          b=b_packed.data_ptr(), reg=reg_t.data_ptr(), P=P.data_ptr() if P is not None else None,
                          out_vals=vals.data_ptr())
    _lib.check(lib.otg_batched_plan(ctypes.byref(t), int(layout.rows_np.max()), _lib.stream_handle(dev)),
               "otg_batched_plan")
    return P, vals.view(layout.B, 3)


def _fixed_dim(dims):
    """The shared point dimension when it has a register-tiled kernel, else 0."""
    d = np.asarray(dims)
    return int(d[0]) if d.size and (d == d[0]).all() and int(d[0]) in (2, 3, 8, 16) else 0


def batched_sqdist(layout, X_packed, Y_packed, x_off, y_off, dims, want_max=False):
    """Cost blocks sum_k (x_ik - y_jk)^2 for every problem of the layout."""
    lib = _lib.load()
    dev = layout.device
    M = torch.empty(layout.total_m, dtype=layout.dtype, device=dev)
    mx = torch.empty(layout.B, dtype=layout.dtype, device=dev) if want_max else None
    dims_t = torch.as_tensor(np.asarray(dims, dtype=np.int32), device=dev)
    xo = torch.as_tensor(np.asarray(x_off, dtype=np.int64), device=dev)
    yo = torch.as_tensor(np.asarray(y_off, dtype=np.int64), device=dev)
    t = _lib.OtgCostTable(dtype=_lib.dtype_code(layout.dtype), nprob=layout.B, X=X_packed.data_ptr(),
                          Y=Y_packed.data_ptr(), x_off=xo.data_ptr(), y_off=yo.data_ptr(),
                          rows=layout.rows.data_ptr(), cols=layout.cols.data_ptr(), dim=dims_t.data_ptr(),
                          max_dim=int(np.max(dims)), M=M.data_ptr(), m_off=layout.m_off.data_ptr(),
                          ldm=layout.ldm.data_ptr(), max_out=mx.data_ptr() if mx is not None else None,
                          fixed_dim=_fixed_dim(dims))
    _lib.check(lib.otg_batched_sqdist(ctypes.byref(t), int(layout.rows_np.max()), _lib.stream_handle(dev)),
               "otg_batched_sqdist")
    return M, mx


# ---------------------------------------------------------------------------
# ot.batch drop-ins
# ---------------------------------------------------------------------------
def _uniform_batch(M):
    layout = RaggedLayout([M.shape[1]] * M.shape[0], [M.shape[2]] * M.shape[0], M.dtype, M.device)
    if layout.ldm_np[0] == M.shape[2] and M.is_contiguous() and M.data_ptr() % 16 == 0:
        Mp = M.reshape(-1)
    else:
        Mp = pack_dense(layout, M)
    return layout, Mp


def _unpack_rows(layout, packed, width_np, off_np):
    B = layout.B
    w = int(width_np[0])
    return packed.view(B, w)


_TRANSPOSE_CHUNK = 65535  # problems per transpose launch (its grid's z extent)


def _transposed(layout, Mp):
    """The layout and packed cost blocks of the transposed problems (one
    transpose pass, otg_transpose_batched, in launches of at most 65535
    problems)."""
    lib = _lib.load()
    B, n, m = layout.B, int(layout.rows_np[0]), int(layout.cols_np[0])
    lt = RaggedLayout([m] * B, [n] * B, layout.dtype, layout.device)
    ld, ldt = int(layout.ldm_np[0]), int(lt.ldm_np[0])
    Mt = torch.empty(lt.total_m, dtype=layout.dtype, device=layout.device)
    for z0 in range(0, B, _TRANSPOSE_CHUNK):
        nb = min(_TRANSPOSE_CHUNK, B - z0)
        _lib.check(lib.otg_transpose_batched(_lib.dtype_code(layout.dtype), _lib.ptr(Mp[z0 * n * ld:]), nb, n, m,
                                             ld, n * ld, _lib.ptr(Mt[z0 * m * ldt:]), ldt, m * ldt,
                                             _lib.stream_handle(layout.device)), "otg_transpose_batched")
    return lt, Mt


def _solve_uniform(Md, a, b, reg, method, max_iter, tol, kl, per_problem=False):
    """Uniform batch in the ot.batch order (u first, row-marginal check every
    10th iteration): the sinkhorn_log (or scaling) order of the transposed
    problems (a and b swapped) on the work-balanced kernel.  The whole batch
    stops on its largest error unless ``per_problem``."""
    layout, Mp = _uniform_batch(Md)
    ap, bp = a.reshape(-1).contiguous(), b.reshape(-1).contiguous()
    lt, Mt = _transposed(layout, Mp)
    vt, ut, status, niter, err, reg_t = run_multi(lt, Mt, bp, ap, reg, max_iter, tol, joint=not per_problem,
                                                  scaling=method == _lib.OTG_METHOD_KNOPP)
    u, v = ut, vt
    del Mt
    P, vals = batched_plan(layout, Mp, u, v, ap, bp, reg_t, method, kl=kl)
    B, n, m = Md.shape
    ld = int(layout.ldm_np[0])
    T = P.view(B, n, ld)[:, :, :m]
    if ld != m:
        T = T.contiguous()
    return T, u.view(B, n), v.view(B, m), vals, niter, status


def _batch_dims(K, a, b, name="M"):
    """(B, n, m) of a batch cost (or kernel) and the check of its weights:
    each (B, n) / (B, m), or one (n,) / (m,) histogram for the whole batch
    (the reference's arithmetic broadcasts it); on the caller's arrays,
    before any device work."""
    sK = shape_of(K)
    if len(sK) != 3:
        raise ValueError("%s must be a (B, n, m) batch, got shape %s" % (name, sK))
    B, n, m = sK
    check_shape("a", a, [(B, n), (n,)])
    check_shape("b", b, [(B, m), (m,)])
    return B, n, m


def _per_problem(w, B, k):
    """(B, k) device weights from (B, k) or a broadcast (k,) histogram."""
    return w.expand(B, k).contiguous() if w.dim() == 1 else w.contiguous()


def solve_batch(M, reg, a=None, b=None, max_iter=1000, tol=1e-5, solver="log_sinkhorn", reg_type="entropy",
                grad="envelope", per_problem=False):
    """GPU ``ot.batch.solve_batch`` (``ot/batch/_linear.py:236``).
    ``per_problem`` (no reference counterpart): every problem stops on its
    own error instead of the batch's largest."""
    if solver not in ("log_sinkhorn", "sinkhorn"):
        raise ValueError(f"Unknown solver: {solver}")
    if reg_type.lower() not in ("entropy", "kl"):
        raise ValueError(f"Unknown reg_type: {reg_type}")
    _batch_dims(M, a, b)
    bd = Boundary(M, a, b)
    Md = bd.to_dev(M)
    B, n, m = Md.shape
    ad = torch.full((B, n), 1.0 / n, dtype=Md.dtype, device=Md.device) if a is None else \
        _per_problem(bd.to_dev(a, Md.dtype), B, n)
    bv = torch.full((B, m), 1.0 / m, dtype=Md.dtype, device=Md.device) if b is None else \
        _per_problem(bd.to_dev(b, Md.dtype), B, m)
    method = _lib.OTG_METHOD_LOG if solver == "log_sinkhorn" else _lib.OTG_METHOD_KNOPP
    T, u, v, vals, niter, _ = _solve_uniform(Md, ad, bv, float(reg), method, max_iter, tol,
                                             reg_type.lower() == "kl", per_problem)
    value_linear = vals[:, 0].to(Md.dtype)
    value = (vals[:, 0] + float(reg) * vals[:, 1]).to(Md.dtype)
    log = {"n_iter": int(niter.max().item())}
    return OTResult(value=bd.out(value), value_linear=bd.out(value_linear),
                    potentials=(bd.out(u), bd.out(v)), plan=bd.out(T), log=log)


def dist_batch(X1, X2=None, metric="sqeuclidean", p=2, nx=None):
    """GPU ``ot.batch.dist_batch`` (``ot/batch/_linear.py:178``) for the
    'sqeuclidean' and 'euclidean' metrics."""
    metric = metric.lower()
    if metric not in ("sqeuclidean", "euclidean"):
        raise NotImplementedError("pot_gb300 dist_batch: metric '%s' is not on the GPU path" % metric)
    bd = Boundary(X1, X2)
    X = bd.to_dev(X1)
    Y = X if X2 is None else bd.to_dev(X2, X.dtype)
    B, n, d = X.shape
    m = Y.shape[1]
    layout = RaggedLayout([n] * B, [m] * B, X.dtype, X.device)
    Mp, _ = batched_sqdist(layout, X.reshape(-1).contiguous(), Y.reshape(-1).contiguous(),
                           np.arange(B) * n * d, np.arange(B) * m * d, [d] * B)
    ld = int(layout.ldm_np[0])
    M = Mp.view(B, n, ld)[:, :, :m]
    if metric == "euclidean":
        M = torch.sqrt(M)
    return bd.out(M.contiguous())


def solve_sample_batch(X_a, X_b, reg, a=None, b=None, metric="sqeuclidean", p=2, max_iter=1000, tol=1e-5,
                       solver="log_sinkhorn", reg_type="entropy", grad="envelope", per_problem=False):
    """GPU ``ot.batch.solve_sample_batch`` (``ot/batch/_linear.py:360``)."""
    bd = Boundary(X_a, X_b, a, b)
    M = dist_batch(bd.to_dev(X_a), bd.to_dev(X_b), metric=metric, p=p)
    res = solve_batch(M, reg, a=None if a is None else bd.to_dev(a, M.dtype),
                      b=None if b is None else bd.to_dev(b, M.dtype), max_iter=max_iter, tol=tol, solver=solver,
                      reg_type=reg_type, grad=grad, per_problem=per_problem)
    return OTResult(value=bd.out(res.value), value_linear=bd.out(res.value_linear),
                    potentials=tuple(bd.out(x) for x in res.potentials), plan=bd.out(res.plan), log=res.log)


def bregman_log_projection_batch(K, a=None, b=None, nx=None, max_iter=10000, tol=1e-5, grad="detach",
                                 per_problem=False):
    """GPU ``ot.batch.bregman_log_projection_batch`` (``_utils.py:165``):
    ``K = -M/reg`` is solved as cost ``-K`` with unit regularisation."""
    _batch_dims(K, a, b, "K")
    bd = Boundary(K, a, b)
    Kd = bd.to_dev(K)
    B, n, m = Kd.shape
    ad = torch.ones((B, n), dtype=Kd.dtype, device=Kd.device) / n if a is None else \
        _per_problem(bd.to_dev(a, Kd.dtype), B, n)
    bv = torch.ones((B, m), dtype=Kd.dtype, device=Kd.device) / m if b is None else \
        _per_problem(bd.to_dev(b, Kd.dtype), B, m)
    T, u, v, _, niter, _ = _solve_uniform((-Kd).contiguous(), ad, bv, 1.0, _lib.OTG_METHOD_LOG, max_iter, tol, False,
                                          per_problem)
    log_T = Kd + u[:, :, None] + v[:, None, :]
    return {"T": bd.out(T), "log_T": bd.out(log_T), "n_iters": int(niter.max().item()),
            "potentials": (bd.out(u), bd.out(v))}


def bregman_projection_batch(K, a=None, b=None, nx=None, max_iter=10000, tol=1e-5, grad="detach",
                             per_problem=False):
    """GPU ``ot.batch.bregman_projection_batch`` (``_utils.py:46``): the
    affinity ``K`` is solved as cost ``-log K`` with unit regularisation."""
    _batch_dims(K, a, b, "K")
    bd = Boundary(K, a, b)
    Kd = bd.to_dev(K)
    B, n, m = Kd.shape
    ad = torch.ones((B, n), dtype=Kd.dtype, device=Kd.device) / n if a is None else \
        _per_problem(bd.to_dev(a, Kd.dtype), B, n)
    bv = torch.ones((B, m), dtype=Kd.dtype, device=Kd.device) / m if b is None else \
        _per_problem(bd.to_dev(b, Kd.dtype), B, m)
    T, f, g, _, niter, _ = _solve_uniform((-torch.log(Kd)).contiguous(), ad, bv, 1.0, _lib.OTG_METHOD_KNOPP,
                                          max_iter, tol, False, per_problem)
    return {"T": bd.out(T), "n_iters": int(niter.max().item()), "potentials": (bd.out(f), bd.out(g))}


# ---------------------------------------------------------------------------
# Native ragged API
# ---------------------------------------------------------------------------
class RaggedResult:
    """Per-problem results of a ragged solve (device tensors)."""

    def __init__(self, layout, u, v, status, niter, err, reg, M=None):
        self.layout, self.u, self.v = layout, u, v
        self.status, self.niter, self.err, self.reg, self.M = status, niter, err, reg, M

    def potentials(self, p):
        L = self.layout
        return (self.u[int(L.r_off_np[p]):int(L.r_off_np[p] + L.rows_np[p])],
                self.v[int(L.c_off_np[p]):int(L.c_off_np[p] + L.cols_np[p])])


def solve_sample_ragged(Xs, Ys, reg, as_=None, bs=None, reg_relative=False, max_iter=100000, tol=1e-6,
                        method="sinkhorn_log", warmstart=None, dtype=torch.float32, device=None, engine="multi",
                        autotune=False):
    """Entropic OT between B point-cloud pairs of uneven sizes and dims, in
    one persistent launch.  ``reg`` is a scalar or one value per problem; with
    ``reg_relative`` it multiplies each problem's largest cost.  Per problem
    the iteration order and stopping test are those of ``ot.sinkhorn(...,
    method='sinkhorn_log')`` (v first, column-marginal L2 error).  With
    ``autotune`` the launch schedule of this workload class is searched
    first if the tuner has none cached (``pot_gb300.tune``)."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    B = len(Xs)
    rows = [x.shape[0] for x in Xs]
    cols = [y.shape[0] for y in Ys]
    dims = [x.shape[1] for x in Xs]
    layout = RaggedLayout(rows, cols, dtype, device)
    X = torch.cat([torch.as_tensor(np.asarray(x), dtype=dtype).reshape(-1) for x in Xs]).to(device)
    Y = torch.cat([torch.as_tensor(np.asarray(y), dtype=dtype).reshape(-1) for y in Ys]).to(device)
    x_off = np.concatenate([[0], np.cumsum([r * d for r, d in zip(rows, dims)])[:-1]])
    y_off = np.concatenate([[0], np.cumsum([c * d for c, d in zip(cols, dims)])[:-1]])
    M, mx = batched_sqdist(layout, X, Y, x_off, y_off, dims, want_max=reg_relative)
    reg_t = torch.as_tensor(reg, dtype=torch.float64, device=device).reshape(-1)
    if reg_t.numel() == 1:
        reg_t = reg_t.expand(B).contiguous()
    if reg_relative:
        reg_t = reg_t * mx.double()
    ap = (torch.cat([torch.as_tensor(np.asarray(a), dtype=dtype) for a in as_]) if as_ is not None else
          torch.cat([torch.full((r,), 1.0 / r, dtype=dtype) for r in rows])).to(device)
    bp = (torch.cat([torch.as_tensor(np.asarray(b), dtype=dtype) for b in bs]) if bs is not None else
          torch.cat([torch.full((c,), 1.0 / c, dtype=dtype) for c in cols])).to(device)
    code = _lib.OTG_METHOD_LOG if method == "sinkhorn_log" else _lib.OTG_METHOD_KNOPP
    wu = wv = None
    if warmstart is not None:
        wu, wv = warmstart
    if engine == "multi" and code == _lib.OTG_METHOD_LOG:
        if autotune:
            tune.tune_multi(layout, M, ap, bp, reg_t)
        u, v, status, niter, err, reg_t = run_multi(layout, M, ap, bp, reg_t, max_iter, tol, warm_u=wu)
    else:
        u, v, status, niter, err, reg_t = run_batched(layout, M, ap, bp, reg_t, code, max_iter, tol, u_first=0,
                                                      warm_u=wu, warm_v=wv)
    return RaggedResult(layout, u, v, status, niter, err, reg_t, M)


# ---------------------------------------------------------------------------
# Equal-size cloud pairs with the cost rebuilt on the tensor cores
# ---------------------------------------------------------------------------
def _pairs_problem(X, Y, anderson=0):
    lib = _lib.load()
    P, n, d = X.shape
    m = Y.shape[1]
    wsb = lib.otg_pairs_workspace_bytes(P, n, m, d, int(anderson))
    ws = torch.empty(wsb, dtype=torch.uint8, device=X.device)
    q = _lib.OtgPairsProblem(X=X.data_ptr(), Y=Y.data_ptr(), npairs=P, d=d, n=n, m=m, anderson_depth=int(anderson),
                             workspace=ws.data_ptr(), workspace_bytes=wsb)
    return lib, q, ws


def pairs_max_cost(X, Y):
    """Largest squared distance max_ij |x_i - y_j|^2 of every pair of X
    (P, n, d) and Y (P, m, d), float32 device tensors: (P,) float64, from
    one max-only pass on the tensor cores (otg_pairs_max_cost)."""
    X, Y = X.float().contiguous(), Y.float().contiguous()
    lib, q, ws = _pairs_problem(X, Y)
    out = torch.empty(X.shape[0], dtype=torch.float64, device=X.device)
    _lib.check(lib.otg_pairs_max_cost(ctypes.byref(q), _lib.ptr(out), _lib.stream_handle(X.device)),
               "otg_pairs_max_cost")
    return out


def run_pairs(X, Y, reg, a=None, b=None, max_iter=100000, tol=1e-6, warm_u=None, check_period=10, anderson=0,
              timeout_ms=0, sum_window_log2=0.0):
    """Log-domain solves of P equal-size cloud pairs, X (P, n, d), Y (P, m, d)
    float32 on the device, squared-Euclidean cost never stored: every pass
    rebuilds cost tiles from the points on the tensor cores
    (otg_sinkhorn_pairs).  Per pair the iteration and stop test of
    ``run_multi`` (sinkhorn_log order, column-marginal L2 error every
    ``check_period`` iterations, each pair on its own; ``anderson`` > 0 mixes
    the v updates).  ``reg``: (P,) absolute values.  ``sum_window_log2`` > 0
    narrows the acceptance window of the shifted sums (rows outside it go
    through the fix-up pass; the results are the same).  Returns (u, v,
    status, niter, err) with u (P, n), v (P, m) natural-log potentials."""
    X, Y = X.float().contiguous(), Y.float().contiguous()
    P, n, _ = X.shape
    m = Y.shape[1]
    dev = X.device
    lib, q, ws = _pairs_problem(X, Y, anderson)
    reg_t = torch.as_tensor(reg, dtype=torch.float64, device=dev).reshape(-1)
    if reg_t.numel() == 1:
        reg_t = reg_t.expand(P).contiguous()
    a = torch.full((P, n), 1.0 / n, dtype=torch.float32, device=dev) if a is None else a.float().contiguous()
    b = torch.full((P, m), 1.0 / m, dtype=torch.float32, device=dev) if b is None else b.float().contiguous()
    u = torch.empty((P, n), dtype=torch.float32, device=dev)
    v = torch.empty((P, m), dtype=torch.float32, device=dev)
    status = torch.empty(P, dtype=torch.int32, device=dev)
    niter = torch.empty(P, dtype=torch.int32, device=dev)
    err = torch.empty(P, dtype=torch.float64, device=dev)
    wu = None if warm_u is None else warm_u.float().reshape(P, n).contiguous()
    q.a, q.b, q.reg = a.data_ptr(), b.data_ptr(), reg_t.data_ptr()
    q.warm_u = wu.data_ptr() if wu is not None else None
    q.max_iter, q.check_period, q.stop_thr, q.timeout_ms = int(max_iter), int(check_period), float(tol), int(timeout_ms)
    q.sum_window_log2 = float(sum_window_log2)
    q.out_u, q.out_v = u.data_ptr(), v.data_ptr()
    q.status, q.niter, q.err = status.data_ptr(), niter.data_ptr(), err.data_ptr()
    _lib.check(lib.otg_sinkhorn_pairs(ctypes.byref(q), _lib.stream_handle(dev)), "otg_sinkhorn_pairs")
    return u, v, status, niter, err


# ---------------------------------------------------------------------------
# Batched (fused) Gromov-Wasserstein
# ---------------------------------------------------------------------------
def _bgemm(A, B, ta, tb, out, alpha=1.0, beta=0.0):
    """out_z = alpha op(A_z) op(B_z) + beta out_z over a batch (csrc/mlp.cu)."""
    lib = _lib.load()
    Bz = A.shape[0]
    M = A.shape[2] if ta else A.shape[1]
    K = A.shape[1] if ta else A.shape[2]
    N = B.shape[1] if tb else B.shape[2]
    _lib.check(lib.otg_gemm_batched(_lib.dtype_code(A.dtype), int(ta), int(tb), M, N, K, float(alpha),
                                    _lib.ptr(A), A.shape[2], A.stride(0), _lib.ptr(B), B.shape[2], B.stride(0),
                                    float(beta), _lib.ptr(out), out.shape[2], out.stride(0), Bz,
                                    _lib.stream_handle(A.device)), "otg_gemm_batched")
    return out


class _BatchPlanes:
    """High/low half planes of a batch of equal-shape operands, each padded
    to whole 128 tiles and stacked (problem z from row z * rows)."""

    def __init__(self, B, rows, cols, device):
        self.B, self.rows, self.cols = B, -(-rows // 128) * 128, -(-cols // 128) * 128
        self.hi = torch.zeros(B * self.rows, self.cols, dtype=torch.float16, device=device)
        self.lo = torch.zeros_like(self.hi)

    def fill(self, X, scale=1.0, transpose=False):
        """planes of scale * X_z (or its transpose) for X of shape (B, r, c)."""
        lib = _lib.load()
        X = X.contiguous()
        _, r, c = X.shape
        _lib.check(lib.otg_split_half_batched(_lib.ptr(X), r, c, c, r * c, float(scale), int(transpose),
                                              _lib.ptr(self.hi), _lib.ptr(self.lo), self.cols, self.rows * self.cols,
                                              self.B, _lib.stream_handle(X.device)), "otg_split_half_batched")
        return self


class _BatchTensorProduct:
    """``out_z = s_acc hC1_z T_z hC2_z^T + s_vec (rowv_z,i + colv_z,j)
    [+ s_add addend_z]`` for a float32 batch of equal-shape problems: two
    tcgen05 split-GEMM launches per product over the whole batch (one grid
    z-slice per problem), the operands as stacked high/low half planes with
    exact power-of-two prescales (the batch's largest entries), fp32-grade
    products.  ``hC1^T T hC2`` (asymmetric costs) uses the transposed planes.
    Replaces the einsum chain of ``tensor_product_batch``
    (``ot/batch/_quadratic.py:535-572``)."""

    def __init__(self, hC1, hC2, qmax, tmax, transposed=False):
        from .gromov import pow2_scale
        self.B, self.n, self.m = hC1.shape[0], hC1.shape[1], hC2.shape[1]
        dev = hC1.device
        B, n, m = self.B, self.n, self.m
        self.lib = _lib.load()
        c1max = float(hC1.abs().max())
        self.s1 = pow2_scale(c1max)
        self.s2 = pow2_scale(float(hC2.abs().max()))
        self.sT = pow2_scale(tmax)
        # (hC1 T)_ij <= max|hC1| sum_k T_kj = max|hC1| q_j
        self.e1 = pow2_scale(self.s1 * c1max * qmax * self.sT)
        self.A1 = _BatchPlanes(B, n, n, dev).fill(hC1, self.s1)
        self.B2 = _BatchPlanes(B, m, m, dev).fill(hC2, self.s2)
        self.A1t = _BatchPlanes(B, n, n, dev).fill(hC1, self.s1, transpose=True) if transposed else None
        self.B2t = _BatchPlanes(B, m, m, dev).fill(hC2, self.s2, transpose=True) if transposed else None
        self.Tt = _BatchPlanes(B, m, n, dev)
        self.P1 = _BatchPlanes(B, n, m, dev)
        self.flag = torch.zeros(1, dtype=torch.int32, device=dev)

    def _gemm(self, A, Bp, k, **kw):
        g = _lib.OtgSplitGemm(a_hi=_lib.ptr(A.hi), a_lo=_lib.ptr(A.lo), a_rows=A.rows, lda=A.cols,
                              b_hi=_lib.ptr(Bp.hi), b_lo=_lib.ptr(Bp.lo), b_rows=Bp.rows, ldb=Bp.cols,
                              k_alloc=-(-k // 64) * 64, abort_flag=_lib.ptr(self.flag), timeout_ms=0,
                              batch=self.B, **kw)
        _lib.check(self.lib.otg_gemm_split3(ctypes.byref(g), _lib.stream_handle(self.flag.device)),
                   "otg_gemm_split3")

    def product(self, T, out, s_acc, s_vec, rowv, colv, addend=None, s_add=0.0, transposed=False):
        n, m = self.n, self.m
        A1, B2 = (self.A1t, self.B2t) if transposed else (self.A1, self.B2)
        self.Tt.fill(T, self.sT, transpose=True)
        # P1 = e1 (s1 hC1)(sT T) as planes; acc of the second GEMM = e1 s1 sT s2 (hC1 T hC2^T)
        self._gemm(A1, self.Tt, n, mode=0, scale=self.e1, out_hi=_lib.ptr(self.P1.hi),
                   out_lo=_lib.ptr(self.P1.lo), ld_h=self.P1.cols, M=n, N=m)
        rowv, colv = rowv.contiguous(), colv.contiguous()
        self._gemm(self.P1, B2, m, mode=1, scale=1.0, s_acc=s_acc / (self.s1 * self.sT * self.e1 * self.s2),
                   s_vec=s_vec, out=_lib.ptr(out), ld_o=m, M=n, N=m, rowv=_lib.ptr(rowv), colv=_lib.ptr(colv),
                   o_bstride=n * m, rowv_bstride=n, colv_bstride=m,
                   addend=_lib.ptr(addend) if addend is not None else None, ld_add=m if addend is not None else 0,
                   addend_bstride=n * m if addend is not None else 0, s_add=float(s_add))
        return out

    def check_abort(self):
        if int(self.flag.item()) != 0:
            raise RuntimeError("pot_gb300: a device-side wait of the tensor-core GEMM timed out")


def solve_gromov_batch(C1, C2, reg=1e-2, a=None, b=None, loss="sqeuclidean", symmetric=None, M=None, alpha=None,
                       T_init=None, max_iter=50, tol=1e-5, max_iter_inner=50, tol_inner=1e-5, grad="envelope",
                       logits=None, per_problem=False):
    """GPU ``ot.batch.solve_gromov_batch`` (``ot/batch/_quadratic.py:269-498``)
    for the squared loss and scalar costs: per outer step the tensor product
    ``constC - hC1 T hC2^T`` (batched GEMMs), ``Mk = (1 - alpha) M + 2 alpha
    L x T``, and the batched log projection of ``-Mk/reg + log T`` (the
    whole batch stopping on its largest inner error, as in the reference;
    ``per_problem=True``: every problem on its own).  The outer loop stops on
    the largest mean plan change (``:458-471``)."""
    if not isinstance(loss, str):
        raise ValueError(f"Unknown loss function: {loss}")
    if loss != "sqeuclidean":
        raise NotImplementedError("pot_gb300 solve_gromov_batch: loss '%s' is not on the GPU path" % loss)
    s1, s2 = shape_of(C1), shape_of(C2)
    if len(s1) == 3 and len(s2) == 3:
        if s1[1] != s1[2] or s2[1] != s2[2] or s1[0] != s2[0]:
            raise ValueError("C1 and C2 must be (B, n, n) and (B, m, m) batches, got %s and %s" % (s1, s2))
        check_shape("a", a, [(s1[0], s1[1]), (s1[1],)])
        check_shape("b", b, [(s1[0], s2[1]), (s2[1],)])
        check_shape("M", M, [(s1[0], s1[1], s2[1])])
        check_shape("T_init", T_init, [(s1[0], s1[1], s2[1])])
    bd = Boundary(C1, C2, a, b, M, T_init)
    C1d = bd.to_dev(C1)
    C2d = bd.to_dev(C2, C1d.dtype)
    if C1d.dim() != 3 or C2d.dim() != 3:
        raise NotImplementedError("pot_gb300 solve_gromov_batch: vector-valued (4-D) costs are not on the GPU path")
    dt, dev = C1d.dtype, C1d.device
    B, n, m = C1d.shape[0], C1d.shape[1], C2d.shape[1]
    ad = torch.ones((B, n), dtype=dt, device=dev) / n if a is None else _per_problem(bd.to_dev(a, dt), B, n)
    bv = torch.ones((B, m), dtype=dt, device=dev) / m if b is None else _per_problem(bd.to_dev(b, dt), B, m)
    tr = lambda X: X.transpose(1, 2).contiguous()  # noqa: E731
    if symmetric is None:
        symmetric = bool(torch.allclose(C1d, tr(C1d), atol=1e-10) and torch.allclose(C2d, tr(C2d), atol=1e-10))
    fC1, fC2 = C1d * C1d, C2d * C2d
    if not symmetric:
        fC1, fC2 = 0.5 * (fC1 + tr(fC1)), 0.5 * (fC2 + tr(fC2))
    hC1, hC2 = (2.0 * C1d).contiguous(), C2d.contiguous()
    hC1t, hC2t = (tr(hC1), tr(hC2)) if not symmetric else (None, None)
    if M is None and alpha is None:
        Md, alpha = torch.zeros((B, n, m), dtype=dt, device=dev), 1.0
    elif M is not None and alpha is None:
        raise ValueError("If M is provided, alpha must also be provided for Fused Gromov-Wasserstein problem")
    elif M is None and alpha is not None:
        raise ValueError("If alpha is provided, M must also be provided for Fused Gromov-Wasserstein problem")
    else:
        Md = bd.to_dev(M, dt).contiguous()
        if tuple(Md.shape) != (B, n, m):
            raise ValueError(f"Shape of M {tuple(Md.shape)} does not match the batch size {B} and dimensions {n}, {m}")
        if alpha < 0 or alpha > 1:
            raise ValueError("Alpha must be in [0, 1] for Fused Gromov-Wasserstein problem")

    def const_parts(p, q):
        return torch.einsum("bij,bj->bi", fC1, p), torch.einsum("bij,bj->bi", fC2, q)

    def const_of(p, q):
        r, c = const_parts(p, q)
        return r[:, :, None] + c[:, None, :]

    if T_init is None:
        const = torch.sqrt(ad.sum(1) * bv.sum(1))
        T = torch.einsum("bi,bj->bij", ad, bv) / const[:, None, None]
    else:
        T = bd.to_dev(T_init, dt).contiguous()

    if dt == torch.float32:
        # tensor cores: the fused products write s_acc dot + s_vec constC (+ addend) directly
        tp = _BatchTensorProduct(hC1, hC2, float(bv.max()), min(float(ad.max()), float(bv.max())),
                                 transposed=not symmetric)
        buf = torch.empty((B, n, m), dtype=dt, device=dev)

        def lin_minus_dot(T, s_dot, s_const, rowv, colv, addend=None, s_add=0.0):
            """s_dot * dot(T) + s_const * (rowv_i + colv_j) [+ s_add addend]"""
            Tc = T.contiguous()
            if symmetric:
                return tp.product(Tc, buf, s_dot, s_const, rowv, colv, addend, s_add)
            tp.product(Tc, buf, 0.5 * s_dot, s_const, rowv, colv, addend, s_add)
            return tp.product(Tc, buf, 0.5 * s_dot, 0.0, rowv, colv, buf, 1.0, transposed=True)

        rv0, cv0 = const_parts(ad, bv)
        has_lin = alpha != 1

        def cost_of(T):   # Mk = (1 - alpha) M + 2 alpha (constC - dot)
            return lin_minus_dot(T, -2.0 * alpha, 2.0 * alpha, rv0, cv0, Md if has_lin else None,
                                 (1 - alpha) if has_lin else 0.0)

        def quad_of(T):   # const_of(T marginals) - dot(T)
            r, c = const_parts(T.sum(2), T.sum(1))
            return lin_minus_dot(T, -1.0, 1.0, r, c)
    else:
        tmp = torch.empty((B, n, m), dtype=dt, device=dev)
        dotb = torch.empty((B, n, m), dtype=dt, device=dev)

        def dot(T):
            _bgemm(hC1, T, 0, 0, tmp)
            _bgemm(tmp, hC2, 0, 1, dotb)                 # hC1 T hC2^T
            if not symmetric:
                _bgemm(hC1t, T, 0, 0, tmp)
                _bgemm(tmp, hC2t, 0, 1, dotb, 0.5, 0.5)  # average with hC1^T T hC2
            return dotb

        constC = const_of(ad, bv)

        def cost_of(T):
            return (1 - alpha) * Md + 2 * alpha * (constC - dot(T))

        def quad_of(T):
            return const_of(T.sum(2), T.sum(1)) - dot(T)

    log_T = torch.log(T + 1e-15)
    it = 0
    u = v = None
    for it in range(max_iter):
        T_prev = T
        Mk = cost_of(T)
        K = -Mk / reg + log_T
        T, u, v, _, _, _ = _solve_uniform((-K).contiguous(), ad, bv, 1.0, _lib.OTG_METHOD_LOG, max_iter_inner,
                                          tol_inner, False, per_problem)
        log_T = K + u[:, :, None] + v[:, None, :]
        if float(torch.amax(torch.mean(torch.abs(T_prev - T), dim=(1, 2)))) < tol:
            break
    vl = (Md * T).sum((1, 2))
    vq = (quad_of(T) * T).sum((1, 2))
    if dt == torch.float32:
        tp.check_abort()
    return OTResult(value=bd.out((1 - alpha) * vl + alpha * vq), value_linear=bd.out((1 - alpha) * vl),
                    value_quad=bd.out(alpha * vq), plan=bd.out(T), potentials=(bd.out(u), bd.out(v)),
                    log={"n_iter": it})
