"""Benchmark of the entropic-OT hot path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl reference]

Prints ONE JSON line (rank 0).

Default workload ("warmstart"): learned warm start vs plain zero-initialised
log-domain Sinkhorn on batches of Gaussian-mixture cloud pairs (n = m = 2048
points in R^16, 1-6 isotropic components per cloud, uniform weights,
reg = 0.02 x max cost, marginal error 1e-6).  A step solves the whole batch:
cost blocks, (warm start,) and the persistent solve; `value` is the warm
arm's solves/s with the clouds resident in HBM, `plain` the zero-init arm's.
The cost blocks (16 MiB per pair) exceed L2 many times over.  `e2e` runs the
public entry point with host (numpy) clouds, copies included.

`--impl reference` times the reference's CPU algorithm (the float64 numpy
restatement of sinkhorn_log) on a bounded sample of the same workload, over
all host cores (one process per core).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

# ---------------------------------------------------------------------------
# replicas: under torchrun every rank solves its own batch on its own GPU (the
# pairs are independent, so nothing is exchanged on the data path); ranks only
# meet at barriers around the timed regions and to take the slowest time.
# ---------------------------------------------------------------------------
_WS = {"rank": 0, "world": 1, "local": 0}


def replica_setup(backend=None):
    """Join the process group when launched with WORLD_SIZE > 1 (nccl with
    GPUs, gloo without, unless `backend` says); returns (rank, world,
    local_rank)."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
        if not dist.is_initialized():
            dist.init_process_group(backend)
        if backend == "nccl":
            torch.cuda.set_device(local)
    _WS.update(rank=rank, world=world, local=local)
    return rank, world, local


def replica_barrier():
    if _WS["world"] > 1:
        import torch.distributed as dist
        dist.barrier()


def replica_max(x):
    """Largest value of `x` over the ranks (the slowest replica's time)."""
    if _WS["world"] == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", _WS["local"]) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "Sinkhorn solves/s at marginal err 1e-6, warm vs plain, 1 GB300; % roofline"
WS_N, WS_D, WS_REG, WS_TOL = 2048, 16, 0.02, 1e-6
# DRAM traffic / algorithmic bytes of multi_sinkhorn_kernel, from one ncu capture of the
# same workload on 128 pairs (profiles/multi_sinkhorn_warmstart_gmm2048.md); the launch's
# traffic scales with the problem-iterations it processes
MULTI_TRAFFIC_RATIO = 132.02 / 133.61  # ncu dram bytes / algorithmic bytes, one plain-arm launch on 128 pairs
EVAL_SEED = 10_000_000


def peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained"), "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "src": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 3 + k and s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------------------------
# warm vs plain (default workload)
# ---------------------------------------------------------------------------
def run_warmstart(args, pk):
    import torch
    from pot_gb300 import _lib
    from pot_gb300.warmstart import pipeline as wp

    dev = torch.device("cuda", _WS["local"])
    B = args.batch
    # each replica solves its own held-out pairs
    X, Y = wp.gen_pairs(EVAL_SEED + _WS["rank"] * B, B, WS_N, WS_D, dev)
    net = wp.default_net(dev)
    st = torch.cuda.current_stream()

    OM = wp.REFINE_OMEGA
    AD = wp.REFINE_ANDERSON
    # arms: (start, omega, iterations between stop tests, Anderson window).
    # Headline: the multiscale prior with Anderson-mixed updates against the
    # plain zero-started iteration, both testing the reference's criterion
    # (column-marginal L2 error < 1e-6) at every iteration.  Ablations: the
    # learned residual network on top of the prior, each component alone,
    # over-relaxation instead of Anderson mixing, and the reference's
    # every-10th-iteration test schedule.
    # The last field is the engine: "multi" reads stored cost blocks (the
    # headline, HBM-bound), "online" rebuilds the cost tiles from the points on
    # the tensor cores every pass (otg_sinkhorn_pairs).
    ARMS = {"warm": ("prior", 1.0, 1, AD, "multi"), "plain": (None, 1.0, 1, 0, "multi"),
            "online_warm": ("prior", 1.0, 1, AD, "online"), "online_plain": (None, 1.0, 1, 0, "online"),
            "learned_anderson": ("net", 1.0, 1, AD, "multi"), "zero_anderson": (None, 1.0, 1, AD, "multi"),
            "prior_plain": ("prior", 1.0, 1, 0, "multi"), "prior_relaxed": ("prior", OM, 1, 0, "multi"),
            "plain_ref_schedule": (None, 1.0, 10, 0, "multi"), "warm_ref_schedule": ("prior", 1.0, 10, AD, "multi")}

    if args.arms:  # a subset (profiling runs); the headline needs both warm and plain
        keep = set(args.arms.split(",")) | {"warm", "plain"}
        ARMS = {k: v for k, v in ARMS.items() if k in keep}

    def step(arm, ev=None):
        init, om, per, ad, eng = ARMS[arm]
        ps = wp.PairSolver(X, Y, engine=eng)
        wu = None
        if init == "net":
            wu = wp.warm_potential(net, X, Y, ps, WS_REG)
        elif init == "prior":
            wu = wp.prior_potential(X, Y, ps, WS_REG)
        out = ps.solve(WS_REG, WS_TOL, warm_u=wu, events=ev, omega=om, check_period=per, anderson=ad)
        return ps, out

    for _ in range(args.warmup):
        for arm in ARMS:
            step(arm)
    torch.cuda.synchronize()
    res = {}
    with ClockSampler(_WS["local"]) as cs:
        for arm in ARMS:
            replica_barrier()
            torch.cuda.synchronize()
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            kev = []
            l0 = _lib.LAUNCHES[0]
            t0.record(st)
            for _ in range(args.steps):
                e = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ps, out = step(arm, e)
                kev.append(e)
            t1.record(st)
            torch.cuda.synchronize()
            replica_barrier()
            ms = replica_max(t0.elapsed_time(t1) / args.steps)
            kms = statistics.mean(a.elapsed_time(b) for a, b in kev)
            nit = out[3].cpu().numpy().astype(np.int64)
            stt = out[2].cpu().numpy()
            err = out[4].cpu().numpy()
            L = ps.layout
            passes = (nit + 2) + (nit + 1)  # column passes incl. the final check pass, row passes
            alg = float((passes * L.rows_np * L.ldm_np * 4).sum())
            res[arm] = {"ms": ms, "kernel_ms": kms, "alg_bytes": alg, "niter_mean": float(nit.mean()),
                        "niter_max": int(nit.max()), "converged": int((stt == 0).sum()),
                        "max_err": float(err.max()), "launches": (_lib.LAUNCHES[0] - l0) // args.steps}
    w, p = res["warm"], res["plain"]
    achieved = p["alg_bytes"] / (p["kernel_ms"] * 1e-3) / 1e9
    # e2e through the public entry point with host clouds in pinned memory
    # (the host-to-device copy of every step's inputs is inside the timed
    # region; results come back as host tensors)
    Xh, Yh = X.cpu().pin_memory(), Y.cpu().pin_memory()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(args.warmup):  # untimed, like the device arms (first-call allocations)
        wp.solve_cloud_pairs(Xh, Yh, WS_REG, WS_TOL, warm=True, check_period=1)
    torch.cuda.synchronize()
    replica_barrier()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_res = wp.solve_cloud_pairs(Xh, Yh, WS_REG, WS_TOL, warm=True, check_period=1)
    e2e_s = replica_max((time.perf_counter() - t) / e2e_steps)
    lu, lv, ni = e2e_res[0], e2e_res[1], e2e_res[2]
    W = _WS["world"]
    return {
        "value": W * B / (w["ms"] * 1e-3), "unit": "solves/s", "ms_per_step": w["ms"], "dtype": "f32",
        "plain": {"value": W * B / (p["ms"] * 1e-3), "ms_per_step": p["ms"], "niter_mean": p["niter_mean"],
                  "niter_max": p["niter_max"], "converged": p["converged"], "max_marginal_err": p["max_err"]},
        "warm": {"niter_mean": w["niter_mean"], "niter_max": w["niter_max"], "converged": w["converged"],
                 "max_marginal_err": w["max_err"]},
        "speedup_warm_vs_plain": p["ms"] / w["ms"],
        "warm_pipeline": "coarse multiscale prior (Voronoi-weighted 256-point problem solved on the GPU + one "
                         "c-transform to every source point), then the solve with Anderson-mixed v updates over "
                         "the last %d iterates (u the exact row update of the mixed v); every pair of both arms "
                         "stops at the first iteration whose column-marginal L2 error is below %g" % (AD, WS_TOL),
        "ablation": {k: {"value": W * B / (res[k]["ms"] * 1e-3), "niter_mean": res[k]["niter_mean"],
                         "speedup_vs_plain": p["ms"] / res[k]["ms"], "start": ARMS[k][0] or "zero",
                         "omega": ARMS[k][1], "check_period": ARMS[k][2], "anderson": ARMS[k][3],
                         "engine": ARMS[k][4],
                         "max_marginal_err": res[k]["max_err"], "converged": res[k]["converged"]}
                     for k in ARMS if k not in ("warm", "plain")},
        # the reference's own schedule (stop test every 10th iteration) for both arms
        "speedup_warm_vs_plain_ref_schedule": (res["plain_ref_schedule"]["ms"] / res["warm_ref_schedule"]["ms"]
                                               if "warm_ref_schedule" in res else None),
        "speedup_warm_vs_plain_ref_schedule_plain": (res["plain_ref_schedule"]["ms"] / w["ms"]
                                                     if "plain_ref_schedule" in res else None),
        # the same two arms on the online engine (no cost blocks; cost tiles from the points)
        "engine_online": ({"warm": W * B / (res["online_warm"]["ms"] * 1e-3),
                           "plain": W * B / (res["online_plain"]["ms"] * 1e-3),
                           "speedup_warm_vs_plain": res["online_plain"]["ms"] / res["online_warm"]["ms"],
                           "unit": "solves/s"} if "online_warm" in res and "online_plain" in res else None),
        "config": {"workload": "learned warm start vs plain log-Sinkhorn, %d GMM cloud pairs n=m=%d d=%d, "
                               "reg=%.2f x max cost, stopThr=%g, float32" % (B, WS_N, WS_D, WS_REG, WS_TOL),
                   "pairs_per_step": W * B, "replicas": W, "l2": "inputs larger than L2 (%.1f GiB of cost blocks)" % (
                       B * WS_N * WS_N * 4 / 2**30),
                   "held_out_seeds": [EVAL_SEED, EVAL_SEED + B - 1]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": p["alg_bytes"] * MULTI_TRAFFIC_RATIO,
                     "traffic_src": "ncu capture on 128 pairs, scaled by problem-iterations",
                     "kernel": "multi_sinkhorn_kernel (plain arm)",
                     "alg_bytes_per_launch": p["alg_bytes"], "launch_ms": p["kernel_ms"],
                     "peak_src": pk["src"] + " (of measured)" if pk["src"] == "measured" else pk["src"]},
        "e2e": {"value": W * B / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(Xh.nbytes + Yh.nbytes),
                "d2h_bytes_per_step": int(lu.nbytes + lv.nbytes + ni.nbytes)},
        "gpu_launches": int(w["launches"] * args.steps),
        "clocks": cs.summary(),
    }


# ---------------------------------------------------------------------------
# other workloads (one JSON line each; not the default)
# ---------------------------------------------------------------------------
def _timed(fn, st):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    out = fn()
    e1.record(st)
    torch.cuda.synchronize()
    return out, e0.elapsed_time(e1)


def gmm_clouds(n, d, comps, mean_std, std, seed, device):
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    means = torch.randn(comps, d, generator=g, device=device) * mean_std
    def cloud():
        c = torch.randint(0, comps, (n,), generator=g, device=device)
        return (means[c] + torch.randn(n, d, generator=g, device=device) * std).contiguous()
    return cloud(), cloud(), g


def run_online(args, pk):
    """Online (lazy) log-Sinkhorn: n = m = args.n points in R^64, 8-component
    mixture (means ~ N(0, 4I), covariance 0.5 I), weights uniform x
    Dirichlet(50), reg = 0.01 x median cost (4096-point subsample),
    stopThr 1e-6; cost never stored."""
    import torch
    from pot_gb300 import _lib
    from pot_gb300.empirical import online_sinkhorn
    dev = torch.device("cuda:0")
    n, d = args.n, 64
    X, Y, g = gmm_clouds(n, d, 8, 2.0, 0.5 ** 0.5, 7, dev)
    gam = torch.distributions.Gamma(torch.full((n,), 50.0, device=dev), torch.ones(n, device=dev))
    a = gam.sample(); a = (a / a.sum()).float().contiguous()
    b = gam.sample(); b = (b / b.sum()).float().contiguous()
    k = min(4096, n)
    reg = 0.01 * float(torch.cdist(X[:k].double(), Y[:k].double()).pow(2).median())
    st = torch.cuda.current_stream()
    for _ in range(args.warmup):
        online_sinkhorn(X, Y, reg, a, b, 2, 0.0)
    iters = args.iters
    (res, ms) = _timed(lambda: online_sinkhorn(X, Y, reg, a, b, iters, 0.0), st)
    per_it = ms / iters
    from pot_gb300.empirical import LAST_STATS
    fixups = LAST_STATS["fixup_units"]
    flop = 4.0 * n * n * d
    achieved = flop / (per_it * 1e-3) / 1e12
    full = None
    if args.full:
        (res2, ms2) = _timed(lambda: online_sinkhorn(X, Y, reg, a, b, args.full, 1e-6), st)
        full = {"ms": ms2, "niter": res2[3], "status": res2[2], "last_err": res2[4][-1] if res2[4] else None}
    return {"metric": "online log-Sinkhorn iterations/s", "value": 1000.0 / per_it, "unit": "iterations/s",
            "ms_per_step": per_it, "dtype": "f32 (fp16 hi/lo x3 tensor-core dot products)",
            "config": {"workload": "online log-Sinkhorn n=m=%d d=64 GMM(8), reg=0.01 x median cost (%.4g)" % (n, reg),
                       "timed_iterations": iters, "l2": "points %.0f MiB, cost never stored" % (2 * n * d * 4 / 2**20),
                       "fixup_row_blocks": fixups},
            "full_solve": full,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / pk["bf16_tflops"], "issued_multiplier": 3,
                         "issued_frac": 3 * achieved / pk["bf16_tflops"], "traffic": None,
                         "kernel": "online_pass_kernel", "alg_flop_per_iteration": flop}}


def aux_online(pk, n=65536, iters=20):
    """The online-cost workload's iteration (n = m = 65536 points in R^64,
    8-component mixture, reg = 0.01 x median cost): `iters` iterations timed
    with CUDA events, algorithmic tensor FLOP 4 n m d per iteration."""
    import torch
    from pot_gb300.empirical import online_sinkhorn
    dev = torch.device("cuda", _WS["local"])
    d = 64
    X, Y, _ = gmm_clouds(n, d, 8, 2.0, 0.5 ** 0.5, 7, dev)
    a = torch.full((n,), 1.0 / n, device=dev)
    k = min(4096, n)
    reg = 0.01 * float(torch.cdist(X[:k].double(), Y[:k].double()).pow(2).median())
    st = torch.cuda.current_stream()
    online_sinkhorn(X, Y, reg, a, a, 2, 0.0)
    _, ms = _timed(lambda: online_sinkhorn(X, Y, reg, a, a, iters, 0.0), st)
    per_it = ms / iters
    flop = 4.0 * n * n * d
    achieved = flop / (per_it * 1e-3) / 1e12
    return {"workload": "online log-Sinkhorn iteration, n=m=%d d=64 GMM(8), reg=0.01 x median cost" % n,
            "value": 1000.0 / per_it, "unit": "iterations/s", "ms_per_iteration": per_it, "timed_iterations": iters,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / pk["bf16_tflops"], "issued_multiplier": 3,
                         "issued_frac": 3 * achieved / pk["bf16_tflops"], "traffic": None,
                         "kernel": "online_pass_kernel (+ online_finalize_kernel)",
                         "alg_flop_per_iteration": flop}}


def aux_gw(pk, n=8192, reps=5):
    """The entropic-GW workload's gradient (n = m = 8192, C1 / C2 from
    N(0, I3) / N(0, I8) points, each / max): both tensor-core GEMMs of
    constC - C1 T hC2^T, median of `reps` CUDA-event timings, algorithmic
    FLOP 4 n^3."""
    import torch
    from pot_gb300 import gromov as pgw
    dev = torch.device("cuda", _WS["local"])
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    xs = torch.randn(n, 3, generator=g, device=dev, dtype=torch.float64)
    xt = torch.randn(n, 8, generator=g, device=dev, dtype=torch.float64)
    C1 = torch.cdist(xs, xs).pow(2)
    C1 /= C1.max()
    C2 = torch.cdist(xt, xt).pow(2)
    C2 /= C2.max()
    C1, C2 = C1.float().contiguous(), C2.float().contiguous()
    del xs, xt
    st = torch.cuda.current_stream()
    pd = torch.full((n,), 1.0 / n, device=dev)
    tp = pgw.TensorProduct(C1, C2, pd, pd)
    T = torch.outer(pd, pd)
    M = torch.empty(n, n, device=dev)
    tp.grad(T, M)
    kms = [_timed(lambda: tp.grad(T, M), st)[1] for _ in range(reps)]
    tp.check_abort()
    gemm_ms = statistics.median(kms)
    flop = 4.0 * n ** 3
    achieved = flop / (gemm_ms * 1e-3) / 1e12
    return {"workload": "entropic-GW gradient constC - C1 T hC2^T, n=m=%d" % n, "value": 1000.0 / gemm_ms,
            "unit": "gradients/s", "ms_per_gradient": gemm_ms,
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / pk["bf16_tflops"], "issued_multiplier": 3,
                         "issued_frac": 3 * achieved / pk["bf16_tflops"], "traffic": None,
                         "kernel": "gemm_split3_kernel (both GEMMs of one gradient)",
                         "alg_flop_per_gradient": flop}}


def run_gw(args, pk):
    """Entropic GW, n = m = args.n: C1 = sqeuclid of N(0, I3) points, C2 of
    N(0, I8) points, each / max; uniform p, q; square loss; eps = 5e-3;
    args.outer outer iterations; inner log-Sinkhorn at 1e-7 warm-started
    from the previous potentials; float32 with tensor-core products."""
    import torch
    from pot_gb300 import gromov as pgw
    dev = torch.device("cuda:0")
    n = args.n
    g = torch.Generator(device=dev); g.manual_seed(3)
    xs = torch.randn(n, 3, generator=g, device=dev, dtype=torch.float64)
    xt = torch.randn(n, 8, generator=g, device=dev, dtype=torch.float64)
    C1 = torch.cdist(xs, xs).pow(2); C1 /= C1.max()
    C2 = torch.cdist(xt, xt).pow(2); C2 /= C2.max()
    C1, C2 = C1.float().contiguous(), C2.float().contiguous()
    st = torch.cuda.current_stream()
    pd = torch.full((n,), 1.0 / n, device=dev)
    tp = pgw.TensorProduct(C1, C2, pd, pd)
    T = torch.outer(pd, pd)
    M = torch.empty(n, n, device=dev)
    for _ in range(args.warmup):
        tp.grad(T, M)
    kms = []
    for _ in range(max(args.steps, 3)):
        (_, ms) = _timed(lambda: tp.grad(T, M), st)
        kms.append(ms)
    gemm_ms = statistics.median(kms)
    flop = 4.0 * n ** 3  # two n^3 GEMMs
    achieved = flop / (gemm_ms * 1e-3) / 1e12
    (res, ms) = _timed(lambda: pgw.entropic_gromov_wasserstein_log(C1, C2, epsilon=5e-3, max_iter=args.outer,
                                                                  numItermax=100000, stopThr=1e-7), st)
    T, lg = res
    return {"metric": "entropic GW outer iterations/s", "value": args.outer / (ms * 1e-3), "unit": "outer iterations/s",
            "ms_per_step": ms / args.outer, "dtype": "f32 (fp16 hi/lo x3 tensor-core GEMMs)",
            "config": {"workload": "entropic GW n=m=%d, eps=5e-3, %d outer iterations, inner log-Sinkhorn 1e-7 warm"
                                   % (n, args.outer), "inner_niter": lg["inner_niter"], "gw_dist": lg["gw_dist"]},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": achieved / pk["bf16_tflops"], "issued_multiplier": 3,
                         "issued_frac": 3 * achieved / pk["bf16_tflops"], "traffic": None,
                         "kernel": "gemm_split3_kernel (both GEMMs of one gradient)", "gemm_ms": gemm_ms,
                         "alg_flop_per_gradient": flop}}


def run_ragged(args, pk):
    """4096 independent problems, n, m ~ U{32..1024}, d in {3, 16}, points ~
    U[0,1]^d, a, b ~ Dirichlet(1), reg = 10^U[-3,-1] x max cost, stopThr
    1e-6, float32, one persistent launch."""
    import torch
    from pot_gb300 import batch as pb
    rng = np.random.default_rng(0)
    B = args.batch
    Xs, Ys, As, Bs, regs = [], [], [], [], []
    for k in range(B):
        n, m = rng.integers(32, 1025, size=2)
        d = 3 if k % 2 == 0 else 16
        Xs.append(rng.random((n, d))); Ys.append(rng.random((m, d)))
        As.append(rng.dirichlet(np.ones(n))); Bs.append(rng.dirichlet(np.ones(m))); regs.append(10 ** rng.uniform(-3, -1))
    st = torch.cuda.current_stream()
    from pot_gb300 import tune
    # untimed: the autotuner picks the launch schedule of this workload class
    # (timed candidate launches on this batch), then warm-up solves
    pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=10, tol=1e-6, autotune=True)
    for _ in range(args.warmup):
        pb.solve_sample_ragged(Xs[:64], Ys[:64], regs[:64], As[:64], Bs[:64], reg_relative=True, max_iter=1000, tol=1e-6)
    (res, ms) = _timed(lambda: pb.solve_sample_ragged(Xs, Ys, regs, As, Bs, reg_relative=True, max_iter=100000,
                                                      tol=1e-6), st)
    sched = tune.lookup(res.layout)
    trials = next(iter(tune.tuner().trials.values()), [])
    nit = res.niter.cpu().numpy().astype(np.int64)
    L = res.layout
    alg = float((((nit + 2) + (nit + 1)) * L.rows_np * L.ldm_np * 4).sum())
    return {"metric": "batched Sinkhorn solves/s", "value": B / (ms * 1e-3), "unit": "solves/s", "ms_per_step": ms,
            "dtype": "f32", "config": {"workload": "%d uneven problems n,m~U[32,1024], d in {3,16}, reg=10^U[-3,-1] x "
                                                   "max cost, stopThr=1e-6" % B,
                                       "niter_median": float(np.median(nit)), "niter_max": int(nit.max()),
                                       "niter_p99": float(np.percentile(nit, 99)),
                                       "niter_top10": sorted(nit.tolist())[-10:],
                                       "status_counts": np.bincount(res.status.cpu().numpy(), minlength=4).tolist(),
                                       "schedule": dict(sched._asdict()) if sched else None,
                                       "tuning_trials_ms": [[list(c), "fill" if f else "tail", round(t, 3)]
                                                            for c, f, t in trials]},
            "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": alg / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], "traffic": None,
                         "kernel": "multi_sinkhorn_kernel (+ cost build)", "alg_bytes": alg}}


def run_dense(args, pk):
    """One dense log-domain solve: n = m = args.n points in R^2, N(0, I) vs
    N((1,1), 0.5 I), cost / max, reg = 0.05, stopThr 1e-6, float32 (the
    plain dense workload scaled up until the cost exceeds L2)."""
    import torch
    from pot_gb300 import bregman, _lib
    dev = torch.device("cuda:0")
    n = args.n
    g = torch.Generator(device=dev); g.manual_seed(0)
    x = torch.randn(n, 2, generator=g, device=dev, dtype=torch.float64)
    y = torch.randn(n, 2, generator=g, device=dev, dtype=torch.float64) * 0.5 ** 0.5 + 1.0
    M = torch.cdist(x, y).pow(2); M /= M.max(); M = M.float().contiguous()
    a = torch.full((n,), 1.0 / n, device=dev)
    st = torch.cuda.current_stream()
    for _ in range(args.warmup):
        bregman.solve_dense(M, a, a, 0.05, _lib.OTG_METHOD_LOG, 10000, 1e-6)
    kms = []
    for _ in range(args.steps):
        (r, ms) = _timed(lambda: bregman.solve_dense(M, a, a, 0.05, _lib.OTG_METHOD_LOG, 10000, 1e-6,
                                                     read_back=False), st)
        kms.append(ms)
    bregman.read_result(r)
    ms = statistics.median(kms)
    alg = ((r.niter + 2) + (r.niter + 1)) * n * n * 4.0
    return {"metric": "dense Sinkhorn solves/s", "value": 1000.0 / ms, "unit": "solves/s", "ms_per_step": ms,
            "dtype": "f32", "config": {"workload": "dense log-Sinkhorn n=m=%d, reg=0.05, stopThr=1e-6" % n,
                                       "iterations": r.niter + 1, "l2": "M = %.2f GiB" % (n * n * 4 / 2**30)},
            "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": alg / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], "traffic": None,
                         "kernel": "dense_sinkhorn_kernel", "alg_bytes_per_launch": alg}}


def run_small(args, pk):
    """The reference's CPU-sized case, many times: dense problems n = m = 1024
    in R^2 (x ~ N(0, I), y ~ N((1,1), 0.5 I)), a = b uniform, cost / max,
    reg = 0.05, stopThr = 1e-9, numItermax = 1000, float64, method 'sinkhorn';
    plan, loss and log per solve.  Direct calls (one persistent solve launch,
    plan and loss kernels, one result read) against replays of one captured
    CUDA graph of the same launches; wall time per solve on the host, since
    the cost (8 MiB) sits in L2 and the solve is latency-bound."""
    import torch
    import pot_gb300 as pg
    from pot_gb300.graphs import SinkhornGraph
    dev = torch.device("cuda:0")
    n, reg, P = 1024, 0.05, 32
    g = torch.Generator(device=dev); g.manual_seed(0)
    probs = []
    for _ in range(P):
        x = torch.randn(n, 2, generator=g, device=dev, dtype=torch.float64)
        y = torch.randn(n, 2, generator=g, device=dev, dtype=torch.float64) * 0.5 ** 0.5 + 1.0
        M = torch.cdist(x, y).pow(2); M /= M.max()
        probs.append(M.contiguous())
    a = torch.full((n,), 1.0 / n, device=dev, dtype=torch.float64)
    gr = SinkhornGraph(n, n, reg, method="sinkhorn", numItermax=1000, stopThr=1e-9, dtype=torch.float64, device=dev)

    def direct(M):
        Pl, lg = pg.sinkhorn(a, a, M, reg, numItermax=1000, stopThr=1e-9, log=True)
        return lg["niter"], float(torch.sum(Pl * M))

    def graph(M):
        _, lg = gr(a, a, M, log=True)
        return lg["niter"], lg["loss"]

    out = {}
    for name, fn in (("direct", direct), ("graph", graph)):
        for _ in range(args.warmup):
            fn(probs[0])
        torch.cuda.synchronize()
        t = time.perf_counter()
        its = []
        for _ in range(args.steps):
            for M in probs:
                its.append(fn(M))
        torch.cuda.synchronize()
        out[name] = {"s": (time.perf_counter() - t) / (args.steps * P), "niter": its}
    nit = np.array([i for i, _ in out["graph"]["niter"]])
    assert [i for i, _ in out["direct"]["niter"]] == list(nit)
    ms = out["graph"]["s"] * 1e3
    alg = float(((nit + 1) * 2 * n * n * 8).mean())
    return {"metric": "dense Sinkhorn solves/s (n=m=1024, float64)", "value": 1.0 / out["graph"]["s"],
            "unit": "solves/s", "ms_per_step": ms, "dtype": "f64",
            "direct": {"value": 1.0 / out["direct"]["s"], "ms_per_solve": out["direct"]["s"] * 1e3},
            "config": {"workload": "plain dense ot.sinkhorn n=m=1024 in R^2, reg=0.05, stopThr=1e-9, float64, %d "
                                   "seeded problems resident on the device, each solve replayed from one CUDA "
                                   "graph (plan + loss + log read back)" % P,
                       "niter_mean": float(nit.mean()), "l2": "cost 8 MiB, L2-resident (latency-bound)"},
            "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": alg / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], "traffic": None,
                         "kernel": "dense_sinkhorn_kernel (graph replay, host wall time)",
                         "alg_bytes_per_launch": alg}}


def run_greenkhorn(args, pk):
    """Greenkhorn (ot.sinkhorn(method='greenkhorn')) on the reference's
    CPU-sized dense case: n = m = 1024 in R^2, x ~ N(0, I), y ~ N((1,1), 0.5 I),
    a = b uniform, cost / max, reg = 0.05, stopThr = 1e-9, float64, step
    budget 10^5 so that every problem converges.  The step chain runs in one
    CTA (latency-bound: a step is a dependent sequence of block reductions);
    wall time per solve on the host, plan and log read back.  The CPU baseline
    is the numpy restatement of the reference's loop on one problem."""
    import torch
    import pot_gb300 as pg
    dev = torch.device("cuda:0")
    n, reg, P = 1024, 0.05, 8
    g = torch.Generator(device=dev); g.manual_seed(1)
    probs = []
    for _ in range(P):
        x = torch.randn(n, 2, generator=g, device=dev, dtype=torch.float64)
        y = torch.randn(n, 2, generator=g, device=dev, dtype=torch.float64) * 0.5 ** 0.5 + 1.0
        M = torch.cdist(x, y).pow(2); M /= M.max()
        probs.append(M.contiguous())
    a = torch.full((n,), 1.0 / n, device=dev, dtype=torch.float64)

    def solve(M):
        Pl, lg = pg.greenkhorn(a, a, M, reg, numItermax=100000, stopThr=1e-9, log=True)
        return lg["n_iter"]

    for _ in range(args.warmup):
        solve(probs[0])
    torch.cuda.synchronize()
    t = time.perf_counter()
    steps = []
    for _ in range(args.steps):
        for M in probs:
            steps.append(solve(M) + 1)
    torch.cuda.synchronize()
    s = (time.perf_counter() - t) / (args.steps * P)
    st = np.array(steps, dtype=np.float64)
    out = {"metric": "greenkhorn solves/s (n=m=1024, float64)", "value": 1.0 / s, "unit": "solves/s",
           "ms_per_step": s * 1e3, "dtype": "f64",
           "coordinate_steps_per_s": float(st.mean() / s), "us_per_coordinate_step": float(s / st.mean() * 1e6),
           "config": {"workload": "ot.sinkhorn(method='greenkhorn') n=m=1024 in R^2, reg=0.05, stopThr=1e-9, "
                                  "float64, %d seeded problems resident on the device; K and its transpose built "
                                  "per solve, step chain in one CTA, plan + log read back" % P,
                      "steps_mean": float(st.mean()), "l2": "K and K^T 16 MiB, L2-resident (latency-bound)"}}
    if not args.no_cpu:
        import oracle
        Mh = probs[0].cpu().numpy()
        ah = np.full(n, 1.0 / n)
        t = time.perf_counter()
        _, lo = oracle.greenkhorn(ah, ah, Mh, reg, numItermax=100000, stopThr=1e-9)
        cs = time.perf_counter() - t
        out["cpu_baseline"] = {"value": 1.0 / cs, "unit": "solves/s", "cores": 1, "kind": "port",
                               "sample": "1 problem of the workload, numpy restatement of the reference loop, "
                                         "%d steps (%.1f us per step)" % (lo["n_iter"] + 1,
                                                                          cs / (lo["n_iter"] + 1) * 1e6)}
    return out


def run_solve(args, pk):
    """One arm of the warm-start workload alone (profiling runs): `args.batch`
    cloud pairs (n = m = 2048, d = 16), plain zero-started solve or (with
    --warm) prior + Anderson, stop test every iteration, on the stored-cost
    engine (multi_sinkhorn_kernel) or the online engine (otg_sinkhorn_pairs);
    the first `warmup` solves are untimed."""
    import torch
    from pot_gb300.warmstart import pipeline as wp
    dev = torch.device("cuda", _WS["local"])
    X, Y = wp.gen_pairs(EVAL_SEED, args.batch, WS_N, WS_D, dev)
    st = torch.cuda.current_stream()

    def one():
        ps = wp.PairSolver(X, Y, engine=args.engine)
        wu = wp.prior_potential(X, Y, ps, WS_REG) if args.warm else None
        return ps.solve(WS_REG, WS_TOL, warm_u=wu, check_period=1, anderson=wp.REFINE_ANDERSON if args.warm else 0)

    for _ in range(args.warmup):
        one()
    ms = []
    for _ in range(args.steps):
        out, t = _timed(one, st)
        ms.append(t)
    per = statistics.median(ms)
    return {"metric": "cloud-pair solves/s (one arm)", "value": args.batch / (per * 1e-3), "unit": "solves/s",
            "ms_per_step": per, "dtype": "f32",
            "config": {"workload": "%s arm, %d GMM cloud pairs n=m=%d d=%d, reg=%.2f x max cost, stopThr=%g, "
                                   "test every iteration, engine %s" % ("warm" if args.warm else "plain",
                                                                         args.batch, WS_N, WS_D, WS_REG, WS_TOL,
                                                                         args.engine),
                       "niter_mean": float(out[3].double().mean()), "converged": int((out[2] == 0).sum())}}


def run_warm_eval(args, pk):
    """Held-out evaluation of the warm start on 10 batches of 1024 pairs
    (seeds after the headline batch's): the warm arm (multiscale prior +
    Anderson-mixed updates) against the plain iteration, both testing the
    column-marginal error (1e-6) at every iteration; mean stop index,
    relative error of the prior and of prior + learned residual against each
    batch's converged potential, and device time per batch (seeds EVAL_SEED
    .. EVAL_SEED + 10239, never used in training)."""
    import torch
    from pot_gb300.warmstart import pipeline as wp
    dev = torch.device("cuda:0")
    net = wp.default_net(dev)
    B, nb = 1024, 10
    res = {"warm": [], "plain": [], "err": [], "prior_err": []}
    t_warm = t_plain = 0.0
    st = torch.cuda.current_stream()

    def arm_run(X, Y, arm):
        ps = wp.PairSolver(X, Y)
        wu = wp.prior_potential(X, Y, ps, WS_REG) if arm == "warm" else None
        return ps, ps.solve(WS_REG, WS_TOL, warm_u=wu, check_period=1,
                            anderson=wp.REFINE_ANDERSON if arm == "warm" else 0)

    X, Y = wp.gen_pairs(EVAL_SEED, B, WS_N, WS_D, dev)
    for _ in range(max(1, args.warmup)):  # untimed: module loads, allocator pools
        for arm in ("warm", "plain"):
            arm_run(X, Y, arm)
    for k in range(nb):
        X, Y = wp.gen_pairs(EVAL_SEED + k * B, B, WS_N, WS_D, dev)
        for arm in ("warm", "plain"):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            ps, out = arm_run(X, Y, arm)
            e1.record(st)
            torch.cuda.synchronize()
            dt = e0.elapsed_time(e1) * 1e-3
            if arm == "warm":
                t_warm += dt
                # error of the prediction against this batch's converged potential
                f = WS_REG * (out[0] - out[0].mean(1, keepdim=True))
                F, prior = wp.inputs(ps, X, Y, WS_REG)
                pred = prior + wp.predict(net, X, Y, ps.maxc, F)
                res["err"].append(float(wp.relative_error(pred, f).median()))
                res["prior_err"].append(float(wp.relative_error(prior, f).median()))
            else:
                t_plain += dt
            assert bool((out[2] == 0).all()), "a pair did not converge"
            res[arm].append(float(out[3].double().mean()))
            del ps
    n = B * nb
    return {"metric": "held-out warm-start evaluation (10240 pairs)", "value": n / t_warm, "unit": "solves/s",
            "dtype": "f32", "plain_value": n / t_plain, "speedup_warm_vs_plain": t_plain / t_warm,
            "mean_stop_index": {"warm": float(np.mean(res["warm"])), "plain": float(np.mean(res["plain"]))},
            "median_rel_error_potential": {"prior_plus_network": float(np.mean(res["err"])),
                                           "prior_only": float(np.mean(res["prior_err"]))},
            "warm_pipeline": "multiscale prior + Anderson(%d), stop test every iteration (both arms)"
                             % wp.REFINE_ANDERSON,
            "config": {"workload": "%d held-out GMM cloud pairs n=m=%d d=%d, reg=%.2f x max cost, stopThr=%g, "
                                   "seeds %d..%d, device time per batch (CUDA events) incl. cost blocks and warm "
                                   "start"
                                   % (n, WS_N, WS_D, WS_REG, WS_TOL, EVAL_SEED, EVAL_SEED + n - 1)}}


def run_tail(args, pk):
    """Cost of one iteration once few problems remain: the batch kernel alone
    against the cluster tail (fixed iteration counts, stop threshold 0, so
    every problem runs them all), float32, reg = 0.001 x raw squared distance,
    points ~ U[0,1]^3."""
    import torch
    from pot_gb300 import batch as pb
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev); g.manual_seed(5)
    out = {}
    for shape in ([(375, 190), (191, 179)], [(64, 64)], [(800, 800)]):
        rows = np.array([r for r, _ in shape]); cols = np.array([c for _, c in shape])
        layout = pb.RaggedLayout(rows, cols, torch.float32, dev)
        Ms = [torch.cdist(torch.rand(n, 3, generator=g, device=dev), torch.rand(m, 3, generator=g, device=dev)).pow(2)
              for n, m in shape]
        Mp = pb.pack_dense(layout, Ms)
        a = torch.cat([torch.full((int(n),), 1.0 / n, device=dev) for n in rows])
        b = torch.cat([torch.full((int(m),), 1.0 / m, device=dev) for m in cols])
        key = " + ".join("%dx%d" % sh for sh in shape)
        out[key] = {}
        for name, tp in (("batch_kernel", -1), ("cluster_tail", 0)):
            for _ in range(args.warmup):
                pb.run_multi(layout, Mp, a, b, 0.001, 200, 0.0, tail_problems=tp)
            its = 6000
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            pb.run_multi(layout, Mp, a, b, 0.001, its, 0.0, tail_problems=tp)
            e1.record()
            torch.cuda.synchronize()
            out[key][name] = e0.elapsed_time(e1) / its * 1e3
    first = out["375x190 + 191x179"]
    return {"metric": "us per iteration, last problems of a batch", "value": first["cluster_tail"], "unit": "us",
            "higher_is_better": False, "dtype": "f32", "per_shape_us": out,
            "config": {"workload": "problems left at the end of a batch, fixed 6000 iterations, float32"}}


def _lib_log():
    from pot_gb300 import _lib
    return _lib.OTG_METHOD_LOG


def run_batch(args, pk):
    """ot.batch.solve_batch on a uniform batch: args.batch problems of
    n = m = args.n (default 1024) points in R^16 (the warm-start clouds),
    cost / max, reg = 0.05, tol 1e-6, solver 'log_sinkhorn' (the batch
    order: u first, row-marginal check), float32."""
    import torch
    from pot_gb300 import batch as pb
    from pot_gb300.warmstart import pipeline as wp
    dev = torch.device("cuda:0")
    B, n = args.batch, min(args.n, 4096)
    X, Y = wp.gen_pairs(EVAL_SEED, B, n, WS_D, dev)
    ps = wp.PairSolver(X, Y)
    M = ps.M.view(B, n, n) / ps.maxc.view(B, 1, 1)
    st = torch.cuda.current_stream()
    ones = torch.full((B, n), 1.0 / n, device=dev)
    # the solver call of solve_batch, which reports per-problem stop indices
    solve = lambda: pb._solve_uniform(M, ones, ones, 0.05, _lib_log(), 10000, 1e-6, False)  # noqa: E731
    for _ in range(args.warmup):
        solve()
    kms = []
    for _ in range(args.steps):
        (res, ms) = _timed(solve, st)
        kms.append(ms)
    ms = statistics.median(kms)
    nit = res[4].cpu().numpy().astype(np.int64)
    # algorithmic passes over each cost block: u and v per iteration plus the
    # final check pass, and the plan (read the cost, write the plan); the
    # transpose the batch order costs here is not counted
    alg = float((((2 * nit + 3) + 2) * n * n * 4.0).sum())
    return {"metric": "batched Sinkhorn solves/s (ot.batch.solve_batch)", "value": B / (ms * 1e-3),
            "unit": "solves/s", "ms_per_step": ms, "dtype": "f32",
            "config": {"workload": "%d problems %dx%d (GMM clouds d=16, cost / max), reg=0.05, tol=1e-6, "
                                   "log_sinkhorn" % (B, n, n), "niter_mean": float(nit.mean())},
            "roofline": {"bound": "hbm", "achieved": alg / (ms * 1e-3) / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": alg / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], "traffic": None,
                         "kernel": "multi_sinkhorn_kernel on the transposed blocks (+ transpose, plan)",
                         "alg_bytes": alg}}


def _oracle_pair_solve(args):
    """One float64 oracle solve of a workload pair (run in a worker process)."""
    x, y = args
    import oracle
    M = oracle.sqeuclidean(x, y)
    reg = WS_REG * M.max()
    t = time.perf_counter()
    _, lg = oracle.sinkhorn_log([], [], M, reg, numItermax=100000, stopThr=WS_TOL)
    return time.perf_counter() - t, lg["niter"]


def cpu_pairs(count, seed):
    import torch
    from pot_gb300.warmstart import pipeline as wp
    X, Y = wp.gen_pairs(seed, count, WS_N, WS_D, torch.device("cpu"))
    return X.double().numpy(), Y.double().numpy()


def cpu_baseline(cores, sample):
    """Reference CPU algorithm (oracle sinkhorn_log, float64) over `sample`
    pairs of the workload, `cores` worker processes; solves/s."""
    import multiprocessing as mp
    X, Y = cpu_pairs(sample, EVAL_SEED)
    t = time.perf_counter()
    if cores > 1:
        with mp.get_context("spawn").Pool(cores) as pool:
            out = pool.map(_oracle_pair_solve, [(X[k], Y[k]) for k in range(sample)])
    else:
        out = [_oracle_pair_solve((X[k], Y[k])) for k in range(sample)]
    wall = time.perf_counter() - t
    return {"value": sample / wall, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": "%d workload pairs (float64 numpy sinkhorn_log restatement, zero init), mean niter %.1f"
                      % (sample, float(np.mean([o[1] for o in out])))}


def reference_arm(cores, steps, warmup):
    """The reference's CPU algorithm on the host cores: W untimed then K
    timed steps, each a bounded sample of the workload (one pair per core,
    fresh seeds per step) solved in `cores` worker processes; solves/s over
    the timed steps."""
    import multiprocessing as mp
    per = max(cores, 4)
    done, wall, nits = 0, 0.0, []
    with mp.get_context("spawn").Pool(cores) as pool:
        for k in range(warmup + steps):
            X, Y = cpu_pairs(per, EVAL_SEED + k * per)
            t = time.perf_counter()
            out = pool.map(_oracle_pair_solve, [(X[i], Y[i]) for i in range(per)])
            dt = time.perf_counter() - t
            if k >= warmup:
                done += per
                wall += dt
                nits += [o[1] for o in out]
    return {"value": done / wall, "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": "%d steps of %d workload pairs each (float64 numpy sinkhorn_log restatement, zero init), "
                      "mean niter %.1f" % (steps, per, float(np.mean(nits)))}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="warmstart")
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-aux", action="store_true")
    ap.add_argument("--arms", default="", help="warm-start workload: comma list of ablation arms to run")
    ap.add_argument("--engine", default="multi", help="solve workload: multi (stored cost) or online")
    ap.add_argument("--warm", action="store_true", help="solve workload: prior + Anderson instead of plain")
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--iters", type=int, default=20)
    ap.add_argument("--full", type=int, default=0)
    ap.add_argument("--outer", type=int, default=50)
    args = ap.parse_args()
    rank, _, _ = replica_setup()
    if args.impl == "reference":
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        cb = reference_arm(cores, args.steps, args.warmup)
        line = {"metric": METRIC, "value": cb["value"], "unit": "solves/s", "impl": "reference",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": "plain log-Sinkhorn (reference CPU algorithm), GMM cloud pairs n=m=%d d=%d, "
                                       "reg=%.2f x max cost, stopThr=%g" % (WS_N, WS_D, WS_REG, WS_TOL)},
                "cpu_baseline": cb, "e2e": {"value": cb["value"], "unit": "solves/s",
                                            "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    pk = peaks()
    if args.workload != "warmstart":
        fn = {"online": run_online, "gw": run_gw, "ragged": run_ragged, "dense": run_dense,
              "batch": run_batch, "small": run_small, "tail": run_tail, "solve": run_solve,
              "warm_eval": run_warm_eval, "greenkhorn": run_greenkhorn}[args.workload]
        line = {"n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "data": "synthetic"}
        line.update(fn(args, pk))
        print(json.dumps(line))
        return
    res = run_warmstart(args, pk)
    line = {"metric": METRIC, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded Gaussian-mixture clouds generated on the device)"}
    line.update(res)
    if not args.no_aux:
        # the tensor-core kernels of the other workloads, measured in the same run
        line["aux"] = {"online": aux_online(pk), "gw_gradient": aux_gw(pk)}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(1, 3)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
