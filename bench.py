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

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "Sinkhorn solves/s at marginal err 1e-6, warm vs plain, 1 GB300; % roofline"
WS_N, WS_D, WS_REG, WS_TOL = 2048, 16, 0.02, 1e-6
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

    dev = torch.device("cuda:0")
    B = args.batch
    X, Y = wp.gen_pairs(EVAL_SEED, B, WS_N, WS_D, dev)
    net = wp.default_net(dev)
    st = torch.cuda.current_stream()

    def step(warm, ev=None):
        ps = wp.PairSolver(X, Y)
        wu = wp.warm_potential(net, X, Y, ps, WS_REG) if warm else None
        out = ps.solve(WS_REG, WS_TOL, warm_u=wu, events=ev)
        return ps, out

    for _ in range(args.warmup):
        step(True)
        step(False)
    torch.cuda.synchronize()
    res = {}
    with ClockSampler() as cs:
        for arm in ("warm", "plain"):
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            kev = []
            l0 = _lib.LAUNCHES[0]
            t0.record(st)
            for _ in range(args.steps):
                e = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ps, out = step(arm == "warm", e)
                kev.append(e)
            t1.record(st)
            torch.cuda.synchronize()
            ms = t0.elapsed_time(t1) / args.steps
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
    # e2e through the public entry point with host clouds
    Xh, Yh = X.cpu().numpy(), Y.cpu().numpy()
    e2e_steps = max(1, min(args.steps, 3))
    torch.cuda.synchronize()
    t = time.perf_counter()
    for _ in range(e2e_steps):
        lu, lv, ni = wp.solve_cloud_pairs(Xh, Yh, WS_REG, WS_TOL, warm=True, net=net)
    e2e_s = (time.perf_counter() - t) / e2e_steps
    return {
        "value": B / (w["ms"] * 1e-3), "unit": "solves/s", "ms_per_step": w["ms"], "dtype": "f32",
        "plain": {"value": B / (p["ms"] * 1e-3), "ms_per_step": p["ms"], "niter_mean": p["niter_mean"],
                  "niter_max": p["niter_max"], "converged": p["converged"], "max_marginal_err": p["max_err"]},
        "warm": {"niter_mean": w["niter_mean"], "niter_max": w["niter_max"], "converged": w["converged"],
                 "max_marginal_err": w["max_err"]},
        "speedup_warm_vs_plain": p["ms"] / w["ms"],
        "config": {"workload": "learned warm start vs plain log-Sinkhorn, %d GMM cloud pairs n=m=%d d=%d, "
                               "reg=%.2f x max cost, stopThr=%g, float32" % (B, WS_N, WS_D, WS_REG, WS_TOL),
                   "pairs_per_step": B, "l2": "inputs larger than L2 (%.1f GiB of cost blocks)" % (
                       B * WS_N * WS_N * 4 / 2**30),
                   "held_out_seeds": [EVAL_SEED, EVAL_SEED + B - 1]},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / pk["hbm_gbs"], "traffic": None, "kernel": "multi_sinkhorn_kernel (plain arm)",
                     "alg_bytes_per_launch": p["alg_bytes"], "launch_ms": p["kernel_ms"],
                     "peak_src": pk["src"] + " (of measured)" if pk["src"] == "measured" else pk["src"]},
        "e2e": {"value": B / e2e_s, "unit": "solves/s", "h2d_bytes_per_step": int(Xh.nbytes + Yh.nbytes),
                "d2h_bytes_per_step": int(lu.nbytes + lv.nbytes + ni.nbytes)},
        "gpu_launches": int(w["launches"] * args.steps),
        "clocks": cs.summary(),
    }


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="warmstart")
    ap.add_argument("--batch", type=int, default=1024)
    ap.add_argument("--impl", default="ours")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        cores = os.cpu_count() or 1
        cb = cpu_baseline(cores, max(cores, 4))
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
    res = run_warmstart(args, pk)
    line = {"metric": METRIC, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "data": "synthetic (seeded Gaussian-mixture clouds generated on the device)"}
    line.update(res)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(1, 3)
    if rank == 0:
        print(json.dumps(line))


if __name__ == "__main__":
    main()
