"""Autotuner for the schedule of the work-balanced batch solver
(``csrc/multi.cu``, ``otg_sinkhorn_multi``).

The schedule divides the work of one launch and leaves each problem's
iteration unchanged (results agree to rounding of the merge order):

- ``ctas_per_sm``: resident CTAs per SM of the persistent grid (0: the most
  the registers allow, 4 in float32, 2 in float64);
- ``units_per_warp``: column-pass units aimed at per warp when problems are
  split into row chunks (default 8);
- ``cap_fill`` / ``cap_tail``: the most row chunks per problem while the
  batch fills the GPU (16) and once few problems remain (64).

A schedule is chosen per workload class, keyed on the dtype and log2 buckets
of the batch size, the mean rows, the mean columns and the spread of the
per-problem work.  The search is a coordinate descent from the default
schedule: each candidate runs a fixed number of iterations (stop threshold
0, so every problem runs them all) timed with CUDA events on the launching
stream, the fill-phase parameters on the caller's whole batch and the tail
cap on its largest few problems.  Results are cached in memory and in a JSON
file (``POT_GB300_TUNE_CACHE``, default ``schedules.json`` next to the built
library in ``pot_gb300/_lib``, an untracked build directory).
"""
import json
import math
import os
from collections import namedtuple

import numpy as np

Schedule = namedtuple("Schedule", ["ctas_per_sm", "units_per_warp", "cap_fill", "cap_tail"])
DEFAULT = Schedule(0, 8, 16, 64)

# candidate values per axis (float64 holds at most 2 CTAs per SM)
SPACE = {
    "ctas_per_sm": {"f32": (2, 3, 4), "f64": (1, 2)},
    "units_per_warp": (4, 8, 16),
    "cap_fill": (8, 16, 32),
    "cap_tail": (16, 32, 64),
}
FILL_AXES = ("ctas_per_sm", "units_per_warp", "cap_fill")
TAIL_AXES = ("cap_tail",)


def _bucket(x):
    return int(round(math.log2(max(float(x), 1.0))))


def schedule_key(dtype_tag, rows, cols):
    """Workload class of a batch: dtype and log2 buckets of the batch size,
    the mean rows, the mean columns and the spread (largest over mean work)."""
    rows = np.asarray(rows, dtype=np.float64)
    cols = np.asarray(cols, dtype=np.float64)
    work = rows * cols
    return "multi/%s/B%d/n%d/m%d/s%d" % (dtype_tag, _bucket(len(rows)), _bucket(rows.mean()), _bucket(cols.mean()),
                                        _bucket(work.max() / max(work.mean(), 1.0)))


def cache_path():
    return os.environ.get("POT_GB300_TUNE_CACHE",
                          os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "schedules.json"))


class Tuner:
    """Schedule cache and coordinate-descent search (timing functions are
    passed in, so the search runs without a GPU in tests)."""

    def __init__(self, path=None):
        self.path = path if path is not None else cache_path()
        self.table = {}
        self.trials = {}
        if self.path and os.path.exists(self.path):
            try:
                with open(self.path) as f:
                    raw = json.load(f)
                self.table = {k: Schedule(*v) for k, v in raw.items()}
            except (OSError, ValueError, TypeError):
                self.table = {}

    def get(self, key):
        return self.table.get(key)

    def put(self, key, sched):
        self.table[key] = Schedule(*sched)
        if not self.path:
            return
        try:
            os.makedirs(os.path.dirname(self.path) or ".", exist_ok=True)
            tmp = self.path + ".tmp"
            with open(tmp, "w") as f:
                json.dump({k: list(v) for k, v in sorted(self.table.items())}, f, indent=1)
            os.replace(tmp, self.path)
        except OSError:
            pass  # an unwritable cache only costs a re-tune

    def search(self, key, dtype_tag, time_fill, time_tail=None, reps=2, start=DEFAULT):
        """Coordinate descent over the fill axes (timed by ``time_fill``) and
        the tail axis (``time_tail``); returns and caches the best schedule.
        Each time function takes a Schedule and returns milliseconds."""
        best = Schedule(*start)
        if best.ctas_per_sm == 0:
            best = best._replace(ctas_per_sm=max(SPACE["ctas_per_sm"][dtype_tag]))
        trials = []
        seen = {}

        def timed(fn, s):
            if (fn is time_fill, s) not in seen:
                seen[(fn is time_fill, s)] = min(fn(s) for _ in range(reps))
                trials.append((tuple(s), fn is time_fill, seen[(fn is time_fill, s)]))
            return seen[(fn is time_fill, s)]

        for axes, fn in ((FILL_AXES, time_fill), (TAIL_AXES, time_tail)):
            if fn is None:
                continue
            t_best = timed(fn, best)
            for ax in axes:
                vals = SPACE[ax][dtype_tag] if isinstance(SPACE[ax], dict) else SPACE[ax]
                for v in vals:
                    if v == getattr(best, ax):
                        continue
                    cand = best._replace(**{ax: v})
                    t = timed(fn, cand)
                    if t < t_best:
                        best, t_best = cand, t
        self.trials[key] = trials
        self.put(key, best)
        return best


_TUNER = None


def tuner():
    global _TUNER
    if _TUNER is None:
        _TUNER = Tuner()
    return _TUNER


def lookup(layout):
    """The cached schedule of this batch's workload class, or None."""
    return tuner().get(schedule_key(_tag(layout.dtype), layout.rows_np, layout.cols_np))


def _tag(dtype):
    import torch
    return "f64" if dtype == torch.float64 else "f32"


def tune_multi(layout, M_packed, a_packed, b_packed, reg, iters=20, tail_problems=2, reps=2, force=False):
    """Choose (and cache) the schedule for this batch's workload class by
    timing candidate launches on the batch itself; returns the Schedule."""
    import torch
    from . import batch as pb
    key = schedule_key(_tag(layout.dtype), layout.rows_np, layout.cols_np)
    t = tuner()
    if not force and t.get(key) is not None:
        return t.get(key)
    st = torch.cuda.current_stream(layout.device)

    def run_timed(lay, M, a, b, r, s):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        # the batch kernel's own schedule is timed: no cluster-tail handoff
        pb._run_multi_once(lay, M, a, b, r, iters, 0.0, schedule=s, tail_problems=-1)
        e1.record(st)
        torch.cuda.synchronize(layout.device)
        return e0.elapsed_time(e1)

    def time_fill(s):
        return run_timed(layout, M_packed, a_packed, b_packed, reg, s)

    time_tail = None
    if layout.B > tail_problems:
        big = np.argsort(-(layout.rows_np * layout.cols_np), kind="stable")[:tail_problems]
        sub = pb.RaggedLayout(layout.rows_np[big], layout.cols_np[big], layout.dtype, layout.device)
        Ms = pb.pack_dense(sub, [layout.block(M_packed, int(p)) for p in big])
        sa = torch.cat([a_packed[int(layout.r_off_np[p]):int(layout.r_off_np[p] + layout.rows_np[p])] for p in big])
        sb = torch.cat([b_packed[int(layout.c_off_np[p]):int(layout.c_off_np[p] + layout.cols_np[p])] for p in big])
        rt = torch.as_tensor(reg, dtype=torch.float64, device=layout.device).reshape(-1)
        sr = rt.expand(layout.B)[torch.as_tensor(big, device=layout.device)].contiguous() if rt.numel() > 1 \
            else rt.expand(tail_problems).contiguous()

        def time_tail(s):
            return run_timed(sub, Ms, sa, sb, sr, s)

    return t.search(key, _tag(layout.dtype), time_fill, time_tail, reps=reps)
