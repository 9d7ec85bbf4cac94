"""Float64 oracle fixtures at the benchmark configurations (run on a CPU).

    python tests/golden/gen_config_fixtures.py [online|ragged|all]

Each fixture holds seeded synthetic inputs of one benchmark configuration,
at a size the float64 oracle solves in minutes (too slow to run inside a
test), and the oracle's results:

- ``online_gmm4096_d64``: the online-cost workload (8-component Gaussian
  mixture in R^64, means ~ N(0, 4 I), covariances 0.5 I; weights uniform
  times a Dirichlet(50) perturbation, renormalised; reg = 0.01 x median
  cost) on its 4096-point subsample; oracle ``sinkhorn_log`` on the stored
  float64 cost (the reference's log-domain solver, ``ot/bregman/
  _sinkhorn.py:690-918``) at stopThr 1e-6 and converged (1e-10).
- ``ragged_cfg3``: a sample of the uneven-batch workload (n, m ~ U{32..1024},
  d in {3, 16}, points ~ U[0,1]^d, a, b ~ Dirichlet(1), reg = 10^U[-3,-1] x
  max cost) with each problem's oracle ``sinkhorn_log`` at stopThr 1e-6.

The points are stored as float32 (what the GPU solvers read); the oracle
runs on those values in float64.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle  # noqa: E402


def gmm(rng, n, d, k, mean_std, std):
    means = rng.standard_normal((k, d)) * mean_std
    return (means[rng.integers(0, k, n)] + rng.standard_normal((n, d)) * std).astype(np.float32)


def weights(rng, n):
    w = np.full(n, 1.0 / n) * rng.dirichlet(np.full(n, 50.0)) * n
    return w / w.sum()


def online(path):
    rng = np.random.default_rng(2)
    n, d = 4096, 64
    X = gmm(rng, n, d, 8, 2.0, np.sqrt(0.5))
    Y = gmm(rng, n, d, 8, 2.0, np.sqrt(0.5))
    a, b = weights(rng, n), weights(rng, n)
    C = oracle.sqeuclidean(X.astype(np.float64), Y.astype(np.float64))
    reg = 0.01 * float(np.median(C))
    out = dict(X=X, Y=Y, a=a, b=b, reg=reg)
    for tag, thr in (("", 1e-6), ("conv_", 1e-10)):
        t = time.time()
        P, lg = oracle.sinkhorn_log(a, b, C, reg, numItermax=100000, stopThr=thr)
        print("online %s: niter %d, %.0f s" % (tag or "1e-6", lg["niter"], time.time() - t), flush=True)
        out[tag + "log_u"], out[tag + "log_v"] = lg["log_u"], lg["log_v"]
        out[tag + "niter"] = lg["niter"]
        out[tag + "loss"] = float(np.sum(P * C))
    np.savez_compressed(path, **out)


def ragged(path):
    rng = np.random.default_rng(3)
    B = 24
    out = {}
    sizes, regs = [], []
    for k in range(B):
        n, m = (int(v) for v in rng.integers(32, 1025, 2))
        d = 3 if k % 2 == 0 else 16
        X = rng.random((n, d)).astype(np.float32)
        Y = rng.random((m, d)).astype(np.float32)
        a, b = rng.dirichlet(np.ones(n)), rng.dirichlet(np.ones(m))
        rel = 10 ** rng.uniform(-3, -1)
        C = oracle.sqeuclidean(X.astype(np.float64), Y.astype(np.float64))
        P, lg = oracle.sinkhorn_log(a, b, C, rel * C.max(), numItermax=100000, stopThr=1e-6)
        out.update({"X%d" % k: X, "Y%d" % k: Y, "a%d" % k: a, "b%d" % k: b, "log_u%d" % k: lg["log_u"],
                    "log_v%d" % k: lg["log_v"], "niter%d" % k: lg["niter"]})
        sizes.append((n, m, d))
        regs.append(rel)
        print("ragged %d: %dx%d d=%d rel %.1e niter %d" % (k, n, m, d, rel, lg["niter"]), flush=True)
    np.savez_compressed(path, sizes=np.array(sizes), reg_rel=np.array(regs), **out)


if __name__ == "__main__":
    which = sys.argv[1] if len(sys.argv) > 1 else "all"
    if which in ("online", "all"):
        online(os.path.join(HERE, "online_gmm4096_d64.npz"))
    if which in ("ragged", "all"):
        ragged(os.path.join(HERE, "ragged_cfg3.npz"))
