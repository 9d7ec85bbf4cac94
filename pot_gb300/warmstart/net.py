"""The warm-start network: forward, backward and AdamW on the GPU through the
kernels of ``csrc/mlp.cu``.

Architecture (d-dimensional clouds, P pairs of n source / m target points):
    hx = relu(relu(X W1x + b1x) W2x + b2x)      per source point
    hy = relu(relu(Y W1y + b1y) W2y + b2y)      per target point
    sX = mean_i hx,  sY = mean_j hy             pooled summaries
    z  = [x_i, sX, sY]
    f_i = relu(relu(z W3 + b3) W4 + b4) W5 + b5
z may carry extra per-point inputs (the soft-min distances of x_i to the
target measure at several temperatures).  The clouds are first centred on
their joint mean and scaled by 1 / sqrt(max cost), so f is in units of the
max-normalised cost.
"""
import ctypes
import math

import numpy as np
import torch

from .. import _lib

PARAM_SHAPES = None


def param_shapes(d, h1=64, h2=64, h3=128, dz=None):
    z = (d if dz is None else dz) + 2 * h2
    return [("W1x", (d, h1)), ("b1x", (h1,)), ("W2x", (h1, h2)), ("b2x", (h2,)),
            ("W1y", (d, h1)), ("b1y", (h1,)), ("W2y", (h1, h2)), ("b2y", (h2,)),
            ("W3", (z, h3)), ("b3", (h3,)), ("W4", (h3, h3)), ("b4", (h3,)),
            ("W5", (h3, 1)), ("b5", (1,))]


def init_params(d, seed=0, h1=64, h2=64, h3=128, dz=None):
    rng = np.random.default_rng(seed)
    out = {}
    for name, shp in param_shapes(d, h1, h2, h3, dz):
        if name.startswith("W"):
            out[name] = (rng.standard_normal(shp) * math.sqrt(2.0 / shp[0])).astype(np.float32)
        else:
            out[name] = np.zeros(shp, dtype=np.float32)
    out["W5"] *= 0.1
    return out


def _p(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


class WarmStartNet:
    """Parameters live in one flat device buffer (views per tensor), so the
    AdamW step is one kernel launch over all of them."""

    def __init__(self, d, params=None, device=None, seed=0, h1=64, h2=64, h3=128, dz=None):
        self.d, self.h1, self.h2, self.h3 = d, h1, h2, h3
        self.dz = d if dz is None else dz
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.shapes = param_shapes(d, h1, h2, h3, self.dz)
        sizes = [int(np.prod(s)) for _, s in self.shapes]
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        self.flat = torch.zeros(int(self.offsets[-1]), dtype=torch.float32, device=self.device)
        self.grad = torch.zeros_like(self.flat)
        self.m = torch.zeros_like(self.flat)
        self.v = torch.zeros_like(self.flat)
        self.step_count = 0
        src = params if params is not None else init_params(d, seed, h1, h2, h3, self.dz)
        self.load(src)
        self.lib = _lib.load()

    def view(self, buf, name):
        k = [n for n, _ in self.shapes].index(name)
        shp = self.shapes[k][1]
        return buf[int(self.offsets[k]):int(self.offsets[k + 1])].view(*shp)

    def P(self, name):
        return self.view(self.flat, name)

    def G(self, name):
        return self.view(self.grad, name)

    def load(self, params):
        for name, _ in self.shapes:
            self.P(name).copy_(torch.as_tensor(np.asarray(params[name]), dtype=torch.float32))

    def state(self):
        return {name: self.P(name).detach().cpu().numpy().copy() for name, _ in self.shapes}

    # -- primitive launches ------------------------------------------------
    def _st(self):
        return _lib.stream_handle(self.device)

    def _gemm(self, ta, tb, M, N, K, A, lda, B, ldb, C, ldc, beta=0.0, bias=None, relu=False, alpha=1.0):
        _lib.check(self.lib.otg_gemm_f32(int(ta), int(tb), M, N, K, alpha, _p(A), lda, _p(B), ldb, beta, _p(C), ldc,
                                         _p(bias), int(relu), self._st()), "otg_gemm_f32")

    def _linear(self, X, W, b, relu):
        R, K = X.shape
        N = W.shape[1]
        Y = torch.empty(R, N, dtype=torch.float32, device=self.device)
        self._gemm(0, 0, R, N, K, X, K, W, N, Y, N, bias=b, relu=relu)
        return Y

    def _linear_bwd(self, X, W, dY, Wname, bname, need_dx=True):
        """dY already masked; fills dW, db; returns dX."""
        R, K = X.shape
        N = W.shape[1]
        dW, db = self.G(Wname), self.G(bname)
        self._gemm(1, 0, K, N, R, X, K, dY, N, dW, N)              # dW = X^T dY
        _lib.check(self.lib.otg_mlp_colsum(_p(dY), R, N, _p(db), self._st()), "otg_mlp_colsum")
        if not need_dx:
            return None
        dX = torch.empty(R, K, dtype=torch.float32, device=self.device)
        self._gemm(0, 1, R, K, N, dY, N, W, N, dX, K)              # dX = dY W^T
        return dX

    def _relu_bwd(self, dY, Y):
        _lib.check(self.lib.otg_mlp_relu_bwd(_p(dY), _p(Y), dY.numel(), self._st()), "otg_mlp_relu_bwd")

    # -- network -------------------------------------------------------------
    def forward(self, X, Y, P, n, m, Z=None, keep=False):
        """X: (P*n, d), Y: (P*m, d) normalised clouds, Z: (P*n, dz) per-point
        head inputs (default X) -> f (P*n,)."""
        d = self.dz
        Z = X if Z is None else Z
        hx1 = self._linear(X, self.P("W1x"), self.P("b1x"), True)
        hx2 = self._linear(hx1, self.P("W2x"), self.P("b2x"), True)
        hy1 = self._linear(Y, self.P("W1y"), self.P("b1y"), True)
        hy2 = self._linear(hy1, self.P("W2y"), self.P("b2y"), True)
        sX = torch.empty(P, self.h2, dtype=torch.float32, device=self.device)
        sY = torch.empty(P, self.h2, dtype=torch.float32, device=self.device)
        _lib.check(self.lib.otg_mlp_segment_mean(_p(hx2), P, n, self.h2, _p(sX), self._st()), "segment_mean")
        _lib.check(self.lib.otg_mlp_segment_mean(_p(hy2), P, m, self.h2, _p(sY), self._st()), "segment_mean")
        z = torch.empty(P * n, d + 2 * self.h2, dtype=torch.float32, device=self.device)
        _lib.check(self.lib.otg_mlp_concat3(_p(Z), _p(sX), _p(sY), P, n, d, self.h2, _p(z), self._st()), "concat3")
        h3 = self._linear(z, self.P("W3"), self.P("b3"), True)
        h4 = self._linear(h3, self.P("W4"), self.P("b4"), True)
        f = self._linear(h4, self.P("W5"), self.P("b5"), False)
        if keep:
            self._cache = (X, Y, P, n, m, hx1, hx2, hy1, hy2, z, h3, h4)
        return f.view(-1)

    def infer(self, X, Y, P, n, m, Z):
        """The forward pass for prediction: fused kernels (encoder + pooling,
        head with the summaries folded into a per-pair bias) for the shipped
        sizes, no activations stored; the layer-by-layer forward otherwise."""
        sX = torch.empty(P, self.h2, dtype=torch.float32, device=self.device)
        sY = torch.empty(P, self.h2, dtype=torch.float32, device=self.device)
        f = torch.empty(P * n, dtype=torch.float32, device=self.device)
        lib, st = self.lib, self._st()
        rc = lib.otg_mlp_encode_pool(_p(X), P, n, self.d, self.h1, self.h2, _p(self.P("W1x")), _p(self.P("b1x")),
                                     _p(self.P("W2x")), _p(self.P("b2x")), _p(sX), st)
        if rc == -5:  # OTG_ERR_UNSUPPORTED: not the shipped sizes
            return self.forward(X, Y, P, n, m, Z=Z)
        _lib.check(rc, "otg_mlp_encode_pool")
        _lib.check(lib.otg_mlp_encode_pool(_p(Y), P, m, self.d, self.h1, self.h2, _p(self.P("W1y")),
                                           _p(self.P("b1y")), _p(self.P("W2y")), _p(self.P("b2y")), _p(sY), st),
                   "otg_mlp_encode_pool")
        rc = lib.otg_mlp_head(_p(Z), P, n, self.dz, self.h2, self.h3, _p(sX), _p(sY), _p(self.P("W3")),
                              _p(self.P("b3")), _p(self.P("W4")), _p(self.P("b4")), _p(self.P("W5")),
                              _p(self.P("b5")), _p(f), st)
        if rc == -5:
            return self.forward(X, Y, P, n, m, Z=Z)
        _lib.check(rc, "otg_mlp_head")
        return f

    def backward(self, df):
        X, Y, P, n, m, hx1, hx2, hy1, hy2, z, h3, h4 = self._cache
        d = self.dz
        df = df.view(-1, 1)
        dh4 = self._linear_bwd(h4, self.P("W5"), df, "W5", "b5")
        self._relu_bwd(dh4, h4)
        dh3 = self._linear_bwd(h3, self.P("W4"), dh4, "W4", "b4")
        self._relu_bwd(dh3, h3)
        dz = self._linear_bwd(z, self.P("W3"), dh3, "W3", "b3")
        dsX = torch.empty(P, self.h2, dtype=torch.float32, device=self.device)
        dsY = torch.empty(P, self.h2, dtype=torch.float32, device=self.device)
        _lib.check(self.lib.otg_mlp_concat3_bwd(_p(dz), P, n, d, self.h2, _p(dsX), _p(dsY), self._st()), "concat3_bwd")
        for side, s_grad, h1, h2, rows, inp in (("x", dsX, hx1, hx2, n, X), ("y", dsY, hy1, hy2, m, Y)):
            dh2 = torch.empty_like(h2)
            _lib.check(self.lib.otg_mlp_segment_mean_bwd(_p(s_grad), P, rows, self.h2, _p(dh2), 0, self._st()),
                       "segment_mean_bwd")
            self._relu_bwd(dh2, h2)
            dh1 = self._linear_bwd(h1, self.P("W2" + side), dh2, "W2" + side, "b2" + side)
            self._relu_bwd(dh1, h1)
            self._linear_bwd(inp, self.P("W1" + side), dh1, "W1" + side, "b1" + side, need_dx=False)
        self._cache = None

    def loss_and_grad(self, f, t, P, n):
        loss = torch.empty(1, dtype=torch.float64, device=self.device)
        df = torch.empty_like(f)
        _lib.check(self.lib.otg_mlp_centered_mse(_p(f), _p(t), P, n, _p(loss), _p(df), self._st()), "centered_mse")
        return loss, df

    def adamw(self, lr, b1=0.9, b2=0.999, eps=1e-8, wd=1e-4):
        self.step_count += 1
        _lib.check(self.lib.otg_mlp_adamw(_p(self.flat), _p(self.grad), _p(self.m), _p(self.v), self.flat.numel(),
                                          lr, b1, b2, eps, wd, self.step_count, self._st()), "otg_mlp_adamw")


def normalise_pairs(X, Y, maxc):
    """Centre each pair on the joint mean of its points and scale by
    1/sqrt(max cost): the cost then lies in [0, 1] and the network sees the
    translation- and scale-free geometry.  X: (P, n, d), Y: (P, m, d),
    maxc: (P,) max squared distance."""
    mu = torch.cat([X, Y], 1).mean(1, keepdim=True)
    s = torch.rsqrt(maxc.clamp_min(1e-30)).view(-1, 1, 1).to(X.dtype)
    return ((X - mu) * s).contiguous(), ((Y - mu) * s).contiguous()
