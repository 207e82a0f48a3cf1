"""The learned initial guess: training data from plain solves, training with the
library's own CUDA kernels, and the model file.

A problem of the training set is a seeded Lamb-Oseen field omega = G/(pi rc^2)
exp(-|x - c|^2 / rc^2) with G in [0.5, 2], core radius rc in [0.1, 0.3] and centre c in
[-0.5, 0.5]^2, sampled on a 1000 x 1000 lattice over [-1,1]^2 with +/-0.25h jitter
(N = 10^6), sigma = h/0.8. The plain FP64 solver produces its weights; every fine cell
(2 sigma edge) of the solved problem is a patch (features of its 3 x 3 neighbourhood,
targets = the centre cell's normalised weights). Patches whose field amplitude is
negligible are mostly skipped.
"""
import ctypes
import math
import os

import numpy as np

from . import _native as N
from . import workloads as W
from ._native import PrbfError

MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "guess_mlp.npz")
IN, HID, OUT = 256, 256, 16
_F = ctypes.POINTER(ctypes.c_float)
_D = ctypes.POINTER(ctypes.c_double)


def _fp(a):
    return a.ctypes.data_as(_F)


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def _check_shapes(X, T=None, M=None):
    """X holds rows of IN features, T and M rows of OUT values, one per row of X."""
    if X.ndim != 2 or X.shape[1] != IN:
        raise ValueError(f"features must be [n, {IN}], got {X.shape}")
    for name, a in (("T", T), ("M", M)):
        if a is not None and a.shape != (X.shape[0], OUT):
            raise ValueError(f"{name} must be [{X.shape[0]}, {OUT}], got {a.shape}")


def _check_points(x, *arrays):
    for a in arrays:
        if a is not None and a.shape[0] != x.shape[0]:
            raise ValueError(f"arrays of {a.shape[0]} and {x.shape[0]} points")


def param_count():
    return int(N.lib().prbf_mlp_param_count())


class Network:
    """The per-cell MLP on one GPU (prbf_mlp)."""

    def __init__(self, seed=0, device=0):
        h = ctypes.c_void_p()
        st = N.lib().prbf_mlp_create(int(device), int(seed), ctypes.byref(h))
        if st:
            raise PrbfError(st, "prbf_mlp_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            N.lib().prbf_mlp_destroy(self.h)
            self.h = None

    __del__ = close

    def _chk(self, st, what):
        if st:
            raise PrbfError(st, what)

    @property
    def weights(self):
        w = np.empty(param_count(), np.float32)
        self._chk(N.lib().prbf_mlp_get_weights(self.h, _fp(w)), "get_weights")
        return w

    @weights.setter
    def weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        if w.size != param_count():
            raise ValueError(f"{w.size} weights, the network has {param_count()}")
        self._chk(N.lib().prbf_mlp_set_weights(self.h, _fp(w)), "set_weights")

    def forward(self, X):
        X = np.ascontiguousarray(X, np.float32)
        _check_shapes(X)
        Y = np.empty((X.shape[0], OUT), np.float32)
        self._chk(N.lib().prbf_mlp_forward(self.h, X.shape[0], _fp(X), _fp(Y)), "forward")
        return Y

    def loss_grad(self, X, T, M):
        X, T, M = (np.ascontiguousarray(a, np.float32) for a in (X, T, M))
        _check_shapes(X, T, M)
        g = np.empty(param_count(), np.float32)
        loss = ctypes.c_float(0)
        self._chk(N.lib().prbf_mlp_loss_grad(self.h, X.shape[0], _fp(X), _fp(T), _fp(M),
                                             ctypes.byref(loss), _fp(g)), "loss_grad")
        return float(loss.value), g

    def train(self, X, T, M, epochs=40, batch=512, lr=1e-3, seed=1):
        X, T, M = (np.ascontiguousarray(a, np.float32) for a in (X, T, M))
        _check_shapes(X, T, M)
        hist = np.zeros(max(epochs, 1), np.float32)
        self._chk(N.lib().prbf_mlp_train(self.h, X.shape[0], _fp(X), _fp(T), _fp(M), int(epochs),
                                         int(batch), float(lr), int(seed), _fp(hist)), "train")
        return hist[:epochs]


def patches(ctx, x, y, f, g=None):
    """Features X [npatch, 256], per-patch output scale and (with g) targets T and masks M."""
    x, y, f = (np.ascontiguousarray(a, np.float64) for a in (x, y, f))
    g = None if g is None else np.ascontiguousarray(g, np.float64)
    _check_points(x, y, f, g)
    L = N.lib()
    npatch = ctypes.c_int(0)
    ctx._check(L.prbf_guess_patches(ctx.h, len(x), _dp(x), _dp(y), _dp(f), _dp(g), None, None, None,
                                    None, ctypes.byref(npatch)))
    n = npatch.value
    X = np.empty((n, IN), np.float32)
    S = np.empty(n, np.float32)
    T = np.empty((n, OUT), np.float32) if g is not None else None
    M = np.empty((n, OUT), np.float32) if g is not None else None
    ctx._check(L.prbf_guess_patches(ctx.h, len(x), _dp(x), _dp(y), _dp(f), _dp(g), _fp(X), _fp(S),
                                    _fp(T) if T is not None else None,
                                    _fp(M) if M is not None else None, ctypes.byref(npatch)))
    return (X, S, T, M) if g is not None else (X, S)


def lamb_oseen_core(x, y, G, rc, xc, yc):
    return G / (math.pi * rc * rc) * np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / (rc * rc))


def training_problem(seed, m=1000):
    """One seeded Lamb-Oseen problem of the training distribution (N = m^2 jittered)."""
    rng = np.random.default_rng(seed)
    G, rc = rng.uniform(0.5, 2.0), rng.uniform(0.1, 0.3)
    xc, yc = rng.uniform(-0.5, 0.5, 2)
    x, y, h = W.lattice_2d(m, jitter=0.25, seed=seed + 7919)
    f = lamb_oseen_core(x, y, G, rc, xc, yc)
    return W.Problem("lamb_oseen_train_%d" % seed, x, y, None, f, h / 0.8, 8, 24, 24, exact=f,
                     meta={"G": G, "rc": rc, "centre": (xc, yc), "h": h})


def make_dataset(seeds, per_problem=12500, m=1000, device=0, rng_seed=0):
    """Patches (features, targets, masks) of plain FP64 solves of the given problems."""
    from .api import Context
    rng = np.random.default_rng(rng_seed)
    Xs, Ts, Ms = [], [], []
    for sd in seeds:
        p = training_problem(sd, m)
        with Context(dim=2, sigma=p.sigma, nsigma_box=8, sigma_buffer=24, sigma_trunc=24,
                     device=device) as c:
            g, st = c.interpolate(p.x, p.y, None, p.f)
            X, S, T, M = patches(c, p.x, p.y, p.f, g)
        # keep the patches where the field is not negligible against the problem's peak
        # (features hold f / max|f|)
        sig = np.flatnonzero(np.abs(X[:, 2::4]).max(axis=1) > 1e-3)
        pick = sig if len(sig) <= per_problem else rng.choice(sig, per_problem, replace=False)
        Xs.append(X[pick])
        Ts.append(T[pick])
        Ms.append(M[pick])
    return np.concatenate(Xs), np.concatenate(Ts), np.concatenate(Ms)


def save(weights, path=MODEL_PATH, **meta):
    os.makedirs(os.path.dirname(path), exist_ok=True)
    np.savez_compressed(path, weights=np.asarray(weights, np.float32),
                        **{k: np.asarray(v) for k, v in meta.items()})


def load(path=MODEL_PATH):
    d = np.load(path)
    return d["weights"].astype(np.float32)


def install(ctx, weights=None):
    """Puts the trained weights in a Context so PRBF_GUESS_LEARNED solves can use them."""
    w = load() if weights is None else np.ascontiguousarray(weights, np.float32)
    if w.size != param_count():
        raise ValueError(f"{w.size} weights, the network has {param_count()}")
    ctx._check(N.lib().prbf_guess_set_weights(ctx.h, _fp(w)))


def guess(ctx, x, y, f):
    x, y, f = (np.ascontiguousarray(a, np.float64) for a in (x, y, f))
    _check_points(x, y, f)
    g0 = np.empty_like(x)
    ctx._check(N.lib().prbf_guess_eval(ctx.h, len(x), _dp(x), _dp(y), _dp(f), _dp(g0)))
    return g0


def train_default(out=MODEL_PATH, nproblems=8, per_problem=12500, epochs=60, device=0, log=print):
    """The model shipped in data/: 8 training problems (seeds 1000..1007), ~10^5 patches."""
    import time
    t0 = time.time()
    X, T, M = make_dataset(range(1000, 1000 + nproblems), per_problem=per_problem, device=device)
    log("dataset: %d patches in %.1f s" % (len(X), time.time() - t0))
    net = Network(seed=20261203, device=device)
    t1 = time.time()
    hist = net.train(X, T, M, epochs=epochs, batch=512, lr=1e-3, seed=7)
    hist2 = net.train(X, T, M, epochs=max(epochs // 3, 1), batch=512, lr=2e-4, seed=8)
    log("training: %.1f s, loss %.4g -> %.4g -> %.4g" % (time.time() - t1, hist[0], hist[-1], hist2[-1]))
    save(net.weights, out, loss=np.concatenate([hist, hist2]), npatch=len(X))
    return net


if __name__ == "__main__":
    train_default()
