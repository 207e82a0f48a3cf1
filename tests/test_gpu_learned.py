"""The learned initial guess: the CUDA network against the FP64 oracle (forward and
gradients), training, and what the trained network gains on held-out problems."""
import os

import numpy as np
import pytest

from oracle import mlp as OM
from petrbf_gb300 import learned as L
from petrbf_gb300 import workloads as W
from petrbf_gb300.api import Context

pytestmark = pytest.mark.gpu


def _small_patches():
    p = L.training_problem(4242, m=200)
    with Context(dim=2, sigma=p.sigma) as c:
        g, st = c.interpolate(p.x, p.y, None, p.f)
        X, S, T, M = L.patches(c, p.x, p.y, p.f, g)
    return X, S, T, M


def _informative(X):
    return np.flatnonzero(np.abs(X[:, 2::4]).max(axis=1) > 1e-3)


# The network's GEMMs take BF16 operands on the tensor cores; the oracle rounds the same
# operands to BF16 and sums in FP64. What remains is FP32 accumulation and the rare operand
# whose FP32 and FP64 values round to neighbouring BF16 numbers (2^-8 apart).
RTOL_NET = 2e-3


@pytest.mark.parametrize("nrows", [48, 300])
def test_forward_and_gradients_match_cpu_oracle(nrows):
    X, S, T, M = _small_patches()
    idx = _informative(X)[:nrows]  # patches with signal (300: several 128-row tiles, a ragged one)
    X, T, M = X[idx], T[idx], M[idx]
    net = L.Network(seed=3)
    w = net.weights
    Y = net.forward(X)
    Yo = OM.forward(w, X)[-1]
    assert np.abs(Y - Yo).max() <= RTOL_NET * max(1.0, np.abs(Yo).max())
    loss, g = net.loss_grad(X, T, M)
    loss_o, g_o = OM.loss_grad(w, X, T, M)
    assert abs(loss - loss_o) <= RTOL_NET * loss_o
    assert np.linalg.norm(g - g_o) <= RTOL_NET * np.linalg.norm(g_o)
    # and far from the network without the operand rounding: the rounding is modelled
    _, g_fp = OM.loss_grad(w, X, T, M, bf16_operands=False)
    assert np.linalg.norm(g - g_o) < np.linalg.norm(g - g_fp)


def test_training_reduces_the_loss():
    X, S, T, M = _small_patches()
    k = _informative(X)
    X, T, M = X[k], T[k], M[k]
    net = L.Network(seed=5)
    hist = net.train(X, T, M, epochs=15, batch=256, lr=1e-3, seed=1)
    assert hist[-1] < 0.3 * hist[0]


@pytest.mark.skipif(not os.path.exists(L.MODEL_PATH), reason="trained model not present")
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_trained_guess_reduces_iterations_on_held_out_problem(precision):
    p = L.training_problem(777, m=500)  # held out (training used seeds 1000..1007, m=1000)
    with Context(dim=2, sigma=p.sigma, precision=precision) as c:
        g0, st0 = c.interpolate(p.x, p.y, None, p.f)
    with Context(dim=2, sigma=p.sigma, precision=precision, guess="learned") as c:
        L.install(c)
        g1, st1 = c.interpolate(p.x, p.y, None, p.f)
    assert st0.reason == 2 and st1.reason == 2
    # guess_rel_resid: the guess's true residual relative to ||f|| (mixed), its
    # preconditioned residual relative to ||B f|| (plain)
    assert st1.guess_used == 1 and st1.guess_rel_resid < (0.1 if precision == "mixed" else 0.5)
    # the same final residual, reached in fewer Krylov (or refinement) iterations
    if precision == "fp64":
        assert st1.its < st0.its
    else:
        assert st1.true_rel_resid <= 1e-13
        assert (st1.outer_its, st1.its) < (st0.outer_its, st0.its)
    assert np.linalg.norm(g1 - g0) <= 1e-6 * np.linalg.norm(g0)
