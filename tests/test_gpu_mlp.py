"""The damping controller's MLP kernels against the FP64 oracle (oracle/mlp.py).

Forward and gradient are FP32 on the GPU; tolerances are relative to the largest
magnitude: outputs 1e-5, loss 1e-5, gradient 1e-4 (FP32 accumulation over the
batch through two GELU layers).  Adam is checked step by step against its
published update rule.  The controller hook is checked for its fallback: with an
all-zero network (accept logit 0, no proposal) the LM iterations are the plain
Nielsen ones.
"""
import numpy as np
import pytest
import torch

import spgo_gb300.scenes as scenes
from spgo_gb300 import learned
from spgo_gb300.solver import BatchSolver
from oracle import mlp as M
from oracle import solver as S

pytestmark = pytest.mark.gpu


def batch(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(0.0, 1.5, (n, M.D_IN)).astype(np.float32)
    T = np.stack([rng.normal(0.0, 2.0, n), rng.integers(0, 2, n)], 1).astype(np.float32)
    return X, T


def rel(a, b):
    return float(np.abs(np.asarray(a, np.float64) - b).max() / max(np.abs(b).max(), 1e-30))


@pytest.mark.parametrize("n", [1, 37, 1000])
def test_forward_matches_oracle(built_lib, cuda_device, n):
    theta = M.init(seed=3)
    X, _ = batch(n, 10 + n)
    ctl = learned.Controller(theta)
    out = ctl.forward(X)
    ref, _ = M.forward(theta.astype(np.float64), X.astype(np.float64))
    assert rel(out, ref) < 1e-5


@pytest.mark.parametrize("n", [1, 129, 4096])
def test_gradient_matches_oracle(built_lib, cuda_device, n):
    theta = M.init(seed=5)
    X, T = batch(n, 20 + n)
    ctl = learned.Controller(theta)
    loss, g = ctl.grad(X, T)
    ref_loss, ref_g = M.loss_and_grad(theta.astype(np.float64), X.astype(np.float64), T.astype(np.float64))
    assert abs(loss - ref_loss) / abs(ref_loss) < 1e-5
    assert rel(g.cpu().numpy(), ref_g) < 1e-4


def test_adam_matches_update_rule(built_lib, cuda_device):
    theta = M.init(seed=7)
    X, T = batch(256, 7)
    ctl = learned.Controller(theta)
    th = theta.astype(np.float64)
    m = np.zeros_like(th)
    v = np.zeros_like(th)
    lr, b1, b2, e = 1e-3, 0.9, 0.999, 1e-8
    import ctypes as C
    st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for step in range(1, 4):
        _, g = ctl.grad(X, T)
        gn = g.cpu().numpy().astype(np.float64)
        ctl.L.spgo_mlp_adam(C.c_void_p(ctl.theta.data_ptr()), C.c_void_p(g.data_ptr()),
                            C.c_void_p(ctl.m.data_ptr()), C.c_void_p(ctl.v.data_ptr()), step, C.c_float(lr), st)
        torch.cuda.synchronize()
        m = b1 * m + (1 - b1) * gn
        v = b2 * v + (1 - b2) * gn * gn
        th = th - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + e)
        # continue the reference from the GPU's parameters so FP32 rounding does not accumulate
        got = ctl.theta.cpu().numpy().astype(np.float64)
        assert np.abs(got - th).max() < 1e-6 + 1e-5 * np.abs(th).max()
        th = got


def test_training_reduces_loss(built_lib, cuda_device):
    """GPU training on a fixed regression target lowers the loss by 10x."""
    rng = np.random.default_rng(0)
    X = rng.normal(0.0, 1.0, (2048, M.D_IN)).astype(np.float32)
    T = np.stack([np.tanh(X[:, 0] - 0.5 * X[:, 5]), (X[:, 2] > 0)], 1).astype(np.float32)
    ctl = learned.Controller(seed=1)
    hist = ctl.train(learned.Traces(X, T), epochs=40, batch=256, lr=3e-3)
    assert hist[-1] < 0.1 * hist[0]


def test_deployed_network_folds_standardisation(built_lib, cuda_device):
    """The deployed parameters on raw features equal the trained network on
    standardised features."""
    rng = np.random.default_rng(4)
    X = (rng.normal(0.0, 1.0, (300, M.D_IN)) * rng.uniform(0.1, 30.0, M.D_IN) + rng.normal(0, 20, M.D_IN))
    ctl = learned.Controller(M.init(seed=9))
    ctl.fit_normalization(X)
    got = ctl.forward(X.astype(np.float32))
    ref, _ = M.forward(ctl.theta.cpu().numpy().astype(np.float64), (X - ctl.mu) / ctl.sd)
    assert rel(got, ref) < 1e-4


def f32_obs(p):
    q = p.copy()
    q.obs_uv = p.obs_uv.astype(np.float32).astype(np.float64)
    q.anchor_uv = p.anchor_uv.astype(np.float32).astype(np.float64)
    q.intrinsics = p.intrinsics.astype(np.float32).astype(np.float64)
    return q


def test_zero_controller_is_nielsen(built_lib, cuda_device):
    """An all-zero network never overrides (logit 0): the iterations are the plain
    schedule's, and both reach the FP64 oracle's cost."""
    probs = [scenes.circle_scene(s, n, l) for s, n, l in [(501, 8, 300), (502, 12, 500)]]
    res = [S.lm_solve(f32_obs(p), S.Loss(), max_iters=30, tol=1e-6) for p in probs]
    runs = []
    for ctl in (None, torch.zeros(M.N_PARAMS, dtype=torch.float32, device="cuda")):
        bs = BatchSolver(probs, precision="fp64")
        bs.set_params(loss="l2", max_iters=30, tol=1e-6, use_graph=0)
        bs.set_controller(ctl)
        runs.append(bs.solve())
        bs.close()
    for b, r in enumerate(res):
        assert runs[0][b]["iterations"] == runs[1][b]["iterations"]
        assert abs(runs[0][b]["cost"] - runs[1][b]["cost"]) / r.cost < 1e-12
        assert abs(runs[1][b]["cost"] - r.cost) / r.cost < 1e-6


def test_trained_controller_beats_nielsen_on_heldout(built_lib, cuda_device):
    """The shipped network (trained on other seeds) reaches the plain FP64 solver's
    cost in fewer LM iterations than the plain schedule, on held-out problems."""
    import os
    if not os.path.exists(learned.DEFAULT_WEIGHTS):
        pytest.fail("controller weights missing")
    probs = scenes.config3(seed=2500, n_problems=192)
    bs = BatchSolver(probs, precision="fp64")
    bs.set_params(loss="l2", max_iters=30, tol=1e-6)
    targets = np.array([s["cost"] for s in bs.solve()])
    bs.close()
    ctl = learned.Controller.load(device="cuda")
    plain, _, _ = learned.iterations_to_target(probs, None, targets, precision="mixed")
    lrn, costs, _ = learned.iterations_to_target(probs, ctl, targets, precision="mixed")
    # mean LM iterations until the plain FP64 cost is reached (a miss counts 31)
    assert lrn.mean() < 0.9 * plain.mean(), (lrn.mean(), plain.mean())


def test_controller_features_match_the_lm_state(built_lib, cuda_device):
    """The 16 inputs (one warp per problem, the logarithms spread over the lanes)
    against what the status read-back implies: log cost per residual, log of the
    cost ratio, log lambda, the iteration index; all finite and inside [-40, 40]."""
    probs = [scenes.circle_scene(s, n, l) for s, n, l in [(91, 6, 80), (92, 9, 150), (93, 12, 300)]]
    bs = BatchSolver(probs, precision="mixed")
    bs.set_params(loss="l2", max_iters=30, tol=1e-6)
    bs.reset()
    bs.iterate(3)
    F = bs.features()
    st = bs.status()
    assert np.isfinite(F).all() and np.abs(F).max() <= 40.0
    for b, p in enumerate(probs):
        s = st[b]
        assert F[b, 0] == pytest.approx(np.log10(s["cost"]) - np.log10(4 * p.n_obs), abs=1e-5)
        assert F[b, 1] == pytest.approx(np.log10(s["cost"]) - np.log10(s["cost0"]), abs=1e-5)
        assert F[b, 5] == pytest.approx(np.log10(s["lam"]), abs=1e-5)
        assert F[b, 10] == pytest.approx(s["iterations"] / 30.0, abs=1e-6)
        assert F[b, 14] == np.rint(F[b, 14]) and F[b, 14] >= 1.0   # log2 of nu, a power of two
    bs.close()
