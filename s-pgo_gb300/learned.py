"""Learned LM damping controller: trace collection, GPU training, evaluation.

The controller is a 16 -> 64 -> 64 -> 2 MLP (``include/spgo.h``,
``csrc/k_mlp.cu``).  Training data come from plain Nielsen-LM runs: at every
iteration of every problem still running, the solver probes the step cost for a
grid of damping factors f (lambda * f) without changing its state; the target
for the first output is log10 of the factor with the lowest cost, the target
for the second is whether that factor gives a lower cost than the schedule's
own lambda (f = 1).  Inputs are standardised with the training set's mean and
spread, folded into the first layer when the network is deployed, so the
solver's kernels read raw features.  Training runs the library's own
forward/backward/Adam kernels.  At solve time the BF16 network sets lambda at
the first iteration and after accepted steps when its second output says the
schedule should be overridden; a rejected step always falls back to Nielsen
(S-PGO itself has no damping schedule, so there is no reference counterpart).
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import native as nat
from .solver import BatchSolver

FACTORS = np.array([1e-6, 1e-4, 1e-3, 1e-2, 1e-1, 1.0, 10.0, 100.0, 1000.0])
SHAPES = [(64, 16), (64,), (64, 64), (64,), (2, 64), (2,)]
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "controller_weights.npz")


def _vp(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


@dataclasses.dataclass
class Traces:
    X: np.ndarray   # [n, 16]
    T: np.ndarray   # [n, 2]


def targets_from_probe(costs: np.ndarray, F: float, factors=FACTORS):
    """(t0, t1) of one problem-iteration from the probed step costs (see module doc)."""
    one = int(np.argmin(np.abs(np.log10(factors))))
    c = np.where(np.isfinite(costs), costs, np.inf)
    k = int(np.argmin(c))
    t0 = float(np.log10(factors[k]))
    t1 = 1.0 if c[k] < c[one] - 1e-9 * abs(F) else 0.0
    return t0, t1


def collect_traces(problems, max_iters=30, tol=1e-6, device="cuda", precision="mixed",
                   factors=FACTORS) -> Traces:
    """Plain-LM traces with per-iteration damping probes (see module doc)."""
    bs = BatchSolver(problems, precision=precision, device=device)
    bs.set_params(loss="l2", max_iters=max_iters, tol=tol, use_graph=0)
    bs.reset()
    X, T = [], []
    for _ in range(max_iters):
        costs = bs.probe(factors)              # also linearises at the current states
        feats = bs.features()
        st = bs.status()
        running = [b for b, s in enumerate(st) if s["status"] == nat.STATUS_RUNNING]
        if not running:
            break
        for b in running:
            X.append(feats[b])
            T.append(targets_from_probe(costs[:, b], st[b]["cost"], factors))
        bs.iterate(1)
    bs.close()
    return Traces(np.asarray(X, np.float32), np.asarray(T, np.float32))


def init_params(seed=0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    parts = []
    for shape in SHAPES:
        parts.append(rng.normal(0.0, np.sqrt(2.0 / shape[1]), shape).ravel() if len(shape) == 2 else np.zeros(shape))
    return np.concatenate(parts).astype(np.float32)


class Controller:
    """MLP parameters on the device (``theta``, acting on standardised inputs),
    trained with the library's kernels; ``deployed()`` gives the parameters the
    solver runs (standardisation folded into the first layer)."""

    def __init__(self, theta: Optional[np.ndarray] = None, mu: Optional[np.ndarray] = None,
                 sd: Optional[np.ndarray] = None, device="cuda", seed=0):
        self.L = nat.lib()
        self.device = torch.device(device)
        if theta is None:
            theta = init_params(seed)
        self.theta = torch.tensor(np.asarray(theta, np.float32), device=self.device)
        assert self.theta.numel() == nat.MLP_PARAMS
        self.mu = np.zeros(nat.MLP_INPUTS) if mu is None else np.asarray(mu, np.float64)
        self.sd = np.ones(nat.MLP_INPUTS) if sd is None else np.asarray(sd, np.float64)
        self.m = torch.zeros_like(self.theta)
        self.v = torch.zeros_like(self.theta)
        self.step = 0

    # -- persistence -----------------------------------------------------------------
    def save(self, path: str):
        np.savez(path, theta=self.theta.cpu().numpy(), mu=self.mu, sd=self.sd)

    @classmethod
    def load(cls, path: str = DEFAULT_WEIGHTS, device="cuda") -> "Controller":
        d = np.load(path)
        return cls(d["theta"], d["mu"], d["sd"], device=device)

    def deployed(self) -> torch.Tensor:
        th = self.theta.detach().cpu().numpy().astype(np.float64)
        W1 = th[:64 * 16].reshape(64, 16) / self.sd[None, :]
        b1 = th[64 * 16:64 * 17] - W1 @ self.mu
        out = th.copy()
        out[:64 * 16] = W1.ravel()
        out[64 * 16:64 * 17] = b1
        return torch.tensor(out.astype(np.float32), device=self.device)

    def _norm(self, X: np.ndarray) -> np.ndarray:
        return ((np.asarray(X, np.float64) - self.mu) / self.sd).astype(np.float32)

    # -- kernels ---------------------------------------------------------------------
    def grad(self, X: np.ndarray, T: np.ndarray):
        """(mean loss, gradient w.r.t. theta) of a batch, from the CUDA kernels."""
        n = X.shape[0]
        dX = torch.tensor(self._norm(X), device=self.device)
        dT = torch.tensor(np.asarray(T, np.float32), device=self.device)
        g = torch.zeros(nat.MLP_PARAMS, dtype=torch.float32, device=self.device)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        out = torch.zeros(2 * n, dtype=torch.float32, device=self.device)
        cache = torch.zeros(nat.MLP_CACHE_PER_SAMPLE * n, dtype=torch.float32, device=self.device)
        st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        nat.check(self.L.spgo_mlp_grad(_vp(self.theta), _vp(dX), _vp(dT), n, _vp(g), _vp(loss), _vp(out),
                                       _vp(cache), st), "mlp_grad")
        torch.cuda.synchronize(self.device)
        return float(loss.item()), g

    def forward(self, X: np.ndarray) -> np.ndarray:
        """FP32 outputs of the deployed network on raw features."""
        n = X.shape[0]
        dX = torch.tensor(np.asarray(X, np.float32), device=self.device)
        out = torch.zeros(2 * n, dtype=torch.float32, device=self.device)
        params = self.deployed()
        st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        nat.check(self.L.spgo_mlp_forward(_vp(params), _vp(dX), n, _vp(out), C.c_void_p(0), st), "mlp_fwd")
        torch.cuda.synchronize(self.device)
        return out.cpu().numpy().reshape(n, 2)

    def adam_step(self, g: torch.Tensor, lr: float):
        self.step += 1
        st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        nat.check(self.L.spgo_mlp_adam(_vp(self.theta), _vp(g), _vp(self.m), _vp(self.v), self.step, float(lr), st),
                  "mlp_adam")

    def fit_normalization(self, X: np.ndarray):
        X = np.asarray(X, np.float64)
        self.mu = X.mean(0)
        self.sd = np.maximum(X.std(0), 1e-3)

    def _grad_dev(self, dX: torch.Tensor, dT: torch.Tensor, g: torch.Tensor, loss: torch.Tensor,
                  out: torch.Tensor, cache: torch.Tensor, st):
        nat.check(self.L.spgo_mlp_grad(_vp(self.theta), _vp(dX), _vp(dT), int(dX.shape[0]), _vp(g), _vp(loss),
                                       _vp(out), _vp(cache), st), "mlp_grad")

    def train(self, tr: Traces, epochs=60, batch=512, lr=2e-3, seed=0, fit_norm=True) -> List[float]:
        """Adam on the mean loss; the standardised traces stay on the device and
        every step is three kernel launches (forward, backward, Adam)."""
        if fit_norm:
            self.fit_normalization(tr.X)
        n = tr.X.shape[0]
        Xd = torch.tensor(self._norm(tr.X), device=self.device)
        Td = torch.tensor(np.asarray(tr.T, np.float32), device=self.device)
        gen = torch.Generator(device=self.device)
        gen.manual_seed(seed)
        g = torch.zeros(nat.MLP_PARAMS, dtype=torch.float32, device=self.device)
        loss = torch.zeros(1, dtype=torch.float32, device=self.device)
        out = torch.zeros(2 * batch, dtype=torch.float32, device=self.device)
        cache = torch.zeros(nat.MLP_CACHE_PER_SAMPLE * batch, dtype=torch.float32, device=self.device)
        ep_loss = torch.zeros(epochs, dtype=torch.float64, device=self.device)
        st = C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)
        for ep in range(epochs):
            perm = torch.randperm(n, device=self.device, generator=gen)
            Xp, Tp = Xd[perm].contiguous(), Td[perm].contiguous()
            for s0 in range(0, n, batch):
                m = min(batch, n - s0)
                self._grad_dev(Xp[s0:s0 + m], Tp[s0:s0 + m], g, loss, out, cache, st)
                self.adam_step(g, lr)
                ep_loss[ep] += loss[0].double() * m
        torch.cuda.synchronize(self.device)
        return (ep_loss / n).cpu().tolist()


def iterations_to_target(problems, controller: Optional[Controller], targets: np.ndarray, max_iters=30,
                         tol=1e-6, device="cuda", precision="mixed"):
    """Per problem, LM iterations until its cost is within rel 1e-6 of targets[b]
    (max_iters + 1 if never), plus the final costs and the solve wall time."""
    import time
    bs = BatchSolver(problems, precision=precision, device=device)
    bs.set_params(loss="l2", max_iters=max_iters, tol=tol, use_graph=0)
    bs.set_controller(controller.deployed() if controller is not None else None)
    bs.reset()
    B = len(problems)
    hit = np.full(B, max_iters + 1)
    t0 = time.perf_counter()
    for it in range(1, max_iters + 1):
        bs.iterate(1)
        st = bs.status()
        for b in range(B):
            if hit[b] > max_iters and st[b]["cost"] <= targets[b] * (1.0 + 1e-6):
                hit[b] = it
        if all(s["status"] != nat.STATUS_RUNNING for s in st):
            break
    wall = time.perf_counter() - t0
    costs = np.array([s["cost"] for s in bs.status()])
    bs.close()
    return hit, costs, wall
