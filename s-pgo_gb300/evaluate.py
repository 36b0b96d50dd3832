"""Evaluation harness: estimation-error metrics and the divergence-rate study.

Metrics (the reference's, restated):
- incremental-pose error: ||Log_SE3(inv(T_true) T_est)|| per incremental pose, summed
  over the window (CUDAmanager.py:100-109, PythonUtils/Manager.py:76-80);
- depth error: |1 / alpha_est - 1 / alpha_true| per landmark, summed
  (PythonUtils/Manager.py:82-95).

Divergence-rate study (ConvegenceTests.py:17-63): many seeded windows, each
stepped with the reference's undamped Gauss-Newton `step(1)` (pose step size 0.5)
for a number of steps, recording the summed pose error after every step; a run
counts as diverged when its final error exceeds 0.5.  Here every trial of the
study is one problem of a single batch, so one batched launch sequence steps all
of them at once; `mode="lm"` runs the Nielsen LM iteration instead.  The windows
come from the reference's own scene distribution (`scene="reference"`:
`scenes.reference_scene`, identity initial poses, inverse depth 1, noise-free
pixels, as the reference feeder sets them up) or from the project's circle scenes
(`scene="circle"`: 1 px noise, perturbed ground truth).

    python s-pgo_gb300/evaluate.py [--trials 100] [--steps 50] [--mode gn|lm] [--scene reference|circle]
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time
from typing import Dict, List

import numpy as np


def _pkg():
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if repo not in sys.path:
        sys.path.insert(0, repo)
    import __graft_entry__
    return __graft_entry__.load_package()


def incremental_pose_errors(est: np.ndarray, true: np.ndarray) -> np.ndarray:
    """||Log_SE3(inv(T_true) T_est)|| for each incremental pose ([N, 4, 4] each)."""
    _pkg()
    from spgo_gb300 import se3
    return np.array([np.linalg.norm(se3.log_se3(se3.inv(t) @ e)) for e, t in zip(est, true)])


def depth_errors(alpha_est: np.ndarray, alpha_true: np.ndarray) -> np.ndarray:
    """|1 / alpha_est - 1 / alpha_true| per landmark."""
    return np.abs(1.0 / np.asarray(alpha_est, np.float64) - 1.0 / np.asarray(alpha_true, np.float64))


def convergence_study(trials: int = 100, steps: int = 50, n_poses: int = 10, landmarks_per_frame: int = 96,
                      step_size: float = 0.5, seed: int = 0, mode: str = "gn", precision: str = "mixed",
                      threshold: float = 0.5, scene: str = "reference", device="cuda") -> Dict:
    """Batched divergence-rate study; returns the error matrix [trials, steps], the
    per-step wall time of the batched step, and the divergence rate."""
    _pkg()
    import torch
    from spgo_gb300 import scenes
    from spgo_gb300.solver import BatchSolver
    rng = np.random.Generator(np.random.PCG64(seed))
    seeds = rng.integers(0, 2**31 - 1, trials)
    if scene == "reference":
        probs = [scenes.reference_scene(int(s), n_poses, landmarks_per_frame, name=f"trial{t}")
                 for t, s in enumerate(seeds)]
    elif scene == "circle":
        probs = [scenes.circle_scene(int(s), n_poses, n_poses * landmarks_per_frame, name=f"trial{t}")
                 for t, s in enumerate(seeds)]
    else:
        raise ValueError(f"unknown scene {scene!r}")
    bs = BatchSolver(probs, precision=precision, device=device)
    if mode == "gn":
        bs.set_params(loss="cauchy", loss_scale=3.0, near_boost=True, eps=1e-4)
    else:
        bs.set_params(loss="l2", max_iters=steps, tol=0.0, use_graph=0)
        bs.reset()
    errors = np.zeros((trials, steps))
    depth = np.zeros(trials)
    times = np.zeros(steps)
    for k in range(steps):
        torch.cuda.synchronize(bs.device)
        t0 = time.perf_counter()
        if mode == "gn":
            bs.gn_step(1, step_size)
        else:
            bs.iterate(1)
        torch.cuda.synchronize(bs.device)
        times[k] = time.perf_counter() - t0
        poses, alphas = bs.get_state()
        for t, p in enumerate(probs):
            errors[t, k] = incremental_pose_errors(poses[t], p.gt_poses).sum()
            if k == steps - 1:
                depth[t] = depth_errors(alphas[t], p.gt_alpha).sum()
    bs.close()
    diverged = errors[:, -1] > threshold
    return {"errors": errors, "step_seconds": times, "depth_error_sum": depth, "diverged": diverged,
            "divergence_rate": float(diverged.mean())}


def main(argv: List[str] | None = None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--trials", type=int, default=100)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--mode", choices=["gn", "lm"], default="gn")
    ap.add_argument("--precision", choices=["mixed", "fp64"], default="mixed")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--scene", choices=["reference", "circle"], default="reference")
    ap.add_argument("--save", default="", help="prefix: <prefix>_errors.txt ([trials, steps] summed pose "
                    "errors, as the reference's study writes them) and <prefix>_timing.txt (ns per batched "
                    "step: one step of every trial together)")
    args = ap.parse_args(argv)
    r = convergence_study(args.trials, args.steps, mode=args.mode, precision=args.precision, seed=args.seed,
                          scene=args.scene)
    e = r["errors"]
    if args.save:
        np.savetxt(args.save + "_errors.txt", e)
        np.savetxt(args.save + "_timing.txt", 1e9 * r["step_seconds"])
    print(json.dumps({"trials": args.trials, "steps": args.steps, "mode": args.mode, "precision": args.precision,
                      "scene": args.scene,
                      "divergence_rate": r["divergence_rate"], "diverged": np.nonzero(r["diverged"])[0].tolist(),
                      "final_error_median": float(np.median(e[:, -1])),
                      "first_error_median": float(np.median(e[:, 0])),
                      "depth_error_sum_median": float(np.median(r["depth_error_sum"])),
                      "ms_per_batched_step": float(1e3 * np.median(r["step_seconds"]))}))


if __name__ == "__main__":
    main()
