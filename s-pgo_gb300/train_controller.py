"""Train the learned LM damping controller on the GPU and save its weights.

    python s-pgo_gb300/train_controller.py [--batches 8] [--config1 8] [--epochs 80]
                                            [--eval-batches 4] [--out PATH]

1. Seeded problems: ``--batches`` batches of the 256-problem config-3 generator
   (batch seeds 1000 + k) and ``--config1`` problems of the config-1 generator
   (N = 100 corridor, 20k landmarks; seeds 5000 + k), generated in a process pool.
2. Traces: the plain Nielsen-LM solver runs each set to 30 iterations; at every
   iteration of every problem still running it probes the step cost for lambda x
   {1e-6 .. 1e3} (``learned.collect_traces``) and records the 16 features.
3. Training: Adam on the library's own forward/backward/Adam kernels.
4. Evaluation on held-out config-3 batches (batch seeds 2000 + k): LM iterations
   until the cost is within relative 1e-6 of the plain FP64 GPU solver's converged
   cost, plain schedule vs learned, in mixed and FP64 precision.

Prints one JSON summary line and writes the weights (theta, feature mean and
spread) to ``--out`` (default: the package's controller_weights.npz).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import sys
import time

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _load():
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import __graft_entry__
    return __graft_entry__.load_package()


def _gen_config3(seed):
    _load()
    from spgo_gb300 import scenes
    return scenes.config3(seed=seed)


def _gen_config1(seed):
    _load()
    from spgo_gb300 import scenes
    return [scenes.config1(seed=seed)]


def generate(fn, seeds, workers):
    ctx = mp.get_context("spawn")
    with ctx.Pool(min(workers, len(seeds))) as pool:
        parts = pool.map(fn, seeds)
    return [p for part in parts for p in part]


def evaluate(problems, controller, max_iters=30):
    import torch
    from spgo_gb300 import learned
    from spgo_gb300.solver import BatchSolver
    bs = BatchSolver(problems, precision="fp64")
    bs.set_params(loss="l2", max_iters=max_iters, tol=1e-6)
    sts = bs.solve()
    torch.cuda.synchronize()
    targets = np.array([s["cost"] for s in sts])
    bs.close()
    out = {}
    for name, prec, ctl in [("plain_fp64", "fp64", None), ("plain_mixed", "mixed", None),
                            ("learned_mixed", "mixed", controller), ("learned_fp64", "fp64", controller)]:
        hit, costs, wall = learned.iterations_to_target(problems, ctl, targets, max_iters=max_iters, precision=prec)
        reached = hit <= max_iters
        out[name] = {"reached_frac": float(reached.mean()),
                     "mean_iters_to_target": float(hit.mean()),          # a miss counts max_iters + 1
                     "mean_iters_reached": float(hit[reached].mean()) if reached.any() else None,
                     "lower_final_frac": float((costs < targets * (1 - 1e-6)).mean())}
    base = out["plain_fp64"]["mean_iters_to_target"]
    for k in ("learned_mixed", "learned_fp64"):
        out[k]["iteration_ratio_vs_plain_fp64"] = base / out[k]["mean_iters_to_target"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--batches", type=int, default=8)
    ap.add_argument("--config1", type=int, default=8)
    ap.add_argument("--eval-batches", type=int, default=4)
    ap.add_argument("--epochs", type=int, default=80)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 4)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    _load()  # the pool returns problems of the package's classes: load it here first
    t0 = time.time()
    train3 = generate(_gen_config3, [1000 + k for k in range(args.batches)], args.workers)
    train1 = generate(_gen_config1, [5000 + k for k in range(args.config1)], args.workers) if args.config1 else []
    held = generate(_gen_config3, [2000 + k for k in range(args.eval_batches)], args.workers)
    t_gen = time.time() - t0

    import torch
    from spgo_gb300 import learned
    t1 = time.time()
    parts = [learned.collect_traces(train3[i:i + 1024]) for i in range(0, len(train3), 1024)]
    if train1:
        parts.append(learned.collect_traces(train1))
    tr = learned.Traces(np.concatenate([p.X for p in parts]), np.concatenate([p.T for p in parts]))
    t_tr = time.time() - t1
    t2 = time.time()
    ctl = learned.Controller(seed=0)
    hist = ctl.train(tr, epochs=args.epochs, lr=args.lr)
    t_train = time.time() - t2
    out = args.out or learned.DEFAULT_WEIGHTS
    ctl.save(out)
    t3 = time.time()
    ev = evaluate(held, ctl)
    summary = {"train_problems": {"config3": len(train3), "config1": len(train1)}, "samples": int(tr.X.shape[0]),
               "heldout_problems": len(held), "epochs": args.epochs, "loss_first_last": [hist[0], hist[-1]],
               "seconds": {"generate": round(t_gen, 1), "traces": round(t_tr, 1), "train": round(t_train, 1),
                           "evaluate": round(time.time() - t3, 1)},
               "eval": ev, "weights": os.path.relpath(out, REPO)}
    print(json.dumps(summary))
    torch.cuda.synchronize()


if __name__ == "__main__":
    main()
