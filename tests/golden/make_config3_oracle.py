"""Generate the config-3 oracle fixture: the FP64 oracle's LM on the first 64
problems of the seeded config-3 batch.

    python tests/golden/make_config3_oracle.py [processes]

For problems 0..63 of ``scenes.config3_specs(3)`` (N ~ U[8, 32] poses,
L ~ U[200, 3000] landmarks, circle generator, pixels rounded to FP32 as the
solver's plan stores them) it runs ``oracle.solver.lm_solve`` (L2, Nielsen
damping, lambda0 1e-4, at most 30 iterations or a relative decrease below 1e-6)
and stores, per problem, the spec, the final cost, the iterations and the final
incremental poses (3x4, float64) in ``config3_oracle.npz`` next to this script.
The GPU parity test compares the plain FP64 GPU solver with it; a CPU test
re-runs the oracle on the smallest of these problems and checks it against the
stored result.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
N_PROB = 64
MAX_ITERS = 30
TOL = 1e-6


def oracle_run(spec):
    """The FP64 oracle's LM on one config-3 problem: (cost, iterations, poses [N][12])."""
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    if REPO not in sys.path:
        sys.path.insert(0, REPO)
    import __graft_entry__
    __graft_entry__.load_package()
    import spgo_gb300.scenes as scenes
    from oracle import solver as S
    seed, n, l = spec
    p = scenes.round_pixels_f32(scenes.circle_scene(seed, n, l))
    r = S.lm_solve(p, S.Loss(), max_iters=MAX_ITERS, tol=TOL)
    return float(r.cost), int(r.iterations), np.asarray(p.poses, dtype=np.float64)[:, :3, :].reshape(n, 12)


def main():
    sys.path.insert(0, REPO)
    import __graft_entry__
    __graft_entry__.load_package()
    import spgo_gb300.scenes as scenes
    procs = int(sys.argv[1]) if len(sys.argv) > 1 else (os.cpu_count() or 1)
    specs = scenes.config3_specs(3)[:N_PROB]
    with mp.get_context("spawn").Pool(procs) as pool:
        res = pool.map(oracle_run, specs, chunksize=1)
    nmax = max(n for _, n, _ in specs)
    poses = np.zeros((N_PROB, nmax, 12))
    for k, (_, _, P) in enumerate(res):
        poses[k, :P.shape[0]] = P
    np.savez_compressed(os.path.join(HERE, "config3_oracle.npz"),
                        specs=np.array(specs, dtype=np.int64),
                        cost=np.array([c for c, _, _ in res]),
                        iterations=np.array([i for _, i, _ in res], dtype=np.int32),
                        poses=poses)
    print("wrote", os.path.join(HERE, "config3_oracle.npz"))


if __name__ == "__main__":
    main()
