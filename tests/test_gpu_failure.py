"""Failure paths that must end in a status, not a hang or a NaN.

The bounded device-side waits (the multi-CTA substitutions of wide reduced systems,
the tensor-core Schur pipeline) give up after ``spgo_params.wait_us``.  Shortening
that limit to one microsecond makes the substitutions' waits for earlier blocks run
out: the step must be rejected, counted as a timeout (not as a factorisation
failure), and leave the state finite; with the default limit restored the same
solver must solve normally.  Nothing here faults, traps or hangs the GPU: every wait
stays bounded, only its limit changes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_wait_limit_rejects_step_and_recovers(built_lib, cuda_device):
    import spgo_gb300.scenes as scenes
    from spgo_gb300.solver import BatchSolver
    # 60 poses: P = 360, too wide for one CTA's shared memory -> multi-CTA substitutions
    p = scenes.corridor_scene(5, n_poses=60, n_landmarks=2500)
    bs = BatchSolver([p], precision="mixed", device=cuda_device)
    assert bs.sizes.max_params == 360
    p0, a0 = bs.poses.clone(), bs.alpha.clone()
    bs.set_params(loss="l2", max_iters=4, tol=1e-12, wait_us=1)
    st = bs.solve()[0]
    assert st["wait_timeouts"] >= 1, st
    assert np.isfinite(st["cost"])
    assert np.all(np.isfinite(bs.poses.cpu().numpy())) and np.all(np.isfinite(bs.alpha.cpu().numpy()))
    # every timed-out step was rejected: the state moved only on accepted steps
    if st["accepted"] == 0:
        assert np.array_equal(bs.poses.cpu().numpy(), p0.cpu().numpy())
    # the default limit again: the same solver solves normally
    bs.poses.copy_(p0)
    bs.alpha.copy_(a0)
    bs.set_params(max_iters=10, wait_us=0)
    st = bs.solve()[0]
    assert st["wait_timeouts"] == 0 and st["factor_failures"] == 0
    assert st["accepted"] >= 1 and st["cost"] < st["cost0"]
    bs.close()
