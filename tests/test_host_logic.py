"""Host-side logic that needs no GPU: seeded scenes and the drop-in staging."""
import numpy as np

import spgo_gb300.scenes as scenes
from spgo_gb300.solver import CudaSolver


def test_scenes_are_seeded():
    a, b = scenes.circle_scene(4, 8, 200), scenes.circle_scene(4, 8, 200)
    assert np.array_equal(a.obs_uv, b.obs_uv) and np.array_equal(a.poses, b.poses)
    c = scenes.circle_scene(5, 8, 200)
    assert not np.array_equal(a.obs_uv[:10], c.obs_uv[:10])


def test_config_sizes():
    p0 = scenes.config0()
    p0.validate()
    assert p0.n_poses == 10 and p0.n_landmarks == 500
    p1 = scenes.config1()
    assert p1.n_poses == 100 and p1.n_landmarks == 20000
    assert 350_000 < p1.n_obs < 450_000
    lo, hi = p1.span()
    assert (hi - lo).max() <= 96


def test_scene_geometry_consistent():
    """Ground-truth state reprojects the noise-free pixels (noise is N(0, 1 px))."""
    from oracle import solver as S
    p = scenes.circle_scene(9, 6, 100)
    q = p.copy()
    q.poses, q.alpha = p.gt_poses, p.gt_alpha
    r = S.linearize(q, S.Loss()).raw_r
    assert np.sqrt(np.mean(r ** 2)) < 2.5


def test_cudasolver_staging_matches_reference_layout():
    """writeObservations / getObservation / getCalibration shapes (Solver.pyx:34-88)."""
    s = CudaSolver(3, 2)
    intr = np.array([320, 320, 320, 240, 320, 320, 320, 240], np.float32)
    Trl = np.eye(4, dtype=np.float32)
    Trl[0, 3] = 0.2
    s.loadCalibration(intr, Trl.reshape(16))
    rng = np.random.default_rng(0)
    for f in range(6):
        a = f // 2
        for t in range(a, 4):
            s.writeObservations(a, t, f, np.r_[rng.uniform(0, 600, 2), 1.0].astype(np.float32),
                                np.r_[rng.uniform(0, 600, 2), 1.0].astype(np.float32))
    l, r = s.getObservation(2, 3)
    assert l.shape == (3, 1) and r.shape == (3, 1)
    i, T = s.getCalibration()
    assert i.shape == (4, 2) and T.shape == (4, 4)
    assert np.array_equal(s.getIncrementalPose(1), np.eye(4, dtype=np.float32))
    assert s.getInverseDepths().shape == (6,) and np.all(s.getInverseDepths() == 1)
    p = s._problem()
    p.validate()
    assert p.n_landmarks == 6 and list(p.host) == [0, 0, 1, 1, 2, 2]
    assert np.allclose(p.anchor_uv[3], s.getObservation(1, 3)[0][:2, 0])


def test_evaluation_metrics():
    """Pose error = ||Log_SE3(inv(T_true) T_est)|| (the reference's metric) and the
    summed depth error, on known perturbations."""
    from spgo_gb300 import evaluate, se3
    from oracle import lie
    rng = np.random.default_rng(3)
    true = np.stack([lie.exp_se3(rng.normal(0, 0.3, 6)) for _ in range(4)])
    xis = rng.normal(0, 0.05, (4, 6))
    est = np.stack([t @ lie.exp_se3(x) for t, x in zip(true, xis)])
    e = evaluate.incremental_pose_errors(est, true)
    assert np.allclose(e, np.linalg.norm(xis, axis=1), rtol=1e-9, atol=1e-12)
    assert np.allclose(evaluate.incremental_pose_errors(true, true), 0.0, atol=1e-12)
    a = np.array([0.5, 0.25, 0.1])
    assert np.allclose(evaluate.depth_errors(a, a * 2.0), [1.0, 2.0, 5.0])
    for _ in range(5):
        xi = rng.normal(0, 0.8, 6)
        assert np.abs(se3.log_se3(lie.exp_se3(xi)) - xi).max() < 1e-12
