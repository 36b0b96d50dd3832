"""The reference scene generator against golden vectors from the reference's own
simulator (``tests/golden/make_reference_scene.py``), and its properties."""
import os

import numpy as np
import pytest

from spgo_gb300 import evaluate, scenes
from oracle import solver as S

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_scene.npz")


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


def _cases(gold):
    return range(int(gold["n_cases"]))


def test_camera_poses_match_reference_stream(gold):
    """SamplePoses with numpy's and torch's generators seeded as in the fixture: the
    same draws in the same order give the same poses (float32 in the reference)."""
    torch = pytest.importorskip("torch")
    for c in _cases(gold):
        s, n, m = (int(x) for x in gold[f"c{c}_case"])
        rng = np.random.RandomState(s)
        torch.manual_seed(s)
        W = scenes.reference_camera_poses(rng, n + 1, axis_draw=lambda: torch.randn(3).double().numpy())
        assert np.abs(W - gold[f"c{c}_W"]).max() < 2e-6


def test_points_match_reference_stream(gold):
    for c in _cases(gold):
        s, n, m = (int(x) for x in gold[f"c{c}_case"])
        pts = scenes.reference_points(np.random.RandomState(1000 + s), n * m)
        assert np.abs(pts - gold[f"c{c}_pts"]).max() < 1e-12


def test_fed_observations_match_reference_feeder(gold):
    """Projection, validity rule, anchoring and the anchor pixel on the reference's
    own poses and points: frames bit-exact, pixels to FP64 rounding."""
    for c in _cases(gold):
        p = scenes.reference_scene_from(gold[f"c{c}_W"], gold[f"c{c}_pts"])
        p.validate()
        assert np.array_equal(p.host, gold[f"c{c}_host"])
        assert np.array_equal(p.obs_ptr, gold[f"c{c}_obs_ptr"])
        assert np.array_equal(p.obs_frame, gold[f"c{c}_obs_frame"])
        assert np.abs(p.obs_uv - gold[f"c{c}_obs_uv"]).max() < 1e-9
        assert np.abs(p.anchor_uv - gold[f"c{c}_anchor_uv"]).max() < 1e-9


def test_reference_scene_is_consistent_with_the_oracle():
    """Noise-free pixels: at the ground truth the oracle's cost is zero for every
    landmark whose anchor observation was fed; the others carry the reference's
    (0, 0) anchor pixel.  Seeded draws are reproducible."""
    import dataclasses
    p = scenes.reference_scene(7, n_poses=6, landmarks_per_frame=40)
    q = scenes.reference_scene(7, n_poses=6, landmarks_per_frame=40)
    assert np.array_equal(p.obs_uv, q.obs_uv) and np.array_equal(p.gt_poses, q.gt_poses)
    assert np.allclose(p.poses, np.eye(4)) and np.all(p.alpha == 1.0)
    assert np.all(p.obs_frame >= np.repeat(p.host, np.diff(p.obs_ptr)))
    fed = ~np.all(p.anchor_uv == 0.0, axis=1)
    keep = np.nonzero(fed)[0]
    cnt = np.diff(p.obs_ptr)
    sel = np.concatenate([np.arange(p.obs_ptr[l], p.obs_ptr[l + 1]) for l in keep])
    g = dataclasses.replace(p, host=p.host[keep], anchor_uv=p.anchor_uv[keep],
                            obs_ptr=np.concatenate([[0], np.cumsum(cnt[keep])]), obs_frame=p.obs_frame[sel],
                            obs_uv=p.obs_uv[sel], poses=p.gt_poses.copy(), alpha=p.gt_alpha[keep].copy())
    assert S.cost(g, S.Loss()) < 1e-12


def test_reference_gn_study_converges_on_cpu():
    """The divergence study's step (undamped GN, Cauchy, step 0.5) on one reference
    window with the oracle: the summed pose error falls from the identity start."""
    p = scenes.reference_scene(3)
    e0 = evaluate.incremental_pose_errors(p.poses, p.gt_poses).sum()
    S.reference_gn_step(p, iterations=20, step_size=0.5)
    e1 = evaluate.incremental_pose_errors(p.poses, p.gt_poses).sum()
    assert e0 > 1.0 and e1 < 0.05
