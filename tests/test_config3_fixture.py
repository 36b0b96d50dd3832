"""The committed config-3 oracle fixture (``tests/golden/config3_oracle.npz``, the
FP64 oracle's LM on problems 0..63 of the seeded config-3 batch, used by the GPU
parity test) against the oracle itself: its problem list is the batch's, and the
oracle re-run here on the two smallest of those problems gives the stored final
cost, iteration count and poses."""
import os

import numpy as np

import spgo_gb300.scenes as scenes
from oracle import solver as S

FIXTURE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "config3_oracle.npz")


def test_fixture_matches_oracle():
    ref = np.load(FIXTURE)
    specs = scenes.config3_specs(3)
    n = len(ref["specs"])
    assert n >= 64
    assert [tuple(int(v) for v in x) for x in ref["specs"]] == [tuple(x) for x in specs[:n]]
    size = [int(s[1]) * int(s[2]) for s in ref["specs"]]
    for k in np.argsort(size)[:2]:
        seed, N, L = (int(v) for v in ref["specs"][k])
        p = scenes.round_pixels_f32(scenes.circle_scene(seed, N, L))
        r = S.lm_solve(p, S.Loss(), max_iters=30, tol=1e-6)
        assert abs(r.cost - ref["cost"][k]) <= 1e-9 * ref["cost"][k]
        assert r.iterations == ref["iterations"][k]
        assert np.abs(p.poses[:, :3, :].reshape(N, 12) - ref["poses"][k, :N]).max() < 1e-9
