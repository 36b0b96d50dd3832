"""The wide-problem refinement's prefix over the poses (s-pgo_gb300/csrc/k_refine.cu,
k_rs_scan_large), restated on the CPU: per component the poses are cut into 42
segments of ceil(N / 42), each segment summed, the segment sums scanned (exclusive),
and each segment walked again from its offset.  The result must be the inclusive
prefix of the per-pose terms for every N (segments past the end are empty), equal to
the serial sum up to FP64 reassociation."""
import math

import numpy as np

SEGS = 42


def segmented_prefix(val):
    N = val.shape[0]
    out = np.zeros_like(val)
    L = (N + SEGS - 1) // SEGS
    for k in range(val.shape[1]):
        seg = []
        for s in range(SEGS):
            i0, i1 = s * L, min(N, s * L + L)
            seg.append(sum(val[i, k] for i in range(i0, i1)) if i0 < i1 else 0.0)
        off, acc = [], 0.0
        for v in seg:
            off.append(acc)
            acc += v
        for s in range(SEGS):
            acc = off[s]
            for i in range(s * L, min(N, s * L + L)):
                acc += val[i, k]
                out[i, k] = acc
    return out


def test_segmented_prefix_matches_serial():
    rng = np.random.default_rng(11)
    for N in (1, 2, 41, 42, 43, 83, 84, 85, 500, 1001):
        val = rng.standard_normal((N, 6)) * 10.0 ** rng.integers(-3, 4, size=(N, 6))
        got = segmented_prefix(val)
        want = np.cumsum(val, axis=0)
        scale = np.cumsum(np.abs(val), axis=0)
        assert np.all(np.abs(got - want) <= 1e-13 * scale + 1e-300), N
        # every pose is written once per component
        assert np.isfinite(got).all() and got.shape == val.shape
    assert math.ceil(500 / SEGS) == 12
