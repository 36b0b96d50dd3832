"""The Jacobian pass's enumeration of a chunk's in-window (landmark, frame) pairs
(s-pgo_gb300/csrc/k_linearize.cu, k_jacobian_acc, phase C.2), restated on the CPU.

Per window row i the kernel keeps the mask of the chunk's landmarks whose window
[lo, hi) holds frame f0 + i (a warp ballot) and the exclusive prefix of the rows'
landmark counts.  Pair j is found by a binary search over that prefix (steps 64..1,
windows of up to 96 rows) and a select of the (j - prefix)-th set bit by halving
popcounts.  The enumeration must visit every in-window pair exactly once, and the
pairs of one row in increasing landmark order (a warp's lanes on distinct slab
columns)."""
import numpy as np


def popc(x):
    return bin(x & 0xFFFFFFFF).count("1")


def kernel_pairs(lo, hi, f0, nb):
    cnt = len(lo)
    rmask, rsp, run = [], [], 0
    for i in range(nb):
        m = 0
        for s in range(32):
            if s < cnt and lo[s] <= f0 + i < hi[s]:
                m |= 1 << s
        rmask.append(m)
        rsp.append(run)
        run += popc(m)
    rsp.append(run)
    out = []
    for j in range(rsp[nb]):
        row = 0
        for step in (64, 32, 16, 8, 4, 2, 1):
            if row + step < nb and rsp[row + step] <= j:
                row += step
        m, r, slot = rmask[row], j - rsp[row], 0
        for w in (16, 8, 4, 2, 1):
            c = popc(m & ((1 << w) - 1))
            if r >= c:
                r -= c
                m >>= w
                slot += w
        out.append((slot, f0 + row))
    return out


def test_window_pair_enumeration():
    rng = np.random.default_rng(5)
    for trial in range(400):
        cnt = int(rng.integers(1, 33))
        host = int(rng.integers(0, 60))
        nbmax = int(rng.choice([4, 20, 32, 96]))
        # landmarks of one host frame sorted by (lo, hi), as the planner orders them
        los, his = [], []
        for _ in range(cnt):
            a = int(rng.integers(0, 8))
            b = int(rng.integers(0, 8)) if rng.random() < 0.8 else 0
            lo = max(0, host - a)
            hi = max(lo, min(host + b, lo + nbmax))
            los.append(lo)
            his.append(hi)
        order = sorted(range(cnt), key=lambda s: (los[s], his[s]))
        lo = [los[s] for s in order]
        hi = [his[s] for s in order]
        f0 = lo[0]
        nb = max(1, max(hi) - f0)
        got = kernel_pairs(lo, hi, f0, nb)
        want = {(s, i) for s in range(cnt) for i in range(lo[s], hi[s])}
        assert len(got) == len(set(got)) == len(want)
        assert set(got) == want
        # a row's pairs are consecutive and in increasing landmark order
        for (s1, i1), (s2, i2) in zip(got, got[1:]):
            assert i2 > i1 or (i2 == i1 and s2 > s1)
