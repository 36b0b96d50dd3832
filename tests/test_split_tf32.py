"""Accuracy of the split-TF32 products the tensor-core Schur kernel issues, restated
on the CPU (numpy, no GPU).

csrc/k_schur_tc.cu scales each slab value and splits it as x = hi + lo: hi is x
rounded to TF32's 10 stored mantissa bits (add 0x1000 to the FP32 bit pattern,
clear the low 13 bits), lo is x - hi (exact in FP32) rounded the same way.  The
MMA forms hi_a hi_b + hi_a lo_b + lo_a hi_b with FP32 accumulation; a product of
two TF32 values (11 significant bits each) is exact in FP32, so the error is the
dropped lo_a lo_b term plus the rounding of lo, about 2^-21 of the product.  The
kernel's comment claims ~21 mantissa bits for this; single-pass TF32 has ~11.
"""
import numpy as np


def tf32_round(x):
    """The kernel's tf32_round: round half away from zero to 10 stored mantissa bits."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32)
    return ((u + np.uint32(0x1000)) & np.uint32(0xFFFFE000)).view(np.float32)


def split(x):
    x = np.asarray(x, dtype=np.float32)
    hi = tf32_round(x)
    lo = tf32_round((x - hi).astype(np.float32))
    return hi, lo


def split_dot(a, b):
    """sum_k a_k b_k as the three MMAs accumulate it (FP32 adds of exact products)."""
    ah, al = split(a)
    bh, bl = split(b)
    acc = np.float32(0)
    for terms in (ah.astype(np.float64) * bh, ah.astype(np.float64) * bl, al.astype(np.float64) * bh):
        for t in terms:
            assert np.float32(t) == t   # every TF32 x TF32 product is exact in FP32
            acc = np.float32(acc + np.float32(t))
    return acc


def test_tf32_round_keeps_ten_mantissa_bits():
    rng = np.random.default_rng(1)
    x = (rng.normal(size=4096) * 10.0 ** rng.uniform(-6, 6, 4096)).astype(np.float32)
    h = tf32_round(x)
    assert np.all(h.view(np.uint32) & np.uint32(0x1FFF) == 0)
    rel = np.abs(h.astype(np.float64) - x) / np.abs(x.astype(np.float64))
    assert rel.max() <= 2.0 ** -11 * (1 + 1e-6)          # half a unit in the 11th bit
    hi, lo = split(x)
    assert np.all(np.abs(lo.astype(np.float64)) <= 2.0 ** -11 * np.abs(x.astype(np.float64)) * (1 + 1e-6))


def test_split_product_carries_about_21_bits():
    rng = np.random.default_rng(2)
    a = rng.normal(size=(2000,)).astype(np.float32)
    b = rng.normal(size=(2000,)).astype(np.float32)
    exact = a.astype(np.float64) * b
    ah, al = split(a)
    bh, bl = split(b)
    three = (ah.astype(np.float64) * bh + ah.astype(np.float64) * bl + al.astype(np.float64) * bh)
    rel3 = np.abs(three - exact) / np.abs(exact)
    one = ah.astype(np.float64) * bh
    rel1 = np.abs(one - exact) / np.abs(exact)
    assert rel3.max() < 2.0 ** -20          # worst case about 2^-21
    assert rel1.max() > 2.0 ** -13          # single pass: about 2^-11
    assert np.median(rel3) < np.median(rel1) * 2.0 ** -9


def test_split_dot_of_a_chunk_within_bound():
    """One chunk's 32-term diagonal entry sum_k (w_k s_k)^2, split-TF32 with FP32
    accumulation (modelled as three FP32 sums of exact products), stays within
    2^-19 of the exact value: per product ~2^-21 plus the FP32 accumulation.  On a
    diagonal entry every dropped lo^2 term has the same sign, so this is a few
    times the typical error of a plain FP32 dot product, never more than FP32's own
    worst case for 32 terms (32 x 2^-24 = 2^-19); the GPU tests bound the whole
    S_L product (2e-6 of max|A|)."""
    rng = np.random.default_rng(3)
    worst_split = worst_fp32 = 0.0
    for _ in range(200):
        x = (rng.normal(size=32) * rng.uniform(0.1, 10.0)).astype(np.float32)
        exact = float(np.dot(x.astype(np.float64), x.astype(np.float64)))
        s = float(split_dot(x, x))
        f = np.float32(0)
        for v in x:
            f = np.float32(f + np.float32(v) * np.float32(v))
        worst_split = max(worst_split, abs(s - exact) / exact)
        worst_fp32 = max(worst_fp32, abs(float(f) - exact) / exact)
    assert worst_split < 2.0 ** -19
    assert worst_fp32 < 2.0 ** -19
    # single-pass TF32 on the same entries is ~2^-11: the split buys ~8 bits
    one = max(abs(float(np.sum(tf32_round(x).astype(np.float64) ** 2)) - float(np.dot(x.astype(np.float64), x)))
              / float(np.dot(x.astype(np.float64), x)) for x in
              (rng.normal(size=32).astype(np.float32) for _ in range(50)))
    assert one > 2.0 ** 6 * worst_split
