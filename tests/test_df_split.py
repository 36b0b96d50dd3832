"""The mixed path's pair reduction splits the FP64 pair records into double-float
pairs with integer operations (``df_split_double`` in
``s-pgo_gb300/csrc/dfloat.cuh``): h = the double with its mantissa truncated to 24
bits, l = the remaining 29 bits rounded to 24 bits, scaled.  Restated here bit for
bit in numpy and checked on doubles from 1e-30 to 1e30 (the records' values lie
far inside), both signs, and the edge cases."""
import numpy as np


def split(x):
    x = np.asarray(x, dtype=np.float64)
    u = x.view(np.uint64)
    hi32 = (u >> np.uint64(32)).astype(np.uint32)
    lo32 = (u & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    e = ((hi32 >> np.uint32(20)) & np.uint32(0x7FF)).astype(np.int64) - 1023
    sign = hi32 & np.uint32(0x80000000)
    hb = sign | (np.clip(e + 127, 0, 255).astype(np.uint32) << np.uint32(23)) | \
        ((hi32 & np.uint32(0xFFFFF)) << np.uint32(3)) | (lo32 >> np.uint32(29))
    h = hb.view(np.float32)
    el = e - 52
    scale = np.where(el >= -126, (np.clip(el + 127, 1, 254).astype(np.uint32) << np.uint32(23)).view(np.float32),
                     np.float32(0))
    l = (((lo32 & np.uint32(0x1FFFFFFF)).astype(np.float32) * scale).view(np.uint32) | sign).view(np.float32)
    tiny = e < -126
    big = e > 127
    nan = big & (e == 1024) & (((hi32 & np.uint32(0xFFFFF)) | lo32) != 0)
    h = np.where(tiny, np.float32(0), h)
    l = np.where(tiny | big, np.float32(0), l)
    h = np.where(big, np.where(nan, np.float32(np.nan), np.copysign(np.float32(np.inf), x).astype(np.float32)), h)
    return h.astype(np.float32), l.astype(np.float32)


def test_split_is_exact_to_48_bits():
    rng = np.random.default_rng(7)
    x = rng.standard_normal(200000) * 10.0 ** rng.uniform(-30, 30, 200000)
    h, l = split(x)
    back = h.astype(np.float64) + l.astype(np.float64)
    # 48 bits where the low part's weight stays in the float range (|x| >= 2^-74);
    # below that the low part is dropped and h alone carries 24 bits
    full = np.abs(x) >= 2.0 ** -74
    assert np.all(np.abs(back - x)[full] <= 2.0 ** -47 * np.abs(x)[full])
    assert np.all(np.abs(back - x)[~full] <= 2.0 ** -23 * np.abs(x)[~full])
    # h is x truncated toward zero to float: |h| <= |x|, |x - h| < one float ulp of h
    assert np.all(np.abs(h.astype(np.float64)) <= np.abs(x))
    assert np.all(np.abs(x - h) < np.spacing(np.abs(h)).astype(np.float64))
    assert np.all(np.sign(h) == np.sign(x)) and np.all((l == 0) | (np.sign(l) == np.sign(x)))


def test_split_edge_cases():
    h, l = split(np.array([0.0, -0.0, 1e-40, -1e-300, 1.0, -2.0, 3e38, 1e39, -1e300, np.inf, -np.inf, np.nan]))
    assert h[0] == 0 and l[0] == 0 and h[1] == 0 and h[2] == 0 and h[3] == 0
    assert h[4] == 1.0 and l[4] == 0 and h[5] == -2.0 and l[5] == 0
    assert np.isfinite(h[6]) and abs(float(h[6]) + float(l[6]) - 3e38) <= 3e38 * 2.0 ** -47
    assert h[7] == np.inf and h[8] == -np.inf and h[9] == np.inf and h[10] == -np.inf
    assert np.isnan(h[11])
