"""The mixed path's SE(3) update, restated on the CPU (numpy, no GPU) and compared
with the FP64 exp map.

k_update_poses<float> (csrc/k_solve.cu) replaces T_k <- T_k Exp(xi) (the reference's
updateEstimation / ExpSE3, src/Optimization/Solver_cuda.cu:511-551, SE3.cu:3-38) by
T + T (Exp(xi) - I): the increment D = Exp(xi) - I in FP32 (Rodrigues coefficients
by their Taylor series below 0.5 rad, by sin / cos above), the product T D and the
sum in double-float, the result stored as FP64.  The claim: the increment keeps
FP32 precision relative to itself, and the pose otherwise keeps ~48 bits, so tiny
late-iteration steps on poses metres from the origin are not lost.
"""
import numpy as np

from dfloat_numpy import add, df, mul_f
from oracle import lie

f32, f64 = np.float32, np.float64


def series_coeffs(t2):
    """The kernel's series for (sin t / t, (1 - cos t) / t^2, (t - sin t) / t^3)."""
    t4 = t2 * t2
    t6, t8 = t4 * t2, t4 * t4
    a = 1 - t2 / 6 + t4 / 120 - t6 / 5040 + t8 / 362880
    b = 0.5 - t2 / 24 + t4 / 720 - t6 / 40320 + t8 / 3628800
    c = 1 / 6 - t2 / 120 + t4 / 5040 - t6 / 362880 + t8 / 39916800
    return a, b, c


def increment_fp32(xi):
    """D = Exp(xi) - I (n, 3, 4) in FP32 as the kernel forms it."""
    p = xi[:, :3].astype(f32)
    r = xi[:, 3:].astype(f32)
    t2 = (p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1] + p[:, 2] * p[:, 2]).astype(f32)
    th = np.sqrt(t2)
    sa, sb, sc = (np.asarray(v, f32) for v in series_coeffs(t2))
    with np.errstate(divide="ignore", invalid="ignore"):
        sn, cs, sh = np.sin(th), np.cos(th), np.sin(f32(0.5) * th)
        fa, fb, fc = sn / th, f32(2) * sh * sh / t2, (th - sn) / (t2 * th)
    small = th < f32(0.5)
    a, b, c = np.where(small, sa, fa), np.where(small, sb, fb), np.where(small, sc, fc)
    z = np.zeros_like(p[:, 0])
    S = np.stack([z, -p[:, 2], p[:, 1], p[:, 2], z, -p[:, 0], -p[:, 1], p[:, 0], z], -1).reshape(-1, 3, 3)
    S2 = np.einsum('nik,nkj->nij', S, S).astype(f32)
    D = np.zeros((len(xi), 3, 4), f32)
    D[:, :, :3] = a[:, None, None] * S + b[:, None, None] * S2
    J = np.eye(3, dtype=f32)[None] + b[:, None, None] * S + c[:, None, None] * S2
    D[:, :, 3] = np.einsum('nij,nj->ni', J, r).astype(f32)
    return D


def update_mixed(T0, xi):
    """T + T D with T D and the sum in double-float, stored as FP64 (n, 3, 4)."""
    D = increment_fp32(xi)
    out = np.zeros_like(T0)
    for i in range(3):
        for j in range(4):
            td = mul_f(df(T0[:, i, 0]), D[:, 0, j])
            td = add(td, mul_f(df(T0[:, i, 1]), D[:, 1, j]))
            td = add(td, mul_f(df(T0[:, i, 2]), D[:, 2, j]))
            v = add(df(T0[:, i, j]), td)
            out[:, i, j] = v[0].astype(f64) + v[1]
    return out, D


def random_poses(rng, n, trans_m):
    T = np.zeros((n, 3, 4))
    for k in range(n):
        T[k, :, :3] = lie.exp_so3(rng.normal(size=3))
        T[k, :, 3] = rng.uniform(-trans_m, trans_m, 3)
    return T


def reference(T0, xi):
    out = np.zeros_like(T0)
    for k in range(len(T0)):
        T = np.eye(4)
        T[:3] = T0[k]
        out[k] = (T @ lie.exp_se3(xi[k]))[:3]
    return out


def test_series_truncation_below_half_radian():
    """Truncated after t^8, the series stays within 1e-10 of the functions up to 0.5 rad
    (references in cancellation-free forms; (t - sin t) / t^3 only where FP64 resolves it)."""
    t = np.linspace(1e-6, 0.5, 2001)
    a, b, c = series_coeffs(t * t)
    rel = lambda x, y: np.max(np.abs(x - y) / np.abs(y))
    assert rel(a, np.sin(t) / t) < 1e-10
    assert rel(b, 2.0 * np.sin(0.5 * t) ** 2 / t ** 2) < 1e-10
    m = t > 1e-2
    assert rel(c[m], ((t - np.sin(t)) / t ** 3)[m]) < 1e-10


def test_mixed_update_matches_fp64_exp_map():
    rng = np.random.default_rng(4)
    n = 400
    T0 = random_poses(rng, n, 30.0)
    # rotation steps from 1e-9 to 1 rad (both branches), translation steps to 0.2 m
    ang = 10.0 ** rng.uniform(-9, 0, n)
    axis = rng.normal(size=(n, 3))
    axis /= np.linalg.norm(axis, axis=1, keepdims=True)
    xi = np.concatenate([axis * ang[:, None], rng.normal(size=(n, 3)) * 10.0 ** rng.uniform(-9, -0.7, (n, 1))], -1)
    got, D = update_mixed(T0, xi)
    ref = reference(T0, xi)
    dmax = np.abs(D.astype(f64)).max(axis=(1, 2))
    err = np.abs(got - ref).max(axis=(1, 2))
    # FP32 relative precision of the increment, plus ~48-bit rounding of the sum
    assert np.all(err <= 1e-6 * dmax + 1e-12 * (1.0 + np.abs(T0).max(axis=(1, 2))))
    # with the pose held in FP32 (as the reference's float32 state is), its own rounding
    # (~1e-6 m at 30 m) swamps the small steps
    fp32 = np.einsum('nik,nkj->nij', T0[:, :, :3].astype(f32), D).astype(f64) + T0.astype(f32)
    tiny = dmax < 1e-6
    assert tiny.sum() > 20
    assert np.median(np.abs(fp32 - ref).max(axis=(1, 2))[tiny]) > 100 * np.median(err[tiny])
