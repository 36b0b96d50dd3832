"""The mixed path's double-float reprojection residuals, restated on the CPU (numpy
float32, no GPU) and compared with the FP64 oracle.

csrc/k_linearize.cu's cost pass forms every residual from double-float values
(pairs of floats, csrc/dfloat.cuh: Knuth two-sum, two-product by FMA): the anchor
point R_a t_a with t_a = ((u - cx)/fx/alpha, (v - cy)/fy/alpha, 1/alpha), the
centre difference c_a - c_n, the rotation into camera n (a three-term dot product),
and r = ((z - c) t_z - f t_x) / t_z with only the final division in plain FP32.
The frame tables hold each global rotation and centre as a float pair.  Plain
FP32 on ~300 px quantities loses ~1e-5 px, which moves the cost at the 1e-6
relative level the LM stopping rule and gain ratio work at; this file checks the
restated double-float path stays near the FP64 residuals and well below that.
"""
import numpy as np

import spgo_gb300.scenes as scenes
from dfloat_numpy import add, df, div, dot3, mul, mul_f, neg, two_sum
from oracle import solver as S

f32, f64 = np.float32, np.float64


def residuals_double_float(p):
    """(O, 4) residuals (uL, vL, uR, vR) as the cost pass forms them."""
    G = S.global_poses(p.poses)
    cams = [G, G @ np.asarray(p.T_rl, f64)]
    lm, a, n = S._expand(p)
    intr = np.asarray(p.intrinsics, f64).astype(f32)
    uv = np.asarray(p.anchor_uv, f64).astype(f32)[lm]
    z = np.asarray(p.obs_uv, f64).astype(f32)
    al = df(np.asarray(p.alpha, f64)[lm])
    one = (np.ones(len(lm), f32), np.zeros(len(lm), f32))
    t3 = [div(div(two_sum(uv[:, 0], -np.full(len(lm), intr[2])), (np.full(len(lm), intr[0]), 0 * one[1])), al),
          div(div(two_sum(uv[:, 1], -np.full(len(lm), intr[3])), (np.full(len(lm), intr[1]), 0 * one[1])), al),
          div(one, al)]
    Ra = [df(G[a][:, k, :]) for k in range(3)]            # rows of the anchor's left rotation
    X = []
    for k in range(3):
        v = mul((Ra[k][0][:, 0], Ra[k][1][:, 0]), t3[0])
        v = add(v, mul((Ra[k][0][:, 1], Ra[k][1][:, 1]), t3[1]))
        v = add(v, mul((Ra[k][0][:, 2], Ra[k][1][:, 2]), t3[2]))
        X.append(v)
    out = np.zeros((len(lm), 4), f64)
    for cam in range(2):
        Gn = cams[cam][n]
        ca, cn = df(G[a][:, :3, 3]), df(Gn[:, :3, 3])
        Xc = []
        for k in range(3):
            d = add(two_sum(ca[0][:, k], -cn[0][:, k]), (ca[1][:, k] - cn[1][:, k], 0 * one[1]))
            Xc.append(add(X[k], d))
        Rh, Rl = df(Gn[:, :3, :3])
        tt = [dot3([Rh[:, 0, k], Rh[:, 1, k], Rh[:, 2, k]], [Rl[:, 0, k], Rl[:, 1, k], Rl[:, 2, k]], Xc)
              for k in range(3)]
        fx, fy, cx, cy = (np.full(len(lm), intr[4 * cam + q]) for q in range(4))
        nu = add(mul(two_sum(z[:, 2 * cam], -cx), tt[2]), neg(mul_f(tt[0], fx)))
        nv = add(mul(two_sum(z[:, 2 * cam + 1], -cy), tt[2]), neg(mul_f(tt[1], fy)))
        itz = f32(1) / tt[2][0]
        out[:, 2 * cam] = (nu[0] + nu[1]) * itz
        out[:, 2 * cam + 1] = (nv[0] + nv[1]) * itz
    return out


def residuals_plain_fp32(p):
    """The same residuals with every quantity a single float (for comparison)."""
    G = S.global_poses(p.poses).astype(f32)
    cams = [G, (S.global_poses(p.poses) @ np.asarray(p.T_rl, f64)).astype(f32)]
    lm, a, n = S._expand(p)
    intr = np.asarray(p.intrinsics, f64).astype(f32)
    uv = np.asarray(p.anchor_uv, f64).astype(f32)[lm]
    al = np.asarray(p.alpha, f64).astype(f32)[lm]
    t = np.stack([(uv[:, 0] - intr[2]) / intr[0] / al, (uv[:, 1] - intr[3]) / intr[1] / al, f32(1) / al], -1)
    Xw = np.einsum('oij,oj->oi', G[a][:, :3, :3], t) + G[a][:, :3, 3]
    z = np.asarray(p.obs_uv, f64).astype(f32)
    out = np.zeros((len(lm), 4), f64)
    for cam in range(2):
        Gn = cams[cam][n]
        tn = np.einsum('oji,oj->oi', Gn[:, :3, :3], Xw - Gn[:, :3, 3])
        fx, fy, cx, cy = intr[4 * cam:4 * cam + 4]
        out[:, 2 * cam] = z[:, 2 * cam] - (fx * tn[:, 0] / tn[:, 2] + cx)
        out[:, 2 * cam + 1] = z[:, 2 * cam + 1] - (fy * tn[:, 1] / tn[:, 2] + cy)
    return out


def test_double_float_residuals_match_fp64():
    p = scenes.circle_scene(21, 10, 300)
    # FP32 pixels and intrinsics, as the device sees them; the oracle then works in FP64
    p.obs_uv = np.asarray(p.obs_uv, f64).astype(f32).astype(f64)
    p.anchor_uv = np.asarray(p.anchor_uv, f64).astype(f32).astype(f64)
    p.intrinsics = np.asarray(p.intrinsics, f64).astype(f32).astype(f64)
    lm, a, n = S._expand(p)
    _, _, cams = S._camera_terms(p, S.global_poses(p.poses), lm, a, n)
    ref = np.concatenate([cams[0][0], cams[1][0]], -1)          # (O, 4) FP64 residuals
    r_df, r_32 = residuals_double_float(p), residuals_plain_fp32(p)
    err_df, err_32 = np.abs(r_df - ref), np.abs(r_32 - ref)
    # a few FP32 ulps of |r| from the final division (the perturbed start puts some
    # points thousands of px off), plus ~1e-6 px from the double-float numerator
    assert np.all(err_df <= 3e-7 * np.abs(ref) + 1e-6)
    assert np.median(err_32) > 20 * np.median(err_df)          # ~1e-5 px against ~2e-7 px
    # the cost: double-float well inside the 1e-6 relative level the LM decisions use
    cost = lambda r: 0.5 * float(np.sum(r * r))
    c_ref = cost(ref)
    assert abs(cost(r_df) - c_ref) / c_ref < 1e-7
    assert abs(cost(r_32) - c_ref) / c_ref > 10 * abs(cost(r_df) - c_ref) / c_ref
