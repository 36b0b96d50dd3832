"""Generate golden vectors from the reference's own CPU solver.

Run in a container where the S-PGO sources are mounted (default
``/root/reference``):

    python tests/golden/make_golden.py [/path/to/S-PGO]

It imports ``PythonUtils/Optimizer.py`` through ``oracle.ref_shim``, builds a
seeded scene in the reference's own layout (landmark l anchored at
``map_value_to_index(l, L, N)``, observed left and right in every frame
n >= anchor; ``CUDAmanager.py:69-79``) and records:

* ``getJacobiansAndResidual`` -> J_T, J_alpha (one non-zero per row), r
  (``Optimizer.py:291-373``);
* ``getHessians`` -> H_TT, g_TT, H_aa (diagonal), g_aa, BB (``Optimizer.py:376-383``);
* two consecutive ``Optimizer.step`` calls -> poses and inverse depths after
  each (``Optimizer.py:135-289``);
* ``LieUtils.Exp_SE3`` / ``J_l_SO3`` / ``J_l_inv_SO3`` on seeded twists.

The fixtures are small ``.npz`` files committed next to this script.
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import lie, ref_shim  # noqa: E402


def make_scene(rng, N, L):
    """Ground-truth frames moving along +x looking down +z, points 3-8 m ahead."""
    Gt = np.zeros((N + 1, 4, 4))
    for k in range(N + 1):
        T = np.eye(4)
        if k > 0:
            T[:3, :3] = lie.exp_so3(rng.normal(0, 0.03, 3))
            T[:3, 3] = np.array([0.25 * k, 0.02 * k, 0.05 * k]) + rng.normal(0, 0.02, 3)
        Gt[k] = T
    anchors = np.array([min(int(l / L * N), N - 1) for l in range(L)])
    pts = np.zeros((L, 3))
    for l in range(L):
        a = anchors[l]
        p_cam = np.array([rng.uniform(-1.5, 1.5), rng.uniform(-1.0, 1.0), rng.uniform(3.0, 8.0)])
        pts[l] = Gt[a, :3, :3] @ p_cam + Gt[a, :3, 3]
    return Gt, anchors, pts


def project(K, T_cam_to_g, X):
    Tinv = lie.inv_se3(T_cam_to_g)
    t = Tinv[:3, :3] @ X + Tinv[:3, 3]
    p = K @ (t / t[2])
    return p


def build(seed, N, L, noise_px, pose_noise, depth_noise):
    rng = np.random.default_rng(seed)
    K = np.array([[320.0, 0, 320.0], [0, 320.0, 240.0], [0, 0, 1.0]])      # StereoSetup.py:12-19
    T_l_r = np.eye(4)
    T_l_r[0, 3] = -0.2                                                     # StereoSetup.py:26-31
    T_r_l = np.linalg.inv(T_l_r)
    Gt, anchors, pts = make_scene(rng, N, L)
    obs = {}
    for f in range(N + 1):
        for l in range(L):
            for right in (False, True):
                T = Gt[f] @ T_r_l if right else Gt[f]
                p = project(K, T, pts[l]).reshape(3, 1)
                p[:2, 0] += rng.normal(0, noise_px, 2)
                obs.setdefault(f, {}).setdefault(l, {})[right] = p
    inc_true = np.stack([np.linalg.inv(Gt[k + 1]) @ Gt[k] for k in range(N)])
    inc_est = np.stack([inc_true[k] @ lie.exp_se3(rng.normal(0, pose_noise, 6)) for k in range(N)])
    alpha_true = np.zeros(L)
    for l in range(L):
        Ta = lie.inv_se3(Gt[anchors[l]])
        alpha_true[l] = 1.0 / (Ta[:3, :3] @ pts[l] + Ta[:3, 3])[2]
    alpha_est = alpha_true * (1.0 + rng.normal(0, depth_noise, L))
    return dict(K=K, T_r_l=T_r_l, obs=obs, anchors=anchors, inc_est=inc_est,
                alpha_est=alpha_est, inc_true=inc_true, alpha_true=alpha_true)


def obs_arrays(sc, N, L):
    """CSR layout (landmark-major, frames ascending) of the reference's observation set."""
    host, auv, ptr, fr, uv = [], [], [0], [], []
    for l in range(L):
        a = int(sc["anchors"][l])
        host.append(a)
        auv.append(sc["obs"][a][l][False][:2, 0])
        for n in range(a, N + 1):
            fr.append(n)
            uv.append(np.concatenate([sc["obs"][n][l][False][:2, 0], sc["obs"][n][l][True][:2, 0]]))
        ptr.append(len(fr))
    return (np.array(host, np.int32), np.array(auv), np.array(ptr, np.int64),
            np.array(fr, np.int32), np.array(uv))


def run(ref_root, seed, N, L, out_name):
    opt_mod = ref_shim.install(ref_root)
    sc = build(seed, N, L, noise_px=1.0, pose_noise=0.02, depth_noise=0.05)
    opt = opt_mod.Optimizer(n=N, m=L)
    opt.estimated_incremental_poses = [p.copy() for p in sc["inc_est"]]
    opt.estimated_inverse_depths = [float(x) for x in sc["alpha_est"]]
    J_T, J_alpha, r = opt.getJacobiansAndResidual(sc["obs"])
    H_TT, g_TT, H_aa, g_aa, BB = opt.getHessians(sc["obs"])
    rows = J_alpha.shape[0]
    col = np.argmax(np.abs(J_alpha), axis=1)
    ja = J_alpha[np.arange(rows), col]
    assert np.count_nonzero(J_alpha) <= rows
    assert np.allclose(H_aa, np.diag(np.diag(H_aa)))
    # two CPU steps (Optimizer.step keeps step size / previous norm between calls)
    steps_p, steps_a = [], []
    for _ in range(2):
        opt.step(sc["obs"])
        steps_p.append(np.stack(opt.estimated_incremental_poses))
        steps_a.append(np.array([float(x) for x in opt.estimated_inverse_depths]))
    host, auv, ptr, fr, uv = obs_arrays(sc, N, L)
    # Lie pins
    LU = opt_mod.LieUtils()
    rng = np.random.default_rng(seed + 1000)
    xis = np.concatenate([rng.normal(0, 1.0, (16, 6)), rng.normal(0, 1e-6, (4, 6))])
    exp_se3 = np.stack([LU.Exp_SE3(x.reshape(6, 1)) for x in xis])
    jl = np.stack([LU.J_l_SO3(x[:3].reshape(3, 1)) for x in xis])
    jl_inv = np.stack([LU.J_l_inv_SO3(x[:3].reshape(3, 1)) for x in xis])
    np.savez_compressed(
        os.path.join(HERE, out_name),
        n_poses=N, intrinsics=np.array([320.0, 320.0, 320.0, 240.0, 320.0, 320.0, 320.0, 240.0]),
        T_rl=sc["T_r_l"], host=host, anchor_uv=auv, obs_ptr=ptr, obs_frame=fr, obs_uv=uv,
        poses=sc["inc_est"], alpha=sc["alpha_est"],
        ref_J_T=J_T, ref_j_alpha=ja, ref_j_alpha_col=col, ref_r=r.reshape(-1),
        ref_H_TT=H_TT, ref_g_TT=g_TT.reshape(-1), ref_H_aa_diag=np.diag(H_aa),
        ref_g_aa=g_aa.reshape(-1), ref_BB=BB,
        ref_step_poses=np.stack(steps_p), ref_step_alpha=np.stack(steps_a),
        lie_xi=xis, ref_exp_se3=exp_se3, ref_jl=jl, ref_jl_inv=jl_inv,
    )
    print("wrote", out_name, "rows", rows, "P", 6 * N, "L", L)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    run(root, 7, 3, 9, "ref_small.npz")
    run(root, 11, 6, 30, "ref_medium.npz")
