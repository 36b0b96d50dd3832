"""Seeded synthetic stereo scenes for the benchmark configurations.

The reference ships only an unseeded simulator (``PythonUtils/Simulator.py``,
``PythonUtils/utils.py``); these generators are project-written and every draw
comes from ``numpy.random.Generator(PCG64(seed))``.

Size convention: ``n_poses`` N incremental poses, N + 1 frames, frame 0 fixed
(the reference's ``Solver(N, M)``: P = 6N pose parameters).

* ``circle_scene``  (config 0 / config 3 problems): N + 1 frames evenly spaced
  on a circle of radius 5 m facing its centre; pinhole fx = fy = 500,
  cx = 320, cy = 240, 640x480; stereo baseline 0.12 m; landmarks uniform in a
  10 m box around the centre.
* ``corridor_scene`` (configs 1 and 2): frames along a sinusoidal path (0.3 m
  per frame) looking sideways at a band of landmarks 3.5-8 m away, so each
  landmark is seen by about 20 consecutive frames; optional covisibility cap
  and uniform outliers.

Every landmark is anchored in a uniformly chosen frame that sees it, as
(u, v, inverse depth), and observed left and right in every frame where both
projections are in-bounds at depth 0.5-30 m.  Pixel noise N(0, 1 px).  The
initial state perturbs frames 1..N by a 0.02 rad rotation (random axis) and
N(0, 0.05 m) translation, and the inverse depths by x(1 + N(0, 0.1)).
"""
from __future__ import annotations

import numpy as np

from .problem import Problem
from . import se3

W_IMG, H_IMG = 640.0, 480.0
INTR = np.array([500.0, 500.0, 320.0, 240.0, 500.0, 500.0, 320.0, 240.0])
BASELINE_M = 0.12
DEPTH_MIN, DEPTH_MAX = 0.5, 30.0
ALPHA_MIN, ALPHA_MAX = 1.0 / 30.0, 1.0 / 0.2


class _TooFew(Exception):
    pass


def _look_at(center, target, down=np.array([0.0, 1.0, 0.0])):
    z = target - center
    z = z / np.linalg.norm(z)
    x = np.cross(down, z)
    x /= np.linalg.norm(x)
    y = np.cross(z, x)
    T = np.eye(4)
    T[:3, :3] = np.stack([x, y, z], 1)
    T[:3, 3] = center
    return T


def _visible(u, v, z):
    return (z >= DEPTH_MIN) & (z <= DEPTH_MAX) & (u >= 0) & (u < W_IMG) & (v >= 0) & (v < H_IMG)


def _build(rng, W, pts, cand, n_keep, window=None, outlier_frac=0.0, name=""):
    """Observe ``pts`` from world camera poses ``W`` (F,4,4); ``cand`` (L,C) frame candidates.

    ``pts`` is oversampled; the first ``n_keep`` points seen by at least two
    frames become the landmarks."""
    F = W.shape[0]
    N = F - 1
    T_rl = np.eye(4)
    T_rl[0, 3] = BASELINE_M
    # move the world into frame 0's camera frame (frame 0 is the identity)
    W0inv = se3.inv(W[0])
    Ws = np.einsum('ij,fjk->fik', W0inv, W)
    P = pts @ W0inv[:3, :3].T + W0inv[:3, 3]
    L = P.shape[0]
    Tcw_l = se3.inv(Ws)
    Tcw_r = se3.inv(np.einsum('fij,jk->fik', Ws, T_rl))
    valid_c = cand >= 0
    cidx = np.where(valid_c, cand, 0)
    Xl = P[:, None, :]
    Rl = Tcw_l[cidx, :3, :3]
    tl = Tcw_l[cidx, :3, 3]
    Rr = Tcw_r[cidx, :3, :3]
    tr = Tcw_r[cidx, :3, 3]
    pl = np.einsum('lcij,lcj->lci', Rl, np.broadcast_to(Xl, cidx.shape + (3,))) + tl
    pr = np.einsum('lcij,lcj->lci', Rr, np.broadcast_to(Xl, cidx.shape + (3,))) + tr
    K = INTR
    zl = pl[..., 2]
    zr = pr[..., 2]
    zls = np.where(np.abs(zl) > 1e-9, zl, 1e-9)
    zrs = np.where(np.abs(zr) > 1e-9, zr, 1e-9)
    ul = K[0] * pl[..., 0] / zls + K[2]
    vl = K[1] * pl[..., 1] / zls + K[3]
    ur = K[4] * pr[..., 0] / zrs + K[6]
    vr = K[5] * pr[..., 1] / zrs + K[7]
    vis = valid_c & _visible(ul, vl, zl) & _visible(ur, vr, zr)
    nvis = vis.sum(1)
    keep = nvis >= 2
    first = np.nonzero(keep)[0][:n_keep]
    if len(first) < n_keep:
        raise _TooFew()
    keep = np.zeros(L, bool)
    keep[first] = True
    # host: uniform among the frames that see the landmark
    host_slot = np.full(L, -1)
    r = rng.random(L)
    for l in np.nonzero(keep)[0]:
        slots = np.nonzero(vis[l])[0]
        host_slot[l] = slots[min(int(r[l] * len(slots)), len(slots) - 1)]
    host = np.where(keep, cand[np.arange(L), np.maximum(host_slot, 0)], -1)
    if window is not None:
        half = window // 2
        vis &= np.abs(cand - host[:, None]) <= half
    vis[~keep] = False
    lm_ids = np.nonzero(keep)[0]
    host = host[lm_ids]
    vis = vis[lm_ids]
    frames = cand[lm_ids]
    uvs = np.stack([ul, vl, ur, vr], -1)[lm_ids]
    P = P[lm_ids]
    Lk = len(lm_ids)
    # CSR, frames ascending per landmark
    order = np.argsort(np.where(vis, frames, 1 << 30), axis=1, kind='stable')
    fr_sorted = np.take_along_axis(frames, order, 1)
    vis_sorted = np.take_along_axis(vis, order, 1)
    uv_sorted = np.take_along_axis(uvs, order[..., None], 1)
    cnt = vis_sorted.sum(1)
    obs_ptr = np.zeros(Lk + 1, np.int64)
    obs_ptr[1:] = np.cumsum(cnt)
    obs_frame = fr_sorted[vis_sorted].astype(np.int32)
    obs_uv = uv_sorted[vis_sorted].astype(np.float64)
    obs_uv = obs_uv + rng.normal(0.0, 1.0, obs_uv.shape)
    lm_of_obs = np.repeat(np.arange(Lk), cnt)
    is_host = obs_frame == host[lm_of_obs]
    if outlier_frac > 0:
        cand_o = np.nonzero(~is_host)[0]
        pick = cand_o[rng.random(len(cand_o)) < outlier_frac]
        obs_uv[pick, 0] = rng.uniform(0, W_IMG, len(pick))
        obs_uv[pick, 1] = rng.uniform(0, H_IMG, len(pick))
        obs_uv[pick, 2] = rng.uniform(0, W_IMG, len(pick))
        obs_uv[pick, 3] = rng.uniform(0, H_IMG, len(pick))
    anchor_uv = obs_uv[is_host][:, :2].copy()
    assert anchor_uv.shape[0] == Lk
    # ground truth state
    gt_inc = np.stack([se3.inv(Ws[k + 1]) @ Ws[k] for k in range(N)])
    Th = Tcw_l[host]
    gt_alpha = 1.0 / (np.einsum('lj,lj->l', Th[:, 2, :3], P) + Th[:, 2, 3])
    # initial state: perturb frames 1..N, then back to incremental poses
    Wi = Ws.copy()
    for k in range(1, F):
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        dT = np.eye(4)
        dT[:3, :3] = se3.exp_so3(0.02 * axis)
        dT[:3, 3] = rng.normal(0.0, 0.05, 3)
        Wi[k] = Wi[k] @ dT
    init_inc = np.stack([se3.inv(Wi[k + 1]) @ Wi[k] for k in range(N)])
    alpha0 = np.clip(gt_alpha * (1.0 + rng.normal(0.0, 0.1, Lk)), ALPHA_MIN, ALPHA_MAX)
    prob = Problem(n_poses=N, intrinsics=INTR.copy(), T_rl=T_rl, host=host.astype(np.int32),
                   anchor_uv=anchor_uv, obs_ptr=obs_ptr, obs_frame=obs_frame, obs_uv=obs_uv,
                   poses=init_inc, alpha=alpha0, gt_poses=gt_inc, gt_alpha=gt_alpha, name=name)
    return prob


def circle_scene(seed: int, n_poses: int = 10, n_landmarks: int = 500, name: str = "") -> Problem:
    """N + 1 frames on a radius-5 m circle facing the centre; landmarks in a 10 m box."""
    rng = np.random.Generator(np.random.PCG64(seed))
    F = n_poses + 1
    W = np.zeros((F, 4, 4))
    for k in range(F):
        th = 2.0 * np.pi * k / F
        c = np.array([5.0 * np.sin(th), 0.0, -5.0 * np.cos(th)])
        W[k] = _look_at(c, np.zeros(3))
    for factor in (2, 8, 64):
        n_draw = factor * n_landmarks + 64
        pts = rng.uniform(-5.0, 5.0, (n_draw, 3))
        cand = np.broadcast_to(np.arange(F), (n_draw, F)).copy()
        try:
            return _build(rng, W, pts, cand, n_landmarks,
                          name=name or f"circle(N={n_poses},L={n_landmarks},seed={seed})")
        except _TooFew:
            continue
    raise RuntimeError("could not place the landmarks")


def corridor_scene(seed: int, n_poses: int = 100, n_landmarks: int = 20000, step_m: float = 0.3,
                   window: int | None = None, outlier_frac: float = 0.0, name: str = "") -> Problem:
    """Frames along a sinusoidal path looking sideways at a band of landmarks 3.5-8 m away."""
    rng = np.random.Generator(np.random.PCG64(seed))
    F = n_poses + 1
    length = step_m * n_poses
    W = np.zeros((F, 4, 4))
    xs = np.arange(F) * step_m
    for k in range(F):
        x = xs[k]
        c = np.array([x, 0.0, 0.5 * np.sin(2.0 * np.pi * x / 15.0)])
        yaw = 0.15 * np.cos(2.0 * np.pi * x / 15.0)
        tgt = c + np.array([np.sin(yaw), 0.0, np.cos(yaw)])
        W[k] = _look_at(c, tgt)
    n_draw = n_landmarks + n_landmarks // 4 + 64
    pts = np.stack([rng.uniform(-4.0, length + 4.0, n_draw),
                    rng.uniform(-2.0, 2.0, n_draw),
                    rng.uniform(3.5, 8.0, n_draw)], 1)
    # candidate frames: those within +-8 m along the path
    span = int(np.ceil(8.0 / step_m))
    k0 = np.clip(np.round(pts[:, 0] / step_m).astype(np.int64), 0, F - 1)
    cand = k0[:, None] + np.arange(-span, span + 1)[None, :]
    cand = np.where((cand >= 0) & (cand < F), cand, -1)
    return _build(rng, W, pts, cand, n_landmarks, window=window, outlier_frac=outlier_frac,
                  name=name or f"corridor(N={n_poses},L={n_landmarks},seed={seed})")


def config0(seed: int = 0) -> Problem:
    """Plain LM, FP64, CPU-runnable: N = 10, 500 landmarks."""
    return circle_scene(seed, 10, 500, name="config0")


def config1(seed: int = 1) -> Problem:
    """N = 100 on a 30 m sinusoidal path, 20k landmarks, ~400k stereo observations."""
    return corridor_scene(seed, 100, 20000, name="config1")


def config2(seed: int = 2) -> Problem:
    """N = 500, 200k landmarks, ~3M observations, 20-frame window, 5 % outliers."""
    return corridor_scene(seed, 500, 200000, window=20, outlier_frac=0.05, name="config2")


def config3_specs(seed: int = 3, n_problems: int = 256):
    """(problem seed, N, L) of each config-3 problem: N ~ U[8, 32], L ~ U[200, 3000]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    Ns = rng.integers(8, 33, n_problems)
    Ls = rng.integers(200, 3001, n_problems)
    seeds = rng.integers(0, 2**31 - 1, n_problems)
    return [(int(s), int(n), int(l)) for s, n, l in zip(seeds, Ns, Ls)]


def config3(seed: int = 3, n_problems: int = 256):
    """256 circle problems, N ~ U[8, 32], L ~ U[200, 3000], per-problem seeds."""
    return [circle_scene(s, n, l, name=f"config3[{i}]")
            for i, (s, n, l) in enumerate(config3_specs(seed, n_problems))]


def round_pixels_f32(p: Problem) -> Problem:
    """The problem with its pixels rounded to float32, the precision the solver's plan
    stores them in: the FP64 oracle and the GPU solvers then see the same data."""
    p.obs_uv = np.asarray(p.obs_uv, dtype=np.float32).astype(np.float64)
    p.anchor_uv = np.asarray(p.anchor_uv, dtype=np.float32).astype(np.float64)
    return p


# ---------------------------------------------------------------------------
# The reference's own scene distribution, restated with a seeded generator.
# ---------------------------------------------------------------------------

REF_WIDTH, REF_HEIGHT = 640.0, 512.0
REF_INTR = np.array([320.0, 320.0, 320.0, 240.0, 320.0, 320.0, 320.0, 240.0])
REF_BASELINE_M = 0.2
REF_MIN_DEPTH = 0.2


def reference_camera_poses(rng, n_frames: int, axis_draw=None) -> np.ndarray:
    """Camera-to-world poses of ``SamplePoses.create_samples`` (PythonUtils/utils.py:19-80).

    A random walk on a sphere: the polar and azimuth angles each grow by
    U(0, 20 deg) per frame, the radius is U(2.5, 3.5) and each position component
    is scaled by U(0.9, 1.1).  The camera looks at the origin (columns right,
    up, forward; the up hint is (U(0, 0.2), U(0, 0.2), 1)), then a 10 deg
    orientation noise about a random axis is applied the way the reference does
    it: the axis-angle rotation acts on the quaternion's vector part
    (``pp.SO3 * tensor`` is a point action on the homogeneous 4-vector), which
    turns R into Rn R Rn^T.

    ``rng`` needs ``uniform`` and ``normal``; the uniform draws come in the
    reference's order, so ``numpy.random.RandomState(s)`` reproduces the
    reference's stream after ``numpy.random.seed(s)``.  ``axis_draw()`` returns
    the noise axis (the reference draws it from torch's generator); the default
    is ``rng.normal(size=3)``."""
    W = np.zeros((n_frames, 4, 4))
    theta = phi = 0.0
    for k in range(n_frames):
        r = rng.uniform(2.5, 3.5)
        theta += abs(rng.uniform(0.0, 20.0) * np.pi / 180.0)
        phi += abs(rng.uniform(0.0, 20.0) * np.pi / 180.0)
        sx = rng.uniform(0.9, 1.1)
        sy = rng.uniform(0.9, 1.1)
        sz = rng.uniform(0.9, 1.1)
        pos = np.array([r * np.sin(phi) * np.cos(theta) * sx, r * np.sin(phi) * np.sin(theta) * sy,
                        r * np.cos(phi) * sz])
        fwd = -pos / np.linalg.norm(pos)
        ux = rng.uniform(0.0, 0.2)
        uy = rng.uniform(0.0, 0.2)
        up = np.array([ux, uy, 1.0])
        up /= np.linalg.norm(up)
        right = np.cross(up, fwd)
        right /= np.linalg.norm(right)
        up = np.cross(fwd, right)
        R = np.stack([right, up, fwd], 1)
        axis = np.asarray(axis_draw() if axis_draw is not None else rng.normal(size=3), np.float64)
        axis /= np.linalg.norm(axis)
        Rn = se3.exp_so3((10.0 * np.pi / 180.0) * axis)
        W[k] = np.eye(4)
        W[k, :3, :3] = Rn @ R @ Rn.T
        W[k, :3, 3] = pos
    return W


def reference_points(rng, m: int) -> np.ndarray:
    """``get_point_samples`` (PythonUtils/utils.py:133-152): per point a radius
    U(0, 2.5), then a uniform direction (azimuth U(0, 2 pi), cos(polar) U(-1, 1)),
    drawn in the reference's order."""
    pts = np.zeros((m, 3))
    for l in range(m):
        r = rng.uniform(0.0, 2.5)
        az = rng.uniform(0.0, 2.0 * np.pi)
        pol = np.arccos(rng.uniform(-1.0, 1.0))
        pts[l] = r * np.array([np.sin(pol) * np.cos(az), np.sin(pol) * np.sin(az), np.cos(pol)])
    return pts


def reference_scene(seed: int, n_poses: int = 10, landmarks_per_frame: int = 96, pixel_noise: float = 0.0,
                    name: str = "") -> Problem:
    """One window of the reference's divergence study (``CUDAmanager.Manager(n, m)``):
    ``Simulator(n + 1 frames, n * m landmarks)`` (PythonUtils/Simulator.py:12-35) with
    every draw from ``numpy.random.Generator(PCG64(seed))``; see
    ``reference_scene_from`` for the observation and initial-state rules."""
    rng = np.random.Generator(np.random.PCG64(seed))
    N = int(n_poses)
    W = reference_camera_poses(rng, N + 1)
    pts = reference_points(rng, N * int(landmarks_per_frame))
    return reference_scene_from(W, pts, noise_rng=rng if pixel_noise > 0 else None, pixel_noise=pixel_noise,
                                name=name or f"reference(N={N},m={landmarks_per_frame},seed={seed})")


def reference_scene_from(W: np.ndarray, pts: np.ndarray, noise_rng=None, pixel_noise: float = 0.0,
                         name: str = "") -> Problem:
    """The reference feeder's problem for camera-to-world poses ``W`` [N+1, 4, 4] and
    world points ``pts`` [M, 3].

    - StereoSetup (PythonUtils/StereoSetup.py:8-35): fx = fy = 320, cx = 320,
      cy = 240, 640x512, right camera 0.2 m along +x (camera-to-world W T_r_l).
    - An observation is valid when depth >= 0.2 m, u <= 640 and v <= 512 (no lower
      bound on u, v: Simulator.py:53-57), and is fed only when valid in both
      cameras (CUDAmanager.py:69-79).
    - Landmark l is anchored in frame ``map_value_to_index(l, M, N)`` and fed for
      every frame from its anchor to N (CUDAmanager.py:71-73).
    - The anchor pixel is what the reference kernel reads from its observation
      tensor (Solver_cuda.cu:147): the anchor frame's left observation when it was
      fed, else the tensor's initial (0, 0) (include/Solver.hpp:33).
    - The feeder passes the noise-free projections (``simulator.observations``);
      ``pixel_noise`` > 0 adds N(0, pixel_noise) from ``noise_rng`` instead, as the
      simulator's noisy copy does (std 2 px there).
    - Initial state: identity incremental poses and inverse depth 1 (the CUDA
      solver's initial tensors, include/Solver.hpp:36-44).
    """
    W = np.asarray(W, np.float64)
    pts = np.asarray(pts, np.float64)
    F = W.shape[0]
    N = F - 1
    M = pts.shape[0]
    T_rl = np.eye(4)
    T_rl[0, 3] = REF_BASELINE_M
    # general inverses, as the reference takes them (its poses come out of float32
    # and are orthonormal only to float32 rounding)
    Tcw_l = np.linalg.inv(W)
    Tcw_r = np.linalg.inv(np.einsum('fij,jk->fik', W, T_rl))
    K = REF_INTR

    def project(Tcw, fx, fy, cx, cy):
        pc = np.einsum('fij,lj->lfi', Tcw[:, :3, :3], pts) + Tcw[None, :, :3, 3]
        z = pc[..., 2]
        return fx * pc[..., 0] / z + cx, fy * pc[..., 1] / z + cy, z

    ul, vl, zl = project(Tcw_l, *K[:4])
    ur, vr, zr = project(Tcw_r, *K[4:])
    ok_l = (zl >= REF_MIN_DEPTH) & (ul <= REF_WIDTH) & (vl <= REF_HEIGHT)
    ok_r = (zr >= REF_MIN_DEPTH) & (ur <= REF_WIDTH) & (vr <= REF_HEIGHT)
    uv = np.stack([ul, vl, ur, vr], -1)                      # [M, F, 4]
    if pixel_noise > 0:
        uv = uv + noise_rng.normal(0.0, pixel_noise, uv.shape)
    host = np.array([anchor_frame(l, M, N) for l in range(M)], np.int64)
    fed = ok_l & ok_r & (np.arange(F)[None, :] >= host[:, None])
    cnt = fed.sum(1)
    obs_ptr = np.zeros(M + 1, np.int64)
    obs_ptr[1:] = np.cumsum(cnt)
    lm_of, fr_of = np.nonzero(fed)                            # landmark-major, frames ascending
    obs_frame = fr_of.astype(np.int32)
    obs_uv = uv[lm_of, fr_of].astype(np.float64)
    li = np.arange(M)
    anchor_uv = np.where(fed[li, host][:, None], uv[li, host, :2], 0.0)
    gt_inc = np.stack([np.linalg.inv(W[k + 1]) @ W[k] for k in range(N)])   # Simulator.py:67-78
    gt_alpha = 1.0 / zl[li, host]
    return Problem(n_poses=N, intrinsics=K.copy(), T_rl=T_rl, host=host.astype(np.int32),
                   anchor_uv=anchor_uv, obs_ptr=obs_ptr, obs_frame=obs_frame, obs_uv=obs_uv,
                   poses=np.broadcast_to(np.eye(4), (N, 4, 4)).copy(), alpha=np.ones(M),
                   gt_poses=gt_inc, gt_alpha=gt_alpha, name=name)


def anchor_frame(v: int, x: int, n: int) -> int:
    """``map_value_to_index`` (PythonUtils/Optimizer.py:12-18): value v of [0, x] to a
    frame index in [0, n - 1]."""
    vc = max(0, min(v, x))
    return min(int((vc / x) * n), n - 1)
