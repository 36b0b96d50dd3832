"""FP64 SO(3)/SE(3) helpers for the oracle (test infrastructure only).

This module is part of the CPU oracle: only tests, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU baseline use it, as a checker.  Nothing on the product
path imports it.

Conventions follow S-PGO:
  * twist xi = (psi, rho): rotation first, translation second
    (``src/LieUtils/SE3.cu:3-38``, ``PythonUtils/LieUtils.py:101-109``);
  * Exp_SE3(xi) = [[Exp_SO3(psi), J_l(psi) rho], [0, 1]];
  * skew(v) is the cross-product matrix (``src/LieUtils/utils.cu:21-36``).
The reference calls ``cv2.Rodrigues`` for Exp/Log SO(3)
(``PythonUtils/LieUtils.py:22-33``); here the closed-form Rodrigues formula is
written out in numpy FP64 with Taylor branches near zero.
"""
from __future__ import annotations

import numpy as np


def skew(v):
    v = np.asarray(v, dtype=np.float64).reshape(3)
    return np.array([[0.0, -v[2], v[1]],
                     [v[2], 0.0, -v[0]],
                     [-v[1], v[0], 0.0]])


def skew_batch(v):
    """Cross-product matrices for an array of 3-vectors, shape (..., 3, 3)."""
    v = np.asarray(v, dtype=np.float64)
    z = np.zeros(v.shape[:-1])
    return np.stack([np.stack([z, -v[..., 2], v[..., 1]], -1),
                     np.stack([v[..., 2], z, -v[..., 0]], -1),
                     np.stack([-v[..., 1], v[..., 0], z], -1)], -2)


def _coeffs(theta):
    """(sin t / t, (1 - cos t) / t^2, (t - sin t) / t^3) with series near 0."""
    t2 = theta * theta
    if theta < 1e-4:
        a = 1.0 - t2 / 6.0 + t2 * t2 / 120.0
        b = 0.5 - t2 / 24.0 + t2 * t2 / 720.0
        c = 1.0 / 6.0 - t2 / 120.0 + t2 * t2 / 5040.0
    else:
        a = np.sin(theta) / theta
        b = (1.0 - np.cos(theta)) / t2
        c = (theta - np.sin(theta)) / (t2 * theta)
    return a, b, c


def exp_so3(psi):
    psi = np.asarray(psi, dtype=np.float64).reshape(3)
    theta = float(np.linalg.norm(psi))
    a, b, _ = _coeffs(theta)
    S = skew(psi)
    return np.eye(3) + a * S + b * (S @ S)


def left_jacobian_so3(psi):
    psi = np.asarray(psi, dtype=np.float64).reshape(3)
    theta = float(np.linalg.norm(psi))
    _, b, c = _coeffs(theta)
    S = skew(psi)
    return np.eye(3) + b * S + c * (S @ S)


def inv_left_jacobian_so3(psi):
    """J_l^{-1}(psi) (``PythonUtils/LieUtils.py:86-96``)."""
    psi = np.asarray(psi, dtype=np.float64).reshape(3)
    theta = float(np.linalg.norm(psi))
    S = skew(psi)
    if theta < 1e-4:
        k = 1.0 / 12.0 + theta * theta / 720.0
    else:
        k = 1.0 / (theta * theta) - (1.0 + np.cos(theta)) / (2.0 * theta * np.sin(theta))
    return np.eye(3) - 0.5 * S + k * (S @ S)


def log_so3(R):
    """Rotation vector of R (principal branch), robust near 0 and pi."""
    R = np.asarray(R, dtype=np.float64).reshape(3, 3)
    c = np.clip(0.5 * (np.trace(R) - 1.0), -1.0, 1.0)
    w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    theta = float(np.arctan2(0.5 * np.linalg.norm(w), c))
    if theta < 1e-4:
        return 0.5 * (1.0 + theta * theta / 6.0) * w
    if np.pi - theta > 1e-2:
        return theta / (2.0 * np.sin(theta)) * w
    # near pi: a a^T = (sym(R) - c I) / (1 - c)
    M = (0.5 * (R + R.T) - c * np.eye(3)) / (1.0 - c)
    k = int(np.argmax(np.diag(M)))
    axis = M[:, k] / np.sqrt(max(M[k, k], 1e-300))
    axis /= np.linalg.norm(axis)
    if np.dot(axis, w) < 0:
        axis = -axis
    return theta * axis


def exp_se3(xi):
    xi = np.asarray(xi, dtype=np.float64).reshape(6)
    T = np.eye(4)
    T[:3, :3] = exp_so3(xi[:3])
    T[:3, 3] = left_jacobian_so3(xi[:3]) @ xi[3:]
    return T


def log_se3(T):
    T = np.asarray(T, dtype=np.float64).reshape(4, 4)
    psi = log_so3(T[:3, :3])
    rho = inv_left_jacobian_so3(psi) @ T[:3, 3]
    return np.concatenate([psi, rho])


def inv_se3(T):
    T = np.asarray(T, dtype=np.float64)
    Ti = np.zeros_like(T)
    R = T[..., :3, :3]
    Rt = np.swapaxes(R, -1, -2)
    Ti[..., :3, :3] = Rt
    Ti[..., :3, 3] = -np.einsum('...ij,...j->...i', Rt, T[..., :3, 3])
    Ti[..., 3, 3] = 1.0
    return Ti
