"""Small FP64 SE(3) helpers for host-side scene set-up and evaluation.

Twist order (psi, rho) and Exp_SE3 = [[Exp_SO3(psi), J_l(psi) rho], [0, 1]]
follow S-PGO ``src/LieUtils/SE3.cu:3-38``.
"""
from __future__ import annotations

import numpy as np


def skew(v):
    return np.array([[0.0, -v[2], v[1]], [v[2], 0.0, -v[0]], [-v[1], v[0], 0.0]])


def exp_so3(psi):
    psi = np.asarray(psi, dtype=np.float64).reshape(3)
    th = float(np.linalg.norm(psi))
    S = skew(psi)
    if th < 1e-4:
        a, b = 1.0 - th * th / 6.0, 0.5 - th * th / 24.0
    else:
        a, b = np.sin(th) / th, (1.0 - np.cos(th)) / (th * th)
    return np.eye(3) + a * S + b * (S @ S)


def log_so3(R):
    R = np.asarray(R, dtype=np.float64).reshape(3, 3)
    c = np.clip(0.5 * (np.trace(R) - 1.0), -1.0, 1.0)
    w = np.array([R[2, 1] - R[1, 2], R[0, 2] - R[2, 0], R[1, 0] - R[0, 1]])
    th = float(np.arctan2(0.5 * np.linalg.norm(w), c))
    if th < 1e-4:
        return 0.5 * (1.0 + th * th / 6.0) * w
    if np.pi - th > 1e-2:
        return th / (2.0 * np.sin(th)) * w
    # near pi: a a^T = (sym(R) - c I) / (1 - c)
    M = (0.5 * (R + R.T) - c * np.eye(3)) / (1.0 - c)
    k = int(np.argmax(np.diag(M)))
    axis = M[:, k] / np.sqrt(max(M[k, k], 1e-300))
    axis /= np.linalg.norm(axis)
    if np.dot(axis, w) < 0:
        axis = -axis
    return th * axis


def log_se3(T):
    """Twist (psi, rho) with Exp_SE3(psi, rho) = T: rho = J_l(psi)^-1 t."""
    T = np.asarray(T, dtype=np.float64)
    psi = log_so3(T[:3, :3])
    th = float(np.linalg.norm(psi))
    S = skew(psi)
    if th < 1e-4:
        c = 1.0 / 12.0 + th * th / 720.0
    else:
        c = (1.0 - th * np.sin(th) / (2.0 * (1.0 - np.cos(th)))) / (th * th)
    Jinv = np.eye(3) - 0.5 * S + c * (S @ S)
    return np.concatenate([psi, Jinv @ T[:3, 3]])


def inv(T):
    T = np.asarray(T, dtype=np.float64)
    Ti = np.zeros_like(T)
    Rt = np.swapaxes(T[..., :3, :3], -1, -2)
    Ti[..., :3, :3] = Rt
    Ti[..., :3, 3] = -np.einsum('...ij,...j->...i', Rt, T[..., :3, 3])
    Ti[..., 3, 3] = 1.0
    return Ti


def pose_error(T_est, T_ref):
    """(rotation angle [rad], translation distance [m]) of inv(T_ref) T_est."""
    E = inv(T_ref) @ np.asarray(T_est, dtype=np.float64)
    return float(np.linalg.norm(log_so3(E[:3, :3]))), float(np.linalg.norm(E[:3, 3]))
