"""Host-side container for one stereo pose-graph / bundle-adjustment problem.

Layout (landmark-major CSR, the order the CUDA kernels read):

* ``n_poses`` N incremental poses T_curr_to_next[k], k = 0..N-1; frames 0..N,
  frame 0 fixed at the identity (S-PGO ``include/Solver.hpp:36-41``,
  ``src/Optimization/Solver_cuda.cu:452-491``);
* per landmark l: host (anchor) frame ``host[l]``, the left pixel observed in
  the host ``anchor_uv[l]`` and the inverse depth ``alpha[l]``
  (``Solver_cuda.cu:146-157``);
* per stereo observation o (grouped by landmark through ``obs_ptr``, frames
  ascending inside a landmark): target frame ``obs_frame[o]`` and the left and
  right pixels ``obs_uv[o] = (uL, vL, uR, vR)``.  The host frame's own stereo
  observation is part of the list, as in the reference feeder
  (``CUDAmanager.py:69-79``).
"""
from __future__ import annotations

import dataclasses
from typing import Optional

import numpy as np


@dataclasses.dataclass
class Problem:
    n_poses: int
    intrinsics: np.ndarray          # (8,) fx_l, fy_l, cx_l, cy_l, fx_r, fy_r, cx_r, cy_r
    T_rl: np.ndarray                # (4,4) pose of the right camera in the left camera frame
    host: np.ndarray                # (L,) int32
    anchor_uv: np.ndarray           # (L,2) float64
    obs_ptr: np.ndarray             # (L+1,) int64
    obs_frame: np.ndarray           # (O,) int32
    obs_uv: np.ndarray              # (O,4) float64
    poses: np.ndarray               # (N,4,4) float64 incremental poses (state)
    alpha: np.ndarray               # (L,) float64 inverse depths (state)
    gt_poses: Optional[np.ndarray] = None
    gt_alpha: Optional[np.ndarray] = None
    name: str = ""

    @property
    def n_landmarks(self) -> int:
        return int(len(self.host))

    @property
    def n_obs(self) -> int:
        return int(len(self.obs_frame))

    @property
    def n_params(self) -> int:
        return 6 * int(self.n_poses)

    def copy(self) -> "Problem":
        return dataclasses.replace(
            self, poses=np.array(self.poses, dtype=np.float64, copy=True),
            alpha=np.array(self.alpha, dtype=np.float64, copy=True))

    def validate(self) -> None:
        N, L, O = int(self.n_poses), self.n_landmarks, self.n_obs
        if N < 1:
            raise ValueError("n_poses must be >= 1")
        if self.obs_ptr.shape != (L + 1,) or self.obs_ptr[0] != 0 or self.obs_ptr[-1] != O:
            raise ValueError("obs_ptr must be a CSR offset array over the observations")
        if np.any(np.diff(self.obs_ptr) < 0):
            raise ValueError("obs_ptr must be non-decreasing")
        if np.any(self.host < 0) or np.any(self.host > N):
            raise ValueError("host frame out of range")
        if O and (np.any(self.obs_frame < 0) or np.any(self.obs_frame > N)):
            raise ValueError("observation frame out of range")
        if self.poses.shape != (N, 4, 4) or self.alpha.shape != (L,):
            raise ValueError("state shape mismatch")
        for l in range(L) if L < 4096 else []:
            f = self.obs_frame[self.obs_ptr[l]:self.obs_ptr[l + 1]]
            if np.any(np.diff(f) <= 0):
                raise ValueError("frames must be strictly ascending inside a landmark")

    def span(self):
        """Per landmark, the pose-block window [lo, hi) its Jacobian touches."""
        L = self.n_landmarks
        lo = np.array(self.host, dtype=np.int64)
        hi = np.array(self.host, dtype=np.int64)
        cnt = np.diff(self.obs_ptr)
        if self.n_obs:
            lm = np.repeat(np.arange(L), cnt)
            np.minimum.at(lo, lm, self.obs_frame.astype(np.int64))
            np.maximum.at(hi, lm, self.obs_frame.astype(np.int64))
        return lo, hi
