"""Golden vectors for the reference scene generator, from the reference's own code.

Run in a container where the S-PGO sources are mounted (default
``/root/reference``):

    python tests/golden/make_reference_scene.py [/path/to/S-PGO]

For each case it runs, from the reference:

* ``SamplePoses(n).poses`` after ``numpy.random.seed(s)`` and ``torch.manual_seed(s)``
  (``PythonUtils/utils.py:19-80``);
* ``get_point_samples(m)`` after ``numpy.random.seed(1000 + s)``
  (``PythonUtils/utils.py:133-152``);
* ``Simulator.compute_observations`` on those poses and points
  (``PythonUtils/Simulator.py:37-63``) and the feeder's loading rule
  (``CUDAmanager.py:69-79``: anchor ``map_value_to_index(l, M, N)`` from
  ``PythonUtils/Optimizer.py:12-18``, frames anchor..N, both cameras valid),

and stores the poses, points and the fed observation lists in
``ref_scene.npz`` next to this script.

``pypose`` is not installed; ``SamplePoses`` uses three of its operations, which are
restated below in float32 as pypose computes them: ``so3(x).Exp()`` (Rodrigues),
``SO3 * tensor`` with a plain 4-vector (the point action on a homogeneous vector:
rotate the first three entries, keep the fourth) and ``SE3([t, q]).matrix()``
(t, then a unit quaternion in x, y, z, w order).  That restatement is the one
part of this fixture not taken from the reference's own code.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import ref_shim  # noqa: E402

CASES = [(0, 5, 30), (1, 5, 30), (2, 10, 20)]   # (seed, n incremental poses, landmarks per frame)


def _skew(v):
    z = torch.zeros((), dtype=v.dtype)
    return torch.stack([torch.stack([z, -v[2], v[1]]), torch.stack([v[2], z, -v[0]]),
                        torch.stack([-v[1], v[0], z])])


class _SO3:
    def __init__(self, R):
        self.R = R                                       # [1, 3, 3] float32

    def __mul__(self, p):                                # point action on (*, 4)
        p = p.reshape(1, 4)
        v = (self.R @ p[:, :3].unsqueeze(-1)).squeeze(-1)
        return torch.cat([v, p[:, 3:]], 1)


class _so3:
    def __init__(self, x):
        self.x = x.reshape(1, 3).to(torch.float32)

    def Exp(self):
        w = self.x[0]
        th = torch.linalg.norm(w)
        S = _skew(w)
        a = torch.sin(th) / th
        b = (1 - torch.cos(th)) / (th * th)
        R = torch.eye(3) + a * S + b * (S @ S)
        return _SO3(R.unsqueeze(0))


class _SE3:
    def __init__(self, vec):
        self.v = vec.reshape(1, 7).to(torch.float32)

    def matrix(self):
        t = self.v[0, :3]
        x, y, z, w = self.v[0, 3:]
        R = torch.stack([
            torch.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)]),
            torch.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)]),
            torch.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)])])
        T = torch.eye(4)
        T[:3, :3] = R
        T[:3, 3] = t
        return T.unsqueeze(0)


def main(reference_root: str):
    opt_mod = ref_shim.install(reference_root)
    pp = sys.modules["pypose"]
    pp.so3 = _so3
    pp.SE3 = _SE3
    from PythonUtils import utils as ref_utils             # noqa: E402
    from PythonUtils.Simulator import Simulator            # noqa: E402
    from PythonUtils.StereoSetup import StereoSetup        # noqa: E402

    out = {}
    for ci, (s, n, m) in enumerate(CASES):
        F, M = n + 1, n * m
        np.random.seed(s)
        torch.manual_seed(s)
        W = np.stack([np.asarray(P, np.float64) for P in ref_utils.SamplePoses(n=F).poses])
        np.random.seed(1000 + s)
        pts = np.stack([np.asarray(p, np.float64) for p in ref_utils.get_point_samples(m=M)])
        sim = object.__new__(Simulator)
        sim.n, sim.m = F, M
        sim.cam = StereoSetup()
        sim.poses = list(W)
        sim.points = list(pts)
        sim.pixel_noise_std = 2.0
        sim.compute_observations()
        host, frames, uv, ptr, anchor_uv = [], [], [], [0], []
        for l in range(M):
            a = opt_mod.map_value_to_index(v=l, x=M, n=n)
            host.append(a)
            anc = (0.0, 0.0)
            for f in range(a, n + 1):
                if sim.validty[f][l][False] and sim.validty[f][l][True]:
                    pl = sim.observations[f][l][False].reshape(3)
                    pr = sim.observations[f][l][True].reshape(3)
                    frames.append(f)
                    uv.append([pl[0], pl[1], pr[0], pr[1]])
                    if f == a:
                        anc = (pl[0], pl[1])
            ptr.append(len(frames))
            anchor_uv.append(anc)
        out[f"c{ci}_case"] = np.array([s, n, m])
        out[f"c{ci}_W"] = W
        out[f"c{ci}_pts"] = pts
        out[f"c{ci}_host"] = np.array(host, np.int32)
        out[f"c{ci}_obs_ptr"] = np.array(ptr, np.int64)
        out[f"c{ci}_obs_frame"] = np.array(frames, np.int32)
        out[f"c{ci}_obs_uv"] = np.array(uv, np.float64).reshape(-1, 4)
        out[f"c{ci}_anchor_uv"] = np.array(anchor_uv, np.float64)
        print(f"case {ci}: seed {s}, N {n}, M {M}: {len(frames)} fed stereo observations")
    np.savez_compressed(os.path.join(HERE, "ref_scene.npz"), n_cases=np.array(len(CASES)), **out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
