"""The allocation-free cost entry point (spgo_cost_noalloc) against the regular
solver's cost (spgo_export_system on an FP64 plan), through the C ABI.

spgo_cost_noalloc serves callers that cannot allocate device memory (inside a
CUDA graph capture they do not own, under a host framework that owns the
memory pool, on real-time threads).  This file is collected last so that a
run stopping at the first failure has run every other test before it; it
also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import spgo_gb300.native as nat
import spgo_gb300.scenes as scenes
from spgo_gb300.solver import BatchSolver

pytestmark = pytest.mark.gpu

REL_TOL = 1e-12  # the FP64 cost tolerance the parity tests use


def device_problem(p, dev, keep):
    """Upload one problem's arrays (C-ABI layout) and describe them."""
    t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
    arrs = dict(intr=t(p.intrinsics, np.float32), trl=t(np.asarray(p.T_rl).reshape(16), np.float64),
                host=t(p.host, np.int32), auv=t(np.asarray(p.anchor_uv).reshape(-1), np.float32),
                ptr=t(p.obs_ptr, np.int64), fr=t(p.obs_frame, np.int32),
                uv=t(np.asarray(p.obs_uv).reshape(-1), np.float32))
    keep.append(arrs)
    d = nat.DeviceProblem()
    d.n_poses, d.n_landmarks, d.n_obs = int(p.n_poses), p.n_landmarks, p.n_obs
    d.intrinsics, d.T_r_to_l, d.host = arrs["intr"].data_ptr(), arrs["trl"].data_ptr(), arrs["host"].data_ptr()
    d.anchor_uv, d.obs_ptr = arrs["auv"].data_ptr(), arrs["ptr"].data_ptr()
    d.obs_frame, d.obs_uv = arrs["fr"].data_ptr(), arrs["uv"].data_ptr()
    return d


def noalloc_cost(L, d, poses, alpha, params, dev):
    out = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    nat.check(L.spgo_cost_noalloc(C.byref(d), C.c_void_p(poses.data_ptr()), C.c_void_p(alpha.data_ptr()),
                                  C.byref(params), C.c_void_p(out.data_ptr()), C.c_void_p(st)), "cost_noalloc")
    torch.cuda.synchronize(dev)
    return float(out.item())


@pytest.mark.parametrize("loss,kw", [("l2", {}), ("cauchy", dict(loss_scale=3.0, near_boost=True))])
def test_noalloc_cost_matches_solver_twice(built_lib, cuda_device, loss, kw):
    dev = cuda_device
    p = scenes.circle_scene(77, 9, 300)
    bs = BatchSolver([p], precision="fp64", device=dev)
    bs.set_params(loss=loss, **kw)
    keep = []
    d = device_problem(p, dev, keep)
    # call 1: the initial state
    ref1 = bs.export_system(0)["cost"]
    got1 = noalloc_cost(built_lib, d, bs.poses, bs.alpha, bs.params, dev)
    assert abs(got1 - ref1) <= REL_TOL * abs(ref1)
    # call 2, right after: a different state (two Gauss-Newton steps later)
    bs.gn_step(2, 1.0)
    ref2 = bs.export_system(0)["cost"]
    got2 = noalloc_cost(built_lib, d, bs.poses, bs.alpha, bs.params, dev)
    assert abs(got2 - ref2) <= REL_TOL * abs(ref2)
    assert abs(got2 - got1) > 1e-3 * abs(got1)   # the second call really saw the new state


def test_noalloc_rejects_oversize(built_lib, cuda_device):
    d = nat.DeviceProblem()
    d.n_poses, d.n_landmarks, d.n_obs = 4096, 10, 0
    buf = torch.zeros(16, dtype=torch.float64, device=cuda_device)
    d.intrinsics = d.T_r_to_l = d.host = d.anchor_uv = d.obs_ptr = d.obs_frame = d.obs_uv = buf.data_ptr()
    rc = built_lib.spgo_cost_noalloc(C.byref(d), C.c_void_p(buf.data_ptr()), C.c_void_p(buf.data_ptr()),
                                     C.byref(nat.default_params()), C.c_void_p(buf.data_ptr()), None)
    assert rc == nat.SPGO_ERR_UNSUPPORTED
    assert b"allocation-free limits" in built_lib.spgo_last_error()


def test_noalloc_bad_frame_index_gives_nan(built_lib, cuda_device):
    """An observation frame outside [0, n_poses] in the caller's device arrays is
    skipped by the kernel's own checks and turns the cost into NaN (the call itself
    succeeds: the host cannot see device memory)."""
    dev = cuda_device
    p = scenes.circle_scene(77, 9, 300)
    bs = BatchSolver([p], precision="fp64", device=dev)
    keep = []
    good = device_problem(p, dev, keep)
    assert np.isfinite(noalloc_cost(built_lib, good, bs.poses, bs.alpha, bs.params, dev))
    q = p.copy()
    q.obs_frame = np.array(p.obs_frame, copy=True)
    q.obs_frame[5] = 1000  # no such frame
    bad = device_problem(q, dev, keep)
    assert np.isnan(noalloc_cost(built_lib, bad, bs.poses, bs.alpha, bs.params, dev))
    # the next call with valid arrays is unaffected
    assert np.isfinite(noalloc_cost(built_lib, good, bs.poses, bs.alpha, bs.params, dev))
