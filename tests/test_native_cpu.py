"""The C-ABI library without a GPU: it builds, loads, exports every symbol the
header declares, and its host-side planner validates input like the
reference's asserts (src/Optimization/Solver.cpp:41-44)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import spgo_gb300.native as nat
import spgo_gb300.scenes as scenes

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "spgo.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"\b(spgo_[a-z_]+)\s*\(", src)))


def test_exports_every_declared_symbol(built_lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(built_lib, n), n
    assert set(names) == set(nat.EXPORTED)
    assert built_lib.spgo_version() == 1


def host_problem(p, keep, f64=False):
    arrs = dict(intr=np.ascontiguousarray(p.intrinsics, np.float32),
                trl=np.ascontiguousarray(p.T_rl, np.float64).reshape(16),
                host=np.ascontiguousarray(p.host, np.int32),
                auv=np.ascontiguousarray(p.anchor_uv, np.float32).reshape(-1),
                ptr=np.ascontiguousarray(p.obs_ptr, np.int64),
                fr=np.ascontiguousarray(p.obs_frame, np.int32),
                uv=np.ascontiguousarray(p.obs_uv, np.float32).reshape(-1))
    keep.append(arrs)
    h = nat.HostProblem()
    h.n_poses, h.n_landmarks, h.n_obs = int(p.n_poses), p.n_landmarks, p.n_obs
    h.intrinsics = arrs["intr"].ctypes.data
    h.T_r_to_l = arrs["trl"].ctypes.data
    h.host = arrs["host"].ctypes.data
    h.obs_ptr = arrs["ptr"].ctypes.data
    h.obs_frame = arrs["fr"].ctypes.data
    if f64:  # the optional FP64 pixel arrays instead of the float ones
        arrs["auv64"] = np.ascontiguousarray(p.anchor_uv, np.float64).reshape(-1)
        arrs["uv64"] = np.ascontiguousarray(p.obs_uv, np.float64).reshape(-1)
        h.anchor_uv_f64 = arrs["auv64"].ctypes.data
        h.obs_uv_f64 = arrs["uv64"].ctypes.data
    else:
        h.anchor_uv = arrs["auv"].ctypes.data
        h.obs_uv = arrs["uv"].ctypes.data
    return h


def plan(problems, prec=nat.PREC_MIXED, f64=False):
    keep = []
    arr = (nat.HostProblem * len(problems))(*[host_problem(p, keep, f64) for p in problems])
    out = C.c_void_p()
    rc = nat.lib().spgo_plan_create(arr, len(problems), prec, C.byref(out))
    return rc, out


def test_default_params_layout(built_lib):
    """The ctypes mirror of spgo_params matches the C struct: spgo_default_params
    writes nothing past it, and every field reads back its documented default."""
    n = C.sizeof(nat.Params)
    buf = (C.c_ubyte * (n + 64))(*([0xA5] * (n + 64)))
    nat.lib().spgo_default_params(C.cast(buf, C.POINTER(nat.Params)))
    assert all(b == 0xA5 for b in bytes(buf)[n:])
    d = nat.Params.from_buffer_copy(bytes(buf)[:n])
    assert d.max_iters > 0 and d.outer_steps == 2 and d.use_tc == 1
    assert abs(d.outer_tol - 1e-3) < 1e-9 and d.ctl_min_log10 == -6.0 and d.stop_rho == 0.0


@pytest.mark.parametrize("f64", [False, True])
def test_plan_sizes(built_lib, f64):
    ps = [scenes.circle_scene(s, 8 + s, 100 + 37 * s) for s in range(5)]
    rc, pl = plan(ps, f64=f64)
    assert rc == 0
    sz = nat.PlanSizes()
    assert built_lib.spgo_plan_sizes_get(pl, C.byref(sz)) == 0
    assert sz.n_problems == 5
    assert sz.total_poses == sum(p.n_poses for p in ps)
    assert sz.total_landmarks == sum(p.n_landmarks for p in ps)
    assert sz.total_obs == sum(p.n_obs for p in ps)
    assert sz.n_chunks >= sum((p.n_landmarks + 31) // 32 for p in ps)
    assert sz.max_params == 6 * 12
    assert sz.static_bytes > 0 and sz.workspace_bytes > 0
    lm_off = (C.c_int32 * 5)()
    pose_off = (C.c_int32 * 5)()
    assert built_lib.spgo_plan_offsets(pl, lm_off, pose_off) == 0
    assert list(lm_off) == list(np.cumsum([0] + [p.n_landmarks for p in ps])[:-1])
    built_lib.spgo_plan_destroy(pl)


def test_plan_rejects_bad_input(built_lib):
    base = scenes.circle_scene(3, 6, 50)
    bad = base.copy()
    bad.host = base.host.copy()
    bad.host[0] = 99
    assert plan([bad])[0] == -1
    bad = base.copy()
    bad.obs_frame = base.obs_frame.copy()
    bad.obs_frame[1], bad.obs_frame[0] = base.obs_frame[0], base.obs_frame[1]  # not ascending
    assert plan([bad])[0] == -1
    bad = base.copy()
    bad.obs_ptr = base.obs_ptr.copy()
    bad.obs_ptr[-1] += 1
    assert plan([bad])[0] == -1
    msg = built_lib.spgo_last_error().decode()
    assert "obs_ptr" in msg
    rc, _ = plan([base], prec=7)
    assert rc == -1


def test_plan_rejects_too_wide_window(built_lib):
    p = scenes.corridor_scene(1, 120, 400)
    p.obs_frame = p.obs_frame.copy()
    # stretch landmark 0 over more than SPGO_MAX_WINDOW poses
    s, e = p.obs_ptr[0], p.obs_ptr[1]
    p.host = p.host.copy()
    p.host[0] = 0
    p.obs_frame[s:e] = np.linspace(0, 120, e - s).astype(np.int32)
    if e - s >= 2:
        assert plan([p])[0] == -2


def test_host_plan_on_a_worker_thread(built_lib):
    """The planner needs no device: HostPlan builds on another thread (as
    solve_stream does) and reports the same sizes as a plan built here."""
    from concurrent.futures import ThreadPoolExecutor
    from spgo_gb300.solver import HostPlan
    ps = [scenes.circle_scene(s, 5 + s, 60 + 11 * s) for s in range(3)]
    with ThreadPoolExecutor(1) as ex:
        hp = ex.submit(HostPlan, ps, "mixed").result()
    rc, pl = plan(ps)
    assert rc == 0
    a, b = nat.PlanSizes(), nat.PlanSizes()
    assert built_lib.spgo_plan_sizes_get(hp.handle, C.byref(a)) == 0
    assert built_lib.spgo_plan_sizes_get(pl, C.byref(b)) == 0
    assert (a.static_bytes, a.workspace_bytes, a.n_chunks) == (b.static_bytes, b.workspace_bytes, b.n_chunks)
    hp.close()
    built_lib.spgo_plan_destroy(pl)


def test_plan_options_shape_the_schur_work_lists(built_lib):
    """spgo_plan_create_opts: the Schur work shapes change how the (chunk, tile)
    products are split into work items, never which products there are; out-of-range
    options are refused."""
    from spgo_gb300.solver import HostPlan
    ps = [scenes.circle_scene(40 + s, 12 + 6 * s, 900 + 400 * s) for s in range(3)]
    sizes = {}
    for opts in (None, dict(tc_split=16), dict(tc_split=64), dict(simt_split=4, tc_split=8)):
        hp = HostPlan(ps, "mixed", opts)
        sz = nat.PlanSizes()
        assert built_lib.spgo_plan_sizes_get(hp.handle, C.byref(sz)) == 0
        sizes[str(opts)] = sz
        assert sz.tc_split == (opts or {}).get("tc_split", 64)
        assert sz.simt_split == (opts or {}).get("simt_split", 16)
        hp.close()
    base = sizes["None"]
    for sz in sizes.values():
        assert (sz.tc_chunk_tiles, sz.schur_chunk_tiles, sz.n_chunks) == \
            (base.tc_chunk_tiles, base.schur_chunk_tiles, base.n_chunks)
    assert sizes[str(dict(tc_split=16))].n_tc_items > base.n_tc_items
    assert sizes[str(dict(simt_split=4, tc_split=8))].n_schur_items > base.n_schur_items
    for bad in (dict(tc_split=65), dict(simt_split=-1), dict(tc_split=128)):
        with pytest.raises(RuntimeError):
            HostPlan(ps, "mixed", bad)
