"""Host-side solvers over the CUDA library.

* ``BatchSolver``: one or many ``Problem``s in one plan; device memory comes
  from PyTorch (``torch.empty`` on the target device), kernels run on the
  current CUDA stream.  Nielsen LM (``solve``/``iterate``/``status``), the
  reference's Gauss-Newton ``step`` semantics (``gn_step``) and a dense export
  of the linear system for parity checks.
* ``CudaSolver``: the reference binding's class (``src/CythonAPI/Solver.pyx``)
  with the same method names, argument layouts and return shapes, so
  ``CUDAmanager.py``-style callers switch by changing the import.
"""
from __future__ import annotations

import ctypes as C
import collections
from concurrent.futures import ThreadPoolExecutor
from typing import Iterable, Iterator, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import native as nat
from .problem import Problem

_PREC = {"mixed": nat.PREC_MIXED, "fp64": nat.PREC_FP64}
_LOSS = {"l2": nat.LOSS_L2, "cauchy": nat.LOSS_CAUCHY, "huber": nat.LOSS_HUBER}


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


def _to34(poses: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(poses, dtype=np.float64)[:, :3, :4]).reshape(-1, 12)


def _to44(p34: np.ndarray) -> np.ndarray:
    n = p34.shape[0]
    out = np.zeros((n, 4, 4))
    out[:, :3, :] = p34.reshape(n, 3, 4)
    out[:, 3, 3] = 1.0
    return out


class HostPlan:
    """The host half of a ``BatchSolver``: the problems marshalled and planned
    (``spgo_plan_create``: sorting, chunking and the static arrays, written into
    page-locked staging).  It needs no device work, so it can be built on another
    thread while an earlier batch solves (the planner releases the GIL)."""

    def __init__(self, problems: Sequence[Problem], precision: str = "mixed", options: Optional[dict] = None):
        """options: the Schur work shapes (``tc_split``, ``simt_split``;
        ``spgo_plan_options``), None for the defaults."""
        self.L = nat.lib()
        self.problems = list(problems)
        if not self.problems:
            raise ValueError("no problems")
        self.precision = precision
        # host arrays must stay alive until the plan is built (the library copies them);
        # FP64 pixels go in as they are (the planner rounds them while it sorts)
        keep = []
        hp = (nat.HostProblem * len(self.problems))()
        for i, p in enumerate(self.problems):
            arrs = (np.ascontiguousarray(p.intrinsics, dtype=np.float32),
                    np.ascontiguousarray(p.T_rl, dtype=np.float64),
                    np.ascontiguousarray(p.host, dtype=np.int32),
                    np.ascontiguousarray(p.anchor_uv, dtype=np.float64),
                    np.ascontiguousarray(p.obs_ptr, dtype=np.int64),
                    np.ascontiguousarray(p.obs_frame, dtype=np.int32),
                    np.ascontiguousarray(p.obs_uv, dtype=np.float64))
            keep.append(arrs)
            h = hp[i]
            h.n_poses = int(p.n_poses)
            h.n_landmarks = int(arrs[2].shape[0])
            h.n_obs = int(arrs[5].shape[0])
            h.intrinsics = arrs[0].ctypes.data
            h.T_r_to_l = arrs[1].ctypes.data
            h.host = arrs[2].ctypes.data
            h.anchor_uv_f64 = arrs[3].ctypes.data
            h.obs_ptr = arrs[4].ctypes.data
            h.obs_frame = arrs[5].ctypes.data
            h.obs_uv_f64 = arrs[6].ctypes.data
        plan = C.c_void_p()
        opts = nat.PlanOptions()
        for k, v in (options or {}).items():
            setattr(opts, k, int(v))
        nat.check(self.L.spgo_plan_create_opts(hp, len(self.problems), _PREC[precision], C.byref(opts),
                                               C.byref(plan)), "plan_create")
        self.handle = plan

    def close(self):
        if getattr(self, "handle", None):
            self.L.spgo_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchSolver:
    """Solve a batch of independent problems with one set of kernel launches."""

    def __init__(self, problems: Optional[Sequence[Problem]] = None, precision: str = "mixed", device="cuda",
                 stream: Optional[torch.cuda.Stream] = None, plan: Optional[HostPlan] = None,
                 plan_options: Optional[dict] = None):
        """``problems`` are planned here (with the Schur work shapes ``plan_options``,
        see ``HostPlan``), or ``plan`` (a ``HostPlan``, whose ownership passes to this
        solver) was planned beforehand."""
        self.L = nat.lib()
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("BatchSolver runs on a CUDA device only")
        self._stream = stream
        if plan is None:
            plan = HostPlan(problems if problems is not None else [], precision, plan_options)
        self._host_plan = plan
        self.problems = plan.problems
        self.precision = plan.precision
        plan = plan.handle
        self._plan = plan
        sz = nat.PlanSizes()
        nat.check(self.L.spgo_plan_sizes_get(plan, C.byref(sz)), "plan_sizes")
        self.sizes = sz
        B = len(self.problems)
        lm_off = (C.c_int32 * B)()
        pose_off = (C.c_int32 * B)()
        nat.check(self.L.spgo_plan_offsets(plan, lm_off, pose_off), "plan_offsets")
        self.lm_off = np.array(lm_off[:], dtype=np.int64)
        self.pose_off = np.array(pose_off[:], dtype=np.int64)
        dev = self.device
        # 256-byte aligned device buffers (caller-owned, PyTorch allocator)
        self.d_static = self._aligned(sz.static_bytes)
        self.d_ws = self._aligned(sz.workspace_bytes)
        self.poses = torch.zeros(max(1, sz.total_poses) * 12, dtype=torch.float64, device=dev)
        self.alpha = torch.zeros(max(1, sz.total_landmarks), dtype=torch.float64, device=dev)
        self.load_state()
        solver = C.c_void_p()
        nat.check(self.L.spgo_solver_create(plan, C.c_void_p(self._addr(self.d_static)), sz.static_bytes,
                                            C.c_void_p(self._addr(self.d_ws)), sz.workspace_bytes,
                                            C.c_void_p(self.poses.data_ptr()), C.c_void_p(self.alpha.data_ptr()),
                                            self._sp(), C.byref(solver)), "solver_create")
        self._solver = solver  # (the upload runs on the stream; the plan outlives it)
        self.params = nat.default_params()
        self._apply_params()

    # -- memory helpers ---------------------------------------------------------
    def _aligned(self, nbytes: int):
        t = torch.empty(int(nbytes) + 256, dtype=torch.uint8, device=self.device)
        return t

    @staticmethod
    def _addr(t: torch.Tensor) -> int:
        a = t.data_ptr()
        return (a + 255) & ~255

    def _sp(self):
        st = self._stream if self._stream is not None else torch.cuda.current_stream(self.device)
        return C.c_void_p(st.cuda_stream)

    def synchronize(self):
        st = self._stream if self._stream is not None else torch.cuda.current_stream(self.device)
        st.synchronize()

    # -- state ------------------------------------------------------------------
    def load_state(self):
        """Copy every problem's ``poses``/``alpha`` into the device state."""
        P = np.concatenate([_to34(p.poses) for p in self.problems]).reshape(-1)
        A = np.concatenate([np.asarray(p.alpha, dtype=np.float64) for p in self.problems])
        self.poses[:P.size].copy_(torch.from_numpy(P))
        self.alpha[:A.size].copy_(torch.from_numpy(A))

    def get_poses(self, b: int) -> np.ndarray:
        N = int(self.problems[b].n_poses)
        o = int(self.pose_off[b])
        return _to44(self.poses[12 * o:12 * (o + N)].cpu().numpy().reshape(N, 12))

    def get_alpha(self, b: int) -> np.ndarray:
        o = int(self.lm_off[b])
        return self.alpha[o:o + self.problems[b].n_landmarks].cpu().numpy().copy()

    def get_state(self):
        """Every problem's poses ([N, 4, 4]) and inverse depths, from one device-to-host
        copy of each state array (the batched form of get_poses / get_alpha)."""
        self.synchronize()
        P = _to44(self.poses[:12 * int(self.sizes.total_poses)].cpu().numpy().reshape(-1, 12))
        A = self.alpha[:int(self.sizes.total_landmarks)].cpu().numpy()
        poses, alphas = [], []
        for b, p in enumerate(self.problems):
            o, N = int(self.pose_off[b]), int(p.n_poses)
            poses.append(P[o:o + N])
            lo = int(self.lm_off[b])
            alphas.append(A[lo:lo + p.n_landmarks].copy())
        return poses, alphas

    def set_poses(self, b: int, poses: np.ndarray):
        N = int(self.problems[b].n_poses)
        o = int(self.pose_off[b])
        self.poses[12 * o:12 * (o + N)].copy_(torch.from_numpy(_to34(poses).reshape(-1)))

    def set_alpha(self, b: int, alpha: np.ndarray):
        o = int(self.lm_off[b])
        self.alpha[o:o + len(alpha)].copy_(torch.from_numpy(np.asarray(alpha, dtype=np.float64)))

    def store_state(self):
        """Copy the device state back into the ``Problem`` objects."""
        for b, p in enumerate(self.problems):
            p.poses = self.get_poses(b)
            p.alpha = self.get_alpha(b)

    # -- parameters ---------------------------------------------------------------
    def set_params(self, loss: Optional[str] = None, loss_scale=None, near_boost=None, eps=None,
                   alpha_min=None, alpha_max=None, lambda0=None, lambda_max=None, tol=None, max_iters=None,
                   refine_steps=None, use_graph=None, use_tc=None, cost_block=None, lin_block=None,
                   outer_steps=None, wait_us=None, ctl_min_log10=None, outer_tol=None,
                   stop_rho=None):
        p = self.params
        if loss is not None:
            p.loss = _LOSS[loss]
        for name, val in (("loss_scale", loss_scale), ("eps", eps), ("alpha_min", alpha_min),
                          ("alpha_max", alpha_max), ("lambda0", lambda0), ("lambda_max", lambda_max),
                          ("tol", tol)):
            if val is not None:
                setattr(p, name, float(val))
        if near_boost is not None:
            p.near_boost = int(bool(near_boost))
        if max_iters is not None:
            p.max_iters = int(max_iters)
        if refine_steps is not None:
            p.refine_steps = int(refine_steps)
        if use_graph is not None:
            p.use_graph = int(bool(use_graph))
        if use_tc is not None:
            p.use_tc = int(bool(use_tc))
        if cost_block is not None:
            p.cost_block = int(cost_block)
        if lin_block is not None:
            p.lin_block = int(lin_block)
        if outer_steps is not None:
            p.outer_steps = int(outer_steps)
        if wait_us is not None:
            p.wait_us = int(wait_us)
        if ctl_min_log10 is not None:
            p.ctl_min_log10 = float(ctl_min_log10)
        if outer_tol is not None:
            p.outer_tol = float(outer_tol)
        if stop_rho is not None:
            p.stop_rho = float(stop_rho)
        self._apply_params()

    def _apply_params(self):
        nat.check(self.L.spgo_set_params(self._solver, C.byref(self.params)), "set_params")

    # -- solving ------------------------------------------------------------------
    def reset(self):
        nat.check(self.L.spgo_lm_reset(self._solver, self._sp()), "lm_reset")

    def iterate(self, n: int = 1):
        nat.check(self.L.spgo_lm_iterate(self._solver, int(n), self._sp()), "lm_iterate")

    def status(self) -> List[dict]:
        B = len(self.problems)
        out = (nat.ProblemStatus * B)()
        nat.check(self.L.spgo_lm_status(self._solver, out, self._sp()), "lm_status")
        return [dict(cost0=s.cost0, cost=s.cost, lam=s.lambda_, iterations=s.iterations, accepted=s.accepted,
                     status=s.status, factor_failures=s.factor_failures, wait_timeouts=s.wait_timeouts)
                for s in out]

    def trace(self) -> List[dict]:
        """Per problem, the LM iterations since the last reset (up to ``native.TRACE_MAX``):
        ``cost`` after each iteration, the ``lam`` its step was solved with, and whether
        it was ``accepted`` (``spgo_lm_trace``)."""
        B, cap = len(self.problems), nat.TRACE_MAX
        cost = np.zeros(B * cap)
        lam = np.zeros(B * cap)
        acc = np.zeros(B * cap, dtype=np.int32)
        n = np.zeros(B, dtype=np.int32)
        nat.check(self.L.spgo_lm_trace(self._solver, cap, cost.ctypes.data, lam.ctypes.data, acc.ctypes.data,
                                       n.ctypes.data, self._sp()), "lm_trace")
        out = []
        for b in range(B):
            k = int(n[b])
            sl = slice(b * cap, b * cap + k)
            out.append(dict(cost=cost[sl].copy(), lam=lam[sl].copy(), accepted=acc[sl].astype(bool)))
        return out

    def solve(self, check_every: int = 8) -> List[dict]:
        """Reset and run Nielsen LM until every problem stops (see ``spgo_lm_solve``)."""
        it = C.c_int32()
        nat.check(self.L.spgo_lm_solve(self._solver, int(check_every), C.byref(it), self._sp()), "lm_solve")
        return self.status()

    def autotune(self) -> dict:
        """Time the run-time launch shapes on this batch and keep the fastest
        (``spgo_autotune``); returns the choices."""
        out = nat.Params()
        nat.check(self.L.spgo_autotune(self._solver, C.byref(out), self._sp()), "autotune")
        self.params = out
        return dict(cost_block=out.cost_block, lin_block=out.lin_block, use_tc=out.use_tc)

    def autotune_plan_shapes(self, candidates=None, iterations: int = 2, repeats: int = 2) -> dict:
        """Time the plan-time Schur work shapes (``spgo_plan_options``: chunks per
        tensor-core or SIMT work item) on this solver's batch: for each candidate a
        solver of the same problems and parameters is planned, reset and run for
        ``iterations`` LM iterations (best of ``repeats``).  This solver's state is not
        touched; returns ``{"best": options, "ms": {candidate: ms}}``.  A new
        ``BatchSolver(..., plan_options=best)`` uses the choice."""
        if candidates is None:
            candidates = ([dict(tc_split=t) for t in (16, 32, 64)] if self.params.use_tc
                          else [dict(simt_split=k) for k in (8, 16, 32)])
        timings = {}
        for cand in candidates:
            s = BatchSolver(self.problems, precision=self.precision, device=self.device, stream=self._stream,
                            plan_options=cand)
            s.params = nat.Params.from_buffer_copy(self.params)
            nat.check(self.L.spgo_set_params(s._solver, C.byref(s.params)), "set_params")
            best = None
            for _ in range(repeats + 1):
                st = torch.cuda.current_stream(self.device) if self._stream is None else self._stream
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.reset()
                e0.record(st)
                s.iterate(iterations)
                e1.record(st)
                e1.synchronize()
                ms = e0.elapsed_time(e1)
                best = ms if best is None else min(best, ms)
            s.close()
            timings[tuple(sorted(cand.items()))] = best
        key = min(timings, key=timings.get)
        return {"best": dict(key), "ms": {str(dict(k)): round(v, 4) for k, v in timings.items()}}

    def gn_step(self, iterations: int = 1, step_size: float = 1.0):
        nat.check(self.L.spgo_gn_step(self._solver, int(iterations), float(step_size), self._sp()), "gn_step")

    def export_system(self, b: int) -> dict:
        """Dense A, g, B, C, g_a and cost of problem ``b`` at the current state (FP64, small problems)."""
        p = self.problems[b]
        P, L = 6 * int(p.n_poses), p.n_landmarks
        dev = self.device
        A = torch.zeros(P * P, dtype=torch.float64, device=dev)
        g = torch.zeros(P, dtype=torch.float64, device=dev)
        Bm = torch.zeros(max(1, P * L), dtype=torch.float64, device=dev)
        Cv = torch.zeros(max(1, L), dtype=torch.float64, device=dev)
        ga = torch.zeros(max(1, L), dtype=torch.float64, device=dev)
        cost = torch.zeros(1, dtype=torch.float64, device=dev)
        vp = lambda t: C.c_void_p(t.data_ptr())
        nat.check(self.L.spgo_export_system(self._solver, int(b), vp(A), vp(g), vp(Bm), vp(Cv), vp(ga), vp(cost),
                                            self._sp()), "export_system")
        self.synchronize()
        return dict(A=A.cpu().numpy().reshape(P, P), g=g.cpu().numpy(), B=Bm[:P * L].cpu().numpy().reshape(P, L),
                    C=Cv[:L].cpu().numpy(), g_a=ga[:L].cpu().numpy(), cost=float(cost.item()))

    def slab_floats(self) -> int:
        return int(self.sizes.slab_elems)

    def export_reduced(self, b: int, lam: float) -> dict:
        """Damped reduced camera system S = A + lam diag(A) - B D^-1 B^T and g_S of problem b (FP64)."""
        P = 6 * int(self.problems[b].n_poses)
        S = torch.zeros(P * P, dtype=torch.float64, device=self.device)
        gS = torch.zeros(P, dtype=torch.float64, device=self.device)
        nat.check(self.L.spgo_export_reduced(self._solver, int(b), float(lam), C.c_void_p(S.data_ptr()),
                                             C.c_void_p(gS.data_ptr()), self._sp()), "export_reduced")
        self.synchronize()
        return dict(S=S.cpu().numpy().reshape(P, P), gS=gS.cpu().numpy())

    def features(self) -> np.ndarray:
        """The learned controller's 16 inputs per problem at the current state."""
        B = len(self.problems)
        f = torch.zeros(B * nat.MLP_INPUTS, dtype=torch.float32, device=self.device)
        nat.check(self.L.spgo_lm_features(self._solver, C.c_void_p(f.data_ptr()), self._sp()), "lm_features")
        self.synchronize()
        return f.cpu().numpy().reshape(B, nat.MLP_INPUTS)

    def probe(self, factors) -> np.ndarray:
        """Cost of the step taken with lambda * f, for each factor and problem ([n_f, B])."""
        fac = np.ascontiguousarray(factors, dtype=np.float64)
        out = np.zeros(len(fac) * len(self.problems), dtype=np.float64)
        nat.check(self.L.spgo_lm_probe(self._solver, len(fac), fac.ctypes.data_as(C.POINTER(C.c_double)),
                                       out.ctypes.data_as(C.POINTER(C.c_double)), self._sp()), "lm_probe")
        return out.reshape(len(fac), len(self.problems))

    def set_controller(self, params: Optional[torch.Tensor]):
        """Learned damping (FP32 parameter tensor on the device) or None for plain Nielsen."""
        ptr = C.c_void_p(params.data_ptr()) if params is not None else C.c_void_p(0)
        nat.check(self.L.spgo_lm_set_controller(self._solver, ptr, self._sp()), "lm_set_controller")

    def launch_count(self) -> int:
        return int(self.L.spgo_launch_count(self._solver))

    def profile(self, capacity: int):
        """Record CUDA events around each launch (``capacity`` launches; 0 disables)."""
        nat.check(self.L.spgo_profile_enable(self._solver, int(capacity)), "profile_enable")

    def profile_read(self) -> dict:
        """{kind: (total_ms, launches)} since the last read (synchronises the stream)."""
        n = len(nat.PROFILE_KINDS)
        ms = (C.c_double * n)()
        cnt = (C.c_int64 * n)()
        nat.check(self.L.spgo_profile_read(self._solver, ms, cnt, n, self._sp()), "profile_read")
        return {k: (ms[i], int(cnt[i])) for i, k in enumerate(nat.PROFILE_KINDS)}

    def close(self):
        if getattr(self, "_solver", None):
            self.synchronize()
            self.L.spgo_solver_destroy(self._solver)
            self._solver = None
        if getattr(self, "_host_plan", None):
            self._host_plan.close()
            self._host_plan = None
            self._plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _plan_on(device: torch.device, problems, precision, plan_options=None):
    torch.cuda.set_device(device)  # page-locked staging is allocated in this device's context
    return HostPlan(problems, precision, plan_options)


def _drive(device: torch.device, stream: torch.cuda.Stream, plan_future, params, controller, check_every):
    """One batch on one CUDA stream: bind, solve, read back, release."""
    hp = plan_future.result()
    torch.cuda.set_device(device)
    with torch.cuda.stream(stream):
        bs = BatchSolver(device=device, stream=stream, plan=hp)
        try:
            if params:
                bs.set_params(**params)
            if controller is not None:
                bs.set_controller(controller)
            st = bs.solve(check_every=check_every)
            poses, alphas = bs.get_state()
        finally:
            bs.close()
    return st, poses, alphas


def solve_stream(batches: Iterable[Sequence[Problem]], precision: str = "mixed", params: Optional[dict] = None,
                 controller: Optional[torch.Tensor] = None, device="cuda", inflight: int = 2,
                 check_every: int = 8, plan_options: Optional[dict] = None) -> Iterator[Tuple[List[dict], list, list]]:
    """Solve batch after batch (each a sequence of ``Problem``) with Nielsen LM (or
    the learned controller), yielding ``(statuses, poses, inverse_depths)`` per batch
    in order.

    ``inflight`` batches solve at once, each on its own CUDA stream driven by its own
    host thread, so one batch's latency-bound launches fill the SMs another leaves
    idle; one more thread plans the upcoming batches (marshalling, sorting, chunking:
    the planner releases the GIL).  Every batch still has its own upload and
    readback.  Up to ``inflight + 1`` batches are planned ahead of the solving ones.
    ``plan_options``: the Schur work shapes every batch is planned with (``HostPlan``)."""
    dev = torch.device(device)
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    inflight = max(1, int(inflight))
    streams = [torch.cuda.Stream(device=dev) for _ in range(inflight)]
    it = iter(batches)
    plans: collections.deque = collections.deque()    # planned, not yet solving
    pending: collections.deque = collections.deque()  # solving, in batch order
    with ThreadPoolExecutor(1) as planner, ThreadPoolExecutor(inflight) as drivers:
        k = 0

        def plan_ahead():
            while len(plans) < inflight + 1:
                nxt = next(it, None)
                if nxt is None:
                    return
                plans.append(planner.submit(_plan_on, dev, nxt, precision, plan_options))

        def start_one():
            nonlocal k
            if plans:
                pending.append(drivers.submit(_drive, dev, streams[k % inflight], plans.popleft(), params,
                                              controller, check_every))
                k += 1

        plan_ahead()
        for _ in range(inflight):
            start_one()
        plan_ahead()
        while pending:
            res = pending.popleft().result()
            start_one()  # the next batch takes the stream of the batch just finished
            plan_ahead()
            yield res


class CudaSolver:
    """Drop-in for the reference's ``CudaSolver`` (``src/CythonAPI/Solver.pyx:16-107``).

    ``CudaSolver(N, M)``: N incremental poses (N + 1 frames), M landmarks per
    frame, N * M features in all; poses start at the identity and inverse
    depths at 1 (``include/Solver.hpp:20-57``).  Observations are staged on the
    host and uploaded in bulk on the next ``step``.  ``step(k)`` runs k
    undamped Gauss-Newton iterations with the reference's cost (Cauchy c^2 = 9,
    x4 weight for targets within one frame of the anchor, C + 1e-4, pose step
    scaled by ``setStepSize``, inverse depth clamped to [1/30, 5])
    (``src/Optimization/Solver_cuda.cu:557-795``).
    """

    def __init__(self, N: int, M: int, precision: str = "mixed", device="cuda"):
        self._N, self._M = int(N), int(M)
        self._number_of_keyframes = self._N
        self._number_of_observations_per_frame = self._M
        self._precision = precision
        self._device = device
        self._intr = np.zeros(8, dtype=np.float32)
        self._Trl = np.zeros((4, 4), dtype=np.float32)
        self._poses = np.tile(np.eye(4, dtype=np.float64), (self._N, 1, 1))
        self._alpha = np.ones(self._N * self._M, dtype=np.float64)
        self._obs = {}            # (frame, feature) -> (left[3], right[3])
        self._meas = []           # (anchor, target, feature) in write order
        self._step_size = 1.0
        self._solver: Optional[BatchSolver] = None
        self._dirty = True

    # --- calibration / observations (Solver.cpp:29-56) -------------------------------
    def loadCalibration(self, intrinsics_py, T_r_to_l_py):
        self._intr = np.asarray(intrinsics_py, dtype=np.float32).reshape(8).copy()
        self._Trl = np.asarray(T_r_to_l_py, dtype=np.float32).reshape(4, 4).copy()
        self._dirty = True

    def writeObservations(self, anchor_frame_ID, target_frame_ID, global_feat_ID, left_obs_py, right_obs_py):
        a, t, f = int(anchor_frame_ID), int(target_frame_ID), int(global_feat_ID)
        if not (0 <= a <= self._N and 0 <= t <= self._N and 0 <= f < self._N * self._M):
            raise IndexError("frame or feature index out of range")
        if len(self._meas) >= self._N * (self._N + 1) * self._M:
            raise IndexError("measurement buffer full")
        self._obs[(t, f)] = (np.asarray(left_obs_py, dtype=np.float32).reshape(3).copy(),
                             np.asarray(right_obs_py, dtype=np.float32).reshape(3).copy())
        self._meas.append((a, t, f))
        self._dirty = True

    def getObservation(self, keyFrameID, global_feat_ID):
        l, r = self._obs.get((int(keyFrameID), int(global_feat_ID)),
                             (np.zeros(3, np.float32), np.zeros(3, np.float32)))
        return l.reshape(3, 1).copy(), r.reshape(3, 1).copy()

    def getCalibration(self):
        # same shapes as the reference binding (Solver.pyx:74-88)
        return self._intr.reshape(4, 2).copy(), self._Trl.reshape(4, 4).copy()

    # --- state (Solver.cpp:59-128) ---------------------------------------------------
    def writeIncrementalPose(self, keyFrameID, T_curr_to_next_py):
        k = int(keyFrameID)
        T = np.asarray(T_curr_to_next_py, dtype=np.float32).reshape(4, 4)
        self._sync_from_device()
        self._poses[k, :3, :] = T[:3, :]
        self._push_state()

    def getIncrementalPose(self, keyFrameID):
        self._sync_from_device()
        return self._poses[int(keyFrameID)].astype(np.float32)

    def loadInverseDepths(self, inverse_depths_py):
        self._sync_from_device()
        self._alpha = np.asarray(inverse_depths_py, dtype=np.float32).reshape(-1).astype(np.float64)
        self._push_state()

    def getInverseDepths(self):
        self._sync_from_device()
        return self._alpha.astype(np.float32)

    def setStepSize(self, step_size):
        self._step_size = float(np.asarray(step_size).reshape(-1)[0])

    # --- solve ----------------------------------------------------------------------
    def step(self, iterations):
        if self._dirty or self._solver is None:
            self._sync_from_device()
            self._build()
        if self._solver is None:
            return
        self._solver.gn_step(int(iterations), self._step_size)
        self._on_device = True
        # features without measurements still have their inverse depth clamped (Solver_cuda.cu:545-546)
        if int(iterations) > 0:
            rest = np.ones(self._alpha.size, dtype=bool)
            rest[self._feats] = False
            self._alpha[rest] = np.clip(self._alpha[rest], 1.0 / 30.0, 1.0 / 0.2)
        self._solver.synchronize()

    # --- internals ------------------------------------------------------------------------
    _on_device = False

    def _problem(self) -> Optional[Problem]:
        L = self._N * self._M
        anchors = {}
        targets = {}
        for a, t, f in self._meas:
            if f in anchors and anchors[f] != a:
                raise ValueError(f"feature {f} written with two anchors ({anchors[f]}, {a})")
            anchors[f] = a
            targets.setdefault(f, set()).add(t)
        feats = sorted(anchors)
        self._feats = np.array(feats, dtype=np.int64)
        if not feats:
            return None
        host = np.array([anchors[f] for f in feats], dtype=np.int32)
        auv = np.zeros((len(feats), 2))
        ptr = [0]
        fr, uv = [], []
        for i, f in enumerate(feats):
            la = self._obs.get((anchors[f], f))
            if la is not None:
                auv[i] = la[0][:2]
            for t in sorted(targets[f]):
                l, r = self._obs[(t, f)]
                fr.append(t)
                uv.append([l[0], l[1], r[0], r[1]])
            ptr.append(len(fr))
        T_rl = self._Trl.astype(np.float64)
        return Problem(n_poses=self._N, intrinsics=self._intr.astype(np.float64), T_rl=T_rl, host=host,
                       anchor_uv=auv, obs_ptr=np.array(ptr, np.int64), obs_frame=np.array(fr, np.int32),
                       obs_uv=np.array(uv, dtype=np.float64).reshape(-1, 4), poses=self._poses.copy(),
                       alpha=self._alpha[self._feats].copy())

    def _build(self):
        if self._solver is not None:
            self._solver.close()
            self._solver = None
        prob = self._problem()
        if prob is None:
            self._dirty = False
            return
        self._solver = BatchSolver([prob], precision=self._precision, device=self._device)
        self._solver.set_params(loss="cauchy", loss_scale=3.0, near_boost=True, eps=1e-4,
                                alpha_min=1.0 / 30.0, alpha_max=1.0 / 0.2)
        self._dirty = False
        self._on_device = True

    def _sync_from_device(self):
        if self._solver is not None and self._on_device:
            self._poses = self._solver.get_poses(0)
            a = self._solver.get_alpha(0)
            self._alpha[self._feats] = a
            self._on_device = False

    def _push_state(self):
        if self._solver is not None:
            self._solver.set_poses(0, self._poses)
            self._solver.set_alpha(0, self._alpha[self._feats])
            self._on_device = True
