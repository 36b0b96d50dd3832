#!/usr/bin/env python3
"""Benchmark: batched Levenberg-Marquardt solves of the config-3 workload.

Workload (synthetic, seeded): 256 independent stereo pose-graph / bundle-
adjustment problems, N ~ U[8, 32] incremental poses and L ~ U[200, 3000]
landmarks each (circle generator, 1 px noise), every problem run to a
relative cost decrease below 1e-6 or an iteration cap (the plain FP64 solver:
30).  One step = one solve of the whole batch from its initial state.

The chosen form is the mixed path (FP32 Jacobian and Hessian blocks summed
exactly, tensor-core Schur complement, FP32 Cholesky, the step refined against
the accurately summed residual of the whole system), batched, with Nielsen
damping and at most 35 LM iterations (``--max-iters``); ``--controller 1``
puts the learned damping controller in the chosen form instead, and the
controller arm of ``plain_fp64.effects`` always times it.  Its reference point
is the plain FP64 GPU solver (Nielsen LM, no controller, 30 iterations):

* ``value``: solves per second that reach the plain FP64 solver's final cost
  (relative 1e-6): the chosen form's batch solves/s times the fraction of its
  problems that end at or below the plain cost.  Inputs resident in HBM; L2
  flushed (256 MB write) between timed steps.  ``raw_solves_per_s`` is the batch
  rate without that filter.
* ``plain_fp64``: the plain FP64 solver batched (the comparison point) and one
  problem at a time, the fraction of chosen-form problems that reach its cost,
  the iterations they need to, and the effects of batching, precision and the
  learned controller taken one at a time.
* ``e2e``: the same metric through the public API per step: marshal and plan the
  host problems, upload, solve, read back poses and inverse depths
  (``solver.solve_stream``: batches planned on a worker thread ahead of their
  solve, ``--inflight`` batches solving at once on their own CUDA streams).
* ``roofline``: the dominant kernel's algorithmic work per launch (HBM bytes or
  FLOPs) over its CUDA-event duration, against the measured peaks; also the
  whole solve's algorithmic bytes against HBM.
* ``cpu_baseline``: the FP64 CPU oracle on a bounded sample of the batch.
* ``--impl reference``: the CPU oracle alone on host cores (process pool),
  same metric.

With torchrun (N > 1) every rank solves its own seeded batch (replicas, weak
scaling); the timing is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "time-to-converged cost (rel 1e-6) & batched solves/s: chosen vs plain FP64 GPU"
WORKLOAD = ("config3: 256 independent problems, N~U[8,32] poses, L~U[200,3000] landmarks, "
            "run to rel cost change < 1e-6 or 30 LM iterations")
N_PROBLEMS = 256
REACH_TOL = 1e-6


def _env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def _batch_seed(rank: int) -> int:
    """Seed of rank r's 256-problem batch (rank 0: the config-3 batch, seed 3)."""
    return 3 + 7919 * rank


def max_over_ranks(x: float, world: int, device="cpu") -> float:
    """The slowest rank's value (the timed region's wall time), via all_reduce MAX."""
    if world <= 1:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU oracle worker (spawned processes; never forked after CUDA init)
# ---------------------------------------------------------------------------
def _oracle_solve(args):
    seed, n, l = args
    os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
    sys.path.insert(0, REPO)
    import __graft_entry__
    __graft_entry__.load_package()
    import spgo_gb300.scenes as scenes
    from oracle import solver as S
    p = scenes.circle_scene(seed, n, l)
    t0 = time.perf_counter()
    res = S.lm_solve(p, S.Loss(), max_iters=30, tol=1e-6)
    return time.perf_counter() - t0, res.cost, res.iterations


def _config3_specs(seed: int, n: int = N_PROBLEMS):
    """(problem seed, N, L) of the batch's problems (the scene generator's own draw)."""
    import __graft_entry__
    __graft_entry__.load_package()
    import spgo_gb300.scenes as scenes
    return scenes.config3_specs(seed, n)


def _make_pool(workers: int):
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(workers)


def cpu_oracle_sample(pool, specs, n_sample: int):
    """Solve ``n_sample`` problems with the FP64 oracle on an existing pool: solves/s.
    Problems go out one at a time, largest first, so the wall time is not set by one
    large problem left for last."""
    sample = sorted(specs[:n_sample], key=lambda s: -(s[1] * s[2]))
    t0 = time.perf_counter()
    out = pool.map(_oracle_solve, sample, chunksize=1)
    wall = time.perf_counter() - t0
    return n_sample / wall, wall, out


# ---------------------------------------------------------------------------
# clocks
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = os.path.join("/tmp", f"spgo_clocks_{os.getpid()}.csv")

    def start(self):
        """Start sampling every 100 ms and return once the first sample is written
        (nvidia-smi takes a few hundred ms to start; without the wait a short timed
        region would see none of its samples)."""
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        t_end = time.time() + 5.0
        while time.time() < t_end and self.proc.poll() is None:
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.01)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# algorithmic work per launch (roofline numerators)
# ---------------------------------------------------------------------------
def roofline_numerator(kind: str, sizes, probs):
    """(bound, unit, algorithmic amount per launch) of a profiled kernel kind.

    Jacobian pass 24 B per stereo observation + 24 B per landmark; cost pass
    24 O + 16 L; residual pass of the step refinement 24 O + 24 L;
    landmark Schur complement sum over landmarks of 2 (6 k)^2 FLOPs (k = pose blocks
    of the landmark's window); factor + solve P^3 / 3 + 4 P^2 per problem (FP32)."""
    O, L = sizes.total_obs, sizes.total_landmarks
    if kind == "linearize":
        return "hbm", "GB/s", 24.0 * O + 24.0 * L
    if kind == "cost":
        return "hbm", "GB/s", 24.0 * O + 16.0 * L
    if kind == "resid_pass":
        return "hbm", "GB/s", 24.0 * O + 24.0 * L
    if kind == "schur":
        return "tensor", "TFLOP/s", float(sizes.schur_flops_landmark)
    if kind == "factor_solve":
        return "fp32", "TFLOP/s", float(sum((6 * p.n_poses) ** 3 / 3.0 + 4 * (6 * p.n_poses) ** 2 for p in probs))
    return None, None, 0.0


def roofline_peaks(peaks: dict, tc: bool):
    """Denominators by bound: measured HBM copy; tensor = measured cuBLAS BF16 / 2 for
    the TF32 kind the Schur pass issues (the nominal TF32 : BF16 ratio), or the
    BF16 figure itself; FP32 SIMT = nominal 152 SMs x 128 lanes x 2 FLOP x max clock."""
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    bf16 = float(peaks.get("bf16_tflops", 1900.0))
    mhz = float(peaks.get("sm_max_mhz", 2070.0))
    src = "measured" if "hbm_gbs" in peaks else "fallback"
    return {"hbm": (hbm, src + " hbm_gbs"),
            "tensor": (bf16 / 2.0 if tc else bf16, src + (" bf16_tflops / 2 (tf32)" if tc else " bf16_tflops")),
            "fp32": (152 * 128 * 2 * mhz * 1e6 / 1e12, "nominal FP32 SIMT at sm_max_mhz")}


def measured_traffic(kind: str, sizes):
    """DRAM bytes per launch of a profiled kernel kind from the committed ncu capture
    record (profiles/dram_traffic.json), scaled from the captured case to this batch
    by the unit it is quoted per; None when the kind was not captured or its kernel
    sources changed since the capture (their SHA-256 is in the record)."""
    import hashlib
    try:
        rec = json.load(open(os.path.join(REPO, "profiles", "dram_traffic.json")))
    except Exception:
        return None, "no capture record"
    k = rec.get("kernels", {}).get(kind)
    if not k:
        return None, "kind not captured"
    h = hashlib.sha256()
    for f in k["sources"]:
        with open(os.path.join(REPO, f), "rb") as fh:
            h.update(fh.read())
    if h.hexdigest() != k["source_sha256"]:
        return None, "stale: the kernel's sources changed since the capture"
    units = {"obs": sizes.total_obs, "schur_flops": sizes.schur_flops_landmark}[k["per"]]
    return k["bytes_per_unit"] * units, f"ncu capture of {k['case']}, scaled per {k['per']}"


def measured_instructions(kind: str):
    """Executed warp instructions per stereo observation of a kernel kind from the
    committed ncu record (profiles/dram_traffic.json); None if absent or stale."""
    import hashlib
    try:
        rec = json.load(open(os.path.join(REPO, "profiles", "dram_traffic.json")))
    except Exception:
        return None
    k = rec.get("kernels", {}).get(kind)
    if not k or k.get("per") != "obs" or "instructions_per_unit" not in k:
        return None
    h = hashlib.sha256()
    for f in k["sources"]:
        with open(os.path.join(REPO, f), "rb") as fh:
            h.update(fh.read())
    return k["instructions_per_unit"] if h.hexdigest() == k["source_sha256"] else None


def _reached(costs, plain):
    import numpy as np
    return np.asarray(costs) <= np.asarray(plain) * (1.0 + REACH_TOL)


def _iters_to_plain(traces, plain, cost0):
    """Per problem, the LM iterations after which its trace first reaches the plain
    cost (None if it never does)."""
    out = []
    for t, pc, c0 in zip(traces, plain, cost0):
        if c0 <= pc * (1.0 + REACH_TOL):
            out.append(0)
            continue
        hit = [k + 1 for k, c in enumerate(t) if c <= pc * (1.0 + REACH_TOL)]
        out.append(hit[0] if hit else None)
    return out


def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    workers = max(1, os.cpu_count() or 1)
    specs = _config3_specs(_batch_seed(0))
    per_step = max(workers, 16)
    times = []
    with _make_pool(workers) as pool:
        for it in range(args.warmup + args.steps):
            sample = [specs[(it * per_step + k) % len(specs)] for k in range(per_step)]
            _, wall, _ = cpu_oracle_sample(pool, sample, per_step)
            if it >= args.warmup:
                times.append(wall)
    total = sum(times)
    value = per_step * len(times) / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / len(times),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD, "sample_per_step": per_step},
            "cpu_baseline": {"value": value, "unit": "solves/s", "cores": workers, "kind": "port",
                             "sample": f"{per_step} config-3 problems per step, FP64 numpy oracle LM, "
                                       f"one process per core (one pool for the run)"},
            "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    import torch

    rank, world, local = _env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    # CPU baseline first, on a spawned pool made before this process touches the GPU
    specs = _config3_specs(_batch_seed(rank))
    cpu = None
    if rank == 0 and not args.no_cpu:
        workers = max(1, os.cpu_count() or 1)
        n_s = max(workers, 16)
        with _make_pool(workers) as pool:
            rate, wall, _ = cpu_oracle_sample(pool, specs, n_s)
        cpu = {"value": rate, "unit": "solves/s", "cores": workers, "kind": "port",
               "sample": f"first {n_s} problems of the batch, FP64 numpy oracle LM "
                         f"(same stopping rule), one process per core, {wall:.1f} s"}

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import __graft_entry__
    __graft_entry__.load_package()
    import importlib
    importlib.import_module("spgo_gb300.build").build()
    scenes = importlib.import_module("spgo_gb300.scenes")
    sv = importlib.import_module("spgo_gb300.solver")

    probs = scenes.config3(seed=_batch_seed(rank))
    n_obs = sum(p.n_obs for p in probs)
    n_lm = sum(p.n_landmarks for p in probs)
    # a non-default stream: the solver replays its LM iterations as CUDA graphs on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    # learned damping: the shipped network (trained by train_controller.py), if present;
    # the chosen form uses it with --controller 1, the controller arm of the effects always
    net_params = None
    learned = importlib.import_module("spgo_gb300.learned")
    if os.path.exists(learned.DEFAULT_WEIGHTS):
        net_params = learned.Controller.load(device=dev).deployed()
    ctl_params = net_params if args.controller else None

    plain_params = dict(loss="l2", max_iters=30, tol=1e-6, lambda0=1e-4)
    stop_rho = 0.25 if args.stop_rho is None else args.stop_rho
    base_params = dict(plain_params, max_iters=args.max_iters, use_tc=args.tc, stop_rho=stop_rho)
    if args.outer >= 0:
        base_params["outer_steps"] = args.outer
    tuned = None

    plan_opts, plan_tune = None, None

    def make(precision, controller=None):
        """A solver of the batch; controller: deployed network weights or None (Nielsen)."""
        s = sv.BatchSolver(probs, precision=precision, device=dev, stream=stream,
                           plan_options=plan_opts if precision == "mixed" else None)
        if precision == "mixed":
            s.set_params(**base_params)
            if tuned is not None:  # later solvers of the same batch reuse the tuned shapes
                s.set_params(**tuned)
        else:
            s.set_params(**plain_params)
        if controller is not None:
            s.set_controller(controller)
        return s

    bs = make("mixed", ctl_params)
    if args.shapes:
        cb, lb = (int(x) for x in args.shapes.split(","))
        tuned = dict(cost_block=cb, lin_block=lb, use_tc=bs.params.use_tc)
        bs.set_params(**tuned)
    elif args.autotune:
        tuned = bs.autotune()  # launch shapes timed on this batch (untimed, before the warm-up)
        # plan-time Schur work shapes, timed on this batch with the tuned launch shapes; the
        # chosen form is re-planned with the fastest
        plan_tune = bs.autotune_plan_shapes()
        plan_opts = plan_tune["best"]
        bs.close()
        bs = make("mixed", ctl_params)
    else:
        tuned = dict(cost_block=bs.params.cost_block, lin_block=bs.params.lin_block, use_tc=bs.params.use_tc)
    p0, a0 = bs.poses.clone(), bs.alpha.clone()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed_solves(solver, n, warm):
        """(per-solve ms, last statuses) of n solves of `solver` from its initial state
        after `warm` untimed ones (L2 flushed before each)."""
        q0, b0 = solver.poses.clone(), solver.alpha.clone()
        out, st = [], None
        for k in range(warm + n):
            solver.poses.copy_(q0)
            solver.alpha.copy_(b0)
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = solver.solve(check_every=args.check_every)
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if k >= warm:
                out.append(e0.elapsed_time(e1))
        return out, st

    def one_step():
        bs.poses.copy_(p0)
        bs.alpha.copy_(a0)
        return bs.solve(check_every=args.check_every)

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize(dev)
    launches0 = bs.launch_count()
    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    ms = []
    status = None
    for k in range(args.steps):
        flush.fill_(k & 0xFF)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(dev)
        e0.record(stream)
        status = one_step()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        ms.append(e0.elapsed_time(e1))
    torch.cuda.synchronize(dev)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = bs.launch_count() - launches0
    chosen_trace = bs.trace()
    # per-kernel CUDA-event timing (graphs off while the events are recorded): one more
    # step of the same work, after the timed region
    bs.profile(200000)
    bs.profile_read()
    flush.fill_(7)
    torch.cuda.synchronize(dev)
    one_step()
    prof = bs.profile_read()
    bs.profile(0)
    total_ms = float(sum(ms))
    total_ms = max_over_ranks(total_ms, world, dev)
    raw_value = N_PROBLEMS * world * args.steps / (total_ms / 1e3)
    iters = [s["iterations"] for s in status]
    chosen_costs = np.array([s["cost"] for s in status])
    cost0 = np.array([s["cost0"] for s in status])

    # kernel shares and roofline of the dominant kernel
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    pk = roofline_peaks(peaks, bool(args.tc))
    tot = sum(v[0] for v in prof.values()) or 1.0
    kernels = {k: {"ms": round(v[0], 4), "launches": v[1], "share": round(v[0] / tot, 4)} for k, v in prof.items()}
    for k, v in prof.items():
        b_, u_, amt = roofline_numerator(k, bs.sizes, probs)
        if b_ and v[1]:
            ms_ = v[0] / v[1]
            ach = amt / (ms_ / 1e3) / (1e9 if b_ == "hbm" else 1e12)
            kernels[k].update(bound=b_, achieved=round(ach, 3), unit=u_, frac=round(ach / pk[b_][0], 4))
    dom = max((k for k in prof if roofline_numerator(k, bs.sizes, probs)[0] and prof[k][1]),
              key=lambda k: prof[k][0])
    avg_ms = prof[dom][0] / max(1, prof[dom][1])
    bound, unit, amount = roofline_numerator(dom, bs.sizes, probs)
    achieved = amount / (avg_ms / 1e3) / (1e9 if bound == "hbm" else 1e12)
    peak, peak_src = pk[bound]
    traffic, traffic_src = measured_traffic(dom, bs.sizes)
    roof = {"kernel": dom, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
            "algorithmic_per_launch": amount, "avg_launch_ms": avg_ms, "peak_source": peak_src,
            "note": "algorithmic work per launch / CUDA-event launch duration (profiled step after the "
                    "timed region, CUDA graphs off)"}
    # the passes over the observations are bound by instruction issue, not DRAM: their
    # executed warp instructions (from the committed ncu record, per observation) over
    # the launch time, against 4 issue slots per SM per cycle at the sampled SM clock
    issue = {}
    for k in ("linearize", "resid_pass", "cost"):
        ipu = measured_instructions(k)
        if ipu is not None and prof.get(k, (0, 0))[1]:
            ms_ = prof[k][0] / prof[k][1]
            rate = ipu * bs.sizes.total_obs / (ms_ / 1e3)
            peak_i = 152 * 4 * float(clk.get("sm_mhz") or peaks.get("sm_max_mhz", 2070.0)) * 1e6
            issue[k] = {"warp_instructions_per_launch": ipu * bs.sizes.total_obs, "per_s": rate,
                        "peak_per_s": peak_i, "frac": rate / peak_i}
    roof["issue"] = issue
    if "schur" in prof and prof["schur"][1] and bs.sizes.tc_chunk_tiles:
        # the tensor-core kernel executes more than the algorithmic count: 128 x 128 tiles
        # padded to the chunk windows, and three TF32 products per split value pair
        sms = prof["schur"][0] / prof["schur"][1]
        executed = 3.0 * 2.0 * 128 * 128 * 32 * bs.sizes.tc_chunk_tiles
        kernels["schur"]["executed_tflops"] = round(executed / (sms / 1e3) / 1e12, 3)
    # the whole solve against HBM: the algorithmic bytes of every pass over observations
    # and landmarks the profiled solve launched, plus the dense per-problem systems each
    # factorisation reads and writes (A, S_L, factor: 3 x 4 P^2 bytes), over the timed
    # solve's duration (the profiled solve repeats its work with graphs off)
    dense = sum(3 * 4.0 * (6 * p.n_poses) ** 2 for p in probs)
    step_bytes = sum(v[1] * roofline_numerator(k, bs.sizes, probs)[2]
                     for k, v in prof.items() if roofline_numerator(k, bs.sizes, probs)[0] == "hbm")
    step_bytes += prof.get("factor_solve", (0, 0))[1] * dense
    step_ms = total_ms / args.steps
    roof["solve_hbm"] = {"bytes": step_bytes, "ms": step_ms, "gbs": step_bytes / (step_ms / 1e3) / 1e9,
                         "frac": step_bytes / (step_ms / 1e3) / 1e9 / pk["hbm"][0]}

    # the plain FP64 GPU solver (the comparison point): batched, and problem at a time;
    # the mixed path without the controller (precision alone)
    plain = None
    reached_frac = None
    plain_costs = None
    if not args.no_plain:
        s64 = make("fp64")
        ms64, st64 = timed_solves(s64, 1, 1)
        s64.close()
        plain_costs = np.array([s["cost"] for s in st64])
        plain_iters = [s["iterations"] for s in st64]
        sm_ = make("mixed")
        msm, stm = timed_solves(sm_, 1, 1)
        mix_trace = sm_.trace()
        sm_.close()
        mixed_costs = np.array([s["cost"] for s in stm])
        mixed_iters = [s["iterations"] for s in stm]
        reached = _reached(chosen_costs, plain_costs)
        reached_frac = float(reached.mean())
        to_plain = _iters_to_plain([t["cost"] for t in chosen_trace], plain_costs, cost0)
        hit = [k for k in to_plain if k is not None]
        ctl_effect = None
        if net_params is not None:
            # the learned controller on the mixed path against Nielsen on the same path:
            # wall time, problems reaching the plain cost, LM iterations to reach it
            sc_ = make("mixed", net_params)
            msc, stc = timed_solves(sc_, 1, 1)
            ctl_trace = sc_.trace()
            sc_.close()
            ctl_costs = np.array([s["cost"] for s in stc])
            ctl_iters = [s["iterations"] for s in stc]
            ctl_hit = [k for k in _iters_to_plain([t["cost"] for t in ctl_trace], plain_costs, cost0)
                       if k is not None]
            mix_hit = [k for k in _iters_to_plain([t["cost"] for t in mix_trace], plain_costs, cost0)
                       if k is not None]
            ctl_effect = {
                "speedup": min(msm) / min(msc),
                "reached_plain_cost_frac": float(_reached(ctl_costs, plain_costs).mean()),
                "learned_ms": min(msc), "mean_iterations": float(np.mean(ctl_iters)),
                "iteration_ratio": float(np.mean(mixed_iters)) / max(1e-9, float(np.mean(ctl_iters))),
                "iterations_to_plain_cost_mean": float(np.mean(ctl_hit)) if ctl_hit else None,
                "nielsen_iterations_to_plain_cost_mean":
                    float(np.mean(mix_hit)) if mix_hit else None}
        t_serial = None
        if args.plain_serial:
            t_serial = 0.0
            for p in probs:
                s1 = sv.BatchSolver([p], precision="fp64", device=dev, stream=stream)
                s1.set_params(**plain_params)
                torch.cuda.synchronize(dev)
                t0 = time.perf_counter()
                s1.solve(check_every=args.check_every)
                torch.cuda.synchronize(dev)
                t_serial += time.perf_counter() - t0
                s1.close()
        chosen_ms = total_ms / args.steps
        plain = {
            "batched_ms": min(ms64), "batched_solves_per_s": N_PROBLEMS / (min(ms64) / 1e3),
            "mean_iterations": float(np.mean(plain_iters)),
            "chosen_speedup_vs_batched": min(ms64) / chosen_ms,
            "reached_plain_cost_frac": reached_frac,
            "median_rel_cost_diff": float(np.median((chosen_costs - plain_costs) / plain_costs)),
            "chosen_iterations_to_plain_cost_mean": float(np.mean(hit)) if hit else None,
            "chosen_iterations_to_plain_cost_max": int(max(hit)) if hit else None,
            "effects": {
                "precision (mixed vs FP64, both batched, no controller)": {
                    "speedup": min(ms64) / min(msm),
                    "reached_plain_cost_frac": float(_reached(mixed_costs, plain_costs).mean()),
                    "mixed_ms": min(msm), "mean_iterations": float(np.mean(mixed_iters))},
                "controller (learned vs Nielsen, mixed, batched)": ctl_effect,
            },
        }
        if t_serial is not None:
            plain["serial_ms"] = 1e3 * t_serial
            plain["serial_solves_per_s"] = N_PROBLEMS / t_serial
            plain["chosen_speedup_vs_serial"] = (t_serial * 1e3) / chosen_ms
            plain["effects"]["batching (FP64, 256 at once vs one at a time)"] = {"speedup": 1e3 * t_serial / min(ms64)}
    value = raw_value * reached_frac if reached_frac is not None else raw_value

    # end-to-end through the public API with host buffers: every batch is marshalled,
    # planned, uploaded, solved and read back.  Serially (one BatchSolver after
    # another), and as a stream (solve_stream: batches planned on a worker thread
    # ahead of their solve, --inflight batches solving at once), which is the headline.
    e2e_ms, h2d, d2h = [], 0, 0
    for k in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        s2 = make("mixed", ctl_params)
        s2.solve(check_every=args.check_every)
        poses, alphas = s2.get_state()
        torch.cuda.synchronize(dev)
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
        h2d = int(s2.sizes.static_bytes + 8 * (12 * s2.sizes.total_poses + s2.sizes.total_landmarks))
        d2h = int(8 * (12 * s2.sizes.total_poses + s2.sizes.total_landmarks))
        s2.close()
        del poses, alphas
    serial_val = N_PROBLEMS * world / (float(np.mean(e2e_ms)) / 1e3)
    n_stream = max(12, args.steps)
    stream_params = {**base_params, **(tuned or {})}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    stream_reached = []
    for _st, _poses, _alphas in sv.solve_stream([probs] * n_stream, "mixed", stream_params, ctl_params, device=dev,
                                                inflight=args.inflight, check_every=args.check_every,
                                                plan_options=plan_opts):
        if plain_costs is not None:
            stream_reached.append(float(_reached([s["cost"] for s in _st], plain_costs).mean()))
    torch.cuda.synchronize(dev)
    stream_ms = 1e3 * (time.perf_counter() - t0) / n_stream
    stream_frac = float(np.mean(stream_reached)) if stream_reached else 1.0
    e2e_val = N_PROBLEMS * world / (stream_ms / 1e3) * stream_frac

    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
            "data": "synthetic (seeded config-3 generator)",
            "raw_solves_per_s": raw_value, "solves_to_plain_cost_per_s": value,
            "config": {"workload": WORKLOAD, "problems_per_gpu": N_PROBLEMS, "landmarks": n_lm, "obs": n_obs,
                       "precision": "mixed", "outer_refinement_steps": int(bs.params.outer_steps),
                       "chosen_max_iters": int(args.max_iters), "chosen_stop_rho": float(stop_rho),
                       "schur": "tcgen05 split TF32" if tuned["use_tc"] else "SIMT FP32",
                       "damping": "learned MLP + Nielsen fallback" if ctl_params is not None else "Nielsen",
                       "autotuned": tuned, "autotuned_plan": plan_tune,
                       "l2": "256 MB flush written between timed steps",
                       "parallelism": f"replicas x{world} (independent batches)",
                       "iterations_max": int(max(iters)), "iterations_mean": float(np.mean(iters)),
                       "value_definition": "batch solves/s x fraction of problems ending at or below the plain "
                                           "FP64 GPU solver's cost (rel 1e-6, plain: 30 LM iterations)"},
            "roofline": roof, "kernels": kernels, "gpu_launches": int(launches), "clocks": clk,
            "cpu_baseline": cpu, "plain_fp64": plain,
            "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": stream_ms, "steps": n_stream, "inflight": args.inflight,
                    "reached_plain_cost_frac": stream_frac,
                    "api": "solver.solve_stream: batches planned on a worker thread ahead of their solve, "
                           f"{args.inflight} batches solving at once on their own CUDA streams; solves that "
                           "reach the plain FP64 cost per second",
                    "serial_value": serial_val * stream_frac,
                    "serial_ms_per_step": float(np.mean(e2e_ms))}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


SINGLE = {
    1: ("config1: one problem, N = 100 poses on a 30 m sinusoidal path, 20k landmarks (~400k stereo "
        "observations), L2, at most 20 LM iterations", dict(loss="l2")),
    2: ("config2: one problem, N = 500 poses, 200k landmarks (~3M stereo observations), 20-frame "
        "covisibility window, 5 % outliers, Huber (delta 2 px), at most 20 LM iterations",
        dict(loss="huber", loss_scale=2.0)),
}


def run_single(args):
    """Configs 1 and 2: one large problem (reduced systems 600 and 3000 wide, the multi-CTA
    factorisation and substitutions), at most 20 LM iterations (relative decrease below
    1e-6 stops) from the same initial state for the chosen form (mixed) and the plain
    FP64 GPU solver.  value: solves per second of
    the chosen form, times 1 if it ends at or below the plain FP64 cost (rel 1e-6), else 0."""
    import numpy as np
    import torch

    rank, world, local = _env_rank()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import __graft_entry__
    __graft_entry__.load_package()
    import importlib
    importlib.import_module("spgo_gb300.build").build()
    scenes = importlib.import_module("spgo_gb300.scenes")
    sv = importlib.import_module("spgo_gb300.solver")
    workload, loss = SINGLE[args.config]
    p = getattr(scenes, f"config{args.config}")()
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # both solvers stop at a relative decrease below 1e-6 (the config-3 rule) or 20 iterations
    params = dict(loss, max_iters=20, tol=1e-6, lambda0=1e-4)

    def timed(prec, n, warm):
        s = sv.BatchSolver([p], precision=prec, device=dev, stream=stream)
        s.set_params(**params)
        if prec == "mixed":
            s.set_params(use_tc=args.tc, stop_rho=0.0 if args.stop_rho is None else args.stop_rho)
            if args.outer >= 0:
                s.set_params(outer_steps=args.outer)
        q0, a0 = s.poses.clone(), s.alpha.clone()
        ms, st = [], None
        for k in range(warm + n):
            s.poses.copy_(q0)
            s.alpha.copy_(a0)
            flush.fill_(k & 0xFF)
            torch.cuda.synchronize(dev)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            st = s.solve(check_every=args.check_every)[0]
            e1.record(stream)
            torch.cuda.synchronize(dev)
            if k >= warm:
                ms.append(e0.elapsed_time(e1))
        prof = None
        if prec == "mixed":
            s.poses.copy_(q0)
            s.alpha.copy_(a0)
            s.profile(200000)
            s.profile_read()
            s.solve(check_every=args.check_every)
            prof = s.profile_read()
            s.profile(0)
        launches = s.launch_count()
        tr = s.trace()[0]
        s.close()
        return ms, st, prof, launches, tr

    ms64, st64, _, _, _ = timed("fp64", 1, 1)
    clocks = ClockSampler(local)
    clocks.start()
    ms, st, prof, launches, tr = timed("mixed", args.steps, args.warmup)
    clk = clocks.stop()
    reached = bool(st["cost"] <= st64["cost"] * (1.0 + REACH_TOL))
    chosen_ms = float(np.mean(ms))
    hit = [k + 1 for k, c in enumerate(tr["cost"]) if c <= st64["cost"] * (1.0 + REACH_TOL)]
    tot = sum(v[0] for v in prof.values()) or 1.0
    kernels = {k: {"ms": round(v[0], 4), "launches": v[1], "share": round(v[0] / tot, 4)}
               for k, v in prof.items() if v[1]}
    # end to end: marshal and plan the host problem, upload, solve, read back
    e2e = []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        s = sv.BatchSolver([p], precision="mixed", device=dev, stream=stream)
        s.set_params(**params)
        s.solve(check_every=args.check_every)
        s.get_state()
        torch.cuda.synchronize(dev)
        e2e.append(time.perf_counter() - t0)
        h2d = int(s.sizes.static_bytes + 8 * (12 * s.sizes.total_poses + s.sizes.total_landmarks))
        d2h = int(8 * (12 * s.sizes.total_poses + s.sizes.total_landmarks))
        s.close()
    line = {"metric": METRIC, "value": (1e3 / chosen_ms) * (1.0 if reached else 0.0), "unit": "solves/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": chosen_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
            "data": f"synthetic (seeded config-{args.config} generator)",
            "config": {"workload": workload, "poses": int(p.n_poses), "landmarks": int(p.n_landmarks),
                       "obs": int(p.n_obs), "reduced_system": 6 * int(p.n_poses),
                       "chosen_stop_rho": 0.0 if args.stop_rho is None else float(args.stop_rho),
                       "l2": "256 MB flush written between timed steps"},
            "iterations": int(st["iterations"]), "ms_per_iteration": chosen_ms / max(1, st["iterations"]),
            "iterations_to_plain_cost": hit[0] if hit else None,
            "ms_to_plain_cost": chosen_ms / max(1, st["iterations"]) * hit[0] if hit else None,
            "reached_plain_cost": reached, "rel_cost_vs_plain": float((st["cost"] - st64["cost"]) / st64["cost"]),
            "plain_fp64": {"ms": min(ms64), "iterations": int(st64["iterations"]),
                           "ms_per_iteration": min(ms64) / max(1, st64["iterations"]),
                           "chosen_speedup": min(ms64) / chosen_ms},
            "kernels": kernels, "gpu_launches": int(launches), "clocks": clk, "cpu_baseline": None,
            "e2e": {"value": (1.0 / float(np.mean(e2e))) * (1.0 if reached else 0.0), "unit": "solves/s",
                    "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": 1e3 * float(np.mean(e2e))}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--check-every", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--plain-serial", type=int, default=1, help="1: also time the FP64 solver one problem at a time")
    ap.add_argument("--tc", type=int, default=1, help="1: tensor-core Schur complement in the mixed path, 0: SIMT")
    ap.add_argument("--controller", type=int, default=0, help="chosen form's damping: 1 learned (shipped weights), "
                    "0 Nielsen")
    ap.add_argument("--outer", type=int, default=-1, help="refinement steps of the mixed step (-1: library default)")
    ap.add_argument("--max-iters", type=int, default=35, help="LM iteration cap of the chosen form")
    ap.add_argument("--stop-rho", type=float, default=None, help="chosen form: least gain ratio of a step that "
                    "ends the solve by the relative-decrease test (0: any accepted step; default 0.25 on the "
                    "config-3 batch, 0 on the single problems of configs 1 and 2)")
    ap.add_argument("--autotune", type=int, default=1, help="1: time the run-time launch shapes first")
    ap.add_argument("--inflight", type=int, default=4, help="e2e: batches solving at once in solve_stream")
    ap.add_argument("--shapes", default="", help="COST,LIN: cost-pass and Jacobian-pass CTA sizes instead of "
                                                 "autotuning (e.g. 64,128, to profile the shapes it picks)")
    ap.add_argument("--config", type=int, default=3, choices=[1, 2, 3],
                    help="3: the 256-problem batch (headline); 1, 2: one large problem, chosen form against "
                         "the plain FP64 GPU solver")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config in SINGLE:
        return run_single(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
