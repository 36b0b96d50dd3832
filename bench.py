#!/usr/bin/env python3
"""Benchmark: batched Levenberg-Marquardt solves of the config-3 workload.

Workload (synthetic, seeded): 256 independent stereo pose-graph / bundle-
adjustment problems, N ~ U[8, 32] incremental poses and L ~ U[200, 3000]
landmarks each (circle generator, 1 px noise), every problem run to a
relative cost decrease below 1e-6 or 30 LM iterations.  One step = one solve
of the whole batch from its initial state.

* ``value``: solves/s of the chosen form (mixed precision, batched) with the
  inputs resident in HBM; L2 is flushed (256 MB write) between timed steps.
* ``e2e``: the same metric through the public API per step: marshal and plan
  the host problems, upload, solve, read back poses and inverse depths.  The
  headline runs batches through ``solver.solve_stream`` (batches planned on a
  worker thread ahead of their solve, ``--inflight`` batches solving at once on
  their own CUDA streams); ``serial_value`` is one ``BatchSolver`` after another.
* ``plain_fp64``: the plain FP64 GPU solver (problems one at a time), its
  solves/s and how many chosen-form costs reach its converged cost (rel 1e-6).
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
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    Ns = rng.integers(8, 33, n)
    Ls = rng.integers(200, 3001, n)
    seeds = rng.integers(0, 2**31 - 1, n)
    return [(int(s), int(a), int(b)) for s, a, b in zip(seeds, Ns, Ls)]


def cpu_oracle_sample(specs, n_sample: int, workers: int):
    """Solve ``n_sample`` problems with the FP64 oracle in a spawned pool; solves/s."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    with ctx.Pool(workers) as pool:
        out = pool.map(_oracle_solve, specs[:n_sample], chunksize=1)
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
# algorithmic bytes per launch (roofline numerators)
# ---------------------------------------------------------------------------
def roofline_numerator(kind: str, sizes, slab_floats: int, ts: int, probs):
    """(bound, unit, algorithmic amount per launch) for a profiled kernel kind.

    linearisation / cost: HBM bytes (observations 20 B, landmark record 40 B, C/g_a,
    slab written); Schur: FLOPs of the W D^-1 W^T chunk blocks, sum 2 (6 nb)^2 32;
    factor_solve: dense Cholesky + two solve pairs per problem (P^3/3 + 4 P^2)."""
    O, L = sizes.total_obs, sizes.total_landmarks
    if kind == "linearize":
        return "hbm", "GB/s", 20.0 * O + 40.0 * L + 2.0 * ts * L + ts * slab_floats
    if kind == "cost":
        return "hbm", "GB/s", 20.0 * O + 40.0 * L
    if kind == "schur":
        return "tensor", "TFLOP/s", float(sizes.schur_flops)
    if kind == "factor_solve":
        return "fp32", "TFLOP/s", float(sum((6 * p.n_poses) ** 3 / 3.0 + 4 * (6 * p.n_poses) ** 2 for p in probs))
    return None, None, 0.0


# DRAM bytes (read + write) per launch of the profiled kernels on this workload
# (256-problem batch, mixed precision), dram__bytes_read.sum + dram__bytes_write.sum:
# the cost and Jacobian passes at the tuned CTA sizes (64, 128) from
# profiles/ncu_linearize_config3_tuned.md, the rest from
# profiles/ncu_kernels_config3_batch.md
NCU_TRAFFIC = {"cost": 119.64e6, "linearize": 251.50e6, "schur": 224.89e6, "factor_solve": 24.00e6,
               "backsub": 206.67e6}
NCU_TRAFFIC_SOURCE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum, profiles/ncu_linearize_config3_tuned.md "
                      "(cost, linearize) and profiles/ncu_kernels_config3_batch.md (the rest)")


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


def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    workers = max(1, os.cpu_count() or 1)
    specs = _config3_specs(_batch_seed(0))
    per_step = max(workers, 16)
    times = []
    for it in range(args.warmup + args.steps):
        sample = [specs[(it * per_step + k) % len(specs)] for k in range(per_step)]
        _, wall, _ = cpu_oracle_sample(sample, per_step, workers)
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
                                       f"one process per core"},
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
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import __graft_entry__
    __graft_entry__.load_package()
    import importlib
    importlib.import_module("spgo_gb300.build").build()
    scenes = importlib.import_module("spgo_gb300.scenes")
    sv = importlib.import_module("spgo_gb300.solver")
    nat = importlib.import_module("spgo_gb300.native")

    specs = _config3_specs(_batch_seed(rank))
    # CPU baseline first (spawned pool, before the solver does any GPU work)
    cpu = None
    if rank == 0 and not args.no_cpu:
        workers = max(1, os.cpu_count() or 1)
        n_s = max(workers, 16)
        rate, wall, _ = cpu_oracle_sample(specs, n_s, workers)
        cpu = {"value": rate, "unit": "solves/s", "cores": workers, "kind": "port",
               "sample": f"first {n_s} problems of the batch, FP64 numpy oracle LM "
                         f"(same stopping rule), one process per core, {wall:.1f} s"}

    probs = scenes.config3(seed=_batch_seed(rank))
    n_obs = sum(p.n_obs for p in probs)
    n_lm = sum(p.n_landmarks for p in probs)
    # a non-default stream: the solver replays its LM iterations as CUDA graphs on it
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    # learned damping: the shipped network (trained by train_controller.py), if present
    ctl_params = None
    if args.controller:
        learned = importlib.import_module("spgo_gb300.learned")
        if os.path.exists(learned.DEFAULT_WEIGHTS):
            ctl_params = learned.Controller.load(device=dev).deployed()

    tuned = None

    def make(precision):
        s = sv.BatchSolver(probs, precision=precision, device=dev, stream=stream)
        s.set_params(loss="l2", max_iters=30, tol=1e-6, lambda0=1e-4, use_tc=args.tc)
        if tuned is not None:  # later solvers of the same batch reuse the tuned shapes
            s.set_params(**tuned)
        if ctl_params is not None:
            s.set_controller(ctl_params)
        return s

    bs = make("mixed")
    if args.shapes:
        cb, lb = (int(x) for x in args.shapes.split(","))
        tuned = dict(cost_block=cb, lin_block=lb, use_tc=bs.params.use_tc)
        bs.set_params(**tuned)
    elif args.autotune:
        tuned = bs.autotune()  # launch shapes timed on this batch (untimed, before the warm-up)
    else:
        tuned = dict(cost_block=bs.params.cost_block, lin_block=bs.params.lin_block, use_tc=bs.params.use_tc)
    p0, a0 = bs.poses.clone(), bs.alpha.clone()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

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
    value = N_PROBLEMS * world * args.steps / (total_ms / 1e3)
    iters = [s["iterations"] for s in status]
    chosen_costs = np.array([s["cost"] for s in status])

    # kernel shares and roofline of the dominant kernel
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    pk = roofline_peaks(peaks, bool(args.tc))
    tot = sum(v[0] for v in prof.values()) or 1.0
    kernels = {k: {"ms": round(v[0], 4), "launches": v[1], "share": round(v[0] / tot, 4)} for k, v in prof.items()}
    slab_floats = int(bs.slab_floats())
    for k, v in prof.items():
        b_, u_, amt = roofline_numerator(k, bs.sizes, slab_floats, 4, probs)
        if b_ and v[1]:
            ms_ = v[0] / v[1]
            ach = amt / (ms_ / 1e3) / (1e9 if b_ == "hbm" else 1e12)
            kernels[k].update(bound=b_, achieved=round(ach, 3), unit=u_, frac=round(ach / pk[b_][0], 4))
    dom = max(prof, key=lambda k: prof[k][0])
    avg_ms = prof[dom][0] / max(1, prof[dom][1])
    bound, unit, amount = roofline_numerator(dom, bs.sizes, slab_floats, 4, probs)
    if bound:
        achieved = amount / (avg_ms / 1e3) / (1e9 if bound == "hbm" else 1e12)
        peak, peak_src = pk[bound]
    else:
        achieved, peak, peak_src = None, None, None
    roof = {"kernel": dom, "bound": bound, "achieved": achieved, "peak": peak, "unit": unit,
            "frac": (achieved / peak) if achieved else None,
            "traffic": NCU_TRAFFIC.get(dom),
            "traffic_source": NCU_TRAFFIC_SOURCE, "algorithmic_per_launch": amount,
            "avg_launch_ms": avg_ms, "peak_source": peak_src,
            "note": "algorithmic bytes per launch / CUDA-event launch duration (profiled step after the "
                    "timed region, CUDA graphs off)"}

    # plain FP64 GPU solver, one problem at a time (untimed for the headline)
    plain = None
    if not args.no_plain:
        plain_costs, t_plain = [], 0.0
        for p in probs:
            s1 = sv.BatchSolver([p], precision="fp64", device=dev, stream=stream)
            s1.set_params(loss="l2", max_iters=30, tol=1e-6, lambda0=1e-4)
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            st1 = s1.solve(check_every=args.check_every)[0]
            torch.cuda.synchronize(dev)
            t_plain += time.perf_counter() - t0
            plain_costs.append(st1["cost"])
            s1.close()
        plain_costs = np.array(plain_costs)
        reached = chosen_costs <= plain_costs * (1.0 + 1e-6)
        plain = {"solves_per_s": N_PROBLEMS / t_plain, "ms_per_batch": 1e3 * t_plain,
                 "chosen_speedup": (t_plain * 1e3) / (total_ms / args.steps),
                 "reached_plain_cost_frac": float(reached.mean()),
                 "median_rel_cost_diff": float(np.median(np.abs(chosen_costs - plain_costs) / plain_costs))}

    # end-to-end through the public API with host buffers: every batch is marshalled,
    # planned, uploaded, solved and read back.  Serially (one BatchSolver after
    # another), and as a stream (solve_stream: batches planned on a worker thread
    # ahead of their solve, --inflight batches solving at once), which is the headline.
    e2e_ms, h2d, d2h = [], 0, 0
    for k in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        s2 = make("mixed")
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
    stream_params = {**dict(loss="l2", max_iters=30, tol=1e-6, lambda0=1e-4, use_tc=args.tc), **(tuned or {})}
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _st, _poses, _alphas in sv.solve_stream([probs] * n_stream, "mixed", stream_params, ctl_params, device=dev,
                                                inflight=args.inflight, check_every=args.check_every):
        pass
    torch.cuda.synchronize(dev)
    stream_ms = 1e3 * (time.perf_counter() - t0) / n_stream
    e2e_val = N_PROBLEMS * world / (stream_ms / 1e3)

    line = {"metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (mixed)",
            "data": "synthetic (seeded config-3 generator)",
            "config": {"workload": WORKLOAD, "problems_per_gpu": N_PROBLEMS, "landmarks": n_lm, "obs": n_obs,
                       "precision": "mixed", "schur": "tcgen05 split TF32" if tuned["use_tc"] else "SIMT FP32",
                       "damping": "learned MLP + Nielsen fallback" if ctl_params is not None else "Nielsen",
                       "autotuned": tuned,
                       "l2": "256 MB flush written between timed steps",
                       "parallelism": f"replicas x{world} (independent batches)",
                       "iterations_max": int(max(iters)), "iterations_mean": float(np.mean(iters))},
            "roofline": roof, "kernels": kernels, "gpu_launches": int(launches), "clocks": clk,
            "cpu_baseline": cpu, "plain_fp64": plain,
            "e2e": {"value": e2e_val, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "ms_per_step": stream_ms, "steps": n_stream, "inflight": args.inflight,
                    "api": "solver.solve_stream: batches planned on a worker thread ahead of their solve, "
                           f"{args.inflight} batches solving at once on their own CUDA streams",
                    "serial_value": serial_val,
                    "serial_ms_per_step": float(np.mean(e2e_ms))}}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
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
    ap.add_argument("--tc", type=int, default=1, help="1: tensor-core Schur complement in the mixed path, 0: SIMT")
    ap.add_argument("--controller", type=int, default=1, help="1: learned damping (shipped weights), 0: Nielsen")
    ap.add_argument("--autotune", type=int, default=1, help="1: time the run-time launch shapes first")
    ap.add_argument("--inflight", type=int, default=4, help="e2e: batches solving at once in solve_stream")
    ap.add_argument("--shapes", default="", help="COST,LIN: cost-pass and Jacobian-pass CTA sizes instead of "
                                                 "autotuning (e.g. 64,128, to profile the shapes it picks)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
