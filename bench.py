#!/usr/bin/env python
"""Benchmark: agent-steps/s of FLAME GPU 2 workloads on GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Default workload: Boids on MessageSpatial3D, 16,384 agents in [0,64)^3,
radius 2 (32^3 bins), wrapped bounds, 10 model steps per bench step — the
single-instance Spatial3D Boids configuration the metric is quoted on.
A bench step runs the whole 10-step simulation; L2 is flushed (256 MiB write)
between bench steps. `value` times the captured-graph replays with inputs
resident in HBM (CUDA events on the simulation's stream); `e2e` times the
public C-ABI path from host buffers: setPopulationData (H2D), 10 steps,
getPopulationData (D2H), per bench step.

Other workloads: birth_death (1,048,576 agents, 8 f32 + 1 i32 + id, death 0.30,
birth 0.20, 100 steps), spatial3d_large (8,388,608 agents, 256^3 bins,
Gaussian mixture), spatial2d_large (16,777,216 agents, 1024^2 bins).

--impl reference times the reference path's CPU implementation on the host
cores: there is no CPU implementation of this path in FLAME GPU 2, so the
serial oracle (a restatement of the reference's algorithm) stands in, run with
all host threads on the same workload.

Under torchrun (N > 1) every rank runs an independent replica ("replicas
only": the path does not shard); value sums the ranks' agent-steps over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "agent-steps/sec & HBM GB/s fraction (Spatial3D Boids); ensemble agent-steps/s + p50/p99 vs plain"
UNIT = "agent-steps/s"


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix="fg_clocks_", suffix=".csv")
        os.close(fd)

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for nm, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(nm)
        try:
            os.remove(self.path)
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            # host-only ranks (the reference arm without a GPU, the CPU tests)
            dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- workloads

def boids_small_cfg():
    from flamegpu2_gb300 import synth
    return dict(synth.BOIDS_SMALL)


def boids_bytes(n, bins):
    """Algorithmic bytes per launch (each stage input read once, output written once):
    message 28 B (id,x,y,z,fx,fy,fz), agent read 28 B, agent write 24 B."""
    vm, va_r, va_w = 28, 28, 24
    out = {
        "fn:outputdata": n * va_r + n * vm,
        "build:location": 2 * n * vm + 4 * (bins + 1),
        "fn:inputdata": n * vm + 4 * (bins + 1) + n * (va_r + va_w),
        "sort:Boid": 2 * n * 28,
    }
    # the agent sort and the message build as one chain of paired launches
    out["sort+build:Boid/location"] = out["sort:Boid"] + out["build:location"]
    return out


def workloads_mod():
    from flamegpu2_gb300 import workloads
    return workloads


def run_boids_small(args, world, rank, local):
    import torch
    from flamegpu2_gb300 import sim, synth
    cfg = boids_small_cfg()
    n, steps_per = cfg["n"], cfg["steps"]
    bins = 32 ** 3
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pop = synth.boids_population(n, cfg["min_pos"], cfg["max_pos"], cfg["seed"] + rank)
    s = sim.Simulation("boids_spatial3d", synth.boids_params(cfg), device=local, steps=steps_per)
    if args.stage_bytes is not None:
        s.set_stage_bytes(args.stage_bytes)
    s.set_population("Boid", n, pop)
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    # every bench step is the workload itself: ten model steps from the seeded
    # population, restored from a device copy outside the timed region (the
    # flocks a continuing run forms make later steps costlier, so a continuing
    # run would measure a different state at each --steps; the e2e loop and the
    # CPU arms also start every sample from the seeded population)
    dpop = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in pop.items()}

    def restart():
        s.reset_population_device("Boid", n, dpop, n + 1)

    for _ in range(args.warmup):
        restart()
        s.step(steps_per)
    s.synchronize()
    kernels_per_step = s.stats()["kernels_per_step"]
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(args.steps):
        restart()
        with torch.cuda.stream(stream):
            flush.add_(1)  # > L2: evicts the previous bench step's working set
        ev[k][0].record(stream)
        s.step(steps_per)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t0
    s.synchronize()
    device_ms = sum(a.elapsed_time(b) for a, b in ev)
    device_ms = allreduce_max(world, device_ms)
    # per-operation times: a second timed pass of the same bench steps, with a
    # pair of CUDA events captured into the step graphs around every operation
    # (on the stream it runs on), read after each bench step; the pass above
    # carries no such instrumentation
    s.time_ops_in_graphs(True)
    for _ in range(2):
        restart()
        s.step(steps_per)
    s.synchronize()
    s.take_profile()
    for k in range(min(args.steps, 50)):
        restart()
        with torch.cuda.stream(stream):
            flush.add_(1)
        s.step(steps_per)
        s.harvest_profile()
    prof = s.take_profile()
    s.time_ops_in_graphs(False)
    # the roofline kernel's time in the mode of the timed pass (ten model steps
    # replayed as one graph): events around its launches only, every replay read
    dom = max(prof.items(), key=lambda kv: kv[1][0])[0]
    s.time_op_in_graphs(dom)
    for _ in range(2):
        restart()
        s.step(steps_per)
    s.synchronize()
    s.take_profile()
    for k in range(min(args.steps, 50)):
        restart()
        with torch.cuda.stream(stream):
            flush.add_(1)
        s.step(steps_per)
        s.harvest_profile()
    dom_prof = s.take_profile()
    s.time_op_in_graphs(None)
    # e2e through the C ABI from host buffers (pinned), with host copies in the timed region
    def pinned_like(a):
        buf = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory().numpy().view(a.dtype)
        buf[:] = a
        return buf
    pinned = {k: pinned_like(v) for k, v in pop.items()}
    names = ("_id", "x", "y", "z", "fx", "fy", "fz")
    outs = {k: pinned_like(pop[k]) for k in names}
    e2e_n = max(3, min(args.steps, 50))
    barrier(world)
    t1 = time.perf_counter()
    for _ in range(e2e_n):
        s.set_population("Boid", n, pinned)
        s.step(steps_per)
        s.get_population("Boid", outs)
    e2e_s = allreduce_max(world, time.perf_counter() - t1)
    clk = clocks.stop()
    s.close()
    peak, peak_kind = measured_peaks()
    algo = boids_bytes(n, bins)
    stages = {}
    for label, (ms, cnt) in prof.items():
        avg_us = ms * 1000.0 / max(cnt, 1)
        d = {"launches": cnt, "avg_us": round(avg_us, 3)}
        if label in algo:
            d["algorithmic_bytes"] = algo[label]
            d["gbs"] = round(algo[label] / (avg_us * 1e-6) / 1e9, 2)
        stages[label] = d
    dom_ms, dom_n = dom_prof.get(dom, prof[dom])
    dom_avg_s = dom_ms / 1000.0 / max(dom_n, 1)
    achieved = algo.get(dom, 0) / dom_avg_s / 1e9 if dom in algo else None
    agent_steps = n * steps_per * args.steps * world
    value = agent_steps / (device_ms / 1000.0)
    e2e_value = n * steps_per * e2e_n * world / e2e_s
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(device_ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded SplitMix64 uniforms)",
        "config": {"workload": "boids_spatial3d: 16,384 agents, [0,64)^3, r=2 (32^3 bins), wrapped, 10 model steps",
                   "agents": n, "bins": bins, "model_steps_per_bench_step": steps_per,
                   "l2": "flushed between bench steps (256 MiB write)", "parallelism": f"replicas x{world}",
                   "state": "every bench step starts from the seeded population (device copy restored outside the "
                            "timed region), as the e2e loop and the CPU arms do"},
        "wall_s": round(wall, 4),
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT, "h2d_bytes_per_step": 28 * n, "d2h_bytes_per_step": 28 * n,
                "path": "fgs_set_population + fgs_step(10) + fgs_get_population (C ABI, pinned host buffers)"},
        "roofline": workloads_mod()._with_traffic(
            {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 2) if achieved else None, "peak": peak,
             "unit": "GB/s", "frac": round(achieved / peak, 4) if achieved else None, "traffic": None,
             "peak_source": peak_kind, "per_launch_algorithmic_bytes": algo.get(dom)},
            "boids_small_inputdata" if dom == "fn:inputdata" else ""),
        "stages": stages,
        "stage_timing": "stages: CUDA events captured around every operation in single-step graphs (a separate "
                        "instrumented pass; sort and build overlap on two graph branches, so stages do not add up "
                        "to ms_per_step). roofline: the dominant operation alone timed by events inside the same "
                        "ten-step graphs as the timed pass",
        "roofline_kernel_us": round(dom_avg_s * 1e6, 3),
        "roofline_kernel_launches_timed": int(dom_n),
        "gpu_launches": kernels_per_step * steps_per * args.steps,
        "clocks": clk,
    }
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline_boids(cfg, threads=1, budget_s=args.cpu_budget)
    if world == 1 and not args.no_extras:
        # the metric's other halves (ensemble agent-steps/s, served p50/p99 vs
        # the plain path), after the timed region, in reduced form
        out.update(workloads_mod().headline_extras(local))
    return out


def cpu_baseline_boids(cfg, threads: int, budget_s: float):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from flamegpu2_gb300 import synth
    p = O.boids_params(cfg["min_pos"], cfg["max_pos"], cfg["interaction_radius"], cfg["separation_radius"],
                       cfg["time_scale"], cfg["global_scale"], cfg["steer_scale"], cfg["collision_scale"],
                       cfg["match_scale"], cfg["wrap"], cfg["sort_period"])
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], cfg["seed"])
    st = {"id": pop["_id"], **{k: pop[k] for k in ("x", "y", "z", "fx", "fy", "fz")}}
    O.boids_run(p, st, 1, threads=threads)  # load + warm
    reps, t0 = 0, time.perf_counter()
    while True:
        O.boids_run(p, st, cfg["steps"], threads=threads)
        reps += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    value = cfg["n"] * cfg["steps"] * reps / el
    return {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{reps} x (16,384-agent wrapped Boids, 10 steps) in {el:.1f} s, serial oracle"}


def run_reference(args, world, rank):
    """Reference arm: the oracle restatement on the host cores (the reference has no CPU path)."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from flamegpu2_gb300 import synth
    cfg = boids_small_cfg()
    threads = os.cpu_count() or 1
    p = O.boids_params(cfg["min_pos"], cfg["max_pos"], cfg["interaction_radius"], cfg["separation_radius"],
                       cfg["time_scale"], cfg["global_scale"], cfg["steer_scale"], cfg["collision_scale"],
                       cfg["match_scale"], cfg["wrap"], cfg["sort_period"])
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], cfg["seed"])
    st = {"id": pop["_id"], **{k: pop[k] for k in ("x", "y", "z", "fx", "fy", "fz")}}
    for _ in range(args.warmup):
        O.boids_run(p, st, cfg["steps"], threads=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        O.boids_run(p, st, cfg["steps"], threads=threads)
    el = time.perf_counter() - t0
    value = cfg["n"] * cfg["steps"] * args.steps / el
    sample = f"{args.steps} x (16,384-agent wrapped Boids, 10 steps), oracle port, {threads} host threads"
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(el * 1000 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 uniforms)",
        "config": {"workload": "boids_spatial3d: 16,384 agents, [0,64)^3, r=2 (32^3 bins), wrapped, 10 model steps"},
        "cpu_baseline": {"value": round(value, 1), "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(value, 1), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="boids_small",
                    choices=["boids_small", "birth_death", "spatial3d_large", "spatial2d_large", "ensemble", "served"])
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU work for cpu_baseline")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="default line: skip the reduced ensemble and served summaries")
    ap.add_argument("--stage-bytes", type=int, default=None,
                    help="shared memory per block for spatial neighbour staging (0 disables)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        out = run_reference(args, world, rank)
    else:
        if args.workload == "boids_small":
            out = run_boids_small(args, world, rank, local)
        else:
            from flamegpu2_gb300 import workloads
            out = workloads.run(args.workload, args, world, rank, local)
    if rank == 0 and out is not None:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
