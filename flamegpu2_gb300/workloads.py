"""Benchmark workloads other than the default Boids line (selected with
bench.py --workload). Each returns one JSON-able dict in bench.py's format.

  birth_death      1,048,576 agents (8 f32 + counter i32 + id), death p=0.30,
                   birth p=0.20 for survivors, 100 steps; one bench step = the
                   whole 100-step run restarted from the same device-resident
                   population. agent-steps = sum of the populations entering
                   each step.
  spatial3d_large  8,388,608 agents in [0,256)^3, r=1 (256^3 bins), 16-component
                   Gaussian mixture (sigma 2, clipped), 4 f32 payload; one bench
                   step = one model step (build + iterate).
  spatial2d_large  16,777,216 agents uniform in [0,4096)^2, r=4 (1024^2 bins),
                   4 f32 payload; one bench step = one model step.
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
UNIT = "agent-steps/s"


def _bench_common():
    import bench  # the driver script at the repository root
    return bench


def _stage_table(prof: dict, algo: dict) -> dict:
    out = {}
    for label, (ms, cnt) in prof.items():
        d = {"launches": cnt, "avg_us": round(ms * 1000.0 / max(cnt, 1), 3), "total_ms": round(ms, 4)}
        if label in algo:
            d["algorithmic_bytes_total"] = int(algo[label])
            d["gbs"] = round(algo[label] / (ms * 1e-3) / 1e9, 2) if ms > 0 else None
        out[label] = d
    return out


def _roofline(stages: dict, peak: float, peak_kind: str) -> dict:
    cands = [(k, v) for k, v in stages.items() if "gbs" in v and v.get("gbs")]
    if not cands:
        return {"bound": "hbm", "achieved": None, "peak": peak, "unit": "GB/s", "frac": None, "traffic": None}
    k, v = max(cands, key=lambda kv: kv[1]["total_ms"])
    return {"bound": "hbm", "kernel": k, "achieved": v["gbs"], "peak": peak, "unit": "GB/s",
            "frac": round(v["gbs"] / peak, 4), "traffic": None, "peak_source": peak_kind,
            "per_launch_algorithmic_bytes": int(v["algorithmic_bytes_total"] / max(v["launches"], 1))}


# --------------------------------------------------------------- birth/death

def run_birth_death(args, world, rank, local):
    import torch
    from flamegpu2_gb300 import sim, synth
    B = _bench_common()
    n0, steps_per, seed = 1 << 20, 100, 1
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    pop = synth.birth_death_population(n0, seed + rank)
    names = ["_id", "counter"] + [f"f{v}" for v in range(8)]
    resident = {k: torch.from_numpy(pop[k].view(np.int32) if pop[k].dtype == np.uint32 else pop[k]).to(dev)
                for k in names}
    s = sim.Simulation("birth_death", [0.30, 0.20, seed], device=local)

    def reset():
        s.reset_population_device("agent", n0, resident, n0 + 1)

    # populations entering each step (deterministic): one untimed run with reads
    reset()
    pops = []
    for _ in range(steps_per):
        pops.append(s.count("agent"))
        s.step(1)
    agent_steps = int(sum(pops))
    for _ in range(args.warmup):
        reset()
        s.step(steps_per)
    s.synchronize()
    kps = s.stats()["kernels_per_step"]
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    clocks = B.ClockSampler(local)
    clocks.start()
    k_steps = max(1, min(args.steps, 20))
    times = []
    B.barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(k_steps):
        reset()  # outside the event window: restores the initial population
        flush.add_(1)  # 256 MiB > L2: the restored population is read from HBM
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s.step(steps_per)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    device_ms = B.allreduce_max(world, sum(times))
    # op profile of one run (eager, event-bracketed)
    reset()
    s.profile_ops(True)
    s.step(steps_per)
    prof = s.take_profile()
    s.profile_ops(False)
    # e2e: host population in, 100 steps, host population out
    host_in = {k: pop[k] for k in names}
    outs = {k: np.empty(4 * n0, dtype=pop[k].dtype) for k in names}
    t1 = time.perf_counter()
    e2e_n = max(2, min(k_steps, 5))
    for _ in range(e2e_n):
        s.set_population("agent", n0, host_in)
        s.step(steps_per)
        s.get_population("agent", outs)
    e2e_s = B.allreduce_max(world, time.perf_counter() - t1)
    final = s.count("agent")
    s.close()
    row = 44  # 8 f32 + counter + _id
    comp_bytes = sum(pops[t] * row + (pops[t + 1] if t + 1 < steps_per else final) * row for t in range(steps_per))
    peak, peak_kind = B.measured_peaks()
    stages = _stage_table(prof, {"compact:agent": comp_bytes})
    return {
        "metric": B.METRIC, "value": round(agent_steps * k_steps * world / (device_ms / 1000.0), 1), "unit": UNIT,
        "n_gpus": world, "steps": k_steps, "warmup": args.warmup, "ms_per_step": round(device_ms / k_steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 uniforms; model-level hash RNG)",
        "config": {"workload": "birth_death: 1,048,576 agents x 44 B, death 0.30, birth 0.20 of survivors, 100 steps",
                   "agent_steps_per_run": agent_steps, "populations_first": pops[:5], "population_final": final,
                   "l2": "flushed between bench steps (256 MiB write)"},
        "wall_s": round(wall, 4),
        "e2e": {"value": round(agent_steps * e2e_n * world / e2e_s, 1), "unit": UNIT,
                "h2d_bytes_per_step": n0 * row, "d2h_bytes_per_step": final * row},
        "roofline": _roofline(stages, peak, peak_kind), "stages": stages,
        "gpu_launches": kps * steps_per * k_steps, "clocks": clk,
    }


# ---------------------------------------------------------- large spatial

def gaussian_mixture_3d(n: int, edge: float, comps: int, sigma: float, seed: int) -> np.ndarray:
    from flamegpu2_gb300 import synth
    centres = np.stack([synth.uniform(seed, 100 + a, comps, 0.0, edge) for a in range(3)], 1)
    which = (synth.bits(seed, 110, n) % np.uint64(comps)).astype(np.int64)
    pos = centres[which] + np.stack([synth.normal(seed, 120 + a, n, 0.0, sigma) for a in range(3)], 1)
    hi = np.nextafter(np.float32(edge), np.float32(0))
    return np.clip(pos, 0.0, hi).astype(np.float32)


def candidate_pairs(pos: np.ndarray, edge: float, radius: float) -> int:
    """Messages visited by all agents' Moore-neighbourhood iterations (clamped filter)."""
    dims = pos.shape[1]
    g = int(np.ceil(np.float32(edge) / np.float32(radius)))
    cell = np.clip(np.floor(pos / np.float32(radius)).astype(np.int64), 0, g - 1)
    flat = cell[:, 0]
    for a in range(1, dims):
        flat = flat + cell[:, a] * g ** a
    counts = np.bincount(flat, minlength=g ** dims).reshape((g,) * dims)
    padded = np.pad(counts, 1)
    nb = np.zeros_like(counts)
    import itertools
    for off in itertools.product((0, 1, 2), repeat=dims):
        sl = tuple(slice(o, o + g) for o in off)
        nb += padded[sl]
    return int((counts.astype(np.int64) * nb).sum())


def run_spatial_large(name, args, world, rank, local):
    import torch
    from flamegpu2_gb300 import sim, synth
    B = _bench_common()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if name == "spatial3d_large":
        dims, n, edge, r, seed = 3, 8 << 20, 256.0, 1.0, 2 + rank
        pos = gaussian_mixture_3d(n, edge, 16, 2.0, seed)
        desc = "spatial3d_large: 8,388,608 agents, [0,256)^3, r=1 (256^3 bins), 16-component Gaussian mixture sigma 2"
    else:
        dims, n, edge, r, seed = 2, 16 << 20, 4096.0, 4.0, 3 + rank
        hi = np.nextafter(np.float32(edge), np.float32(0))
        pos = np.stack([np.minimum(synth.uniform(seed, a, n, 0.0, edge), hi) for a in range(2)], 1)
        desc = "spatial2d_large: 16,777,216 agents uniform in [0,4096)^2, r=4 (1024^2 bins)"
    bins = int(np.ceil(edge / r)) ** dims
    cols = {"_id": np.arange(1, n + 1, dtype=np.uint32), "x": pos[:, 0].copy(), "y": pos[:, 1].copy()}
    if dims == 3:
        cols["z"] = pos[:, 2].copy()
    for k in range(4):
        cols[f"p{k}"] = synth.uniform(seed, 20 + k, n, 0.0, 1.0)
    cand = candidate_pairs(pos, edge, r)
    s = sim.Simulation("spatial_payload", [dims, 0.0, edge, r], device=local)
    s.set_population("agent", n, cols)
    for _ in range(args.warmup):
        s.step(1)
    s.synchronize()
    kps = s.stats()["kernels_per_step"]
    stream = torch.cuda.ExternalStream(s.stream, device=dev)
    clocks = B.ClockSampler(local)
    clocks.start()
    k_steps = max(1, min(args.steps, 20 if dims == 2 else 3))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(k_steps)]
    B.barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(k_steps):  # working set > L2: no flush needed
        ev[k][0].record(stream)
        s.step(1)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    device_ms = B.allreduce_max(world, sum(a.elapsed_time(b) for a, b in ev))
    s.profile_ops(True)
    s.step(1)
    prof = s.take_profile()
    s.profile_ops(False)
    s.close()
    vm = 4 * dims + 16  # position + 4 payload floats
    va_r, va_w = vm, 16
    algo = {"build:location": 2 * n * vm + 4 * (bins + 1),
            "fn:in": n * vm + 4 * (bins + 1) + n * (va_r + va_w),
            "fn:out": n * va_r + n * vm,
            "sort:agent": 2 * n * (4 + vm)}
    peak, peak_kind = B.measured_peaks()
    stages = _stage_table(prof, algo)
    if "fn:in" in stages:
        stages["fn:in"]["candidate_pairs"] = cand
        stages["fn:in"]["candidate_pairs_per_s"] = round(cand / (stages["fn:in"]["total_ms"] * 1e-3), 1)
    bd = stages.get("build:location", {})
    roof = {"bound": "hbm", "kernel": "build:location (5 kernels: bin, scan, perm, stabilise, long bins)",
            "achieved": bd.get("gbs"), "peak": peak, "unit": "GB/s",
            "frac": round(bd["gbs"] / peak, 4) if bd.get("gbs") else None, "traffic": None,
            "peak_source": peak_kind, "per_launch_algorithmic_bytes": algo["build:location"],
            "note": "iterate is on-chip bound here (see stages.fn:in.candidate_pairs_per_s)"}
    return {
        "metric": B.METRIC, "value": round(n * k_steps * world / (device_ms / 1000.0), 1), "unit": UNIT,
        "n_gpus": world, "steps": k_steps, "warmup": args.warmup, "ms_per_step": round(device_ms / k_steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 uniforms / Box-Muller normals)",
        "config": {"workload": desc, "agents": n, "bins": bins, "candidate_pairs_per_step": cand,
                   "l2": "working set larger than L2"},
        "wall_s": round(wall, 4), "roofline": roof, "stages": stages, "gpu_launches": kps * k_steps, "clocks": clk,
    }


def run(name, args, world, rank, local):
    if name == "birth_death":
        return run_birth_death(args, world, rank, local)
    if name in ("spatial3d_large", "spatial2d_large"):
        return run_spatial_large(name, args, world, rank, local)
    raise SystemExit(f"unknown workload {name}")
