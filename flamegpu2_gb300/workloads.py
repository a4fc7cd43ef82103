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


def _stage_table(prof: dict, algo: dict, per_launch: bool = True) -> dict:
    """prof: label -> (total ms, launches). algo: algorithmic bytes of one
    launch (per_launch) or of all the profiled launches together."""
    out = {}
    for label, (ms, cnt) in prof.items():
        d = {"launches": cnt, "avg_us": round(ms * 1000.0 / max(cnt, 1), 3), "total_ms": round(ms, 4)}
        if label in algo:
            total = algo[label] * cnt if per_launch else algo[label]
            d["algorithmic_bytes_total"] = int(total)
            d["gbs"] = round(total / (ms * 1e-3) / 1e9, 2) if ms > 0 else None
        out[label] = d
    return out


def profiled_value(summary: str, name: str, key: str = ""):
    """A per-launch figure of a workload's roofline kernel from one ncu capture
    summarised in profiles/<summary>.md (line '[key ]<name>: N'); None if absent."""
    import re
    try:
        with open(os.path.join(ROOT, "profiles", summary + ".md")) as f:
            m = re.search(r"^" + re.escape((key + " ") if key else "") + re.escape(name) + r":\s*([0-9.]+)",
                          f.read(), re.M)
    except OSError:
        return None
    return float(m.group(1)) if m else None


def profiled_traffic(summary: str, key: str = ""):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)."""
    t = profiled_value(summary, "traffic_bytes_per_launch", key)
    return int(t) if t is not None else None


def _with_traffic(roof: dict, summary: str, what: str = None, key: str = "") -> dict:
    """Adds the profiled DRAM traffic and, where the summary records the same
    launch's ncu duration (gpu__time_duration.sum), the roofline fraction that
    duration gives: a cross-check of the live event timing, which inside a
    graph also counts the event nodes and the lost programmatic launch overlap."""
    t = profiled_traffic(summary, key)
    if t is not None:
        roof["traffic"] = t
        roof["traffic_source"] = f"profiles/{summary}.md" + (f": {what}" if what else "")
    us = profiled_value(summary, "ncu_duration_us_per_launch", key)
    alg = roof.get("per_launch_algorithmic_bytes")
    if us and alg and roof.get("peak"):
        gbs = alg / (us * 1e-6) / 1e9
        roof["ncu_check"] = {"duration_us": us, "achieved": round(gbs, 2), "frac": round(gbs / roof["peak"], 4)}
    return roof


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
    s.time_ops_in_graphs(True)  # per-operation times from events inside the step graphs

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
    s.take_profile()
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
    # per-operation times of every one of the 100 steps (the population and so
    # the work changes each step): the same graph replays, one step at a time,
    # reading the timing events captured into the graphs after each
    reset()
    s.take_profile()
    for _ in range(steps_per):
        s.step(1)
        s.harvest_profile()
    prof = s.take_profile()
    s.time_ops_in_graphs(False)
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
    stages = _stage_table(prof, {"compact:agent": comp_bytes}, per_launch=False)
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
        "roofline": _with_traffic(_roofline(stages, peak, peak_kind), "birth_death_compact",
                                  "k_compact (the whole stage: the agent-function launch counts the survivors)"),
        "stages": stages,
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
    s.time_ops_in_graphs(True)  # per-operation times from events inside the step graphs
    for _ in range(args.warmup):
        s.step(1)
    s.synchronize()
    s.take_profile()
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
        ev[k][1].synchronize()
        s.harvest_profile()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    device_ms = B.allreduce_max(world, sum(a.elapsed_time(b) for a, b in ev))
    prof = s.take_profile()
    s.close()
    vm = 4 * dims + 16  # position + 4 payload floats
    va_r, va_w = vm, 16
    algo = {"build:location": 2 * n * vm + 4 * (bins + 1),
            "fn:in": n * vm + 4 * (bins + 1) + n * (va_r + va_w),
            "fn:out": n * va_r + n * vm,
            "sort:agent": 2 * n * (4 + vm)}
    pair = "sort+build:agent/location"  # the agent sort and the message build as one chain of paired launches
    algo[pair] = algo["build:location"] + algo["sort:agent"]
    peak, peak_kind = B.measured_peaks()
    stages = _stage_table(prof, algo)
    if "fn:in" in stages:
        stages["fn:in"]["candidate_pairs"] = cand
        stages["fn:in"]["candidate_pairs_per_s"] = round(cand * stages["fn:in"]["launches"] /
                                                         (stages["fn:in"]["total_ms"] * 1e-3), 1)
    paired = pair in stages
    op = pair if paired else "build:location"
    bd = stages.get(op, {})
    what = ("sort+build:agent/location (4 paired launches: scan, placement, stable positions, long bins, each doing "
            "the agent sort and the message build; the keys are computed by the output launch)" if paired else
            "build:location (4 kernels: scan, perm, stabilise, long bins; the bin keys are computed by the output launch)")
    roof = {"bound": "hbm", "kernel": what,
            "achieved": bd.get("gbs"), "peak": peak, "unit": "GB/s",
            "frac": round(bd["gbs"] / peak, 4) if bd.get("gbs") else None, "traffic": None,
            "peak_source": peak_kind, "per_launch_algorithmic_bytes": algo[op],
            "note": "iterate is on-chip bound here (see stages.fn:in.candidate_pairs_per_s)"}
    if paired:
        roof = _with_traffic(roof, "spatial_large_sort_build", "the four paired launches of a simulation step of "
                             "this workload", name)
    else:
        roof = _with_traffic(roof, "spatial_large_build", "the four build kernels a simulation step runs, from a "
                             "standalone build of this size", name)
    cpu = None
    if world == 1 and rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_payload(dims, edge, r, cols, 20_000 if dims == 3 else 1_000_000)
    out = {
        "metric": B.METRIC, "value": round(n * k_steps * world / (device_ms / 1000.0), 1), "unit": UNIT,
        "n_gpus": world, "steps": k_steps, "warmup": args.warmup, "ms_per_step": round(device_ms / k_steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 uniforms / Box-Muller normals)",
        "config": {"workload": desc, "agents": n, "bins": bins, "candidate_pairs_per_step": cand,
                   "l2": "working set larger than L2"},
        "wall_s": round(wall, 4), "roofline": roof, "stages": stages, "gpu_launches": kps * k_steps, "clocks": clk,
    }
    if cpu is not None:
        out["cpu_baseline"] = cpu
    return out


def cpu_baseline_payload(dims, edge, r, cols, m):
    """The serial oracle on a bounded sample of the full-size workload: one
    model step in which the oracle sorts and builds the whole population and
    only m randomly chosen agents run the iterate layer, so each agent's
    iterate costs what it costs at full size. The step time is extrapolated to
    the whole population: t(sort + build) + t(iterate of m) * n / m."""
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import oracle as O
    n = cols["x"].shape[0]
    g = O.grid(dims, [0.0] * dims, [edge] * dims, r)
    st = {"id": cols["_id"], **{k: v for k, v in cols.items() if k != "_id"}}
    sample = np.sort(np.random.default_rng(11).choice(n, m, replace=False))
    _, t_index, t_iter = O.payload_step_sampled(g, False, st, sample)
    step_s = t_index + t_iter * n / m
    return {"value": round(n / step_s, 1), "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"one model step of the full {n:,}-agent population: serial sort + message build of all "
                      f"agents ({t_index:.1f} s) and the iterate of {m:,} random agents ({t_iter:.1f} s), "
                      f"extrapolated to {n:,} agents ({step_s:.0f} s per step)"}


# ------------------------------------------------------------ batched ensemble

def _ensemble_once(specs, pops, steps, batched, device, read_back=True, tuning="off"):
    """One CUDAEnsemble::simulate over the given instances through the public
    API (host populations in, host populations out). Returns timings."""
    from flamegpu2_gb300 import sim, synth
    t0 = time.perf_counter()
    ens = sim.Ensemble("boids_spatial3d", synth.boids_params(dict(synth.BOIDS_SMALL)), device=device, batched=batched,
                       tuning=tuning)
    for sp, pop in zip(specs, pops):
        r = ens.add_run(steps, sp["seed"], "Boid", sp["n"], pop, "location", (0.0, 0.0, 0.0), (sp["edge"],) * 3,
                        sp["radius"])
        ens.set_property(r, "MIN_POSITION", 0.0)
        ens.set_property(r, "MAX_POSITION", sp["edge"])
        ens.set_property(r, "INTERACTION_RADIUS", sp["radius"])
    if ens.simulate() != 0:
        raise RuntimeError("ensemble run failed")
    d2h = 0
    if read_back:
        for i, sp in enumerate(specs):
            for k in ("x", "y", "z", "fx", "fy", "fz"):
                d2h += ens.get(i, "Boid", k, np.float32).nbytes
    wall = time.perf_counter() - t0
    st = ens.stats()
    tun = ens.tuning() if batched else {"tuned": False}
    ens.close()
    return {"wall_s": wall, "step_s": st["step_s"], "simulate_s": st["elapsed_s"], "batched": st["batched"],
            "kernels_per_step": st["kernels_per_step"], "graph_launches": st["graph_launches"], "d2h": d2h,
            "tuning": tun}


def run_ensemble(args, world, rank, local):
    """256 Boids instances, population log-uniform in [1,024, 1,048,576],
    radius uniform in [1, 4], edge 4 r cbrt(N/64) (whole radii), 100 steps:
    one batched simulation (segmented kernels, one graph per step) against the
    same instances run one after another through CUDASimulation."""
    import torch
    from flamegpu2_gb300 import synth
    B = _bench_common()
    torch.cuda.set_device(local)
    count, steps = 256, 100
    specs = synth.ensemble_instances(count, seed=1000 + 1000 * rank, n_lo=1024, n_hi=1 << 20)
    pops = [synth.boids_population(sp["n"], 0.0, sp["edge"], sp["seed"]) for sp in specs]
    total_n = sum(sp["n"] for sp in specs)
    agent_steps = total_n * steps
    for _ in range(args.warmup):  # graphs, pools, code paths
        _ensemble_once(specs[:8], pops[:8], 3, True, local, read_back=False)
    # the launch shape: the committed tuning cache's entry for this GPU and size
    # class; without one, the autotuner measures it here (outside the timed runs)
    probe = _ensemble_once(specs, pops, 1, True, local, read_back=False, tuning="cache")
    if not probe["tuning"].get("tuned"):
        probe = _ensemble_once(specs, pops, 1, True, local, read_back=False, tuning="measure")
    clocks = B.ClockSampler(local)
    clocks.start()
    B.barrier(world)
    k = max(1, min(args.steps, 3))
    runs = [_ensemble_once(specs, pops, steps, True, local, tuning="cache") for _ in range(k)]
    # A/B: the same runs with the fixed launch shapes
    fixed = [_ensemble_once(specs, pops, steps, True, local, tuning="off") for _ in range(k)]
    clk = clocks.stop()
    step_s = B.allreduce_max(world, sum(r["step_s"] for r in runs))
    wall_s = B.allreduce_max(world, sum(r["wall_s"] for r in runs))
    fixed_step_s = B.allreduce_max(world, sum(r["step_s"] for r in fixed))
    # the plain path: the same instances one after another (CUDASimulation per run)
    seq = _ensemble_once(specs, pops, steps, False, local)
    seq_step_s = B.allreduce_max(world, seq["step_s"])
    seq_wall_s = B.allreduce_max(world, seq["wall_s"])
    bins = 0
    for sp in specs:
        cells = int(round(sp["edge"] / np.float32(sp["radius"])))
        bins += cells ** 3
    step_bytes = 136 * total_n + 8 * (bins + count)  # Bd + It, Boids message 28 B
    peak, peak_kind = B.measured_peaks()
    achieved = step_bytes * steps * k / step_s / 1e9
    h2d = total_n * 28
    return {
        "metric": B.METRIC, "value": round(agent_steps * k * world / step_s, 1), "unit": UNIT, "n_gpus": world,
        "steps": k, "warmup": args.warmup, "ms_per_step": round(step_s * 1000.0 / k, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 uniforms; instance sizes and radii from seeds 1000+i)",
        "config": {"workload": "batched ensemble: 256 Boids instances, N log-uniform [1024, 1048576], r U[1,4], "
                               "edge 4 r cbrt(N/64), 100 steps",
                   "instances": count, "agents_total": total_n, "bins_total": bins, "model_steps": steps,
                   "l2": "working set larger than L2",
                   "sequential_plain_path": {
                       "value": round(agent_steps * world / seq_step_s, 1),
                       "e2e": round(agent_steps * world / seq_wall_s, 1),
                       "what": "same instances, one CUDASimulation after another (graphs on)"},
                   "speedup_vs_sequential": round(seq_step_s / (step_s / k), 2),
                   "e2e_speedup_vs_sequential": round(seq_wall_s / (wall_s / k), 2),
                   "kernels_per_step": runs[0]["kernels_per_step"],
                   "tuned": bool(runs[0]["tuning"].get("tuned")), "tuning": runs[0]["tuning"],
                   "fixed_shapes": {"value": round(agent_steps * k * world / fixed_step_s, 1),
                                    "ms_per_step": round(fixed_step_s * 1000.0 / k, 3),
                                    "what": "the same runs with the default launch shapes (tuning off)"},
                   "tuned_over_fixed": round(fixed_step_s / step_s, 3)},
        "wall_s": round(wall_s, 3),
        "e2e": {"value": round(agent_steps * k * world / wall_s, 1), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": runs[0]["d2h"],
                "path": "fge_add_run x256 + fge_simulate + fge_get_variable (C ABI, host buffers)"},
        "roofline": {"bound": "hbm", "kernel": "whole batched step (sort, build, iterate; one graph)",
                     "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": None, "peak_source": peak_kind, "per_launch_algorithmic_bytes": step_bytes},
        "gpu_launches": runs[0]["kernels_per_step"] * steps * k, "clocks": clk,
    }


# ----------------------------------------------------------------- serving

def _served_requests(count, seed):
    """Requests: 50/50 Boids-3D / predator-prey-2D, N log-uniform in
    [1024, 4194304], steps uniform in [10, 1000]."""
    from flamegpu2_gb300 import synth
    reqs = []
    for i in range(count):
        u = (synth.bits(seed, 100 + i, 3) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
        n = int(round(np.exp(np.log(1024) + u[0] * (np.log(4194304) - np.log(1024)))))
        steps = 10 + int(u[1] * 991)
        if u[2] < 0.5:
            edge = 2.0 * max(1, int(np.ceil(32.0 * np.cbrt(n / 16384.0))))  # config-0 density, whole radii
            cfg = dict(synth.BOIDS_SMALL, n=n, max_pos=edge)
            pop = synth.boids_population(n, 0.0, edge, seed + i)
            reqs.append({"model": "boids_spatial3d", "params": synth.boids_params(cfg), "steps": steps, "n": n,
                         "pops": {"Boid": (n, pop)}})
        else:
            # three agents per unit area, a quarter of them predators: the prey's
            # crowding limit (4 others within r) holds them to about 3.5 per unit
            # area, i.e. below twice their initial number, once the predators die out
            n_pred = max(1, n // 4)
            n_prey = n - n_pred
            edge = float(np.ceil(np.sqrt(n / 3.0)))
            prey, pred = synth.predprey_population(n_prey, n_pred, edge, seed + i)
            reqs.append({"model": "predprey2d", "params": [edge, 1.0, 0.05, 0.02, 0.5, seed + i], "steps": steps,
                         "n": n, "pops": {"prey": (n_prey, prey), "predator": (n_pred, pred)}})
    return reqs


def _percentile(v, q):
    return float(np.percentile(np.asarray(v, dtype=np.float64), q)) if v else None


def _srpt_latencies(arrivals, service):
    """Completion minus arrival of each job under preemptive shortest remaining
    service first on one server (event simulation)."""
    n = len(arrivals)
    rem = list(service)
    done = [None] * n
    t, nxt, active = 0.0, 0, []
    order = sorted(range(n), key=lambda i: arrivals[i])
    while nxt < n or active:
        if not active:
            t = max(t, arrivals[order[nxt]])
        while nxt < n and arrivals[order[nxt]] <= t:
            active.append(order[nxt])
            nxt += 1
        j = min(active, key=lambda i: rem[i])
        horizon = arrivals[order[nxt]] if nxt < n else float("inf")
        run = min(rem[j], horizon - t)
        t += run
        rem[j] -= run
        if rem[j] <= 1e-12:
            done[j] = t
            active.remove(j)
    return [done[i] - arrivals[i] for i in range(n)]


def run_served(args, world, rank, local):
    """Poisson request streams served by SimulationServer (continuous
    batching under a 150 GB budget) against the same requests run one after
    another through CUDASimulation (FIFO)."""
    import torch
    from flamegpu2_gb300 import sim
    B = _bench_common()
    torch.cuda.set_device(local)
    count = max(8, min(int(os.environ.get("FG_SERVED_REQUESTS", "32")), 256))
    rates = getattr(args, "served_rates", None) or \
        [float(r) for r in os.environ.get("FG_SERVED_RATES", "10,30,100,300,1000").split(",")]
    reqs = _served_requests(count, 4 + 1000 * rank)
    # warm-up: a few small runs through both paths
    for _ in range(args.warmup):
        srv = sim.Server(device=local)
        for r in reqs[:2]:
            srv.submit(r["model"], r["params"], 3, 0, r["pops"])
        srv.run_until_idle()
        srv.close()
    # plain path, one request after another: service time of each
    # (and the agent-steps of each run: the populations entering each of its steps)
    service, work = [], []
    for r in reqs:
        t0 = time.perf_counter()
        s = sim.Simulation(r["model"], r["params"], device=local)
        for agent, (n, cols) in r["pops"].items():
            s.set_population(agent, n, cols)
        s.step(r["steps"])
        for agent in r["pops"]:
            s.get(agent, "x", np.float32)
        service.append(time.perf_counter() - t0)
        work.append(s.agent_steps())
        s.close()
    per_rate = []
    clocks = B.ClockSampler(local)
    clocks.start()
    launches = 0
    for ri, rate in enumerate(rates):
        from flamegpu2_gb300 import synth
        u = (synth.bits(77 + ri, 0, count) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
        arrivals = np.cumsum(-np.log(1.0 - u) / rate)  # Poisson process: exponential gaps
        t_srv = time.perf_counter()  # the server's clock starts inside its constructor
        srv = sim.Server(device=local, memory_budget=150 << 30, max_active=64)
        if os.environ.get("FG_SERVED_INFLIGHT"):
            srv.set_scheduling(0.0, float(os.environ["FG_SERVED_INFLIGHT"]))
        ids, order = {}, {}
        t_start = time.perf_counter()
        nxt = 0
        while True:
            remaining = srv.poll()
            now = time.perf_counter() - t_start
            while nxt < count and arrivals[nxt] <= now:
                r = reqs[nxt]
                rid = srv.submit(r["model"], r["params"], r["steps"], 0, r["pops"])
                ids[rid] = t_start + arrivals[nxt]
                order[rid] = nxt
                nxt += 1
                remaining += 1
            if nxt >= count and remaining == 0:
                break
            if remaining == 0:
                time.sleep(max(0.0, min(0.001, arrivals[nxt] - now)))
        makespan = time.perf_counter() - t_start
        counters = srv.counters()
        lat, detail = [], []
        for rid in srv.take_completed():
            info = srv.info(rid)
            if info["failed"]:
                raise RuntimeError(f"request {rid} failed: {info['error']}")
            # completion on the host clock minus the scheduled arrival
            lat.append(t_srv + info["completed_s"] - ids[rid])
            i = order[rid]
            detail.append([i, reqs[i]["model"][:5], reqs[i]["n"], reqs[i]["steps"], round(lat[-1], 3),
                           round(info["admitted_s"] - info["arrival_s"], 3)])
        srv.close()
        # the sequential plain path on the same arrivals (single FIFO server)
        done, seq_lat = 0.0, []
        for i in range(count):
            start = max(arrivals[i], done)
            done = start + service[i]
            seq_lat.append(done - arrivals[i])
        # shortest-remaining-service-first on one server, preemptive, from the
        # measured single-run service times: a reference point for the order
        srpt_lat = _srpt_latencies(arrivals, service)
        per_rate.append({"rate_req_s": rate, "throughput": round(sum(work) / makespan, 1),
                         "srpt_ideal": {"p50_s": round(_percentile(srpt_lat, 50), 4),
                                        "p99_s": round(_percentile(srpt_lat, 99), 4)},
                         "p50_s": round(_percentile(lat, 50), 4), "p99_s": round(_percentile(lat, 99), 4),
                         "makespan_s": round(makespan, 3), "scheduler": counters,
                         "requests": sorted(detail) if rate == max(rates) else None,
                         "sequential": {"throughput": round(sum(work) / done, 1),
                                        "p50_s": round(_percentile(seq_lat, 50), 4),
                                        "p99_s": round(_percentile(seq_lat, 99), 4), "makespan_s": round(done, 3)}})
    clk = clocks.stop()
    top = max(per_rate, key=lambda d: d["rate_req_s"])
    return {
        "metric": B.METRIC, "value": top["throughput"], "unit": UNIT,
        "n_gpus": world, "steps": len(rates), "warmup": args.warmup, "ms_per_step": round(top["makespan_s"] * 1000, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 populations; Poisson arrivals)",
        "config": {"workload": f"served request stream: {count} requests, 50/50 Boids-3D / predator-prey-2D, "
                               "N log-uniform [1024, 4194304], steps U[10, 1000], budget 150 GB",
                   "requests": count, "agent_steps": int(sum(work)),
                   "agent_steps_counted": "populations entering each step of each run, summed on the device "
                                          "(CUDASimulation::getAgentStepCount of the plain runs)",
                   "nominal_agent_steps": int(sum(r["n"] * r["steps"] for r in reqs)), "rates": per_rate,
                   "speedup_vs_sequential_at_top_rate": round(top["throughput"] / top["sequential"]["throughput"], 2),
                   "l2": "working sets larger than L2"},
        "e2e": {"value": top["throughput"], "unit": UNIT, "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "path": "fgv_submit / fgv_poll / fgv_take_completed (host populations in and out)"},
        "roofline": None, "gpu_launches": None, "clocks": clk,
    }


def run(name, args, world, rank, local):
    if name == "ensemble":
        return run_ensemble(args, world, rank, local)
    if name == "served":
        return run_served(args, world, rank, local)
    if name == "birth_death":
        return run_birth_death(args, world, rank, local)
    if name in ("spatial3d_large", "spatial2d_large"):
        return run_spatial_large(name, args, world, rank, local)
    raise SystemExit(f"unknown workload {name}")


def headline_extras(local):
    """The ensemble and serving halves of the headline metric ("ensemble
    agent-steps/s + p50/p99 vs plain"), in reduced form for the default bench
    line: one timed pass of the 256-instance batched Boids ensemble (with its
    fixed-shape and sequential plain-path counterparts), and the 32-request
    served stream at 1,000 requests/s (with the sequential plain path on the
    same arrivals). The full lines are the `ensemble` and `served` workloads."""
    import types
    a = types.SimpleNamespace(steps=1, warmup=1, no_cpu_baseline=True, served_rates=[1000.0])
    e = run_ensemble(a, 1, 0, local)
    v = run_served(a, 1, 0, local)
    rate = v["config"]["rates"][-1]
    ec = e["config"]
    return {
        "ensemble": {"workload": ec["workload"], "value": e["value"], "unit": UNIT, "e2e": e["e2e"]["value"],
                     "ms_per_model_step": round(e["ms_per_step"] / ec["model_steps"], 3),
                     "sequential_plain_path": ec["sequential_plain_path"]["value"],
                     "speedup_vs_sequential": ec["speedup_vs_sequential"],
                     "e2e_speedup_vs_sequential": ec["e2e_speedup_vs_sequential"],
                     "tuned_over_fixed": ec["tuned_over_fixed"], "timed_passes": e["steps"]},
        "served": {"workload": v["config"]["workload"], "rate_req_s": rate["rate_req_s"],
                   "value": rate["throughput"], "unit": UNIT,
                   "agent_steps": v["config"]["agent_steps"], "p50_s": rate["p50_s"], "p99_s": rate["p99_s"],
                   "sequential_plain_path": rate["sequential"],
                   "speedup_vs_sequential": round(rate["throughput"] / rate["sequential"]["throughput"], 2)},
    }
