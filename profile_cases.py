"""Small, fixed cases for profiling single kernels (ncu) and per-operation
timings, outside the benchmark's timed loop.

  python profile_cases.py boids --n 1048576
      Boids (wrapped, radius 2) at about one agent per bin: edge =
      4 r cbrt(N/64), the density of the batched-ensemble instances;
      prints per-operation timings (CUDA events, eager) and graph step time.
  python profile_cases.py ensemble --count 32
      The first `count` instances of the 256-instance Boids ensemble, 5 steps,
      as one batched simulation.
  python profile_cases.py payload --dims 2 --n 4194304
      The large spatial workloads' model (position + 4 payload words, squared
      distance test) at population n and the same density (2D uniform, r = 4,
      16 agents per bin; 3D Gaussian mixture, r = 1); per-operation timings and
      graph step time.
  python profile_cases.py build --dims 3
      Five spatial message builds through the C ABI (fg_spatial_build) of the
      large workloads' positions: 8,388,608 Gaussian-mixture messages on 256^3
      bins (--dims 3) or 16,777,216 uniform messages on 1024^2 bins (--dims 2),
      records of position + 4 payload words; prints the mean build time.
      --sorted orders the messages by bin first, as the messages of agents
      that the automatic spatial sort has ordered arrive in a simulation.
  python profile_cases.py sort --dims 3 --sorted
      Five automatic spatial agent sorts through the C ABI
      (fg_spatial_sort_agents) of the same positions with their agent columns
      (8 x 4 bytes in 3D, 7 in 2D); --sorted gives an already sorted population.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np


def boids(n: int, steps: int = 20):
    from flamegpu2_gb300 import sim, synth
    r = 2.0
    cells = int(np.ceil(4.0 * np.cbrt(n / 64.0)))
    edge = float(np.float32(r) * np.float32(cells))
    cfg = dict(synth.BOIDS_SMALL, n=n, max_pos=edge, interaction_radius=r)
    s = sim.Simulation("boids_spatial3d", synth.boids_params(cfg))
    s.set_population("Boid", n, synth.boids_population(n, 0.0, edge, 5))
    s.step(3)
    s.synchronize()
    s.profile_ops(True)
    s.step(5)
    prof = s.take_profile()
    s.profile_ops(False)
    s.step(steps)  # captures the step graphs this call replays
    s.synchronize()
    t = time.perf_counter()
    s.step(steps)
    s.synchronize()
    el = time.perf_counter() - t
    s.close()
    return {"n": n, "edge": edge, "ms_per_step_graph": round(el / steps * 1000, 4),
            "ops_us": {k: round(v[0] / max(v[1], 1) * 1000, 1) for k, v in prof.items()}}


def payload(dims: int, n: int, steps: int = 5):
    """The large spatial workloads' model at population n and their density:
    2D uniform (r = 4, 16 agents per bin), 3D Gaussian mixture (r = 1)."""
    from flamegpu2_gb300 import sim, synth, workloads
    if dims == 2:
        r = 4.0
        edge = float(4.0 * np.sqrt(n / 16.0))
        hi = np.nextafter(np.float32(edge), np.float32(0))
        pos = np.stack([np.minimum(synth.uniform(3, a, n, 0.0, edge), hi) for a in range(2)], 1)
    else:
        r = 1.0
        edge = float(np.ceil(256.0 * np.cbrt(n / float(8 << 20))))
        pos = workloads.gaussian_mixture_3d(n, edge, 16, 2.0, 2)
    cols = {"_id": np.arange(1, n + 1, dtype=np.uint32), "x": pos[:, 0].copy(), "y": pos[:, 1].copy()}
    if dims == 3:
        cols["z"] = pos[:, 2].copy()
    for k in range(4):
        cols[f"p{k}"] = synth.uniform(3, 20 + k, n, 0.0, 1.0)
    s = sim.Simulation("spatial_payload", [dims, 0.0, edge, r])
    s.set_population("agent", n, cols)
    s.step(2)
    s.synchronize()
    s.profile_ops(True)
    s.step(steps)
    prof = s.take_profile()
    s.profile_ops(False)
    s.step(steps)
    s.synchronize()
    t = time.perf_counter()
    s.step(steps)
    s.synchronize()
    el = time.perf_counter() - t
    s.close()
    return {"dims": dims, "n": n, "edge": edge, "ms_per_step_graph": round(el / steps * 1000, 4),
            "ops_us": {k: round(v[0] / max(v[1], 1) * 1000, 1) for k, v in prof.items()}}


def ensemble(count: int, steps: int = 5):
    from flamegpu2_gb300 import sim, synth
    specs = synth.ensemble_instances(count, seed=1000, n_lo=1024, n_hi=1 << 20)
    ens = sim.Ensemble("boids_spatial3d", synth.boids_params(dict(synth.BOIDS_SMALL)))
    for sp in specs:
        pop = synth.boids_population(sp["n"], 0.0, sp["edge"], sp["seed"])
        r = ens.add_run(steps, sp["seed"], "Boid", sp["n"], pop, "location", (0.0, 0.0, 0.0), (sp["edge"],) * 3,
                        sp["radius"])
        ens.set_property(r, "MIN_POSITION", 0.0)
        ens.set_property(r, "MAX_POSITION", sp["edge"])
        ens.set_property(r, "INTERACTION_RADIUS", sp["radius"])
    if ens.simulate() != 0:
        raise RuntimeError("ensemble run failed")
    st = ens.stats()
    ens.close()
    return {"instances": count, "agents": sum(sp["n"] for sp in specs), **st}


def build(dims: int, presorted: bool = False, reps: int = 5):
    import ctypes as C
    import torch
    from flamegpu2_gb300 import capi, synth, workloads
    if dims == 3:
        pos = workloads.gaussian_mixture_3d(1 << 23, 256.0, 16, 2.0, 2)
        g = capi.grid(3, (0, 0, 0), (256, 256, 256), 1.0)
    else:
        n = 1 << 24
        hi = np.nextafter(np.float32(4096.0), np.float32(0))
        pos = np.stack([np.minimum(synth.uniform(3, a, n, 0.0, 4096.0), hi) for a in range(2)], 1)
        g = capi.grid(2, (0, 0), (4096, 4096), 4.0)
    n = pos.shape[0]
    if presorted:
        cell = [np.clip(np.floor((pos[:, a] - np.float32(g.min[a])) / np.float32(g.radius)).astype(np.int64), 0,
                        g.gridDim[a] - 1) for a in range(dims)]
        key = cell[0] + cell[1] * g.gridDim[0] + (cell[2] * g.gridDim[0] * g.gridDim[1] if dims == 3 else 0)
        pos = pos[np.argsort(key, kind="stable")]
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(dims)]
    payload = torch.rand((n, 4), device="cuda")
    rec = capi.record_desc(cols + [payload])
    out = torch.empty((n, rec.words), dtype=torch.int32, device="cuda")
    pbm = torch.empty(g.binCount + 1, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(capi.lib().fg_spatial_build_workspace_size(n, g.binCount))
    st = capi.stream_handle()
    args = (C.byref(g), n, None, cols[0].data_ptr(), cols[1].data_ptr(), cols[2].data_ptr() if dims == 3 else None,
            None, C.byref(rec), out.data_ptr(), pbm.data_ptr(), ws.ptr, ws.nbytes, st)
    capi.check(capi.lib().fg_spatial_build(*args), "fg_spatial_build")
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        capi.check(capi.lib().fg_spatial_build(*args), "fg_spatial_build")
    b.record()
    b.synchronize()
    assert ws.status() == 0
    return {"dims": dims, "sorted_input": presorted, "messages": n, "bins": g.binCount, "record_bytes": rec.words * 4,
            "build_us": round(a.elapsed_time(b) * 1000 / reps, 1)}


def sort(dims: int, presorted: bool = False, reps: int = 5):
    """Automatic spatial agent sorts through the C ABI (fg_spatial_sort_agents)
    of the large workloads' populations: positions as in `build`, eight 4-byte
    columns in 3D (x, y, z, four payload words, an id), seven in 2D."""
    import ctypes as C
    import torch
    from flamegpu2_gb300 import capi, synth, workloads
    if dims == 3:
        pos = workloads.gaussian_mixture_3d(1 << 23, 256.0, 16, 2.0, 2)
        g = capi.grid(3, (0, 0, 0), (256, 256, 256), 1.0)
    else:
        n = 1 << 24
        hi = np.nextafter(np.float32(4096.0), np.float32(0))
        pos = np.stack([np.minimum(synth.uniform(3, a, n, 0.0, 4096.0), hi) for a in range(2)], 1)
        g = capi.grid(2, (0, 0), (4096, 4096), 4.0)
    n = pos.shape[0]
    if presorted:
        cell = [np.clip(np.floor((pos[:, a] - np.float32(g.min[a])) / np.float32(g.radius)).astype(np.int64), 0,
                        g.gridDim[a] - 1) for a in range(dims)]
        key = cell[0] + cell[1] * g.gridDim[0] + (cell[2] * g.gridDim[0] * g.gridDim[1] if dims == 3 else 0)
        pos = pos[np.argsort(key, kind="stable")]
    ins = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(dims)]
    ins += [torch.rand(n, device="cuda") for _ in range(4)]
    ins.append(torch.arange(1, n + 1, dtype=torch.int32, device="cuda"))
    outs = [torch.empty_like(c) for c in ins]
    colarr = capi.columns(list(zip(ins, outs)))
    perm = torch.empty(n, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(capi.lib().fg_spatial_sort_workspace_size(n, C.byref(g)))
    st = capi.stream_handle()
    args = (C.byref(g), n, None, ins[0].data_ptr(), ins[1].data_ptr(), ins[2].data_ptr() if dims == 3 else None,
            colarr, len(ins), perm.data_ptr(), ws.ptr, ws.nbytes, st)
    capi.check(capi.lib().fg_spatial_sort_agents(*args), "fg_spatial_sort_agents")
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        capi.check(capi.lib().fg_spatial_sort_agents(*args), "fg_spatial_sort_agents")
    b.record()
    b.synchronize()
    assert ws.status() == 0
    return {"dims": dims, "sorted_input": presorted, "agents": n, "columns": len(ins), "sort_us":
            round(a.elapsed_time(b) * 1000 / reps, 1)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["boids", "ensemble", "build", "payload", "sort"])
    ap.add_argument("--dims", type=int, default=3)
    ap.add_argument("--sorted", action="store_true")
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--count", type=int, default=32)
    a = ap.parse_args()
    if a.case == "boids":
        out = boids(a.n)
    elif a.case == "ensemble":
        out = ensemble(a.count)
    elif a.case == "payload":
        out = payload(a.dims, a.n)
    elif a.case == "sort":
        out = sort(a.dims, a.sorted)
    else:
        out = build(a.dims, a.sorted)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
