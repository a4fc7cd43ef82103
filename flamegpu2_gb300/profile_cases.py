"""Small, fixed cases for profiling single kernels (ncu) and per-operation
timings, outside the benchmark's timed loop.

  python -m flamegpu2_gb300.profile_cases boids --n 1048576
      Boids (wrapped, radius 2) at about one agent per bin: edge =
      4 r cbrt(N/64), the density of the batched-ensemble instances;
      prints per-operation timings (CUDA events, eager) and graph step time.
  python -m flamegpu2_gb300.profile_cases ensemble --count 32
      The first `count` instances of the 256-instance Boids ensemble, 5 steps,
      as one batched simulation.
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
    t = time.perf_counter()
    s.step(steps)
    s.synchronize()
    el = time.perf_counter() - t
    s.close()
    return {"n": n, "edge": edge, "ms_per_step_graph": round(el / steps * 1000, 4),
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["boids", "ensemble"])
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--count", type=int, default=32)
    a = ap.parse_args()
    out = boids(a.n) if a.case == "boids" else ensemble(a.count)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
