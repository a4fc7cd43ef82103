"""One small Boids run on cuda:0 through the C ABI, checked against the oracle
(used by __graft_entry__.smoke())."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def run_smoke():
    import oracle as O
    from flamegpu2_gb300 import sim, synth
    cfg = dict(synth.BOIDS_SMALL, n=2048, max_pos=32.0)
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], cfg["seed"])
    s = sim.Simulation("boids_spatial3d", synth.boids_params(cfg))
    s.set_population("Boid", cfg["n"], pop)
    s.step(3)
    got = {k: s.get("Boid", k, np.float32) for k in ("x", "y", "z")}
    ids = s.get("Boid", "_id", np.uint32)
    s.close()
    p = O.boids_params(cfg["min_pos"], cfg["max_pos"], cfg["interaction_radius"], cfg["separation_radius"],
                       cfg["time_scale"], cfg["global_scale"], cfg["steer_scale"], cfg["collision_scale"],
                       cfg["match_scale"], cfg["wrap"], cfg["sort_period"])
    ref = O.boids_run(p, {"id": pop["_id"], **{k: pop[k] for k in ("x", "y", "z", "fx", "fy", "fz")}}, 3)
    assert np.array_equal(ids, ref["id"]), "agent order differs from the oracle"
    for k in ("x", "y", "z"):
        err = float(np.abs(got[k] - ref[k]).max())
        assert err <= 1e-4, f"{k} differs from the oracle by {err}"
    print("smoke ok: 2048 Boids x 3 steps match the oracle")


if __name__ == "__main__":
    run_smoke()
