"""Batched ensembles: every instance of one batched simulation (segmented
sort, build and iterate over concatenated buffers) must equal its own plain
single-instance CUDASimulation run, and the sequential fallback must agree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BOIDS_NAMES = ("_id", "x", "y", "z", "fx", "fy", "fz")


def _run_specs(specs, steps, batched=True, stage=96 * 1024):
    from flamegpu2_gb300 import sim, synth
    ens = sim.Ensemble("boids_spatial3d", synth.boids_params(dict(synth.BOIDS_SMALL)), batched=batched, stage_bytes=stage)
    pops = []
    for k, sp in enumerate(specs):
        pop = synth.boids_population(sp["n"], 0.0, sp["edge"], sp["seed"])
        pops.append(pop)
        run = ens.add_run(steps[k] if isinstance(steps, list) else steps, sp["seed"], "Boid", sp["n"], pop,
                          "location", (0.0, 0.0, 0.0), (sp["edge"],) * 3, sp["radius"])
        ens.set_property(run, "MIN_POSITION", 0.0)
        ens.set_property(run, "MAX_POSITION", sp["edge"])
        ens.set_property(run, "INTERACTION_RADIUS", sp["radius"])
    assert ens.simulate() == 0
    st = ens.stats()
    out = [{k: ens.get(i, "Boid", k, np.uint32 if k == "_id" else np.float32) for k in BOIDS_NAMES}
           for i in range(len(specs))]
    ens.close()
    return pops, out, st


def _plain(sp, pop, steps):
    from flamegpu2_gb300 import sim, synth
    cfg = dict(synth.BOIDS_SMALL, n=sp["n"], max_pos=sp["edge"], interaction_radius=sp["radius"])
    s = sim.Simulation("boids_spatial3d", synth.boids_params(cfg))
    s.set_population("Boid", sp["n"], pop)
    s.step(steps)
    out = {k: s.get("Boid", k, np.uint32 if k == "_id" else np.float32) for k in BOIDS_NAMES}
    s.close()
    return out


def test_batched_ensemble_equals_plain_runs():
    from flamegpu2_gb300 import synth
    specs = synth.ensemble_instances(12, seed=1000, n_lo=100, n_hi=40000)
    pops, out, st = _run_specs(specs, 6)
    assert st["batched"] and st["graph_launches"] == 6
    for sp, pop, got in zip(specs, pops, out):
        ref = _plain(sp, pop, 6)
        for k in BOIDS_NAMES:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"instance n={sp['n']} r={sp['radius']:.3f} {k}")


def test_batched_ensemble_per_run_steps_and_sequential_fallback():
    from flamegpu2_gb300 import synth
    specs = synth.ensemble_instances(5, seed=77, n_lo=500, n_hi=5000)
    steps = [3, 1, 4, 4, 2]
    pops, out_b, st_b = _run_specs(specs, steps, batched=True)
    _, out_s, st_s = _run_specs(specs, steps, batched=False)
    assert st_b["batched"] and not st_s["batched"]
    for k in range(len(specs)):
        ref = _plain(specs[k], pops[k], steps[k])
        for v in BOIDS_NAMES:
            np.testing.assert_array_equal(out_b[k][v], ref[v])
            np.testing.assert_array_equal(out_s[k][v], ref[v])


def test_batched_ensemble_matches_oracle():
    import oracle as O
    from flamegpu2_gb300 import synth
    specs = synth.ensemble_instances(4, seed=5, n_lo=300, n_hi=3000)
    pops, out, _ = _run_specs(specs, 5)
    for sp, pop, got in zip(specs, pops, out):
        p = O.boids_params(0.0, sp["edge"], sp["radius"], 0.5, 0.05, 0.15, 0.005, 0.01, 0.03, 1, 1)
        ref = O.boids_run(p, {"id": pop["_id"], **{k: pop[k] for k in ("x", "y", "z", "fx", "fy", "fz")}}, 5)
        np.testing.assert_array_equal(got["_id"], ref["id"])
        for k in ("x", "y", "z", "fx", "fy", "fz"):
            np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
