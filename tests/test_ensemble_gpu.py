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


BD_NAMES = ("_id", "counter") + tuple(f"f{v}" for v in range(8))


def _bd_runs(params, steps, batched):
    """Birth/death ensemble: params = [(n, p_death, p_birth, seed)], steps per run."""
    import ctypes as C
    from flamegpu2_gb300 import sim, synth
    ens = sim.Ensemble("birth_death", [0.3, 0.2, 1.0], batched=batched)
    pops = []
    for (n, pd, pb, seed), st in zip(params, steps):
        pop = synth.birth_death_population(n, seed)
        pops.append(pop)
        r = ens.add_run(st, seed, "agent", n, pop)
        ens.set_property(r, "P_DEATH", pd)
        ens.set_property(r, "P_BIRTH", pb)
        ens.set_property(r, "SEED", seed, C.c_uint64)
    assert ens.simulate() == 0
    out = [{k: ens.get(i, "agent", k, np.uint32 if k == "_id" else (np.int32 if k == "counter" else np.float32))
            for k in BD_NAMES} for i in range(len(params))]
    st = ens.stats()
    ens.close()
    return pops, out, st


@pytest.mark.parametrize("graphs", [True])
def test_batched_birth_death_equals_plain_runs_and_oracle(graphs):
    # births and deaths inside one batched simulation (segmented compaction
    # over every run's rows): each run equals its own plain run and the oracle,
    # order and ids included. Growing runs (low death, high birth) outgrow
    # their row segments several times, shrinking ones empty out.
    import oracle as O
    from flamegpu2_gb300 import sim
    params = [(0, 0.3, 0.2, 3), (1, 0.0, 1.0, 4), (100, 0.3, 0.2, 5), (3000, 0.05, 0.6, 6), (20_000, 0.3, 0.2, 7),
              (5000, 0.9, 0.1, 8), (777, 0.1, 0.5, 9), (40_000, 0.2, 0.3, 10)]
    steps = [10, 12, 12, 12, 7, 12, 12, 9]
    pops, out, st = _bd_runs(params, steps, batched=True)
    assert st["batched"]
    for (n, pd, pb, seed), stp, pop, got in zip(params, steps, pops, out):
        s = sim.Simulation("birth_death", [pd, pb, seed])
        s.set_population("agent", n, pop)
        s.step(stp)
        for k in BD_NAMES:
            dt = np.uint32 if k == "_id" else (np.int32 if k == "counter" else np.float32)
            np.testing.assert_array_equal(got[k], s.get("agent", k, dt), err_msg=f"run n={n} seed={seed} {k}")
        s.close()
        f = np.stack([pop[f"f{v}"] for v in range(8)]) if n else np.zeros((8, 0), np.float32)
        cap = max(4 * n, 1024) * 64
        fo, co, io, _, _ = O.birth_death_run(f, pop["counter"], pop["_id"], n + 1, cap, pd, pb, seed, stp)
        np.testing.assert_array_equal(got["_id"], io)
        np.testing.assert_array_equal(got["counter"], co)
        for v in range(8):
            np.testing.assert_array_equal(got[f"f{v}"], fo[v])
    assert len(out[3]["_id"]) > 3000 * 10  # a run that grew well past its first segment


def test_autotuned_ensemble_same_results_and_cache(tmp_path):
    # the autotuner times launch-shape candidates on the batch itself, keeps the
    # fastest and stores it per GPU / model / size class; the results do not
    # depend on the shape (bit-exact against the untuned run), and a second
    # ensemble of the same size class reads the shape back from the cache
    import json
    from flamegpu2_gb300 import sim, synth
    specs = synth.ensemble_instances(10, seed=300, n_lo=500, n_hi=20000)
    cache = str(tmp_path / "shapes.json")

    def run(tuning):
        ens = sim.Ensemble("boids_spatial3d", synth.boids_params(dict(synth.BOIDS_SMALL)), tuning=tuning,
                           tuning_cache=cache)
        for sp in specs:
            pop = synth.boids_population(sp["n"], 0.0, sp["edge"], sp["seed"])
            r = ens.add_run(4, sp["seed"], "Boid", sp["n"], pop, "location", (0.0, 0.0, 0.0), (sp["edge"],) * 3,
                            sp["radius"])
            ens.set_property(r, "MIN_POSITION", 0.0)
            ens.set_property(r, "MAX_POSITION", sp["edge"])
            ens.set_property(r, "INTERACTION_RADIUS", sp["radius"])
        assert ens.simulate() == 0
        out = [{k: ens.get(i, "Boid", k, np.uint32 if k == "_id" else np.float32) for k in BOIDS_NAMES}
               for i in range(len(specs))]
        t = ens.tuning()
        ens.close()
        return out, t

    base, t0 = run("off")
    assert not t0["tuned"]
    tuned, t1 = run("measure")
    assert t1["tuned"] and t1["source"] == "measured"
    assert t1["shape"]["block"] in (64, 128) and t1["step_ms"] <= t1["default_step_ms"]
    for a, b in zip(base, tuned):
        for k in BOIDS_NAMES:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    doc = json.load(open(cache))
    assert t1["key"] in doc["entries"]
    again, t2 = run("cache")
    assert t2["tuned"] and t2["source"] == "cache" and t2["shape"] == t1["shape"]
    for a, b in zip(base, again):
        for k in BOIDS_NAMES:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
