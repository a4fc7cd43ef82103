"""JSON state files (the reference's JSONStateWriter / JSONStateReader layout):
a run exported part-way and loaded into a new simulation continues exactly as
the uninterrupted run, ids, environment and step counter included."""
import json

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim():
    from flamegpu2_gb300 import sim
    return sim


BOIDS_VARS = ("_id", "x", "y", "z", "fx", "fy", "fz")


def test_boids_export_load_continues_exactly(tmp_path):
    from flamegpu2_gb300 import synth
    S = _sim()
    cfg = dict(synth.BOIDS_SMALL)
    params = synth.boids_params(cfg)
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], 11)
    a = S.Simulation("boids_spatial3d", params)
    a.set_population("Boid", cfg["n"], pop)
    a.step(10)
    whole = {k: a.get("Boid", k, np.uint32 if k == "_id" else np.float32) for k in BOIDS_VARS}
    a.close()
    b = S.Simulation("boids_spatial3d", params)
    b.set_population("Boid", cfg["n"], pop)
    b.step(5)
    path = tmp_path / "boids.json"
    b.export_data(path)
    b.close()
    doc = json.load(open(path))
    assert doc["stats"]["step_count"] == 5
    assert len(doc["agents"]["Boid"]["default"]) == cfg["n"]
    assert set(doc["agents"]["Boid"]["default"][0]) == set(BOIDS_VARS)
    assert doc["environment"]["INTERACTION_RADIUS"] == pytest.approx(cfg["interaction_radius"])
    c = S.Simulation("boids_spatial3d", params)
    c.load_state(path)
    c.step(5)
    resumed = {k: c.get("Boid", k, np.uint32 if k == "_id" else np.float32) for k in BOIDS_VARS}
    c.close()
    for k in BOIDS_VARS:
        np.testing.assert_array_equal(resumed[k], whole[k], err_msg=k)


def test_birth_death_resume_keeps_ids_and_step_counter(tmp_path):
    # the hash RNG is keyed by (seed, id, step): resuming needs the step counter,
    # the ids and the next id back
    from flamegpu2_gb300 import synth
    S = _sim()
    n = 20_000
    pop = synth.birth_death_population(n, 2)
    names = ["_id", "counter"] + [f"f{v}" for v in range(8)]
    dt = {k: np.uint32 if k == "_id" else (np.int32 if k == "counter" else np.float32) for k in names}
    a = S.Simulation("birth_death", [0.30, 0.20, 2])
    a.set_population("agent", n, pop)
    a.step(6)
    whole = {k: a.get("agent", k, dt[k]) for k in names}
    a.close()
    b = S.Simulation("birth_death", [0.30, 0.20, 2])
    b.set_population("agent", n, pop)
    b.step(3)
    path = tmp_path / "bd.json"
    b.export_data(path)
    b.close()
    c = S.Simulation("birth_death", [0.30, 0.20, 2])
    c.load_state(path)
    c.step(3)
    resumed = {k: c.get("agent", k, dt[k]) for k in names}
    c.close()
    for k in names:
        np.testing.assert_array_equal(resumed[k], whole[k], err_msg=k)


def test_state_file_with_two_states_and_array_variables(tmp_path):
    S = _sim()
    n = 300
    s = S.Simulation("condition_split", [])
    x = (np.arange(n) % 2).astype(np.int32)
    y = np.tile(np.array([13, 14, 15, 16], np.int32), (n, 1))
    s.set_population("Agent", n, {"x": x, "y": y}, state="Start")
    s.step(1)
    path = tmp_path / "split.json"
    s.export_data(path)
    e1 = s.get("Agent", "y", np.int32, elements=4, state="End")
    s.close()
    doc = json.load(open(path))
    assert set(doc["agents"]["Agent"]) == {"End", "End2"}  # empty lists are not written
    assert doc["agents"]["Agent"]["End"][0]["y"] == [3, 4, 5, 6]
    t = S.Simulation("condition_split", [])
    t.load_state(path)
    assert t.count("Agent", "End") == n // 2 and t.count("Agent", "Start") == 0
    np.testing.assert_array_equal(t.get("Agent", "y", np.int32, elements=4, state="End"), e1)
    t.close()
