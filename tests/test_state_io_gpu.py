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


# ------------------------------------------------ the reference's IO tests
# tests/test_cases/io/test_io.cu: MiniSim (JSON_WriteRead) and IOTest2.

SCALARS = [("float", np.float32), ("double", np.float64), ("int64_t", np.int64), ("uint64_t", np.uint64),
           ("int32_t", np.int32), ("uint32_t", np.uint32), ("int16_t", np.int16), ("uint16_t", np.uint16),
           ("int8_t", np.int8), ("uint8_t", np.uint8)]
LIMITS = [("float_qnan", np.float32), ("float_snan", np.float32), ("float_inf", np.float32),
          ("float_inf_neg", np.float32), ("double_qnan", np.float64), ("double_snan", np.float64),
          ("double_inf", np.float64), ("double_inf_neg", np.float64)]
CTYPES = {np.float32: "c_float", np.float64: "c_double", np.int64: "c_int64", np.uint64: "c_uint64",
          np.int32: "c_int32", np.uint32: "c_uint32", np.int16: "c_int16", np.uint16: "c_uint16",
          np.int8: "c_int8", np.uint8: "c_uint8"}
SIM_CONFIG = [("input_file", "invalid"), ("step_log_file", "step"), ("exit_log_file", "exit"),
              ("common_log_file", "common"), ("truncate_log_files", "false"), ("random_seed", "654321"),
              ("steps", "123"), ("verbosity", "0"), ("timing", "true")]


def _io_populations():
    # MiniSim: pop_a_out (5 agents of "a") and pop_b_out (5 of "b", in state "2")
    i = np.arange(5)
    a = {k: (1 + j + i).astype(dt) for j, (k, dt) in enumerate(SCALARS)}
    a["float_qnan"] = np.full(5, np.nan, np.float32)
    a["float_snan"] = np.full(5, np.nan, np.float32)
    a["float_inf"] = np.full(5, np.inf, np.float32)
    a["float_inf_neg"] = np.full(5, -np.inf, np.float32)
    a["double_qnan"] = np.full(5, np.nan, np.float64)
    a["double_snan"] = np.full(5, np.nan, np.float64)
    a["double_inf"] = np.full(5, np.inf, np.float64)
    a["double_inf_neg"] = np.full(5, -np.inf, np.float64)
    b = {k: np.stack([np.full(5, 1 + j), i, np.ones(5)], 1).astype(dt) for j, (k, dt) in enumerate(SCALARS)}
    return a, b


def _io_export(path):
    S = _sim()
    s = S.Simulation("io_types", [])
    a, b = _io_populations()
    s.set_population("a", 5, a)
    s.set_population("b", 5, b, state="2")  # the agents in the non-initial state
    for k, v in SIM_CONFIG:
        s.set_config(k, v)
    s.set_config("device_id", 0)
    s.set_config("inLayerConcurrency", False)
    s.export_data(str(path))
    s.close()
    return a, b


def test_state_file_layout_matches_the_reference_writer(tmp_path):
    # the layout src/flamegpu/io/JSONStateWriter.cu writes: config (simulation
    # items in writeConfig's order, cuda), stats, environment (every property;
    # NaN and infinities as null), agents by name, each state with agents
    # (empty ones omitted) as a list of objects keyed by variable name in
    # std::map order, arrays as lists
    path = tmp_path / "io.json"
    _io_export(path)
    doc = json.loads(path.read_text(), object_pairs_hook=lambda kv: kv)
    assert [k for k, _ in doc] == ["config", "stats", "environment", "agents"]
    d = dict(doc)
    cfg = dict(d["config"])
    assert [k for k, _ in cfg["simulation"]] == [k for k, _ in SIM_CONFIG]
    sim_cfg = dict(cfg["simulation"])
    assert sim_cfg["input_file"] == "invalid" and sim_cfg["step_log_file"] == "step"
    assert sim_cfg["exit_log_file"] == "exit" and sim_cfg["common_log_file"] == "common"
    assert sim_cfg["truncate_log_files"] is False and sim_cfg["random_seed"] == 654321
    assert sim_cfg["steps"] == 123 and sim_cfg["verbosity"] == 0 and sim_cfg["timing"] is True
    assert cfg["cuda"] == [("device_id", 0), ("inLayerConcurrency", False)]
    assert dict(d["stats"])["step_count"] == 0
    # the extension keys are plain numbers, which the reference's reader skips
    assert all(k == "step_count" or (k.startswith("next_id:") and isinstance(v, int)) for k, v in d["stats"])
    env = dict(d["environment"])
    for j, (k, dt) in enumerate(SCALARS):
        assert env[k] == 12 + j
        assert env[k + "_a"] == [12 + j, 0, 1]
    for k, _ in LIMITS:
        assert env[k] is None  # JSON has no NaN or infinity
    agents = d["agents"]
    assert [k for k, _ in agents] == ["a", "b"]
    ag = dict(agents)
    assert [k for k, _ in ag["a"]] == ["default"]
    assert [k for k, _ in ag["b"]] == ["2"]  # state "1" holds no agents
    rows_a = dict(ag["a"])["default"]
    assert len(rows_a) == 5
    names_a = sorted(["_id"] + [k for k, _ in SCALARS] + [k for k, _ in LIMITS])  # std::map order
    for i, row in enumerate(rows_a):
        assert [k for k, _ in row] == names_a
        r = dict(row)
        for j, (k, dt) in enumerate(SCALARS):
            assert r[k] == 1 + j + i
        for k, _ in LIMITS:
            assert r[k] is None
    for i, row in enumerate(dict(ag["b"])["2"]):
        r = dict(row)
        assert [k for k, _ in row] == sorted(["_id"] + [k for k, _ in SCALARS])
        for j, (k, dt) in enumerate(SCALARS):
            assert r[k] == [1 + j, i, 1]


def test_json_write_read(tmp_path):
    # MiniSim::run (test_io.cu:255-560): export with one configuration, import
    # into a simulation configured otherwise; configuration, populations and
    # environment come back (NaN and infinities as NaN: JSON has neither)
    import ctypes as C
    S = _sim()
    path = tmp_path / "io.json"
    a, b = _io_export(path)
    s = S.Simulation("io_types", [])
    for k, v in [("step_log_file", ""), ("exit_log_file", ""), ("common_log_file", ""), ("truncate_log_files", True),
                 ("random_seed", 0), ("steps", 0), ("verbosity", 2), ("timing", False)]:
        s.set_config(k, v)
    s.load_state(str(path))
    for k, v in SIM_CONFIG[1:]:
        assert s.get_config(k) == v, k
    assert s.count("a") == 5 and s.count("b", "2") == 5 and s.count("b", "1") == 0
    for k, dt in SCALARS:
        np.testing.assert_array_equal(s.get("a", k, dt), a[k])
        np.testing.assert_array_equal(s.get("b", k, dt, elements=3, state="2"), b[k])
    for k, dt in LIMITS:
        assert np.all(np.isnan(s.get("a", k, dt)))
    for j, (k, dt) in enumerate(SCALARS):
        assert s.get_env(k, getattr(C, CTYPES[dt])) == 12 + j
    for k, dt in LIMITS:
        assert np.isnan(s.get_env(k, getattr(C, CTYPES[dt])))
    s.step(1)  # the loaded simulation runs
    s.close()


def test_agent_ids_export_import(tmp_path):
    # IOTest2.AgentID_JSON_ExportImport (test_io.cu:622-665)
    S = _sim()
    path = tmp_path / "ids.json"
    s = S.Simulation("io_agentid", [])
    s.set_population("agent", 100, {"id_other": np.zeros(100, np.uint32)})
    s.step(1)
    ids = s.get("agent", "_id", np.uint32)
    assert np.all(ids != 0) and len(set(ids.tolist())) == 100
    s.export_data(str(path))
    s.close()
    t = S.Simulation("io_agentid", [])
    t.load_state(str(path))
    np.testing.assert_array_equal(t.get("agent", "_id", np.uint32), ids)
    t.close()


def test_agent_id_collision_in_a_state_file(tmp_path):
    # IOTest2.AgentID_FileInput_IDCollision (test_io.cu:712-735): ids 1, 2, 1
    S = _sim()
    path = tmp_path / "collide.json"
    path.write_text('{"agents":{"agent":{"default":[{"_id":1,"id_other":0},{"_id":2,"id_other":0},'
                    '{"_id":1,"id_other":0}]}}}')
    s = S.Simulation("io_agentid", [])
    with pytest.raises(S.SimError, match="AgentIDCollision"):
        s.load_state(str(path))
    s.close()


def test_unknown_config_items_are_rejected(tmp_path):
    # JSONStateReader.cu:406,414: unknown simulation / CUDA config items are errors
    S = _sim()
    for body in ('{"config":{"simulation":{"not_an_item":1}}}', '{"config":{"cuda":{"not_an_item":1}}}'):
        path = tmp_path / "bad.json"
        path.write_text(body)
        s = S.Simulation("io_agentid", [])
        with pytest.raises(S.SimError, match="JSONError"):
            s.load_state(str(path))
        s.close()
