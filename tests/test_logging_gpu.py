"""Step and exit logs (the reference's LoggingConfig / StepLoggingConfig /
RunLog, CUDASimulation.cu:1949-2022): frames at step 0 and every `frequency`
steps of simulate(), agent counts, environment properties and device
reductions of agent variables, checked against the populations read back."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def test_step_and_exit_logs_of_birth_death():
    from flamegpu2_gb300 import synth
    S = _sim()
    n, steps = 50_000, 9
    pop = synth.birth_death_population(n, 4)
    s = S.Simulation("birth_death", [0.30, 0.20, 4], steps=steps)
    s.configure(steps=steps, seed=0)
    s.set_population("agent", n, pop)
    s.set_step_log(["count:agent:default", "env:P_DEATH", "sum:agent:default:counter"], frequency=3)
    s.set_exit_log(["count:agent:default", "mean:agent:default:f0", "sd:agent:default:f0",
                    "min:agent:default:f3", "max:agent:default:f3", "sum:agent:default:f1",
                    "min:agent:default:counter", "max:agent:default:counter", "sum:agent:default:_id"])
    s.simulate()
    log = s.run_log()
    f = {k: s.get("agent", k, np.float32) for k in ("f0", "f1", "f3")}
    counter = s.get("agent", "counter", np.int32)
    ids = s.get("agent", "_id", np.uint32)
    s.close()
    # frames before the first step and after every third
    assert [fr["step_index"] for fr in log["steps"]] == [0, 3, 6, 9]
    assert log["steps"][0]["agents"]["agent"]["default"][0]["count"] == n
    assert abs(log["steps"][0]["env"]["P_DEATH"] - 0.30) < 1e-7
    ex = log["exit"]
    assert ex["step_index"] == steps
    a = ex["agents"]["agent"]["default"][0]
    m = len(ids)
    assert a["count"] == m == log["steps"][-1]["agents"]["agent"]["default"][0]["count"]
    v = a["variables"]
    f0 = f["f0"].astype(np.float64)
    assert v["f0"]["mean"] == pytest.approx(f0.mean(), rel=1e-12)
    assert v["f0"]["standard_deviation"] == pytest.approx(f0.std(), rel=1e-9)
    # float reductions are logged as floats (9 significant digits: the same float back)
    assert np.float32(v["f3"]["min"]) == f["f3"].min() and np.float32(v["f3"]["max"]) == f["f3"].max()
    assert v["f1"]["sum"] == pytest.approx(f["f1"].astype(np.float64).sum(), rel=1e-12)
    assert v["counter"]["min"] == int(counter.min()) and v["counter"]["max"] == int(counter.max())
    assert v["_id"]["sum"] == int(ids.astype(np.uint64).sum())
    # step frames: the logged counter sums are those of the populations then
    assert log["steps"][-1]["agents"]["agent"]["default"][0]["variables"]["counter"]["sum"] == int(counter.sum())


def test_logs_are_deterministic():
    from flamegpu2_gb300 import synth
    S = _sim()
    outs = []
    for _ in range(2):
        cfg = dict(synth.BOIDS_SMALL)
        s = S.Simulation("boids_spatial3d", synth.boids_params(cfg))
        s.configure(steps=4, seed=0)
        s.set_population("Boid", cfg["n"], synth.boids_population(cfg["n"], 0.0, 64.0, 1))
        s.set_step_log(["mean:Boid:default:fx", "sd:Boid:default:x", "sum:Boid:default:y"], frequency=1)
        s.simulate()
        outs.append(s.run_log()["steps"])
        s.close()
    strip = lambda frames: [{k: v for k, v in fr.items() if k != "step_time"} for fr in frames]
    assert strip(outs[0]) == strip(outs[1])


def test_run_log_layout_matches_the_reference_logger():
    # JSONLogger (src/flamegpu/io/JSONLogger.cu:80-200): top-level config,
    # performance_specs (with the times), steps, exit; a step frame's
    # step_time before step_index, env, agents; the exit frame's rtc_time,
    # init_time, exit_time, total_time first; agents -> agent -> state -> a
    # list of {count, variables -> variable -> reduction -> value}
    import json
    from flamegpu2_gb300 import synth
    S = _sim()
    pop = synth.birth_death_population(5000, 2)
    s = S.Simulation("birth_death", [0.30, 0.20, 2], steps=4)
    s.configure(steps=4, seed=7)
    s.set_population("agent", 5000, pop)
    s.set_step_log(["count:agent:default", "env:P_DEATH", "sum:agent:default:counter", "mean:agent:default:f0"],
                   frequency=2)
    s.set_exit_log(["count:agent:default", "max:agent:default:f3", "min:agent:default:f3"])
    s.simulate()
    log = s.run_log()
    s.close()
    assert list(log) == ["config", "performance_specs", "steps", "exit"]
    assert log["config"] == {"random_seed": 7}
    assert list(log["performance_specs"]) == ["device_name", "device_cc_major", "device_cc_minor", "cuda_version",
                                              "seatbelts", "flamegpu_version"]
    for fr in log["steps"]:
        assert list(fr) == ["step_time", "step_index", "env", "agents"]
        assert list(fr["agents"]) == ["agent"] and list(fr["agents"]["agent"]) == ["default"]
        entry = fr["agents"]["agent"]["default"]
        assert isinstance(entry, list) and len(entry) == 1
        assert list(entry[0]) == ["count", "variables"]
        assert list(entry[0]["variables"]) == ["counter", "f0"]  # std::map order of (name, reduction)
        assert list(entry[0]["variables"]["counter"]) == ["sum"]
        assert list(entry[0]["variables"]["f0"]) == ["mean"]
    ex = log["exit"]
    assert list(ex) == ["rtc_time", "init_time", "exit_time", "total_time", "step_index", "agents"]
    assert list(ex["agents"]["agent"]["default"][0]["variables"]["f3"]) == ["min", "max"]  # Reduction enum order
    json.dumps(log)  # plain JSON throughout
