"""Device agent creation: the reference's DeviceAgentCreationTest known answers
(tests/test_cases/runtime/agent/test_device_agent_creation.cu:53-1338),
restated on the models of examples/agent_creation_tests/agent_creation.cu.

1024 agents with x = i + 1, id = i; a child has id = parent id + 1 and
x = child id + 12, so x - id tells parents (1) from children (12). Births go
to the function's own list (fused with its compaction) or to another state or
agent type (appended after that list's agents), with and without death and an
agent function condition (EvenThreadsOnlyCdn). Also: default values of
unset child variables, array variables, and unique ids across states and
agent types, including ids read on the device through agent_out.getID().
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1024


def _sim(model, params):
    from flamegpu2_gb300 import sim
    return sim.Simulation(model, params)


def _pop(n=N):
    return {"x": np.arange(1, n + 1, dtype=np.float32), "id": np.arange(n, dtype=np.uint32)}


def _summary(s, agent, state="default"):
    n = s.count(agent, state)
    x = s.get(agent, "x", np.float32, state=state) if n else np.zeros(0, np.float32)
    ids = s.get(agent, "id", np.uint32, state=state) if n else np.zeros(0, np.uint32)
    d = x - ids.astype(np.float32)
    p, c = ids[d == 1.0], ids[d == 12.0]
    return {"n": n, "is_1": int(p.size), "is_12": int(c.size), "other": int(n - p.size - c.size),
            "is_1_mod2": (int((p % 2 == 0).sum()), int((p % 2 == 1).sum())),
            "is_12_mod2": (int((c % 2 == 0).sum()), int((c % 2 == 1).sum())),
            "is_12_mod4": tuple(int((c % 4 == k).sum()) for k in range(4))}


def _run(kind, layout, cond, runner="agent", state="default"):
    s = _sim("dac", [kind, layout, cond])
    s.set_population(runner, N, _pop(), state=state)
    s.step(1)
    return s


def _check(got, **want):
    for k, v in want.items():
        assert got[k] == v, (k, got)


# kind: 0 Mandatory, 1 Optional, 2 MandatoryWithDeath, 3 OptionalWithDeath


def test_mandatory_output_same_state():  # :53-92
    s = _run(0, 0, 0)
    _check(_summary(s, "agent"), n=2 * N, is_1=N, is_12=N)


def test_optional_output_same_state():  # :93-132
    s = _run(1, 0, 0)
    _check(_summary(s, "agent"), n=N * 3 // 2, is_1=N, is_12=N // 2)


def test_mandatory_output_different_state():  # :133-174
    s = _run(0, 1, 0, state="a")
    _check(_summary(s, "agent", "a"), n=N, is_1=N)
    _check(_summary(s, "agent", "b"), n=N, is_12=N)


def test_optional_output_different_state():  # :175-216
    s = _run(1, 1, 0, state="a")
    _check(_summary(s, "agent", "a"), n=N, is_1=N)
    _check(_summary(s, "agent", "b"), n=N // 2, is_12=N // 2)


def test_mandatory_output_same_state_with_death():  # :217-257
    s = _run(2, 0, 0)
    _check(_summary(s, "agent"), n=N, is_1=0, is_12=N)


def test_optional_output_same_state_with_death():  # :258-298
    s = _run(3, 0, 0)
    _check(_summary(s, "agent"), n=N, is_1=N // 2, is_12=N // 2)


def test_mandatory_output_different_state_with_death():  # :299-338
    s = _run(2, 1, 0, state="a")
    _check(_summary(s, "agent", "a"), n=0)
    _check(_summary(s, "agent", "b"), n=N, is_12=N)


def test_optional_output_different_state_with_death():  # :339-382
    s = _run(3, 1, 0, state="a")
    _check(_summary(s, "agent", "a"), n=N // 2, is_1=N // 2)
    _check(_summary(s, "agent", "b"), n=N // 2, is_12=N // 2)


def test_mandatory_output_different_agent():  # :383-442
    s = _run(0, 4, 0, runner="agent2")
    _check(_summary(s, "agent2"), n=N, is_1=N, is_1_mod2=(N // 2, N // 2))
    _check(_summary(s, "agent", "b"), n=N, is_12=N, is_12_mod2=(N // 2, N // 2))


def test_optional_output_different_agent():  # :443-494
    s = _run(1, 4, 0, runner="agent2")
    _check(_summary(s, "agent2"), n=N, is_1=N, is_1_mod2=(N // 2, N // 2))
    _check(_summary(s, "agent", "b"), n=N // 2, is_12=N // 2, is_12_mod2=(0, N // 2))


def test_mandatory_output_different_agent_with_death():  # :495-556
    s = _run(2, 4, 0, runner="agent2")
    _check(_summary(s, "agent2"), n=0)
    _check(_summary(s, "agent", "b"), n=N, is_1=0, is_12=N, is_12_mod2=(N // 2, N // 2))


def test_optional_output_different_agent_with_death():  # :557-603
    s = _run(3, 4, 0, runner="agent2")
    _check(_summary(s, "agent2"), n=N // 2, is_1=N // 2, is_1_mod2=(N // 2, 0))
    _check(_summary(s, "agent", "b"), n=N // 2, is_12=N // 2, is_12_mod2=(0, N // 2))


def test_default_variable_value():  # :604-653
    s = _run(0, 5, 0, runner="agent2")
    n = s.count("agent")
    assert n == N
    default = s.get("agent", "default", np.float32)
    ids = s.get("agent", "id", np.uint32)
    is15 = default == 15.0
    assert int(is15.sum()) == N
    assert int((ids[is15] % 4 == 1).sum()) == N // 4
    assert int((ids[is15] % 4 == 3).sum()) == N // 4


def test_mandatory_output_same_state_with_condition():  # :657-720
    s = _run(0, 2, 1, state="a")
    a = _summary(s, "agent", "a")
    _check(a, n=N // 2, is_1=N // 2, is_1_mod2=(0, N // 2))
    _check(_summary(s, "agent", "b"), n=N, is_1=N // 2, is_12=N // 2, is_1_mod2=(N // 2, 0),
           is_12_mod4=(0, N // 4, 0, N // 4))


def test_optional_output_same_state_with_condition():  # :721-778
    s = _run(1, 2, 1, state="a")
    _check(_summary(s, "agent", "a"), n=N // 2, is_1=N // 2, is_1_mod2=(0, N // 2))
    _check(_summary(s, "agent", "b"), n=N // 2 + N // 4, is_12=N // 4, is_1=N // 2, is_1_mod2=(N // 2, 0),
           is_12_mod4=(0, N // 4, 0, 0))


def test_mandatory_output_different_state_with_condition():  # :779-839
    s = _run(0, 3, 1, state="a")
    _check(_summary(s, "agent", "a"), n=N // 2, is_1=N // 2, is_1_mod2=(0, N // 2))
    _check(_summary(s, "agent", "b"), n=N // 2, is_12=N // 2, is_12_mod4=(0, N // 4, 0, N // 4))
    _check(_summary(s, "agent", "c"), n=N // 2, is_1=N // 2, is_1_mod2=(N // 2, 0))


def test_optional_output_different_state_with_condition():  # :840-892
    s = _run(1, 3, 1, state="a")
    _check(_summary(s, "agent", "a"), n=N // 2, is_1=N // 2, is_1_mod2=(0, N // 2))
    _check(_summary(s, "agent", "b"), n=N // 4, is_12=N // 4, is_12_mod4=(0, N // 4, 0, 0))
    _check(_summary(s, "agent", "c"), n=N // 2, is_1=N // 2, is_1_mod2=(N // 2, 0))


def test_mandatory_output_same_state_with_death_with_condition():  # :893-945
    s = _run(2, 0, 1)
    _check(_summary(s, "agent"), n=N, is_1=N // 2, is_1_mod2=(0, N // 2), is_12=N // 2,
           is_12_mod4=(0, N // 4, 0, N // 4))


def test_optional_output_same_state_with_death_with_condition():  # :946-1002
    s = _run(3, 0, 1)
    _check(_summary(s, "agent"), n=N, is_1=N // 2 + N // 4, is_1_mod2=(N // 4, N // 2), is_12=N // 4,
           is_12_mod4=(0, N // 4, 0, 0))


def test_mandatory_output_different_state_with_death_with_condition():  # :1003-1048
    s = _run(2, 1, 1, state="a")
    _check(_summary(s, "agent", "a"), n=N // 2, is_1=N // 2, is_1_mod2=(0, N // 2))
    _check(_summary(s, "agent", "b"), n=N // 2, is_12=N // 2, is_12_mod2=(0, N // 2))


def test_optional_output_different_state_with_death_with_condition():  # :1049-1106
    s = _run(3, 1, 1, state="a")
    _check(_summary(s, "agent", "a"), n=N // 2 + N // 4, is_1=N // 2 + N // 4, is_1_mod2=(N // 4, N // 2))
    _check(_summary(s, "agent", "b"), n=N // 4, is_12=N // 4, is_12_mod4=(0, N // 4, 0, 0))


@pytest.mark.parametrize("default_works", [False, True])
def test_device_birth_array_variables(default_works):  # :1129-1194
    s = _sim("dac_array", [1.0 if default_works else 0.0])
    s.set_population("agent_name", N, {"id": np.arange(N, dtype=np.uint32)})
    s.step(1)
    assert s.count("agent_name") == N
    ids = s.get("agent_name", "id", np.uint32)
    arr = s.get("agent_name", "array_var", np.int32, elements=4)
    y = s.get("agent_name", "y", np.float32)
    assert np.all(ids % 3 == 0)
    ref = np.array([3, 5, 9, 17], np.int32)
    if default_works:
        np.testing.assert_array_equal(arr, np.tile(ref, (N, 1)))
        np.testing.assert_array_equal(y, np.full(N, 14.0, np.float32))
    else:
        np.testing.assert_array_equal(arr - ids[:, None].astype(np.int32), np.tile(ref, (N, 1)))
        np.testing.assert_array_equal(y, 14.0 + ids.astype(np.float32))


def test_agent_ids_unique_across_states():  # :1205-1296
    s = _sim("dac_ids", [0.0])
    for st in ("a", "b"):
        s.set_population("agent", 100, {"id_copy": np.zeros(100, np.uint32)}, state=st)
    s.step(1)
    rows = []
    for st in ("a", "b"):
        n = s.count("agent", st)
        assert n == 200
        rows.append({k: s.get("agent", k, np.uint32, state=st) for k in ("_id", "id_copy", "id_other")})
    ids = np.concatenate([r["_id"] for r in rows])
    copies = np.concatenate([r["id_copy"] for r in rows])
    other = np.concatenate([r["id_other"] for r in rows])
    assert len(set(ids.tolist())) == ids.size == 400
    np.testing.assert_array_equal(ids, copies)
    # parent / child pairs: each names the other (children's id_other is the
    # parent's id; parents' is the id agent_out.getID() returned)
    pair = {int(i): int(o) for i, o in zip(ids, other) if o != 0}
    assert len(pair) == 400
    for i, o in pair.items():
        assert pair[o] == i


def test_agent_ids_of_births_into_another_agent_type():  # :1297-1338
    s = _sim("dac_ids", [1.0])
    s.set_population("agentA", 100, {"id_other": np.zeros(100, np.uint32)})
    s.set_population("agentB", 200, {"id_other": np.zeros(200, np.uint32)})
    s.step(1)
    assert s.count("agentA") == 100
    assert s.count("agentB") == 300
    ids = s.get("agentB", "_id", np.uint32)
    assert len(set(ids.tolist())) == 300
    # each A holds its child's id, each child its parent's
    a_ids = s.get("agentA", "_id", np.uint32)
    a_other = s.get("agentA", "id_other", np.uint32)
    b_other = s.get("agentB", "id_other", np.uint32)
    child_of = dict(zip(a_ids.tolist(), a_other.tolist()))
    for cid, parent in zip(ids[200:].tolist(), b_other[200:].tolist()):
        assert child_of[parent] == cid


def test_births_across_lists_over_many_steps_grow_capacity():
    # agent2 (1024) gives birth into agent state b every step, for 40 steps:
    # the output list grows past its first allocation while steps are replayed
    # in multi-step graphs; every child is kept, in parent order per step
    s = _run(0, 4, 0, runner="agent2")
    s.step(39)
    b = _summary(s, "agent", "b")
    assert b["n"] == 40 * N and b["is_12"] == 40 * N
    ids = s.get("agent", "_id", np.uint32, state="b")
    np.testing.assert_array_equal(ids, np.arange(1, 40 * N + 1, dtype=np.uint32))
    child = s.get("agent", "id", np.uint32, state="b")
    np.testing.assert_array_equal(child, np.tile(np.arange(1, N + 1, dtype=np.uint32), 40))


@pytest.mark.parametrize("graphs", [True, False])
def test_cross_agent_births_match_oracle(graphs):
    # births into another agent type (with death; from a function with a
    # condition and a state transition), order and ids exact against the
    # oracle over 12 steps
    import oracle as O
    from flamegpu2_gb300 import sim
    n = 3000
    rng = np.random.default_rng(4)
    prey = {"_id": np.arange(1, n + 1, dtype=np.uint32), "v": rng.integers(0, 100, n).astype(np.uint32),
            "x": rng.uniform(0, 50, n).astype(np.float32)}
    s = sim.Simulation("cross_birth", [])
    s.configure(steps=1, seed=0, use_graphs=graphs)
    s.set_population("prey", n, prey)
    s.step(12)
    empty = {"_id": np.zeros(0, np.uint32), "v": np.zeros(0, np.uint32), "x": np.zeros(0, np.float32)}
    exp, _ = O.cross_birth_run({("prey", "default"): prey, ("hunter", "roam"): empty, ("hunter", "rest"): empty},
                               {"prey": n + 1, "hunter": 1}, 12)
    for (agent, state), want in exp.items():
        assert s.count(agent, state) == len(want["_id"]), (agent, state)
        for k, dt in (("_id", np.uint32), ("v", np.uint32), ("x", np.float32)):
            np.testing.assert_array_equal(s.get(agent, k, dt, state=state), want[k], err_msg=f"{agent}/{state}/{k}")
    assert len(exp[("hunter", "roam")]["_id"]) > 1000 and len(exp[("prey", "default")]["_id"]) > n
