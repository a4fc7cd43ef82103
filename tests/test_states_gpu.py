"""Agent function conditions and state transitions: the reference's own
known answers (SplitAgents, AllDisabled, transition chains), and an
order-exact comparison with the oracle of a model that combines conditions,
death, birth and two-way transitions."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _get(s, agent, state, names, dtypes):
    return {k: s.get(agent, k, dt, state=state) for k, dt in zip(names, dtypes)}


def test_condition_split_agents():
    # TestAgentFunctionConditions.SplitAgents (test_agent_function_conditions.cu:48-105)
    S = _sim()
    n = 2000
    s = S.Simulation("condition_split", [])
    x = (np.arange(n) % 2).astype(np.int32)
    y = np.tile(np.array([13, 14, 15, 16], np.int32), (n, 1))
    s.set_population("Agent", n, {"x": x, "y": y}, state="Start")
    s.step(1)
    assert s.count("Agent", "Start") == 0
    assert s.count("Agent", "End") == n // 2 and s.count("Agent", "End2") == n // 2
    e1 = _get(s, "Agent", "End", ["x", "_id"], [np.int32, np.uint32])
    e2 = _get(s, "Agent", "End2", ["x", "_id"], [np.int32, np.uint32])
    e1["y"] = s.get("Agent", "y", np.int32, elements=4, state="End")
    e2["y"] = s.get("Agent", "y", np.int32, elements=4, state="End2")
    s.close()
    assert (e1["x"] == 2).all() and (e2["x"] == -1).all()
    np.testing.assert_array_equal(e1["y"].reshape(-1, 4), np.tile([3, 4, 5, 6], (n // 2, 1)))
    np.testing.assert_array_equal(e2["y"].reshape(-1, 4), np.tile([23, 24, 25, 26], (n // 2, 1)))
    # each group keeps its original order
    np.testing.assert_array_equal(e1["_id"], np.arange(2, n + 1, 2))
    np.testing.assert_array_equal(e2["_id"], np.arange(1, n + 1, 2))


def test_condition_all_disabled():
    # TestAgentFunctionConditions.AllDisabled (test_agent_function_conditions.cu:107-130)
    S = _sim()
    s = S.Simulation("condition_none", [])
    s.set_population("Agent", 1000, {"x": np.zeros(1000, np.int32)})
    s.step(3)
    x = s.get("Agent", "x", np.int32)
    y = s.get("Agent", "y", np.int32, elements=4)
    s.close()
    assert (x == -3).all()
    np.testing.assert_array_equal(y, np.tile([23, 24, 25, 26], (1000, 1)))


@pytest.mark.parametrize("graphs", [True, False])
def test_state_chain_moves_one_round_per_step(graphs):
    # TestAgentStateTransitions.Src_10_Dest_10 in spirit
    # (test_agent_state_transition.cu:174-260): one round of agents leaves
    # Start each step and is appended to End in order
    S = _sim()
    rounds, per = 5, 10
    n = rounds * per
    s = S.Simulation("state_chain", [])
    s.configure(steps=1, seed=0, use_graphs=graphs)
    rnd = np.repeat(np.arange(1, rounds + 1, dtype=np.int32), per)
    order = np.random.default_rng(3).permutation(n)
    s.set_population("Agent", n, {"x": np.zeros(n, np.int32), "round": rnd[order]}, state="Start")
    ids = np.arange(1, n + 1, dtype=np.uint32)
    for step in range(rounds):
        s.step(1)
        assert s.count("Agent", "Start") == (rounds - step - 1) * per
        assert s.count("Agent", "End") == (step + 1) * per
        end = _get(s, "Agent", "End", ["_id", "x", "round"], [np.uint32, np.int32, np.int32])
        # rounds in order of leaving; inside a round, the original order
        exp = np.concatenate([ids[rnd[order] == r] for r in range(1, step + 2)])
        np.testing.assert_array_equal(end["_id"], exp)
        np.testing.assert_array_equal(end["x"], end["round"] + 10)
        start = _get(s, "Agent", "Start", ["x"], [np.int32])
        assert (start["x"] == step + 1).all()
    s.close()


@pytest.mark.parametrize("n,steps,graphs", [(1000, 6, True), (4097, 4, True), (300, 5, False), (0, 2, True)])
def test_state_mix_matches_oracle_exactly(n, steps, graphs):
    S = _sim()
    rng = np.random.default_rng(n + steps)
    a = {"_id": np.arange(1, n + 1, dtype=np.uint32), "v": rng.integers(0, 100, n).astype(np.uint32),
         "x": rng.uniform(0, 12, n).astype(np.float32)}
    s = S.Simulation("state_mix", [])
    s.configure(steps=1, seed=0, use_graphs=graphs)
    s.set_population("agent", n, a, state="A")
    for _ in range(steps):
        s.step(1)
    got = {st: _get(s, "agent", st, ["_id", "v", "x"], [np.uint32, np.uint32, np.float32]) for st in ("A", "B")}
    s.close()
    empty = {"_id": np.zeros(0, np.uint32), "v": np.zeros(0, np.uint32), "x": np.zeros(0, np.float32)}
    exp, _ = O.state_mix_run({"A": a, "B": empty}, n + 1, steps)
    for st in ("A", "B"):
        for k in ("_id", "v", "x"):
            np.testing.assert_array_equal(got[st][k], exp[st][k], err_msg=f"state {st} {k}")
