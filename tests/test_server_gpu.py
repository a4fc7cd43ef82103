"""Predator-prey parity with the oracle, and the simulation server: a run
served in a mix of concurrent runs (other models, sizes and seeds, admitted
as slots and the memory budget allow) gives exactly the result it gives
alone, and the result of a plain CUDASimulation run."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

PP = dict(edge=256.0, radius=1.0, p_prey_birth=0.05, p_pred_death=0.02, step=0.5, seed=7, max_crowd=4)
# served runs are limited to four times their largest initial population: a
# dense domain keeps the prey below that (crowding caps them near 3.5 per unit area)
PS = dict(PP, edge=64.0)


def _pp_params(p):
    return [p["edge"], p["radius"], p["p_prey_birth"], p["p_pred_death"], p["step"], p["seed"], p["max_crowd"]]


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _plain_predprey(p, prey, pred, steps):
    S = _sim()
    s = S.Simulation("predprey2d", _pp_params(p))
    s.set_population("prey", len(prey["x"]), prey)
    s.set_population("predator", len(pred["x"]), pred)
    s.step(steps)
    out = ({k: s.get("prey", k, np.uint32 if k == "_id" else np.float32) for k in ("_id", "x", "y")},
           {k: s.get("predator", k, np.uint32 if k == "_id" else np.float32) for k in ("_id", "x", "y")},
           s.agent_steps())
    s.close()
    return out


@pytest.mark.parametrize("n_prey,n_pred,steps", [(20_000, 1_000, 30), (3_000, 2_000, 12), (1, 0, 5), (0, 10, 5)])
def test_predprey_matches_oracle_exactly(n_prey, n_pred, steps):
    from flamegpu2_gb300 import synth
    prey, pred = synth.predprey_population(n_prey, n_pred, PP["edge"], 3)
    gp, gq, _ = _plain_predprey(PP, prey, pred, steps)
    op, oq, _ = O.predprey_run(PP, prey, pred, steps, n_prey + 1)
    for k in ("_id", "x", "y"):
        np.testing.assert_array_equal(gp[k], op[k], err_msg=f"prey {k}")
        np.testing.assert_array_equal(gq[k], oq[k], err_msg=f"predator {k}")


def _boids_request(n, seed):
    from flamegpu2_gb300 import synth
    cfg = dict(synth.BOIDS_SMALL)
    return synth.boids_params(cfg), synth.boids_population(n, cfg["min_pos"], cfg["max_pos"], seed)


def _collect(srv, rid, model):
    if model == "predprey2d":
        return tuple({k: srv.get(rid, a, k, np.uint32 if k == "_id" else np.float32) for k in ("_id", "x", "y")}
                     for a in ("prey", "predator"))
    return ({k: srv.get(rid, "Boid", k, np.uint32 if k == "_id" else np.float32)
             for k in ("_id", "x", "y", "z", "fx", "fy", "fz")},)


def test_server_result_same_alone_and_in_the_mix():
    from flamegpu2_gb300 import synth
    S = _sim()
    prey, pred = synth.predprey_population(12_000, 600, PS["edge"], 5)
    steps = 25
    # alone
    srv = S.Server(max_active=1)
    rid = srv.submit("predprey2d", _pp_params(PS), steps, 0, {"prey": (12_000, prey), "predator": (600, pred)})
    srv.run_until_idle()
    assert srv.take_completed() == [rid]
    assert not srv.info(rid)["failed"], srv.info(rid)["error"]
    alone = _collect(srv, rid, "predprey2d")
    srv.close()
    # in a mix: boids and predator-prey runs of other sizes and seeds around it
    srv = S.Server(max_active=8)
    others = []
    for i in range(6):
        if i % 2 == 0:
            params, pop = _boids_request(2048 * (i + 1), 100 + i)
            others.append(("boids", srv.submit("boids_spatial3d", params, 10 + 5 * i, 0,
                                              {"Boid": (len(pop["x"]), pop)})))
        else:
            p2 = dict(PS, seed=50 + i)
            q1, q2 = synth.predprey_population(3_000 * i, 400, PS["edge"], 200 + i)
            others.append(("pp", srv.submit("predprey2d", _pp_params(p2), 8 + 4 * i, 0,
                                            {"prey": (len(q1["x"]), q1), "predator": (400, q2)})))
        if i == 2:
            rid = srv.submit("predprey2d", _pp_params(PS), steps, 0, {"prey": (12_000, prey), "predator": (600, pred)})
        srv.poll()
    srv.run_until_idle()
    done = srv.take_completed()
    assert sorted(done) == sorted([r for _, r in others] + [rid])
    for r in done:
        assert not srv.info(r)["failed"], srv.info(r)["error"]
    mixed = _collect(srv, rid, "predprey2d")
    for a, b in zip(alone, mixed):
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    mixed_steps = srv.info(rid)["agent_steps"]
    # and the plain CUDASimulation and the oracle agree with both
    plain = _plain_predprey(PS, prey, pred, steps)
    assert mixed_steps == plain[2] > 0  # agent-steps of the run (populations entering each step)
    op, oq, _ = O.predprey_run(PS, prey, pred, steps, 12_001)
    for k in ("_id", "x", "y"):
        np.testing.assert_array_equal(plain[0][k], mixed[0][k])
        np.testing.assert_array_equal(plain[1][k], mixed[1][k])
        np.testing.assert_array_equal(op[k], mixed[0][k])
        np.testing.assert_array_equal(oq[k], mixed[1][k])
    # one boids run of the mix against a plain run
    params, pop = _boids_request(2048, 100)
    s = S.Simulation("boids_spatial3d", params)
    s.set_population("Boid", 2048, pop)
    s.step(10)
    for k in ("x", "fx"):
        np.testing.assert_array_equal(s.get("Boid", k, np.float32), srv.get(others[0][1], "Boid", k, np.float32))
    s.close()
    srv.close()


def test_server_budget_queues_and_isolates_failures():
    from flamegpu2_gb300 import synth
    S = _sim()
    prey, pred = synth.predprey_population(4_000, 200, 40.0, 9)
    # a budget that fits one run at a time: the second waits in the queue
    one = 1 << 20
    srv = S.Server(memory_budget=one, max_active=8)
    a = srv.submit("predprey2d", _pp_params(dict(PS, edge=40.0)), 5, 0, {"prey": (4_000, prey), "predator": (200, pred)})
    b = srv.submit("predprey2d", _pp_params(dict(PS, edge=40.0)), 5, 0, {"prey": (4_000, prey), "predator": (200, pred)})
    srv.poll()
    st = srv.stats()
    assert st["active"] == 1 and st["queued"] == 1
    # a run with an unknown variable fails at submission; the others are unaffected
    with pytest.raises(S.SimError):
        srv.submit("predprey2d", _pp_params(dict(PS, edge=40.0)), 5, 0, {"prey": (1, {"nope": np.zeros(1, np.float32)})})
    # a run whose prey multiply without limit (no predators, no crowding) stops at
    # four times its initial population with OutOfMemory; the others complete
    lone, _ = synth.predprey_population(2_000, 0, 256.0, 10)
    c = srv.submit("predprey2d", _pp_params(dict(PP, max_crowd=1_000_000)), 60, 0,
                   {"prey": (2_000, lone), "predator": (0, {"x": np.zeros(0, np.float32), "y": np.zeros(0, np.float32)})})
    srv.run_until_idle()
    done = srv.take_completed()
    assert sorted(done) == [a, b, c]
    assert srv.info(c)["failed"] and "OutOfMemory" in srv.info(c)["error"]
    assert not srv.info(a)["failed"] and not srv.info(b)["failed"]
    for k in ("_id", "x", "y"):
        np.testing.assert_array_equal(srv.get(a, "prey", k, np.float32 if k != "_id" else np.uint32),
                                      srv.get(b, "prey", k, np.float32 if k != "_id" else np.uint32))
    assert srv.stats()["reserved_bytes"] == 0
    srv.close()
