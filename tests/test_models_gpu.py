"""Model-level parity: agent functions written against the FLAME GPU 2 API run
through CUDASimulation (C ABI) and are compared with the serial oracle and
with the reference tests' known answers."""
import os

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _count_run(dims, mn, mx, r, wrap, optional, pos, do_output=None):
    S = _sim()
    n = pos.shape[0]
    params = [dims] + list(mn) + [0.0] * (3 - len(mn)) + list(mx) + [0.0] * (3 - len(mx)) + [r, int(wrap), int(optional)]
    s = S.Simulation("spatial_count", params)
    cols = {"_id": np.arange(1, n + 1, dtype=np.uint32), "x": pos[:, 0].copy(), "y": pos[:, 1].copy()}
    if dims == 3:
        cols["z"] = pos[:, 2].copy()
    if do_output is not None:
        cols["do_output"] = do_output.astype(np.int32)
    s.set_population("agent", n, cols)
    s.step()
    out = {k: s.get("agent", k, np.uint32) for k in ("_id", "count", "badCount")}
    for k in ("result_x", "result_y", "result_z", "x", "y"):
        out[k] = s.get("agent", k, np.float32)
    s.close()
    return out


@pytest.mark.parametrize("optional", [False, True])
def test_spatial3d_counts_match_reference_expectation(golden, optional):
    pre = "s3d_optional_" if optional else "s3d_mandatory_"
    pos = golden[pre + "pos"].reshape(-1, 3)
    r = _count_run(3, (0, 0, 0), (5, 5, 5), 1.0, False, optional, pos, golden[pre + "do_output"] if optional else None)
    agent = r["_id"] - 1
    np.testing.assert_array_equal(r["count"], golden[pre + "expect"][agent])
    assert int(r["badCount"].sum()) == 0
    # agent order after the automatic spatial sort matches the oracle's stable sort
    o = O.count_model(O.grid(3, (0, 0, 0), (5, 5, 5), 1.0), False, pos[:, 0], pos[:, 1], pos[:, 2],
                      do_output=golden[pre + "do_output"] if optional else None)
    np.testing.assert_array_equal(agent, o["order"])


@pytest.mark.parametrize("optional", [False, True])
def test_spatial2d_counts_match_reference_expectation(golden, optional):
    pre = "s2d_optional_" if optional else "s2d_mandatory_"
    pos = golden[pre + "pos"].reshape(-1, 2)
    r = _count_run(2, (0, 0), (11, 11), 1.0, False, optional, pos, golden[pre + "do_output"] if optional else None)
    np.testing.assert_array_equal(r["count"], golden[pre + "expect"][r["_id"] - 1])
    assert int(r["badCount"].sum()) == 0


@pytest.mark.parametrize("off", [(0.0, 0.0, 0.0), (141.0, -540.0, 200.0), (-1401.5, 5640.3, -2008.8)])
def test_spatial3d_wrapped_lattice(off):
    i, j, k = np.meshgrid(np.arange(35), np.arange(35), np.arange(35), indexing="ij")
    pos = np.stack([(i.ravel() * np.float32(2.0) + np.float32(off[0])),
                    (j.ravel() * np.float32(2.0) + np.float32(off[1])),
                    (k.ravel() * np.float32(2.0) + np.float32(off[2]))], 1).astype(np.float32)
    r = _count_run(3, off, tuple(o + 70 for o in off), 3.5, True, False, pos)
    assert np.all(r["count"] == 27)
    assert np.all(r["badCount"] <= 189)
    assert np.all(r["result_x"] == 0.0) and np.all(r["result_y"] == 0.0) and np.all(r["result_z"] == 0.0)


@pytest.mark.parametrize("off", [(0.0, 0.0), (141.0, 0.0), (0.0, 3440.0), (-2342.0, 0.0), (141.4, -540.7)])
def test_spatial2d_wrapped_lattice(off):
    i, j = np.meshgrid(np.arange(15), np.arange(15), indexing="ij")
    pos = np.stack([(i.ravel() * np.float32(2.0) + np.float32(off[0])),
                    (j.ravel() * np.float32(2.0) + np.float32(off[1]))], 1).astype(np.float32)
    r = _count_run(2, off, tuple(o + 30 for o in off), 3.0, True, False, pos)
    assert np.all(r["count"] == 9)
    assert np.all(r["result_x"] == 0.0) and np.all(r["result_y"] == 0.0)


@pytest.mark.parametrize("optional", [False, True])
def test_spatial3d_counts_and_order_with_agents_outside_the_bounds(optional):
    # a third of the agents outside [0,5)^3: their messages fall in the clamped
    # edge bins, their sort keys past the grid's cells (unclamped); the output
    # launch computes both key sets, and the sort's scan runs past the cells
    rng = np.random.default_rng(17 + optional)
    n = 3000
    pos = rng.uniform(-2.0, 7.0, (n, 3)).astype(np.float32)
    do = (rng.random(n) < 0.6).astype(np.int32) if optional else None
    r = _count_run(3, (0, 0, 0), (5, 5, 5), 1.0, False, optional, pos, do)
    o = O.count_model(O.grid(3, (0, 0, 0), (5, 5, 5), 1.0), False, pos[:, 0], pos[:, 1], pos[:, 2], do_output=do)
    agent = r["_id"] - 1
    np.testing.assert_array_equal(agent, o["order"])
    np.testing.assert_array_equal(r["count"], o["count"])  # both in the sorted order


def test_spatial3d_bounds_not_factor_radius():
    h = np.float32(50.1) / np.float32(2)
    pos = np.array([[h, 0.0, h], [h, 18.0, h], [0.0, h, 0.5], [18.0, h, 0.5], [h, 50.0, 50.1],
                    [h, 50.0, np.float32(50.1) - np.float32(10.11)]], np.float32)
    r = _count_run(3, (0, 0, 0), (50.1, 50.1, 50.1), 10.0, False, False, pos)
    by_id = dict(zip(r["_id"].tolist(), r["count"].tolist()))
    assert [by_id[i] for i in range(1, 7)] == [2, 2, 2, 2, 1, 1]


def test_wrapped_out_of_bounds_raises_device_error():
    # test_spatial_3d.cu:976-979 (Wrapped_OutOfBounds): a location outside the
    # bounds given to the wrapped iterator is a device error, reported on the host.
    S = _sim()
    i, j, k = np.meshgrid(np.arange(35), np.arange(35), np.arange(35), indexing="ij")
    pos = np.stack([(i.ravel() * 2.0 + 141.0 + 200.0), (j.ravel() * 2.0 - 540.0), (k.ravel() * 2.0)], 1).astype(np.float32)
    with pytest.raises(S.SimError, match="DeviceError"):
        _count_run(3, (141.0, -540.0, 0.0), (211.0, -470.0, 70.0), 3.5, True, False, pos)


def test_agent_death_order(golden):
    S = _sim()
    x = golden["death_x"]
    s = S.Simulation("agent_death")
    s.set_population("agent", len(x), {"x": x.astype(np.uint32)})
    s.step()
    np.testing.assert_array_equal(s.get("agent", "x", np.uint32), golden["death_expect"])
    s.close()


@pytest.mark.parametrize("optional", [False, True])
def test_bruteforce_counts(optional):
    S = _sim()
    n = 3000
    rng = np.random.default_rng(2)
    x = rng.integers(-50, 50, n).astype(np.int32)
    do = (rng.random(n) < 0.7).astype(np.int32) if optional else np.ones(n, np.int32)
    s = S.Simulation("bruteforce_count", [int(optional)])
    s.set_population("agent", n, {"x": x, "do_output": do})
    s.step()
    assert np.all(s.get("agent", "count", np.uint32) == int(do.sum()))
    assert np.all(s.get("agent", "sum", np.int32) == int((x * do).sum()))
    s.close()


def _boids_run(cfg, steps, use_graphs=True):
    from flamegpu2_gb300 import synth
    S = _sim()
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], cfg["seed"])
    s = S.Simulation("boids_spatial3d", synth.boids_params(cfg), steps=steps, use_graphs=use_graphs)
    s.set_population("Boid", cfg["n"], pop)
    s.step(steps)
    out = {"_id": s.get("Boid", "_id", np.uint32)}
    for k in ("x", "y", "z", "fx", "fy", "fz"):
        out[k] = s.get("Boid", k, np.float32)
    st = s.stats()
    s.close()
    return pop, out, st


def _boids_oracle(cfg, pop, steps):
    p = O.boids_params(cfg["min_pos"], cfg["max_pos"], cfg["interaction_radius"], cfg["separation_radius"],
                       cfg["time_scale"], cfg["global_scale"], cfg["steer_scale"], cfg["collision_scale"],
                       cfg["match_scale"], cfg["wrap"], cfg["sort_period"])
    st = {"id": pop["_id"], **{k: pop[k] for k in ("x", "y", "z", "fx", "fy", "fz")}}
    return O.boids_run(p, st, steps)


@pytest.mark.parametrize("use_graphs", [True, False])
def test_boids_small_matches_oracle(use_graphs):
    # Boids on MessageSpatial3D, 16,384 agents, 32^3 bins, wrapped, 10 steps.
    from flamegpu2_gb300 import synth
    cfg = dict(synth.BOIDS_SMALL)
    pop, out, st = _boids_run(cfg, 10, use_graphs)
    ref = _boids_oracle(cfg, pop, 10)
    # agent order (auto spatial sort) and ids are exact; so is the float state
    # (same visit order, no FMA contraction on either side), which is stricter
    # than the 1e-4 tolerance on positions that the comparison asks for
    np.testing.assert_array_equal(out["_id"], ref["id"])
    for k in ("x", "y", "z", "fx", "fy", "fz"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    if use_graphs:
        assert st["graph_launches"] == 1  # ten steps replayed as one captured graph


def test_boids_clamped_matches_oracle():
    from flamegpu2_gb300 import synth
    cfg = dict(synth.BOIDS_SMALL, n=6000, wrap=0, min_pos=-0.5, max_pos=0.5, interaction_radius=0.05,
               separation_radius=0.01, time_scale=0.0005, global_scale=0.15, steer_scale=0.055,
               collision_scale=10.0, match_scale=0.015, seed=5)
    pop, out, _ = _boids_run(cfg, 5)
    ref = _boids_oracle(cfg, pop, 5)
    np.testing.assert_array_equal(out["_id"], ref["id"])
    for k in ("x", "y", "z", "fx", "fy", "fz"):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)


def test_birth_death_matches_oracle_exactly():
    from flamegpu2_gb300 import synth
    S = _sim()
    n, steps, seed = 100_000, 25, 1
    pop = synth.birth_death_population(n, seed)
    s = S.Simulation("birth_death", [0.30, 0.20, seed])
    s.set_population("agent", n, pop)
    s.step(steps)
    f = np.stack([s.get("agent", f"f{v}", np.float32) for v in range(8)])
    cnt = s.get("agent", "counter", np.int32)
    ids = s.get("agent", "_id", np.uint32)
    agent_steps = s.agent_steps()
    s.close()
    fo, co, io, nid, pops = O.birth_death_run(np.stack([pop[f"f{v}"] for v in range(8)]), pop["counter"],
                                              pop["_id"], n + 1, 4 * n, 0.30, 0.20, seed, steps)
    # agent-steps counted on the device: the populations entering each step
    assert agent_steps == int(pops.astype(np.int64).sum())
    assert len(ids) == len(io)
    np.testing.assert_array_equal(ids, io)
    np.testing.assert_array_equal(cnt, co)
    np.testing.assert_array_equal(f, fo)


def test_operation_times_from_step_graphs():
    # timing events captured into the step graphs: steps stay graph replays,
    # results are unchanged, and every operation of the step is timed
    from flamegpu2_gb300 import synth
    S = _sim()
    cfg = dict(synth.BOIDS_SMALL)
    params = synth.boids_params(cfg)
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], 3)
    outs = []
    for timed in (False, True):
        s = S.Simulation("boids_spatial3d", params)
        s.set_population("Boid", cfg["n"], pop)
        if timed:
            s.time_ops_in_graphs(True)
        for _ in range(4):
            s.step(1)
            s.harvest_profile()
        prof = s.take_profile()
        st = s.stats()
        outs.append({k: s.get("Boid", k, np.float32) for k in ("x", "fx")})
        s.close()
        if timed:
            assert st["graph_launches"] == 4
            paired = os.environ.get("FLAMEGPU_PAIR_SORT_BUILD") == "1" and os.environ.get("FLAMEGPU_FUSE_KEYS") != "0"
            middle = ("sort+build:Boid/location",) if paired else ("sort:Boid", "build:location")
            for label in ("fn:outputdata", "fn:inputdata") + middle:
                assert label in prof and prof[label][1] >= 2 and prof[label][0] > 0.0, (label, prof)
        else:
            assert prof == {}
    for k in ("x", "fx"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])


def test_population_direct_columns_match_agent_vector_path():
    # every variable given (ids set): copied straight to the device; one left
    # out: the AgentVector path with defaults. Same state, same new ids.
    from flamegpu2_gb300 import synth
    S = _sim()
    n = 20_000
    pop = synth.birth_death_population(n, 4)
    outs = []
    for cols in (pop, {k: v for k, v in pop.items() if k != "counter"}):
        s = S.Simulation("birth_death", [0.30, 0.20, 4])
        s.set_population("agent", n, cols)
        s.step(6)
        names = ["_id", "counter"] + [f"f{v}" for v in range(8)]
        bufs = {k: np.zeros(4 * n, dtype=np.uint32 if k == "_id" else (np.int32 if k == "counter" else np.float32))
                for k in names}
        m = s.get_population("agent", bufs)
        outs.append({k: v[:m].copy() for k, v in bufs.items()})
        s.close()
    for k in outs[0]:
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)
    assert outs[0]["_id"].max() > n  # births took fresh ids past the given ones


def test_parity_holds_without_programmatic_dependent_launch():
    # Every kernel waits for its predecessors before touching memory, so with
    # or without the programmatic-dependency launch attribute the results are
    # those of plain stream order: the bit-exact Boids and birth/death checks
    # run again in a process with the attribute off.
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FLAMEGPU_PDL="0")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-m", "gpu",
                        os.path.join(root, "tests", "test_models_gpu.py"),
                        "-k", "boids_small_matches_oracle or boids_clamped or birth_death_matches"],
                       cwd=root, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "4 passed" in r.stdout, r.stdout[-2000:]


def test_parity_holds_without_key_fusion():
    # The Boids output launch computes the message bins and the agents' sort
    # keys itself (the build's and the sort's key kernels are not run); with
    # that turned off the bit-exact checks hold the same.
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FLAMEGPU_FUSE_KEYS="0")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-m", "gpu",
                        os.path.join(root, "tests", "test_models_gpu.py"),
                        "-k", "boids_small_matches_oracle or boids_clamped or birth_death_matches or key_kernels"],
                       cwd=root, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "5 passed" in r.stdout, r.stdout[-2000:]


@pytest.mark.parametrize("n", [1001, 2048])
def test_population_through_page_locked_buffers(n):
    # page-locked host columns are read and written by one launch through
    # their mapped addresses (16-byte or 4-byte units by alignment and size),
    # pageable ones by one copy each: the same state either way
    import torch
    from flamegpu2_gb300 import synth
    S = _sim()
    cfg = dict(synth.BOIDS_SMALL, n=n, seed=6)
    pop = synth.boids_population(n, cfg["min_pos"], cfg["max_pos"], cfg["seed"])

    def pinned_like(a):
        buf = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory().numpy().view(a.dtype)
        buf[:] = a
        return buf

    names = ("_id", "x", "y", "z", "fx", "fy", "fz")
    res = []
    for locked in (False, True):
        s = S.Simulation("boids_spatial3d", synth.boids_params(cfg))
        cols = {k: pinned_like(v) for k, v in pop.items()} if locked else pop
        outs = {k: (pinned_like(pop[k]) if locked else np.empty_like(pop[k])) for k in names}
        for _ in range(3):
            s.set_population("Boid", n, cols)
            s.step(2)
            assert s.get_population("Boid", outs) == n
            cols = {k: outs[k].copy() for k in names}
            if locked:
                cols = {k: pinned_like(v) for k, v in cols.items()}
        s.close()
        res.append({k: np.array(outs[k]) for k in names})
    for k in names:
        np.testing.assert_array_equal(res[0][k], res[1][k], err_msg=k)


@pytest.mark.parametrize("locked", [False, True])
def test_population_with_unset_ids_gets_ids_assigned(locked):
    # page-locked columns: the transfer launch checks the ids on the device
    # (the host does not read them); pageable: the host checks them. Either
    # way an id left unset (0) sends the population through the path that
    # assigns ids, and the next id follows the largest id given
    import torch
    from flamegpu2_gb300 import synth
    S = _sim()
    n = 4096
    cfg = dict(synth.BOIDS_SMALL, n=n, seed=8)
    pop = synth.boids_population(n, cfg["min_pos"], cfg["max_pos"], cfg["seed"])

    def pinned_like(a):
        buf = torch.empty(a.nbytes, dtype=torch.uint8).pin_memory().numpy().view(a.dtype)
        buf[:] = a
        return buf

    ids = np.arange(1, n + 1, dtype=np.uint32) * 3
    ids[1234] = 0
    pop = dict(pop, _id=ids)
    cols = {k: pinned_like(v) for k, v in pop.items()} if locked else pop
    s = S.Simulation("boids_spatial3d", synth.boids_params(cfg))
    s.set_population("Boid", n, cols)
    got = s.get("Boid", "_id", np.uint32)
    assert len(got) == n and np.all(got != 0) and len(np.unique(got)) == n
    # the ids that were set are kept; the unset one got a fresh id
    keep = np.ones(n, bool)
    keep[1234] = False
    np.testing.assert_array_equal(got[keep], ids[keep])
    # every id set: taken as given, and the population is not left empty by the first try
    ids2 = np.arange(1, n + 1, dtype=np.uint32) * 5
    cols2 = dict(cols, _id=pinned_like(ids2) if locked else ids2)
    s.set_population("Boid", n, cols2)
    np.testing.assert_array_equal(s.get("Boid", "_id", np.uint32), ids2)
    s.step(1)
    assert s.count("Boid") == n
    s.close()


def test_key_kernels_fused_into_the_output_launch():
    # Boids step: outputdata, agent sort (5 kernels), message build (5),
    # inputdata, step end = 13 kernels; the output launch computing both key
    # sets saves the two key kernels (11), and the sort and build then run as
    # one chain of four paired launches (7)
    from flamegpu2_gb300 import synth
    S = _sim()
    cfg = dict(synth.BOIDS_SMALL, n=2000, seed=4)
    s = S.Simulation("boids_spatial3d", synth.boids_params(cfg))
    s.set_population("Boid", cfg["n"], synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], cfg["seed"]))
    s.step(2)
    s.synchronize()
    k = s.stats()["kernels_per_step"]
    s.close()
    if os.environ.get("FLAMEGPU_FUSE_KEYS") == "0":
        assert k == 13, k
    else:
        assert k == (7 if os.environ.get("FLAMEGPU_PAIR_SORT_BUILD") == "1" else 11), k


def test_parity_holds_with_sort_and_build_paired():
    # The agent sort and the message build run as two graph branches by
    # default; as one chain of paired launches (FLAMEGPU_PAIR_SORT_BUILD=1)
    # the bit-exact checks hold the same
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, FLAMEGPU_PAIR_SORT_BUILD="1")
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-p", "no:cacheprovider", "-m", "gpu",
                        os.path.join(root, "tests", "test_models_gpu.py"), os.path.join(root, "tests", "test_payload_gpu.py"),
                        "-k", "boids_small_matches_oracle or boids_clamped or key_kernels or rows_in_bin_order"],
                       cwd=root, env=env, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    assert "7 passed" in r.stdout, r.stdout[-2000:]


def test_steps_replayed_as_one_graph_match_single_steps():
    # step(n) replays up to 16 steps per captured graph when no host work runs
    # between steps; the state after 37 steps (16 + 16 + 5) equals that of 37
    # single steps, and the step counter and per-step timings cover every step
    from flamegpu2_gb300 import synth
    S = _sim()
    cfg = dict(synth.BOIDS_SMALL, n=3000, seed=9)
    pop = synth.boids_population(cfg["n"], cfg["min_pos"], cfg["max_pos"], cfg["seed"])
    outs, stats = [], []
    for many in (False, True):
        s = S.Simulation("boids_spatial3d", synth.boids_params(cfg))
        s.set_population("Boid", cfg["n"], pop)
        if many:
            s.step(37)
        else:
            for _ in range(37):
                s.step(1)
        outs.append({k: s.get("Boid", k, np.float32) for k in ("x", "y", "z", "fx")})
        outs[-1]["_id"] = s.get("Boid", "_id", np.uint32)
        stats.append(s.stats())
        s.close()
    for k in outs[0]:
        np.testing.assert_array_equal(outs[0][k], outs[1][k], err_msg=k)
    assert stats[0]["graph_launches"] == 37 and stats[1]["graph_launches"] == 3
    assert stats[0]["step_counter"] == stats[1]["step_counter"] == 37


def test_agent_steps_of_a_fixed_population():
    # no birth, death or transition: counted on the host, n per step, whether
    # steps are replayed one or ten per graph
    from flamegpu2_gb300 import synth
    S = _sim()
    cfg = dict(synth.BOIDS_SMALL, n=3000)
    s = S.Simulation("boids_spatial3d", synth.boids_params(cfg))
    s.set_population("Boid", 3000, synth.boids_population(3000, cfg["min_pos"], cfg["max_pos"], 2))
    s.step(1)
    s.step(10)
    assert s.agent_steps() == 3000 * 11
    s.close()
