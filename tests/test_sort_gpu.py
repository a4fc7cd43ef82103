"""Automatic spatial agent sort and empty message lists: the reference's
AutomaticSpatialAgentSort known answers
(tests/test_cases/runtime/agent/detail/test_spatial_agent_sort.cu:23-240),
Spatial3DMessageTest.ReadEmpty (tests/test_cases/runtime/messaging/test_spatial_3d.cu:507-540),
and the wrapped iterator on grids of fewer than three bins along an axis,
where the reference's modulo walk visits a bin more than once (against the
oracle's restatement of that walk)."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

AGENT_COUNT = 4


def _sim():
    from flamegpu2_gb300 import sim
    return sim


@pytest.mark.parametrize("variant,expect", [(0, [0, 1, 2, 3]), (1, [3, 2, 1, 0]), (2, [3, 2, 1, 0]),
                                            (3, [3, 2, 1, 0]), (4, [3, 2, 1, 0])])
def test_automatic_spatial_agent_sort(variant, expect):
    # 0 SortingDisabled, 1 SortEveryStep, 2 SortEveryStep_no_default,
    # 3 SortEveryStep_vec2 (packed "xy"), 4 SortEveryStep_vec3 (packed "xyz");
    # agents start in reverse spatial order at (-i, -i, -i)
    S = _sim()
    s = S.Simulation("sort_order", [variant])
    i = np.arange(AGENT_COUNT)
    cols = {"initial_order": i.astype(np.int32)}
    if variant == 3:
        cols["xy"] = np.stack([-i, -i], 1).astype(np.float32)
    elif variant == 4:
        cols["xyz"] = np.stack([-i, -i, -i], 1).astype(np.float32)
    else:
        for k in ("x", "y", "z"):
            cols[k] = (-i).astype(np.float32)
    state = "foobar" if variant == 2 else "default"
    s.set_population("agent", AGENT_COUNT, cols, state=state)
    s.step(1)
    assert s.get("agent", "initial_order", np.int32, state=state).tolist() == expect
    s.close()


def test_read_empty():
    # a message list read before anything has output to it: no messages
    S = _sim()
    s = S.Simulation("read_empty", [])
    s.set_population("agent", 1, {"count": np.array([1], np.uint32)})
    s.step(1)
    assert s.count("agent") == 1
    assert s.get("agent", "count", np.uint32).tolist() == [0]
    s.close()


def _count_run(mx, pos):
    # the neighbour-count model of examples/spatial_tests (test_spatial_3d.cu:855-900), wrapped
    S = _sim()
    n = pos.shape[0]
    s = S.Simulation("spatial_count", [3, 0.0, 0.0, 0.0, mx[0], mx[1], mx[2], 1.0, 1, 0])
    s.set_population("agent", n, {"_id": np.arange(1, n + 1, dtype=np.uint32), "x": pos[:, 0].copy(),
                                  "y": pos[:, 1].copy(), "z": pos[:, 2].copy()})
    s.step()
    out = {k: s.get("agent", k, np.uint32) for k in ("_id", "count", "badCount")}
    for k in ("result_x", "result_y", "result_z"):
        out[k] = s.get("agent", k, np.float32)
    s.close()
    return out


@pytest.mark.parametrize("mx", [(2.0, 4.0, 1.0), (1.0, 2.0, 3.0), (2.0, 2.0, 2.0)])
def test_wrapped_iteration_on_grids_under_three_bins(mx):
    # gridDim 1 or 2 along an axis: the 27-bin modulo walk repeats bins, as the
    # reference's WrapFilter does (MessageSpatial3DDevice.cuh:727-749)
    rng = np.random.default_rng(int(sum(mx) * 10))
    n = 300
    pos = (rng.random((n, 3)) * np.array(mx)).astype(np.float32)
    r = _count_run(mx, pos)
    o = O.count_model(O.grid(3, (0, 0, 0), mx, 1.0), True, pos[:, 0], pos[:, 1], pos[:, 2])
    agent = r["_id"] - 1
    np.testing.assert_array_equal(agent, o["order"])
    np.testing.assert_array_equal(r["count"], o["count"])
    np.testing.assert_array_equal(r["badCount"], o["badCount"])
    for k in ("result_x", "result_y", "result_z"):
        np.testing.assert_array_equal(r[k], o[k], err_msg=k)
