"""HostAgentAPI::getPopulationData (DeviceAgentVector) in host functions: the
calls of the reference's tests/test_cases/runtime/agent/
test_device_agent_vector.cu (update every agent, erase, push_back with fresh
ids; reductions, counts and sorts in the same host function see the view and
a sort reorders it), through examples/host_api/host_population_models.cu.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _errors():
    L = C.CDLL(_sim().MODELS_LIB)
    L.fg_test_host_population_errors.restype = C.c_uint
    return L.fg_test_host_population_errors(1)


def _edit(x, ids, next_id):
    """One step of the model on the host: x += 1, drop multiples of 5, append 1000..1002 with fresh ids."""
    x = x + 1
    keep = x % 5 != 0
    x, ids = x[keep], ids[keep]
    new_ids = np.arange(next_id, next_id + 3, dtype=ids.dtype)
    return np.concatenate([x, [1000, 1001, 1002]]).astype(np.int32), np.concatenate([ids, new_ids]), next_id + 3


@pytest.mark.parametrize("n", [1, 1000, 5003])
def test_edit_erase_push_back(n):
    S = _sim()
    _errors()
    s = S.Simulation("host_population", [], check_each_step=True)
    x = np.arange(n, dtype=np.int32)
    s.set_population("agent", n, {"x": x})
    ids = s.get("agent", "_id", np.uint32)
    next_id = int(ids.max()) + 1
    for _ in range(3):
        s.step(1)
        x, ids, next_id = _edit(x, ids, next_id)
        np.testing.assert_array_equal(s.get("agent", "x", np.int32), x)
        np.testing.assert_array_equal(s.get("agent", "y", np.int32), 2 * x)
        got_ids = s.get("agent", "_id", np.uint32)
        np.testing.assert_array_equal(got_ids[:-3], ids[:-3])  # kept agents keep their ids
        assert len(np.unique(got_ids)) == len(got_ids)
        assert (got_ids[-3:] >= next_id - 3).all()
        ids = got_ids
    s.close()
    assert _errors() == 0


def test_reductions_and_sort_see_the_view():
    S = _sim()
    _errors()
    s = S.Simulation("host_population_sync", [], check_each_step=True)
    n = 3001
    x = np.random.default_rng(5).integers(0, 1000, n).astype(np.int32)
    s.set_population("agent", n, {"x": x})
    s.step(1)
    got = s.get("agent", "x", np.int32)
    s.close()
    assert _errors() == 0
    want = np.concatenate([x + 10, [-5]])
    np.testing.assert_array_equal(got, np.sort(want)[::-1])


@pytest.mark.parametrize("n", [1, 1024])
def test_insert_copies_of_an_agent(n):
    # test_device_agent_vector.cu Insert: n copies of agent 0 inserted n / 2 from the end, fresh ids
    S = _sim()
    s = S.Simulation("host_population_insert", [], check_each_step=True)
    x = np.arange(n, dtype=np.int32)
    s.set_population("agent", n, {"x": x, "y": x + 7})
    ids0 = s.get("agent", "_id", np.uint32)
    s.step(1)
    at = n - n // 2
    want = np.concatenate([x[:at], np.zeros(n, np.int32), x[at:]])
    np.testing.assert_array_equal(s.get("agent", "x", np.int32), want)
    np.testing.assert_array_equal(s.get("agent", "y", np.int32), want + 7)
    ids = s.get("agent", "_id", np.uint32)
    np.testing.assert_array_equal(np.concatenate([ids[:at], ids[at + n:]]), ids0)
    assert len(np.unique(ids)) == 2 * n
    assert (ids[at:at + n] > ids0.max()).all()
    s.close()
