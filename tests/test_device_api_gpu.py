"""DeviceAPI calls beyond variables and messages: isAgent / isState (the
reference's DeviceAPITest.check_agent_name_state known answers,
tests/test_cases/runtime/test_device_api.cu:365-405) and AgentOut::genID
(DeviceAPI.cuh:548-557: the new agent's id claimed before getID returns it),
through the models of examples/device_api_tests/device_api_tests.cu."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_check_agent_name_state():
    from flamegpu2_gb300 import sim
    n = 1024
    s = sim.Simulation("agent_name_state")
    s.set_population("agent", n, {"correct_name": np.full(n, -1, np.int32)}, state="state")
    s.step(1)
    assert s.count("agent", "state") == n
    for var, want in (("correct_name", 1), ("wrong_name", 0), ("correct_state", 1), ("wrong_state", 0)):
        np.testing.assert_array_equal(s.get("agent", var, np.int32, state="state"), np.full(n, want, np.int32), err_msg=var)
    s.close()


@pytest.mark.parametrize("use_graphs", [True, False])
def test_gen_id_claims_the_child_id(use_graphs):
    from flamegpu2_gb300 import sim
    n = 3000
    s = sim.Simulation("gen_id", use_graphs=use_graphs)
    s.set_population("agent", n, {"child": np.zeros(n, np.uint32)})
    s.step(1)
    assert s.count("agent") == 2 * n
    ids = s.get("agent", "_id", np.uint32)
    child = s.get("agent", "child", np.uint32)
    parent = s.get("agent", "parent", np.uint32)
    s.close()
    born = parent != 0
    assert born.sum() == n
    # every parent's stored child id is the id its child carries, and ids are unique
    by_parent = dict(zip(parent[born].tolist(), ids[born].tolist()))
    parents = ~born
    for pid, cid in zip(ids[parents].tolist(), child[parents].tolist()):
        assert by_parent[pid] == cid
    assert np.unique(ids).size == 2 * n
