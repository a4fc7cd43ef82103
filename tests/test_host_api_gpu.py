"""Host functions of a model: agents created by init functions
(HostAgentAPI::newAgent) and reductions of agent variables in exit functions
(HostAgentAPI::sum / min / max / meanStandardDeviation), through ensembles and
plain simulations of the models in examples/host_api/host_api_models.cu.

The first two tests restate known answers of the reference: the sum of sums of
TestCUDAEnsemble.simulate (tests/test_cases/simulation/test_cuda_ensemble.cu:
279-316: 2 runs of 1 and 2 steps over 32 agents whose counters count the
steps, 96) and the closed form of its ensemble example
(examples/cpp/ensemble/src/main.cu:88-96, with each run's properties set
directly so that the closed form holds exactly).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _models():
    from flamegpu2_gb300 import sim
    sim.core()
    L = C.CDLL(sim.MODELS_LIB)
    L.fg_test_counter_total.argtypes = [C.c_int]
    L.fg_test_counter_total.restype = C.c_uint64
    L.fg_test_offset_totals.argtypes = [C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.c_int]
    return L


def test_ensemble_sum_of_sums():
    from flamegpu2_gb300 import sim
    L = _models()
    L.fg_test_counter_total(1)
    pop = 32
    ens = sim.Ensemble("ensemble_counter", [pop])
    expected = 0
    for idx in range(2):
        ens.add_run(idx + 1, 0)
        expected += (idx + 1) * pop
    assert ens.simulate() == 0
    assert L.fg_test_counter_total(1) == expected == 96
    # the populations the init functions created, each counter equal to its run's steps
    for idx in range(2):
        assert ens.count(idx, "Agent") == pop
        np.testing.assert_array_equal(ens.get(idx, "Agent", "counter", np.uint32), np.full(pop, idx + 1, np.uint32))
    ens.close()


def test_ensemble_example_closed_form():
    from flamegpu2_gb300 import sim
    L = _models()
    ia, ra = C.c_int64(), C.c_int64()
    L.fg_test_offset_totals(C.byref(ia), C.byref(ra), 1)
    runs, pop, steps = 60, 1000, 10
    ens = sim.Ensemble("ensemble_offset", [pop])
    expected_init = expected_result = 0
    for i in range(runs):
        r = ens.add_run(steps, 12 + i)
        init, init_offset, offset = i // 10, 1 - i // 50, i
        ens.set_property(r, "init", init, C.c_int32)
        ens.set_property(r, "init_offset", init_offset, C.c_int32)
        ens.set_property(r, "offset", offset, C.c_int32)
        expected_init += init
        expected_result += pop * init + init_offset * ((pop - 1) * pop // 2) + pop * steps * offset
    assert ens.simulate() == 0
    L.fg_test_offset_totals(C.byref(ia), C.byref(ra), 1)
    assert ia.value == expected_init
    assert ra.value == expected_result
    ens.close()


@pytest.mark.parametrize("n", [0, 1, 1000, 70_001])
def test_host_reductions_and_created_agents(n):
    from flamegpu2_gb300 import sim
    s = sim.Simulation("host_probe", [n])
    s.configure(steps=2)
    s.simulate()
    i = np.arange(n)
    x = (i - 100).astype(np.int32)
    f = (i * 0.5).astype(np.float32)
    u = (i % 7).astype(np.uint32)
    assert s.get_env("count", C.c_uint32) == n
    assert s.get_env("sum_x", C.c_int64) == int(x.astype(np.int64).sum())
    # sum<int>: the sum in the variable's own type, which wraps past 2^31 as the reference's does
    total = int(x.astype(np.int64).sum())
    assert s.get_env("sum_x_int", C.c_int32) == ((total + 2 ** 31) % 2 ** 32) - 2 ** 31
    assert s.get_env("min_x", C.c_int32) == (int(x.min()) if n else 0)
    assert s.get_env("max_x", C.c_int32) == (int(x.max()) if n else 0)
    assert s.get_env("max_u", C.c_uint32) == (int(u.max()) if n else 0)
    assert s.get_env("sum_f", C.c_double) == float(f.astype(np.float64).sum())
    if n:
        np.testing.assert_allclose(s.get_env("mean_f", C.c_double), f.astype(np.float64).mean(), rtol=1e-12)
        np.testing.assert_allclose(s.get_env("sd_f", C.c_double), f.astype(np.float64).std(), rtol=1e-9)
    # the created agents, in creation order, with fresh distinct ids
    assert s.count("a") == n
    np.testing.assert_array_equal(s.get("a", "x", np.int32), x)
    np.testing.assert_array_equal(s.get("a", "u", np.uint32), u)
    ids = s.get("a", "_id", np.uint32)
    assert len(np.unique(ids)) == n and np.all(ids != 0)
    s.close()
