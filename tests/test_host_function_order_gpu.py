"""Host function order and exit conditions: the known answers of the
reference's tests/test_cases/simulation/test_host_functions.cu (MiniSim), through
examples/host_api/host_function_order.cu: with SimulationConfig().steps = 0
the simulation runs until the exit condition returns EXIT (its second call),
init, host layer, step, exit condition and exit functions run in that order,
several functions of one kind in the order added, and adding one twice raises
InvalidHostFunc.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

Init, Step, Exit, HostLayer, ExitCondition, Init2, Step2, Exit2, HostLayer2, ExitCondition2 = range(10)


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _order(second, steps):
    S = _sim()
    s = S.Simulation("host_function_order", [int(second)], steps=steps)
    s.simulate()
    s.close()
    L = C.CDLL(S.MODELS_LIB)
    out = np.zeros(64, np.int32)
    n = L.fg_test_function_order(out.ctypes.data_as(C.c_void_p), 64)
    return list(out[:n])


def test_exit_condition_ends_an_unbounded_run():
    # test_host_functions.cu:119-146: eight calls in this order
    assert _order(False, 0) == [Init, HostLayer, Step, ExitCondition, HostLayer, Step, ExitCondition, Exit]


def test_step_limit_before_the_exit_condition():
    assert _order(False, 1) == [Init, HostLayer, Step, ExitCondition, Exit]


def test_several_functions_of_a_kind_run_in_the_order_added():
    # test_host_functions.cu:151-205; the first exit condition's EXIT skips the second
    assert _order(True, 0) == [Init, Init2, HostLayer, HostLayer2, Step, Step2, ExitCondition, ExitCondition2,
                               HostLayer, HostLayer2, Step, Step2, ExitCondition, Exit, Exit2]


def test_duplicates_raise_invalid_host_func():
    L = C.CDLL(_sim().MODELS_LIB)
    L.fg_test_host_function_duplicates.restype = C.c_uint32
    assert L.fg_test_host_function_duplicates() == 63
