"""The reference's brute-force message tests
(tests/test_cases/runtime/messaging/test_brute_force.cu), restated against
the models in examples/bruteforce_tests/bruteforce_tests.cu. Expectations are
computed on the host in message order (the output order of the agents); the
reference draws x from a time-seeded generator, here a seeded one.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 128  # AGENT_COUNT


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _sum_product(xs, sum0=0, product0=1):
    s, p = sum0, product0
    for x in xs:
        s += int(x)
        p *= int(x)
        p = 1 if p > 1000000 else p
        p = -1 if p < -1000000 else p
    return s, p


@pytest.mark.parametrize("variant,optional", [(1, False), (2, False), (1, True), (2, True)])
def test_sum_and_product_of_every_message(variant, optional):
    # Mandatory1 (:73-117), Mandatory2 (:119-172), Optional1 (:174-219), Optional2 (:220-276)
    S = _sim()
    x = np.random.default_rng(variant + 10 * optional).integers(-3, 4, N).astype(np.int32)
    steps = 1 if variant == 1 else 2
    msgs = [v for v in x if (v != 0 or not optional)]
    s_exp, p_exp = _sum_product(msgs)
    if variant == 2:
        s_exp, p_exp = _sum_product([v + 1 for v in x if (v + 1 != 0 or not optional)], s_exp, p_exp)
    s = S.Simulation("bf_sum", [variant, int(optional)])
    s.set_population("Agent", N, {"x": x, "sum": np.zeros(N, np.int32), "product": np.ones(N, np.int32)})
    s.step(steps)
    np.testing.assert_array_equal(s.get("Agent", "sum", np.int32), np.full(N, s_exp, np.int32))
    np.testing.assert_array_equal(s.get("Agent", "product", np.int32), np.full(N, p_exp, np.int32))
    s.close()


def test_optional_none():
    # OptionalNone (:277-314): no agent outputs; nothing is read
    S = _sim()
    s = S.Simulation("bf_optional_none")
    s.set_population("Agent", N, {"index": np.arange(N, dtype=np.uint32),
                                  "message_read": np.full(N, 0xFFFFFFFF, np.uint32)})
    s.step(1)
    np.testing.assert_array_equal(s.get("Agent", "message_read", np.uint32), np.full(N, 0xFFFFFFFF, np.uint32))
    s.close()


def test_read_empty():
    # ReadEmpty (:332-381): a list read before any output has no messages
    S = _sim()
    s = S.Simulation("bf_read_empty")
    s.set_population("agent", 1, {"count": np.array([1], np.uint32)})
    s.step(1)
    assert s.count("agent") == 1
    assert s.get("agent", "count", np.uint32)[0] == 0
    s.close()


def test_array_message_variables():
    # ArrayVariable (:383-418)
    S = _sim()
    s = S.Simulation("bf_array")
    s.set_population("Agent", N, {"index": np.arange(N, dtype=np.uint32)})
    s.step(1)
    got = s.get("Agent", "message_read", np.uint32, elements=3)
    idx = s.get("Agent", "index", np.uint32)
    np.testing.assert_array_equal(got, np.stack([idx * 3, idx * 7, idx * 11], 1))
    s.close()


@pytest.mark.parametrize("persistent", [False, True])
def test_persistence(persistent):
    # PersistenceOff / PersistenceOn (:517-627): the init function creates the
    # agents; output only on even steps; a persistent list is still read on the
    # odd step, a non-persistent one is empty
    S = _sim()
    s = S.Simulation("bf_persistence", [int(persistent)])
    expect_sum = N * (N - 1) // 2
    for step in range(2):
        s.step(1)
        assert s.count("Agent") == N
        count = s.get("Agent", "count", np.uint32)
        total = s.get("Agent", "sum", np.uint32)
        if step % 2 == 0 or persistent:
            np.testing.assert_array_equal(count, np.full(N, N, np.uint32))
            np.testing.assert_array_equal(total, np.full(N, expect_sum, np.uint32))
        else:
            np.testing.assert_array_equal(count, np.zeros(N, np.uint32))
            np.testing.assert_array_equal(total, np.zeros(N, np.uint32))
    s.close()


def test_reserved_message_variable_name():
    # reserved_name (:316-330)
    S = _sim()
    with pytest.raises(S.SimError, match="ReservedName|starts with"):
        S.Simulation("bf_reserved")
