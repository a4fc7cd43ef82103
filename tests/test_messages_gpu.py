"""Message list truncate / append semantics: the reference's
TestMessage_AppendTruncate known answers
(tests/test_cases/runtime/messaging/test_append_truncate.cu:72-320)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1024


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _do_out():
    # the reference draws 70% "output" with a default-seeded mt19937_64; any
    # fixed 70% draw states the same expectations
    rng = np.random.default_rng(7)
    return (rng.uniform(0, 1, N) < 0.7).astype(np.uint32)


@pytest.mark.parametrize("graphs", [True, False])
def test_truncate(graphs):
    S = _sim()
    s = S.Simulation("at_truncate", [])
    s.configure(steps=1, seed=0, use_graphs=graphs)
    s.set_population("Agent", N, {"count": np.zeros(N, np.uint32)})
    for _ in range(2):
        s.step(1)
        assert (s.get("Agent", "count", np.uint32) == N).all()
    s.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_append_keep_data(graphs):
    S = _sim()
    s = S.Simulation("at_append", [])
    s.configure(steps=1, seed=0, use_graphs=graphs)
    s.set_population("Agent", N, {"count0": np.zeros(N, np.uint32)})
    for _ in range(2):
        s.step(1)
        assert (s.get("Agent", "count0", np.uint32) == N).all()
        assert (s.get("Agent", "count1", np.uint32) == N).all()
    s.close()


def test_optional_truncate():
    S = _sim()
    d = _do_out()
    r = int(d.sum())
    s = S.Simulation("at_opt_truncate", [])
    s.set_population("Agent", N, {"do_out": d})
    s.step(1)
    assert (s.get("Agent", "count", np.uint32) == r).all()
    s.step(1)
    assert (s.get("Agent", "count", np.uint32) == N - r).all()
    s.close()


def test_optional_append_keep_data():
    S = _sim()
    d = _do_out()
    r = int(d.sum())
    s = S.Simulation("at_opt_append", [])
    s.set_population("Agent", N, {"do_out": d})
    s.step(1)
    assert (s.get("Agent", "count0", np.uint32) == r).all()
    assert (s.get("Agent", "count1", np.uint32) == N - r).all()
    s.step(1)
    assert (s.get("Agent", "count0", np.uint32) == N - r).all()
    assert (s.get("Agent", "count1", np.uint32) == r).all()
    s.close()


def test_append_keep_data_resize():
    # the second producer has twice the agents of the first: the list grows
    S = _sim()
    s = S.Simulation("at_append_resize", [])
    s.set_population("a", N, {})
    s.set_population("b", 2 * N, {})
    s.set_population("c", 1, {})
    s.step(1)
    assert s.get("c", "c0", np.uint32)[0] == 0
    assert s.get("c", "c1", np.uint32)[0] == N
    assert s.get("c", "c2", np.uint32)[0] == 2 * N
    s.close()
