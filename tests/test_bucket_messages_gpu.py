"""Bucket messages (MessageBucket): the known answers of the reference's tests
(tests/test_cases/runtime/messaging/test_bucket.cu), through the model of
examples/bucket_message_tests/bucket_message_tests.cu:

* Mandatory / Optional / OptionalNone: agent id outputs to bucket
  12 + id / 2 and reads bucket 12 + (id - 1) / 2: the count (iterated and
  size()) and the sum of the ids output there.
* Mandatory_Range: the four buckets from 12 + (id / 8) * 4 read as one range.
* ArrayVariable: an array message variable read back from the agent's bucket.
* PersistenceOff / PersistenceOn: output on even steps only; a
  non-persistent list reads empty on odd steps, a persistent one keeps the
  last output.
* A key past the bounds is a device error; a list without an upper bound
  cannot be built (DataValidation); the description's bound checks
  (DescriptionValidation).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1024


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _run(variant, cols, n=N, steps=1, use_graphs=True, persistent=0):
    S = _sim()
    s = S.Simulation("bucket_messages", [variant, persistent], use_graphs=use_graphs, check_each_step=True)
    s.set_population("agent", n, cols)
    s.step(steps)
    out = {k: s.get("agent", k, np.uint32) for k in ("count1", "count2", "sum")}
    out["id"] = s.get("agent", "id", np.int32)
    s.close()
    return out


def _expected(ids, outputs):
    """Per bucket b = id / 2: the number and the sum of the ids output there."""
    count = np.zeros(N // 2, np.uint32)
    total = np.zeros(N // 2, np.uint32)
    np.add.at(count, ids[outputs] // 2, 1)
    np.add.at(total, ids[outputs] // 2, ids[outputs].astype(np.uint32))
    return count, total


@pytest.mark.parametrize("use_graphs", [True, False])
def test_mandatory(use_graphs):
    ids = np.random.default_rng(1).permutation(N).astype(np.int32)  # any row order
    r = _run(0, {"id": ids}, use_graphs=use_graphs)
    count, total = _expected(np.arange(N), np.ones(N, bool))
    b = np.maximum(r["id"] - 1, 0) // 2
    np.testing.assert_array_equal(r["count1"], count[b])
    np.testing.assert_array_equal(r["count2"], count[b])
    np.testing.assert_array_equal(r["sum"], total[b])


def test_optional():
    # test_bucket.cu:199-214: do_output where a uniform draw exceeds 0.3 (any draw)
    ids = np.arange(N, dtype=np.int32)
    do = (np.random.default_rng(2).random(N) > 0.3).astype(np.int32)
    r = _run(1, {"id": ids, "do_output": do})
    count, total = _expected(ids, do.astype(bool))
    b = np.maximum(r["id"] - 1, 0) // 2
    np.testing.assert_array_equal(r["count1"], count[b])
    np.testing.assert_array_equal(r["count2"], count[b])
    np.testing.assert_array_equal(r["sum"], total[b])


def test_optional_none():
    r = _run(2, {"id": np.arange(N, dtype=np.int32)})
    for k in ("count1", "count2", "sum"):
        np.testing.assert_array_equal(r[k], np.zeros(N, np.uint32))


def test_mandatory_range():
    ids = np.arange(N, dtype=np.int32)
    r = _run(3, {"id": ids})
    count, total = _expected(ids, np.ones(N, bool))
    first = (r["id"] // 8) * 4
    c1 = sum(count[first + j] for j in range(4))
    s1 = sum(total[first + j] for j in range(4))
    np.testing.assert_array_equal(r["count1"], c1)
    np.testing.assert_array_equal(r["count2"], count[r["id"] // 2])
    np.testing.assert_array_equal(r["sum"], s1)


def test_array_variable():
    S = _sim()
    s = S.Simulation("bucket_messages", [4], check_each_step=True)
    idx = np.random.default_rng(3).permutation(N).astype(np.uint32)
    s.set_population("agent", N, {"index": idx, "id": np.arange(N, dtype=np.int32)})
    s.step(1)
    index = s.get("agent", "index", np.uint32)
    read = s.get("agent", "message_read", np.uint32, elements=3)
    s.close()
    np.testing.assert_array_equal(read, np.stack([index * 3, index * 7, index * 11], axis=1))


@pytest.mark.parametrize("persistent", [0, 1])
def test_persistence(persistent):
    # test_bucket.cu:408-496: output to bucket 0 on even steps only
    S = _sim()
    s = S.Simulation("bucket_messages", [5, persistent], check_each_step=True)
    ids = np.arange(N, dtype=np.int32)
    s.set_population("agent", N, {"id": ids})
    want_sum = int(ids.sum())
    for step in range(4):
        s.step(1)
        c = s.get("agent", "count1", np.uint32)
        t = s.get("agent", "sum", np.uint32)
        if step % 2 == 0 or persistent:
            assert (c == N).all() and (t == want_sum).all(), step
        else:
            assert (c == 0).all() and (t == 0).all(), step
    s.close()


def test_bad_key_is_a_device_error():
    S = _sim()
    s = S.Simulation("bucket_messages", [6], check_each_step=True)
    s.set_population("agent", 64, {"id": np.arange(64, dtype=np.int32)})
    with pytest.raises(S.SimError, match="DeviceError"):
        s.step(1)
    s.close()


def test_no_upper_bound_is_invalid():
    # test_bucket.cu:38-47 (DataValidation)
    S = _sim()
    with pytest.raises(S.SimError, match="InvalidMessage"):
        S.Simulation("bucket_messages", [7])


def test_description_validation():
    # test_bucket.cu:23-37 (DescriptionValidation): all eleven checks hold
    S = _sim()
    L = C.CDLL(S.MODELS_LIB)
    L.fg_test_bucket_description.restype = C.c_uint32
    assert L.fg_test_bucket_description() == (1 << 11) - 1
