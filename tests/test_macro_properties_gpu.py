"""Environment macro properties: the known answers of the reference's tests
(tests/test_cases/runtime/environment/test_device_macro_property.cu and
test_host_macro_property.cu), through the model of
examples/macro_property_tests/macro_property_tests.cu:

* the device operations on one agent: +=, +, addAtomic, -=, -, subAtomic,
  pre/post increment and decrement, min, max and CAS (value that succeeds and
  value that fails), exchange over every 4- and 8-byte type;
* host views: a 2 x 3 x 4 x 5 property filled by agents and read on the host,
  written on the host and read by agents, zeroed on the host; the host
  arithmetic over nine types;
* 70,001 agents updating one property at once (count, sum, min, max);
* an index past a dimension is a device error, and so is a property both
  read and updated in one agent function (WriteRead, ReadWrite).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _run(variant, cols, n=1):
    S = _sim()
    s = S.Simulation("macro_properties", [variant], check_each_step=True)
    s.set_population("agent", n, cols)
    s.step(1)
    out = {k: s.get("agent", k, np.uint32) for k in ("a", "b", "c")}
    out["cd"] = s.get("agent", "cd", np.float64)
    for k, t in (("x_i64", np.int64), ("x_u64", np.uint64), ("x_i32", np.int32), ("x_u32", np.uint32),
                 ("x_f64", np.float64), ("x_f32", np.float32)):
        out[k] = s.get("agent", k, t)
    s.close()
    return out


def _errors(reset=True):
    L = C.CDLL(_sim().MODELS_LIB)
    L.fg_test_macro_errors.restype = C.c_uint
    return L.fg_test_macro_errors(1 if reset else 0)


# variant, a, expected b, expected c (None: not checked)
DEVICE_CASES = [
    ("add2", 1, 12, 13, 1),
    ("add3", 2, 12, 13, 13),
    ("sub", 3, 12, 13, None),
    ("sub2", 4, 12, 13, 25),
    ("sub3", 5, 12, 13, 13),
    ("postincrement", 6, 12, 1, 2),
    ("preincrement", 7, 12, 2, 2),
    ("postdecrement", 8, 12, 1, 0),
    ("predecrement", 9, 12, 0, 0),
    ("min", 10, 12, 12, 12),
    ("min2", 10, 45, 25, 25),
    ("max", 11, 45, 45, 45),
    ("max2", 11, 12, 25, 25),
    ("cas", 12, 25, 25, 100),
    ("cas2", 12, 12, 25, 25),
]


@pytest.mark.parametrize("name,variant,a,b,c", DEVICE_CASES, ids=[c[0] for c in DEVICE_CASES])
def test_device_operation(name, variant, a, b, c):
    r = _run(variant, {"a": np.array([a], np.uint32)})
    assert int(r["b"][0]) == b
    if c is not None:
        assert int(r["c"][0]) == c


def test_add_uint_and_double():
    # test_device_macro_property.cu:105-145 (add)
    r = _run(0, {"a": np.array([12], np.uint32)})
    assert int(r["b"][0]) == 13
    assert float(r["cd"][0]) == 13.0


def test_exchange_every_type():
    # test_device_macro_property.cu:632-806 (exchange_int64 ... exchange_float)
    r = _run(13, {})
    for k in ("x_i64", "x_u64", "x_i32", "x_u32", "x_f64", "x_f32"):
        assert r[k][0] == 15, k


def _grid_population():
    i, j, k, w = np.meshgrid(np.arange(2), np.arange(3), np.arange(4), np.arange(5), indexing="ij")
    cols = {"i": i.ravel(), "j": j.ravel(), "k": k.ravel(), "w": w.ravel()}
    return {n: v.astype(np.uint32) for n, v in cols.items()}, 120


def test_host_read():
    # test_host_macro_property.cu:17-77 (ReadTest)
    cols, n = _grid_population()
    cols["a"] = np.arange(n, dtype=np.uint32)
    _errors()
    _run(14, cols, n)
    assert _errors() == 0


def test_host_write():
    # test_host_macro_property.cu:78-151 (WriteTest)
    cols, n = _grid_population()
    cols["a"] = 2 + np.arange(n, dtype=np.uint32)
    r = _run(15, cols, n)
    np.testing.assert_array_equal(r["a"], np.full(n, 12, np.uint32))


def test_host_zero():
    # test_host_macro_property.cu:152-216 (ZeroTest)
    cols, n = _grid_population()
    r = _run(16, cols, n)
    np.testing.assert_array_equal(r["a"], np.ones(n, np.uint32))


def test_host_arithmetic():
    # test_host_macro_property.cu:217-491 (ArithmeticTest)
    _errors()
    S = _sim()
    s = S.Simulation("macro_properties", [17], check_each_step=True)
    s.step(1)
    s.close()
    assert _errors() == 0


def test_contention():
    n = 70001
    ids = (np.arange(n) - n // 2).astype(np.int32)
    r = _run(18, {"id": ids}, n)
    assert (r["a"] == n).all()
    assert (r["cd"] == float(ids.astype(np.int64).sum())).all()
    assert (r["b"].view(np.int32) == ids.min()).all()
    assert (r["c"].view(np.int32) == ids.max()).all()


def test_index_past_a_dimension_is_a_device_error():
    S = _sim()
    s = S.Simulation("macro_properties", [19], check_each_step=True)
    s.set_population("agent", 4, {"a": np.zeros(4, np.uint32)})
    with pytest.raises(S.SimError, match="DeviceError"):
        s.step(1)
    s.close()


@pytest.mark.parametrize("variant", [20, 21], ids=["WriteRead", "ReadWrite"])
def test_read_and_update_in_one_function_is_a_device_error(variant):
    # test_device_macro_property.cu:40-104 (WriteRead, ReadWrite with seatbelts on)
    S = _sim()
    s = S.Simulation("macro_properties", [variant], check_each_step=True)
    s.set_population("agent", 1, {"a": np.array([12], np.uint32)})
    with pytest.raises(S.SimError, match="DeviceError"):
        s.step(1)
    s.close()


def test_separate_functions_may_read_and_update_every_step():
    # the flags clear after every agent function: init / update / read run for several steps
    S = _sim()
    s = S.Simulation("macro_properties", [0], check_each_step=True)
    s.set_population("agent", 1, {"a": np.array([12], np.uint32)})
    s.step(3)
    assert int(s.get("agent", "b", np.uint32)[0]) == 13
    s.close()
