"""Host reductions that run user operators or histograms on the device:
HostAgentAPI::count / histogramEven / reduce / transformReduce
(include/flamegpu/runtime/agent/HostAgentAPI.cuh:226-268) over every scalar
type, as the reference's host-reduction tests use them
(tests/test_cases/runtime/agent/host_reduction/test_count.cu,
test_histogram_even.cu, test_reduce.cu with a max operator,
test_transform_reduce.cu with "a <= 0 ? 1 : 0" and a sum), checked against
numpy on seeded populations; the model is host_reductions in
examples/host_api/host_reduction_models.cu. Integer results are exact (sums
wrap in the variable's type, as the device arithmetic does); floating-point
sums are compared within a relative tolerance of 1e-5 (float) / 1e-12 (double),
since the device folds in a tree order.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TYPES = [("f", np.float32), ("d", np.float64), ("i8", np.int8), ("u8", np.uint8), ("i16", np.int16),
         ("u16", np.uint16), ("i32", np.int32), ("u32", np.uint32), ("i64", np.int64), ("u64", np.uint64)]


def _population(n, seed):
    rng = np.random.default_rng(seed)
    cols = {}
    for k, t in TYPES:
        if np.issubdtype(t, np.floating):
            v = rng.uniform(-5.0, 25.0, n).astype(t)
            v[rng.random(n) < 0.05] = 0
        elif np.issubdtype(t, np.signedinteger):
            v = rng.integers(-5, 25, n).astype(t)
        else:
            v = rng.integers(0, 25, n).astype(t)
        cols[k] = v
    if n > 2:
        cols["i64"][0] = np.int64(1) << 50
        cols["u64"][1] = np.uint64(1) << 60
        cols["i32"][2] = -(1 << 30)
    return cols


def _run(n, seed):
    from flamegpu2_gb300 import sim
    s = sim.Simulation("host_reductions")
    s.set_population("agent", n, _population(n, seed))
    s.step(1)
    s.synchronize()
    s.close()
    L = C.CDLL(sim.MODELS_LIB)
    out = np.zeros(10 * 16, np.uint64)
    L.fg_test_host_reductions(out.ctypes.data_as(C.c_void_p))
    return out.reshape(10, 16)


def _as(word, t):
    return np.frombuffer(np.uint64(word).tobytes()[:np.dtype(t).itemsize], dtype=t)[0]


@pytest.mark.parametrize("n,seed", [(50_000, 3), (300, 4), (1, 5), (0, 6)])
def test_count_histogram_reduce_transform_reduce(n, seed):
    res = _run(n, seed)
    pop = _population(n, seed)
    for k, (name, t) in enumerate(TYPES):
        col = pop[name]
        s = res[k]
        assert int(s[0]) == int(np.count_nonzero(col == 0)), name
        # reduce(max, init 0): max of the values and init
        want_max = max([col.max(), t(0)]) if n else t(0)
        assert _as(s[1], t) == want_max, name
        # reduce(sum, init 7): init combined once
        got = _as(s[2], t)
        if np.issubdtype(t, np.floating):
            want = float(np.sum(col.astype(np.float64))) + 7.0
            np.testing.assert_allclose(float(got), want, rtol=1e-5 if t == np.float32 else 1e-12, atol=1e-3, err_msg=name)
        else:
            bits = 8 * np.dtype(t).itemsize
            total = (sum(int(x) for x in col.tolist()) + 7) % (1 << bits)
            assert int(np.array(got).astype(np.uint64 if bits == 64 else np.int64)) % (1 << bits) == total, name
        assert int(_as(s[3], np.int32)) == int(np.count_nonzero(col <= 0)), name
        inside = col[(col >= 0) & (col < 20)].astype(np.float64)
        bins = np.minimum(np.floor(inside * (10.0 / 20.0)).astype(np.int64), 9)
        np.testing.assert_array_equal(s[4:14].astype(np.int64), np.bincount(bins, minlength=10), err_msg=name)
        assert int(s[14]) == 1, name

