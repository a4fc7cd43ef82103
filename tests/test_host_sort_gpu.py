"""HostAgentAPI::sort (HostAgentAPI.cuh:287-302; the reference radix-sorts
(key, row) pairs with CUB and gathers every variable): ascending and
descending, one key and two, every scalar width, a bit subrange, through
host_sort in examples/host_api/host_sort_models.cu, against numpy's stable
sort of the same order-preserving key bits (ties keep their earlier order)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bits(a, desc=False, begin=0, end=None):
    """The unsigned key whose ascending order is a's (descending: inverted)."""
    w = a.dtype.itemsize * 8
    u = a.view({1: np.uint8, 2: np.uint16, 4: np.uint32, 8: np.uint64}[a.dtype.itemsize]).astype(np.uint64)
    sign = np.uint64(1) << np.uint64(w - 1)
    full = np.uint64((1 << w) - 1) if w < 64 else np.uint64(0xFFFFFFFFFFFFFFFF)
    if np.issubdtype(a.dtype, np.floating):
        u = np.where(u & sign, u ^ full, u ^ sign)
    elif np.issubdtype(a.dtype, np.signedinteger):
        u = u ^ sign
    if desc:
        u = ~u & full
    end = w if end is None else end
    u = u >> np.uint64(begin)
    if end - begin < 64:
        u = u & np.uint64((1 << (end - begin)) - 1)
    return u


def _pop(n, seed):
    rng = np.random.default_rng(seed)
    return {"k": np.arange(n, dtype=np.uint32),
            "f": rng.uniform(-50, 50, n).astype(np.float32),
            "d": rng.normal(0, 1e3, n),
            "i": rng.integers(-20, 20, n).astype(np.int32),
            "u": rng.integers(0, 1 << 62, n, dtype=np.uint64) >> rng.integers(0, 60, n).astype(np.uint64),
            "c": rng.integers(-128, 128, n).astype(np.int8),
            "h": rng.integers(0, 1 << 16, n).astype(np.uint16)}


def _expected_order(mode, p):
    if mode == 0:
        return np.argsort(_bits(p["f"]), kind="stable")
    if mode == 1:
        return np.argsort(_bits(p["f"], desc=True), kind="stable")
    if mode == 2:
        return np.lexsort((_bits(p["f"], desc=True), _bits(p["i"])))
    if mode == 3:
        return np.argsort(_bits(p["u"], desc=True), kind="stable")
    if mode == 4:
        return np.argsort(_bits(p["c"]), kind="stable")
    if mode == 5:
        return np.argsort(_bits(p["d"], begin=4, end=60), kind="stable")
    return np.argsort(_bits(p["h"], desc=True), kind="stable")


@pytest.mark.parametrize("mode", range(7))
@pytest.mark.parametrize("n", [1, 777, 100_003])
def test_host_sort_matches_stable_numpy(mode, n):
    from flamegpu2_gb300 import sim
    p = _pop(n, 31 * mode + n)
    s = sim.Simulation("host_sort", [mode])
    s.set_population("agent", n, p)
    s.step(1)
    k = s.get("agent", "k", np.uint32)
    got = {v: s.get("agent", v, p[v].dtype) for v in ("f", "i", "u", "c")}
    s.close()
    order = _expected_order(mode, p)
    np.testing.assert_array_equal(k, order.astype(np.uint32))
    for v, col in got.items():  # every variable moved with its agent
        np.testing.assert_array_equal(col, p[v][order], err_msg=v)
