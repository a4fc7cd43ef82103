"""Host environment arrays by element and as a whole, the reference's
HostAgentAPI / HostEnvironment / HostRandom type names, and host random
numbers (HostRandom.cuh:22-66), through host_env_random in
examples/host_api/host_env_models.cu (the calls of the reference's
host_functions example, examples/cpp/host_functions/src/main.cu:8-62)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _env(s, name, ctype, n=None):
    from flamegpu2_gb300 import sim
    buf = (ctype * n)() if n else ctype()
    sim._check(sim.core().fgs_get_environment(s._h, name.encode(), C.byref(buf), C.sizeof(buf)))
    return list(buf) if n else buf.value


def _run(seed, n=1000):
    from flamegpu2_gb300 import sim
    s = sim.Simulation("host_env_random", seed=seed)
    s.set_population("agent", n, {"x": np.arange(n, dtype=np.float32)})
    s.step(1)
    out = {"u64_sum": _env(s, "u64_sum", C.c_uint64), "u64_sum_array": _env(s, "u64_sum_array", C.c_uint64),
           "arr_old2": _env(s, "arr_old2", C.c_int), "arr_sum_before": _env(s, "arr_sum_before", C.c_int),
           "arr": _env(s, "arr", C.c_int, 4), "count": _env(s, "count", C.c_uint32),
           "hist": _env(s, "hist", C.c_uint32, 8),
           "random": (_env(s, "r_uniform", C.c_double), _env(s, "r_normal", C.c_double),
                      _env(s, "r_lognormal", C.c_double), _env(s, "r_int", C.c_int), _env(s, "r_poisson", C.c_uint32))}
    s.close()
    return out


def test_environment_arrays_agent_api_and_histogram():
    r = _run(5)
    assert r["u64_sum"] == r["u64_sum_array"] == 36
    assert r["arr_old2"] == 3 and r["arr_sum_before"] == 1 + 2 + 30 + 4
    assert r["arr"] == [5, 6, 7, 8]
    assert r["count"] == 1000
    # x = 0 .. 999 over 8 bins of width 128 from -0.5
    assert r["hist"] == [128] * 7 + [1000 - 7 * 128]


def test_host_random_ranges_and_seeding():
    a, b, c = _run(5)["random"], _run(5)["random"], _run(6)["random"]
    u, nrm, ln, i, p = a
    assert 0.0 <= u < 1.0 and ln > 0.0 and 1 <= i <= 10 and p >= 0 and np.isfinite(nrm)
    assert a == b          # the seed reproduces the host draws
    assert a[0] != c[0]    # another seed draws differently
