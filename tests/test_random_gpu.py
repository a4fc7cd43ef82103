"""Device random numbers (FLAMEGPU->random, AgentRandom).

The reference draws from curand Philox states (RandomManager.cu:46-113,
AgentRandom.cuh:68-170); no reference test pins those values, and the draws
here come from a counter-based hash instead, so these tests check what the
reference documents instead of values: the ranges and distributions of
every kind of draw (uniform float / double in [0, 1), integers in [min,
max], floating point in [min, max), normal, logNormal, Poisson with the
product-of-uniforms method below mean 10 and transformed rejection above),
that a seed reproduces its draws exactly (with or without step graphs) and
that seeds and steps draw differently, and the seatbelt error for min > max.
Each check is five standard errors wide or a goodness-of-fit p-value above
1e-4, on a fixed seed (deterministic pass or fail).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N = 1 << 18
VARS = {"u_f": np.float32, "u_d": np.float64, "u_i": np.int32, "u_r": np.float32, "n_f": np.float32,
        "n_d": np.float64, "ln_f": np.float32, "p_s": np.uint32, "p_l": np.uint32, "p_1": np.uint32}


def _draws(seed, steps=1, params=(3.5, 250.0), use_graphs=True, n=N):
    from flamegpu2_gb300 import sim
    s = sim.Simulation("random_draws", list(params), steps=steps, seed=seed, use_graphs=use_graphs)
    s.set_population("agent", n, {"u_i": np.zeros(n, np.int32)})
    s.step(steps)
    out = {k: s.get("agent", k, t) for k, t in VARS.items()}
    s.close()
    return out


def _near(x, want, se, what):
    assert abs(x - want) <= 5.0 * se, (what, x, want, se)


def _poisson_fit(counts, mean):
    stats = pytest.importorskip("scipy.stats")
    n = counts.size
    hi = int(stats.poisson.ppf(1.0 - 1e-6, mean))
    lo = int(stats.poisson.ppf(1e-6, mean))
    edges = np.arange(lo, hi + 2)
    obs = np.histogram(np.clip(counts, lo, hi), bins=edges)[0].astype(np.float64)
    exp = stats.poisson.pmf(edges[:-1], mean) * n
    exp[0] += stats.poisson.cdf(lo - 1, mean) * n
    exp[-1] += stats.poisson.sf(hi, mean) * n
    # pool sparse cells so every expected count is at least 5
    o2, e2, ao, ae = [], [], 0.0, 0.0
    for o, e in zip(obs, exp):
        ao += o
        ae += e
        if ae >= 5.0:
            o2.append(ao)
            e2.append(ae)
            ao = ae = 0.0
    if ae > 0.0:
        o2[-1] += ao
        e2[-1] += ae
    o2, e2 = np.array(o2), np.array(e2)
    e2 *= o2.sum() / e2.sum()
    return stats.chisquare(o2, e2).pvalue


def test_uniform_normal_lognormal_distributions():
    stats = pytest.importorskip("scipy.stats")
    d = _draws(17)
    for k in ("u_f", "u_d"):
        u = d[k].astype(np.float64)
        assert u.min() >= 0.0 and u.max() < 1.0, k
        _near(u.mean(), 0.5, np.sqrt(1 / 12 / N), k)
        _near(u.var(), 1 / 12, np.sqrt(1 / 180 / N), k)
    # integers in [-3, 7], each value equally likely
    vals, cnt = np.unique(d["u_i"], return_counts=True)
    assert vals.tolist() == list(range(-3, 8))
    p = 1 / 11
    for c in cnt:
        _near(c / N, p, np.sqrt(p * (1 - p) / N), "u_i")
    r = d["u_r"].astype(np.float64)
    assert r.min() >= 2.0 and r.max() < 5.0
    _near(r.mean(), 3.5, 3.0 * np.sqrt(1 / 12 / N), "u_r")
    for k in ("n_f", "n_d"):
        x = d[k].astype(np.float64)
        assert np.isfinite(x).all(), k
        _near(x.mean(), 0.0, 1 / np.sqrt(N), k)
        _near(x.std(), 1.0, 1 / np.sqrt(2 * N), k)
        assert stats.kstest(x, "norm").pvalue > 1e-4, k
    ln = d["ln_f"].astype(np.float64)
    assert (ln > 0.0).all()
    y = np.log(ln)
    _near(y.mean(), 0.0, 0.5 / np.sqrt(N), "ln_f")
    _near(y.std(), 0.5, 0.5 / np.sqrt(2 * N), "ln_f")


@pytest.mark.parametrize("small,large", [(3.5, 250.0), (9.99, 10.0), (0.2, 5000.0)])
def test_poisson_distribution(small, large):
    # both sides of the switch between the two methods (mean 10), and the
    # default mean (1)
    d = _draws(23, params=(small, large))
    for k, mean in (("p_s", small), ("p_l", large), ("p_1", 1.0)):
        c = d[k].astype(np.float64)
        _near(c.mean(), mean, np.sqrt(mean / N), k)
        _near(c.var(), mean, mean * np.sqrt(2.0 / N) + np.sqrt(mean / N), k)
        assert _poisson_fit(d[k].astype(np.int64), mean) > 1e-4, (k, mean)


def test_poisson_of_non_positive_mean_is_zero():
    d = _draws(5, params=(0.0, -4.0), n=4096)
    assert not d["p_s"].any() and not d["p_l"].any()


def test_draws_reproducible_per_seed_and_distinct_per_step():
    a = _draws(99, n=20_000)
    b = _draws(99, n=20_000, use_graphs=False)
    for k in VARS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    c = _draws(100, n=20_000)
    assert np.mean(a["u_d"] == c["u_d"]) < 1e-3
    two = _draws(99, steps=2, n=20_000)  # the second step's draws
    assert np.mean(a["u_d"] == two["u_d"]) < 1e-3
    # agents draw independently: no two agents share a stream
    assert np.unique(a["u_d"]).size > 19_990


def test_uniform_with_min_above_max_is_a_device_error():
    # AgentRandom.cuh:129-137: with seatbelts on, min > max raises DTHROW
    from flamegpu2_gb300 import sim
    s = sim.Simulation("random_bad_range", [], check_each_step=True)
    s.set_population("agent", 64, {"u_i": np.zeros(64, np.int32)})
    with pytest.raises(sim.SimError, match="DeviceError"):
        s.step(1)
        s.synchronize()
    s.close()
