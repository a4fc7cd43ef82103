"""Seeded synthetic populations (counter-based, reproducible on any host).

Value i of stream s under seed k is SplitMix64's finaliser (Steele, Lea &
Flood 2014) of mix64(k ^ (s << 32)) + (i + 1) * 0x9E3779B97F4A7C15; uniforms
use its top 24 bits, so a float32 uniform in [lo, hi) is lo + (hi - lo) * u
evaluated in float32. Used by the benchmark and the tests for the workloads
(Boids, birth/death, large spatial, ensembles).
"""
import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def mix64(z):
    z = np.asarray(z, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


def bits(seed: int, stream: int, n: int, offset: int = 0) -> np.ndarray:
    base = mix64(np.uint64((seed ^ (stream << 32)) & 0xFFFFFFFFFFFFFFFF))
    i = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        return mix64(base + i * _GOLDEN)


def uniform(seed: int, stream: int, n: int, lo: float, hi: float) -> np.ndarray:
    u = (bits(seed, stream, n) >> np.uint64(40)).astype(np.float32) * np.float32(1.0 / 16777216.0)
    return (np.float32(lo) + (np.float32(hi) - np.float32(lo)) * u).astype(np.float32)


def normal(seed: int, stream: int, n: int, mean: float = 0.0, sigma: float = 1.0) -> np.ndarray:
    u1 = 1.0 - (bits(seed, stream, n) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
    u2 = (bits(seed, stream + 1000, n) >> np.uint64(11)).astype(np.float64) / 9007199254740992.0
    return (mean + sigma * np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)).astype(np.float32)


# ------------------------------------------------------------------ workloads

BOIDS_SMALL = dict(  # 16,384 agents in [0,64)^3, r = 2 (32^3 bins), wrapped, 10 steps
    n=16384, min_pos=0.0, max_pos=64.0, interaction_radius=2.0, separation_radius=0.5, time_scale=0.05,
    global_scale=0.15, steer_scale=0.005, collision_scale=0.01, match_scale=0.03, wrap=1, sort_period=1,
    steps=10, seed=0)


def boids_params(cfg: dict) -> list:
    return [cfg["min_pos"], cfg["max_pos"], cfg["interaction_radius"], cfg["separation_radius"], cfg["time_scale"],
            cfg["global_scale"], cfg["steer_scale"], cfg["collision_scale"], cfg["match_scale"], cfg["wrap"],
            cfg["sort_period"]]


def boids_population(n: int, lo: float, hi: float, seed: int) -> dict:
    hi_open = np.nextafter(np.float32(hi), np.float32(lo))  # keep positions strictly inside [lo, hi)
    pop = {"_id": np.arange(1, n + 1, dtype=np.uint32)}
    for s, k in enumerate(("x", "y", "z")):
        pop[k] = np.minimum(uniform(seed, s, n, lo, hi), hi_open)
    for s, k in enumerate(("fx", "fy", "fz")):
        pop[k] = uniform(seed, 3 + s, n, -1.0, 1.0)
    return pop


def birth_death_population(n: int, seed: int) -> dict:
    pop = {"_id": np.arange(1, n + 1, dtype=np.uint32), "counter": np.zeros(n, np.int32)}
    for v in range(8):
        pop[f"f{v}"] = uniform(seed, v, n, 0.0, 1.0)
    return pop


def predprey_population(n_prey: int, n_pred: int, edge: float, seed: int):
    """Prey and predators uniform in [0, edge)^2; ids 1..n per agent type."""
    hi = np.nextafter(np.float32(edge), np.float32(0))
    prey = {"_id": np.arange(1, n_prey + 1, dtype=np.uint32),
            "x": np.minimum(uniform(seed, 10, n_prey, 0.0, edge), hi),
            "y": np.minimum(uniform(seed, 11, n_prey, 0.0, edge), hi)}
    pred = {"_id": np.arange(1, n_pred + 1, dtype=np.uint32),
            "x": np.minimum(uniform(seed, 12, n_pred, 0.0, edge), hi),
            "y": np.minimum(uniform(seed, 13, n_pred, 0.0, edge), hi)}
    return prey, pred


def ensemble_instances(count: int, seed: int = 1000, n_lo: int = 1024, n_hi: int = 1 << 20):
    """Boids ensemble instances: population log-uniform in [n_lo, n_hi], radius
    uniform in [1, 4], domain edge 4 r cbrt(N / 64) rounded up to a whole number
    of radii (so the wrapped iterator's radius divides the width)."""
    out = []
    for i in range(count):
        u = float((bits(seed + i, 0, 1) >> np.uint64(11))[0]) / 9007199254740992.0
        n = int(round(np.exp(np.log(n_lo) + u * (np.log(n_hi) - np.log(n_lo)))))
        r = float(uniform(seed + i, 1, 1, 1.0, 4.0)[0])
        cells = int(np.ceil(4.0 * np.cbrt(n / 64.0)))
        edge = float(np.float32(r) * np.float32(cells))
        out.append({"n": n, "radius": r, "edge": edge, "seed": seed + i})
    return out
