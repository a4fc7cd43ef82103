"""ctypes front-end of the serial host oracle — TEST INFRASTRUCTURE ONLY.

The oracle (fg_oracle.cpp) is a deterministic serial restatement of the
reference's spatial message build, neighbour iteration, auto spatial sort and
birth/death compaction. Only the tests, the smoke check and the CPU-baseline
leg of bench.py import this module; the product never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfg_oracle.so")
_lock = threading.Lock()
_lib = None


class Grid(C.Structure):
    _fields_ = [
        ("dims", C.c_int32),
        ("min", C.c_float * 3),
        ("max", C.c_float * 3),
        ("radius", C.c_float),
        ("width", C.c_float * 3),
        ("gridDim", C.c_uint32 * 3),
        ("binCount", C.c_uint32),
        ("wrapCompatible", C.c_int32),
    ]


class PredPreyParams(C.Structure):
    _fields_ = [("edge", C.c_float), ("radius", C.c_float), ("p_prey_birth", C.c_float),
                ("p_pred_death", C.c_float), ("step", C.c_float), ("seed", C.c_uint64), ("max_crowd", C.c_uint32)]


class BoidsParams(C.Structure):
    _fields_ = [
        ("min_pos", C.c_float), ("max_pos", C.c_float),
        ("interaction_radius", C.c_float), ("separation_radius", C.c_float),
        ("time_scale", C.c_float), ("global_scale", C.c_float), ("steer_scale", C.c_float),
        ("collision_scale", C.c_float), ("match_scale", C.c_float),
        ("wrap", C.c_int32), ("sort_period", C.c_uint32),
    ]


def build() -> str:
    """Compile the oracle shared library (g++, seconds)."""
    subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            src = os.path.join(_HERE, "fg_oracle.cpp")
            if (not os.path.exists(_LIB_PATH)) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
                build()
            L = C.CDLL(_LIB_PATH)
            P = C.POINTER
            u32p, f32p, i32p = P(C.c_uint32), P(C.c_float), P(C.c_int32)
            L.or_grid_init.argtypes = [P(Grid), C.c_int32, f32p, f32p, C.c_float]
            L.or_approx_exactly_divisible.argtypes = [C.c_float, C.c_float]
            L.or_approx_exactly_divisible.restype = C.c_int32
            L.or_bin.argtypes = [P(Grid), C.c_float, C.c_float, C.c_float]
            L.or_bin.restype = C.c_uint32
            L.or_spatial_build.argtypes = [P(Grid), C.c_uint32, f32p, f32p, f32p, u32p, u32p, u32p]
            L.or_neighbours.argtypes = [P(Grid), u32p, C.c_float, C.c_float, C.c_float, C.c_int32, u32p, C.c_uint32]
            L.or_neighbours.restype = C.c_uint32
            L.or_sort_key.argtypes = [P(Grid), C.c_float, C.c_float, C.c_float]
            L.or_sort_key.restype = C.c_uint32
            L.or_sort_max_bit.argtypes = [P(Grid)]
            L.or_sort_max_bit.restype = C.c_int32
            L.or_stable_sort_perm.argtypes = [C.c_uint32, u32p, C.c_int32, u32p]
            L.or_compact.argtypes = [C.c_uint32, u32p, u32p]
            L.or_compact.restype = C.c_uint32
            L.or_boids_run.argtypes = [P(BoidsParams), C.c_uint32, u32p, f32p, f32p, f32p, f32p, f32p, f32p,
                                       C.c_uint32, C.c_uint32, C.c_int32]
            L.or_count_model.argtypes = [P(Grid), C.c_int32, C.c_uint32, u32p, f32p, f32p, f32p, i32p, u32p, u32p,
                                         f32p, f32p, f32p, u32p]
            L.or_birth_death_run.argtypes = [C.c_uint32, C.c_uint32, f32p, i32p, u32p, u32p, C.c_float, C.c_float,
                                             C.c_uint64, C.c_uint32, C.c_uint32, u32p]
            L.or_birth_death_run.restype = C.c_uint32
            L.or_predprey_run.argtypes = [P(PredPreyParams), C.c_uint32, C.c_uint32, u32p, C.c_uint32, f32p, f32p,
                                          u32p, u32p, u32p, f32p, f32p, u32p]
            L.or_payload_run.argtypes = [P(Grid), C.c_int32, C.c_uint32, C.c_uint32, u32p, f32p, f32p, f32p, f32p,
                                         C.c_uint32, C.c_uint32, C.c_int32]
            L.or_payload_step_sampled.argtypes = [P(Grid), C.c_int32, C.c_uint32, u32p, f32p, f32p, f32p, f32p,
                                                  C.c_uint32, u32p, P(C.c_double)]
            L.or_mix64.argtypes = [C.c_uint64]
            L.or_mix64.restype = C.c_uint64
            L.or_hash_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint32]
            L.or_hash_uniform.restype = C.c_float
            _lib = L
    return _lib


def _p(a, ct):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ct))


def grid(dims, mn, mx, radius) -> Grid:
    g = Grid()
    mn3 = (C.c_float * 3)(*[float(v) for v in list(mn) + [0.0] * (3 - len(mn))])
    mx3 = (C.c_float * 3)(*[float(v) for v in list(mx) + [0.0] * (3 - len(mx))])
    lib().or_grid_init(C.byref(g), int(dims), mn3, mx3, C.c_float(radius))
    return g


def approx_exactly_divisible(x, y) -> bool:
    return bool(lib().or_approx_exactly_divisible(C.c_float(x), C.c_float(y)))


def spatial_build(g: Grid, x, y, z=None):
    """Return (pbm[binCount+1], perm[n], bins[n]) of the stable message build."""
    x = np.ascontiguousarray(x, np.float32)
    y = np.ascontiguousarray(y, np.float32)
    z = None if z is None else np.ascontiguousarray(z, np.float32)
    n = x.shape[0]
    pbm = np.zeros(g.binCount + 1, np.uint32)
    perm = np.zeros(n, np.uint32)
    bins = np.zeros(n, np.uint32)
    lib().or_spatial_build(C.byref(g), n, _p(x, C.c_float), _p(y, C.c_float), _p(z, C.c_float),
                           _p(pbm, C.c_uint32), _p(perm, C.c_uint32), _p(bins, C.c_uint32))
    return pbm, perm, bins


def neighbours(g: Grid, pbm, x, y, z=0.0, wrap=False):
    pbm = np.ascontiguousarray(pbm, np.uint32)
    cap = 4096
    out = np.zeros(cap, np.uint32)
    n = lib().or_neighbours(C.byref(g), _p(pbm, C.c_uint32), x, y, z, int(wrap), _p(out, C.c_uint32), cap)
    if n > cap:
        out = np.zeros(n, np.uint32)
        lib().or_neighbours(C.byref(g), _p(pbm, C.c_uint32), x, y, z, int(wrap), _p(out, C.c_uint32), n)
    return out[:n].copy()


def sort_keys(g: Grid, x, y, z=None):
    L = lib()
    n = len(x)
    return np.array([L.or_sort_key(C.byref(g), float(x[i]), float(y[i]), 0.0 if z is None else float(z[i]))
                     for i in range(n)], np.uint32)


def sort_max_bit(g: Grid) -> int:
    return int(lib().or_sort_max_bit(C.byref(g)))


def stable_sort_perm(keys, bits):
    keys = np.ascontiguousarray(keys, np.uint32)
    perm = np.zeros(keys.shape[0], np.uint32)
    lib().or_stable_sort_perm(keys.shape[0], _p(keys, C.c_uint32), int(bits), _p(perm, C.c_uint32))
    return perm


def compact(alive):
    alive = np.ascontiguousarray(alive, np.uint32)
    out = np.zeros(alive.shape[0], np.uint32)
    k = lib().or_compact(alive.shape[0], _p(alive, C.c_uint32), _p(out, C.c_uint32))
    return out[:k].copy()


def boids_params(min_pos, max_pos, interaction_radius, separation_radius, time_scale, global_scale,
                 steer_scale, collision_scale, match_scale, wrap, sort_period=1) -> BoidsParams:
    return BoidsParams(min_pos, max_pos, interaction_radius, separation_radius, time_scale, global_scale,
                       steer_scale, collision_scale, match_scale, int(wrap), int(sort_period))


def boids_run(p: BoidsParams, state: dict, steps: int, first_step: int = 0, threads: int = 1) -> dict:
    """state: dict of numpy arrays id(u32), x,y,z,fx,fy,fz (f32). Returns a new dict."""
    s = {k: np.array(state[k], dtype=(np.uint32 if k == "id" else np.float32), copy=True) for k in
         ("id", "x", "y", "z", "fx", "fy", "fz")}
    n = s["x"].shape[0]
    lib().or_boids_run(C.byref(p), n, _p(s["id"], C.c_uint32), *[_p(s[k], C.c_float) for k in
                                                                  ("x", "y", "z", "fx", "fy", "fz")],
                       steps, first_step, threads)
    return s


def count_model(g: Grid, wrap: bool, x, y, z=None, ids=None, do_output=None):
    """One step of the reference's neighbour-count test model. Returns dict with
    count, badCount, result_x/y/z and the agent order after the auto sort."""
    n = len(x)
    x = np.array(x, np.float32, copy=True)
    y = np.array(y, np.float32, copy=True)
    z = None if z is None else np.array(z, np.float32, copy=True)
    ids = np.arange(1, n + 1, dtype=np.uint32) if ids is None else np.ascontiguousarray(ids, np.uint32)
    cnt = np.zeros(n, np.uint32)
    bad = np.zeros(n, np.uint32)
    rx, ry, rz = (np.zeros(n, np.float32) for _ in range(3))
    order = np.zeros(n, np.uint32)
    do = None if do_output is None else np.ascontiguousarray(do_output, np.int32)
    lib().or_count_model(C.byref(g), int(wrap), n, _p(ids, C.c_uint32), _p(x, C.c_float), _p(y, C.c_float),
                         _p(z, C.c_float), _p(do, C.c_int32), _p(cnt, C.c_uint32), _p(bad, C.c_uint32), _p(rx, C.c_float),
                         _p(ry, C.c_float), _p(rz, C.c_float), _p(order, C.c_uint32))
    return {"count": cnt, "badCount": bad, "result_x": rx, "result_y": ry, "result_z": rz, "order": order,
            "x": x, "y": y, "z": z}


def birth_death_run(f, counter, ids, next_id, cap, p_death, p_birth, seed, steps, first_step=0):
    """f: [8, n] float32; counter int32[n]; ids uint32[n]. Returns (f, counter, ids, next_id, pops)."""
    n = f.shape[1]
    fb = np.zeros((8, cap), np.float32)
    fb[:, :n] = f
    cb = np.zeros(cap, np.int32)
    cb[:n] = counter
    ib = np.zeros(cap, np.uint32)
    ib[:n] = ids
    nid = np.array([next_id], np.uint32)
    pops = np.zeros(max(steps, 1), np.uint32)
    m = lib().or_birth_death_run(n, cap, _p(fb, C.c_float), _p(cb, C.c_int32), _p(ib, C.c_uint32),
                                 _p(nid, C.c_uint32), p_death, p_birth, seed, steps, first_step,
                                 _p(pops, C.c_uint32))
    return fb[:, :m].copy(), cb[:m].copy(), ib[:m].copy(), int(nid[0]), pops[:steps].copy()


def payload_run(g: Grid, wrap: bool, state: dict, steps: int, first_step: int = 0, sort_period: int = 1,
                threads: int = 1) -> dict:
    """The large spatial workloads' model. state: id (u32), x, y[, z], p0..p3 (f32).
    Returns a new dict in the agents' final order."""
    dims = g.dims
    keys = ["x", "y"] + (["z"] if dims == 3 else [])
    s = {"id": np.array(state["id"], np.uint32, copy=True)}
    for k in keys:
        s[k] = np.array(state[k], np.float32, copy=True)
    n = s["x"].shape[0]
    pay = np.ascontiguousarray(np.stack([np.asarray(state[f"p{k}"], np.float32) for k in range(4)]))
    lib().or_payload_run(C.byref(g), int(wrap), int(sort_period), n, _p(s["id"], C.c_uint32), _p(s["x"], C.c_float),
                         _p(s["y"], C.c_float), _p(s.get("z"), C.c_float), _p(pay, C.c_float), steps, first_step,
                         threads)
    for k in range(4):
        s[f"p{k}"] = pay[k].copy()
    return s


def payload_step_sampled(g: Grid, wrap: bool, state: dict, sample) -> tuple:
    """One serial step of the payload model over the whole population in which
    only the agents at sorted positions `sample` iterate. Returns
    (new state, seconds of sort + build, seconds of the sample's iterate)."""
    dims = g.dims
    s = {"id": np.array(state["id"], np.uint32, copy=True)}
    for k in ["x", "y"] + (["z"] if dims == 3 else []):
        s[k] = np.array(state[k], np.float32, copy=True)
    n = s["x"].shape[0]
    pay = np.ascontiguousarray(np.stack([np.asarray(state[f"p{k}"], np.float32) for k in range(4)]))
    smp = np.ascontiguousarray(sample, np.uint32)
    t = np.zeros(2, np.float64)
    lib().or_payload_step_sampled(C.byref(g), int(wrap), n, _p(s["id"], C.c_uint32), _p(s["x"], C.c_float),
                                  _p(s["y"], C.c_float), _p(s.get("z"), C.c_float), _p(pay, C.c_float),
                                  smp.shape[0], _p(smp, C.c_uint32), _p(t, C.c_double))
    for k in range(4):
        s[f"p{k}"] = pay[k].copy()
    return s, float(t[0]), float(t[1])


def hash_uniform(seed, key, step, stream) -> float:
    return float(lib().or_hash_uniform(seed, key, step, stream))


def predprey_run(params: dict, prey: dict, pred: dict, steps: int, next_prey_id: int, cap: int = None):
    """prey/pred: dicts of x, y (f32) and _id (u32). Returns (prey, pred, next_prey_id)."""
    p = PredPreyParams(params["edge"], params["radius"], params["p_prey_birth"], params["p_pred_death"],
                       params["step"], int(params["seed"]), int(params.get("max_crowd", 4)))
    n = len(prey["x"])
    cap = cap or max(4 * n, 1024)
    px = np.zeros(cap, np.float32); px[:n] = prey["x"]
    py = np.zeros(cap, np.float32); py[:n] = prey["y"]
    pid = np.zeros(cap, np.uint32); pid[:n] = prey["_id"]
    qx = np.array(pred["x"], np.float32, copy=True)
    qy = np.array(pred["y"], np.float32, copy=True)
    qid = np.array(pred["_id"], np.uint32, copy=True)
    nprey = np.array([n], np.uint32)
    npred = np.array([len(qx)], np.uint32)
    nid = np.array([next_prey_id], np.uint32)
    lib().or_predprey_run(C.byref(p), steps, 0, _p(nprey, C.c_uint32), cap, _p(px, C.c_float), _p(py, C.c_float),
                          _p(pid, C.c_uint32), _p(nid, C.c_uint32), _p(npred, C.c_uint32), _p(qx, C.c_float),
                          _p(qy, C.c_float), _p(qid, C.c_uint32))
    m, q = int(nprey[0]), int(npred[0])
    return ({"x": px[:m].copy(), "y": py[:m].copy(), "_id": pid[:m].copy()},
            {"x": qx[:q].copy(), "y": qy[:q].copy(), "_id": qid[:q].copy()}, int(nid[0]))


def state_mix_run(pops: dict, next_id: int, steps: int, first_step: int = 0):
    """The "state_mix" model of examples/state_tests/state_tests.cu, serially
    (pure Python: small populations only). pops: {"A": {"_id", "v", "x"},
    "B": {...}} of numpy arrays. Per function, following the reference:
      condition  failing agents first, passing ones after, each in order
                 (CUDAFatAgent::processFunctionCondition, CUDAFatAgent.cu:186-236);
      death      the passing agents that return DEAD are removed, order kept
                 (CUDAFatAgent::processDeath, CUDAFatAgent.cu:105-137);
      transition the surviving passing agents are appended to the end state
                 (CUDAFatAgent::transitionState, CUDAFatAgent.cu:139-184);
      births     appended to the output state after that, in parent order,
                 with consecutive new ids (CUDASimulation.cu:1064-1079,
                 CUDAAgentStateList.cu:189-250).
    Returns (pops, next_id)."""
    f32 = np.float32
    st = {k: [(int(i), int(v), f32(x)) for i, v, x in zip(p["_id"], p["v"], p["x"])] for k, p in pops.items()}

    def run(src, dst, cond, body):
        nonlocal next_id
        fails = [a for a in st[src] if not cond(a)]
        passes = [a for a in st[src] if cond(a)]
        survivors, births = [], []
        for a in passes:
            new, child, alive = body(a)
            if child is not None:
                births.append(child)
            if alive:
                survivors.append(new)
        births = [(next_id + k, v, x) for k, (v, x) in enumerate(births)]
        next_id += len(births)
        if src == dst:
            st[src] = fails + survivors + births
        else:
            st[src] = fails
            st[dst] = st[dst] + survivors + births

    for s in range(first_step, first_step + steps):
        def ab(a):
            i, v, x = a
            x = f32(x + f32(1.0))
            child = (v + 1000, x) if i % 5 == 0 else None
            return (i, v, x), child, i % 7 != 0
        run("A", "B", lambda a: (a[0] + s) % 3 == 0, ab)
        run("B", "A", lambda a: a[0] % 2 == 0, lambda a: ((a[0], a[1], f32(a[2] * f32(2.0))), None, True))
        run("A", "A", lambda a: a[2] > f32(10.0), lambda a: ((a[0], a[1], f32(a[2] - f32(10.0))), None, True))
    out = {}
    for k, lst in st.items():
        out[k] = {"_id": np.array([a[0] for a in lst], np.uint32), "v": np.array([a[1] for a in lst], np.uint32),
                  "x": np.array([a[2] for a in lst], np.float32)}
    return out, next_id


def cross_birth_run(pops: dict, next_id: dict, steps: int, first_step: int = 0):
    """The "cross_birth" model of examples/agent_creation_tests/agent_creation.cu,
    serially (pure Python: small populations only). pops: {("prey", "default"),
    ("hunter", "roam"), ("hunter", "rest")} -> {"_id", "v", "x"}; next_id:
    {agent: next id}. Per function, as state_mix_run, with the births appended
    to the output agent's list after the death compaction and the transition,
    with that agent's next ids (CUDASimulation.cu:1062-1080,
    CUDAAgent.cu:427-450, CUDAAgentStateList.cu:189-250). Returns (pops, next_id)."""
    f32 = np.float32
    st = {k: [(int(i), int(v), f32(x)) for i, v, x in zip(p["_id"], p["v"], p["x"])] for k, p in pops.items()}
    nid = dict(next_id)

    def run(src, dst, out, cond, body):
        fails = [a for a in st[src] if not cond(a)]
        passes = [a for a in st[src] if cond(a)]
        survivors, births = [], []
        for a in passes:
            new, child, alive = body(a)
            if child is not None:
                births.append(child)
            if alive:
                survivors.append(new)
        if src == dst:
            st[src] = fails + survivors
        else:
            st[src] = fails
            st[dst] = st[dst] + survivors
        agent = out[0]
        st[out] = st[out] + [(nid[agent] + k, v, x) for k, (v, x) in enumerate(births)]
        nid[agent] += len(births)

    P, R, S = ("prey", "default"), ("hunter", "roam"), ("hunter", "rest")
    for step in range(first_step, first_step + steps):
        def spawn(a):
            i, v, x = a
            x = f32(x + f32(1.0))
            child = (v + 1000, f32(x * f32(0.5))) if (i + step) % 3 == 0 else None
            return (i, v, x), child, i % 11 != 0

        def hunt(a):
            i, v, x = a
            x = f32(x + f32(2.0))
            child = (v + 7, x) if i % 5 == 0 else None
            return (i, v, x), child, True

        def wake(a):
            i, v, x = a
            return (i, v, f32(x - f32(1.0))), None, True

        run(P, P, R, lambda a: True, spawn)
        run(R, S, P, lambda a: a[0] % 2 == 0, hunt)
        run(S, R, R, lambda a: True, wake)
    out = {k: {"_id": np.array([a[0] for a in v], np.uint32), "v": np.array([a[1] for a in v], np.uint32),
               "x": np.array([a[2] for a in v], np.float32)} for k, v in st.items()}
    return out, nid
