"""ctypes binding of the simulation C ABI (include/flamegpu_gb300/fg_sim.h).

Drives CUDASimulation runs of the models registered in libfg_models.so from
Python (the tests and the benchmark). No computation happens here: every
step runs in the native libraries, and loading fails loudly without them.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import capi

MODELS_LIB = os.path.join(capi.LIBDIR, "libfg_models.so")

SIM_EXPORTS = [
    "fgs_register_model", "fgs_list_models", "fgs_last_error", "fgs_create", "fgs_destroy", "fgs_configure",
    "fgs_set_population", "fgs_set_population_device", "fgs_get_count", "fgs_get_variable", "fgs_get_population",
    "fgs_get_variable_device", "fgs_step", "fgs_simulate", "fgs_synchronize", "fgs_set_environment",
    "fgs_get_environment", "fgs_stream", "fgs_stats", "fgs_step_times", "fgs_profile_ops", "fgs_take_profile",
    "fgs_set_stage_bytes", "fgs_reset_population_device", "fgs_time_ops_in_graphs", "fgs_harvest_profile",
    "fgs_export", "fgs_load_state", "fgs_set_log", "fgs_run_log", "fgs_agent_steps", "fgs_set_config",
    "fgs_get_config", "fgs_time_op_in_graphs",
]

_lock = threading.Lock()
_core = None
_models = None


class SimError(RuntimeError):
    pass


def core():
    """libflamegpu2_gb300.so with the simulation ABI prototypes, plus the model library."""
    global _core, _models
    with _lock:
        if _core is None:
            L = capi.lib()
            vp, u32, i32, sz = C.c_void_p, C.c_uint32, C.c_int32, C.c_size_t
            L.fgs_last_error.restype = C.c_char_p
            L.fgs_list_models.argtypes = [C.c_char_p, sz]
            L.fgs_create.argtypes = [C.c_char_p, C.POINTER(C.c_double), i32, i32]
            L.fgs_create.restype = vp
            L.fgs_destroy.argtypes = [vp]
            L.fgs_configure.argtypes = [vp, u32, C.c_uint64, i32, i32]
            L.fgs_set_population.argtypes = [vp, C.c_char_p, C.c_char_p, u32, i32, C.POINTER(C.c_char_p),
                                             C.POINTER(vp)]
            L.fgs_set_population_device.argtypes = L.fgs_set_population.argtypes
            L.fgs_get_count.argtypes = [vp, C.c_char_p, C.c_char_p, C.POINTER(u32)]
            L.fgs_get_variable.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, vp, sz]
            L.fgs_get_population.argtypes = [vp, C.c_char_p, C.c_char_p, i32, C.POINTER(C.c_char_p), C.POINTER(vp), u32,
                                             C.POINTER(u32)]
            L.fgs_get_variable_device.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_char_p, vp, sz]
            L.fgs_step.argtypes = [vp, u32]
            L.fgs_agent_steps.argtypes = [vp, C.POINTER(C.c_uint64)]
            L.fgs_set_config.argtypes = [vp, C.c_char_p, C.c_char_p]
            L.fgs_time_op_in_graphs.argtypes = [vp, C.c_char_p]
            L.fgs_get_config.argtypes = [vp, C.c_char_p, C.c_char_p, C.c_size_t]
            L.fgs_simulate.argtypes = [vp]
            L.fgs_synchronize.argtypes = [vp]
            L.fgs_set_environment.argtypes = [vp, C.c_char_p, vp, sz]
            L.fgs_get_environment.argtypes = [vp, C.c_char_p, vp, sz]
            L.fgs_stream.argtypes = [vp, C.POINTER(vp)]
            L.fgs_stats.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(u32), C.POINTER(u32)]
            L.fgs_step_times.argtypes = [vp, C.POINTER(C.c_double), u32, C.POINTER(u32)]
            L.fgs_profile_ops.argtypes = [vp, i32]
            L.fgs_set_stage_bytes.argtypes = [vp, u32]
            L.fgs_reset_population_device.argtypes = [vp, C.c_char_p, C.c_char_p, u32, i32, C.POINTER(C.c_char_p),
                                                      C.POINTER(vp), u32]
            L.fgs_take_profile.argtypes = [vp, C.c_char_p, sz]
            L.fgs_time_ops_in_graphs.argtypes = [vp, i32]
            L.fgs_harvest_profile.argtypes = [vp]
            L.fgs_export.argtypes = [vp, C.c_char_p]
            L.fgs_load_state.argtypes = [vp, C.c_char_p]
            L.fgs_set_log.argtypes = [vp, i32, C.c_char_p, u32]
            L.fgs_run_log.argtypes = [vp, C.c_char_p, sz, C.POINTER(sz)]
            _core = L
        if _models is None:
            if not os.path.exists(MODELS_LIB):
                raise RuntimeError(f"{MODELS_LIB} is missing: run flamegpu2_gb300.build.build() first")
            _models = C.CDLL(MODELS_LIB, mode=C.RTLD_GLOBAL)
    return _core


def models() -> list[str]:
    buf = C.create_string_buffer(4096)
    core().fgs_list_models(buf, 4096)
    return [m for m in buf.value.decode().split(",") if m]


def _check(rc):
    if rc != 0:
        raise SimError(core().fgs_last_error().decode())


class Simulation:
    """One CUDASimulation of a registered model."""

    def __init__(self, model: str, params=(), device: int = 0, steps: int = 1, seed: int = 0,
                 use_graphs: bool = True, check_each_step: bool = False):
        L = core()
        self._lib = L
        self._name_arrays = {}
        self._last_ptrs = {}
        arr = (C.c_double * max(1, len(params)))(*[float(p) for p in params])
        self._h = L.fgs_create(model.encode(), arr, len(params), device)
        if not self._h:
            raise SimError(L.fgs_last_error().decode())
        self.configure(steps, seed, use_graphs, check_each_step)

    def close(self):
        if getattr(self, "_h", None):
            core().fgs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def configure(self, steps=1, seed=0, use_graphs=True, check_each_step=False):
        _check(core().fgs_configure(self._h, steps, seed, int(use_graphs), int(check_each_step)))

    def _names(self, names) -> "C.Array":
        """The C array of column names, built once per distinct tuple of names."""
        key = tuple(names)
        cn = self._name_arrays.get(key)
        if cn is None:
            cn = (C.c_char_p * max(1, len(key)))(*[k.encode() for k in key])
            self._name_arrays[key] = cn
        return cn

    def _pointers(self, slot: str, names: tuple, arrs: list) -> "C.Array":
        """The C array of the columns' data pointers. A call passing the same
        (contiguous) array objects as the previous one through this slot reuses
        its array; the slot keeps those arrays alive, so their addresses hold."""
        last = self._last_ptrs.get(slot)
        if last is not None and last[0] == names and len(last[1]) == len(arrs) and \
                all(x is y for x, y in zip(last[1], arrs)):
            return last[2]
        cp = (C.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])
        self._last_ptrs[slot] = (names, arrs, cp)
        return cp

    def set_population(self, agent: str, n: int, columns: dict, state: str = "default"):
        names = tuple(columns)
        arrs = [np.ascontiguousarray(columns[k]) for k in names]
        for k, a in zip(names, arrs):
            if a.shape[0] != n:
                raise ValueError(f"column {k} has {a.shape[0]} rows, expected {n}")
        cp = self._pointers("set", names, arrs)
        _check(self._lib.fgs_set_population(self._h, agent.encode(), state.encode(), n, len(names), self._names(names),
                                            cp))

    def set_population_device(self, agent: str, n: int, columns: dict, state: str = "default"):
        """columns: name -> torch CUDA tensor (kept alive by the caller until this returns)."""
        names = list(columns)
        cn = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
        cp = (C.c_void_p * max(1, len(names)))(*[columns[k].data_ptr() for k in names])
        _check(core().fgs_set_population_device(self._h, agent.encode(), state.encode(), n, len(names), cn, cp))

    def reset_population_device(self, agent: str, n: int, columns: dict, next_id: int, state: str = "default"):
        """Replace the population from torch CUDA tensors holding every variable (incl. _id)."""
        names = list(columns)
        cn = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
        cp = (C.c_void_p * max(1, len(names)))(*[columns[k].data_ptr() for k in names])
        _check(core().fgs_reset_population_device(self._h, agent.encode(), state.encode(), n, len(names), cn, cp,
                                                  next_id))

    def count(self, agent: str, state: str = "default") -> int:
        n = C.c_uint32(0)
        _check(core().fgs_get_count(self._h, agent.encode(), state.encode(), C.byref(n)))
        return n.value

    def get(self, agent: str, var: str, dtype, elements: int = 1, state: str = "default") -> np.ndarray:
        n = self.count(agent, state)
        out = np.empty((n, elements) if elements > 1 else n, dtype=dtype)
        _check(core().fgs_get_variable(self._h, agent.encode(), state.encode(), var.encode(),
                                       out.ctypes.data, out.nbytes))
        return out

    def get_population(self, agent: str, outs: dict, state: str = "default") -> int:
        """Fill caller arrays (name -> numpy array with room for every agent); returns the count."""
        names = tuple(outs)
        arrs = [outs[k] for k in names]
        for k, a in zip(names, arrs):
            if not a.flags.c_contiguous:
                raise ValueError(f"output array {k} is not contiguous")
        cp = self._pointers("get", names, arrs)
        cap = min(o.shape[0] for o in arrs)
        n = C.c_uint32()
        _check(self._lib.fgs_get_population(self._h, agent.encode(), state.encode(), len(names), self._names(names), cp,
                                            cap, C.byref(n)))
        return n.value

    def get_device(self, agent: str, var: str, dst, state: str = "default"):
        """Copy a variable's device column into a torch tensor (async on the sim stream)."""
        _check(core().fgs_get_variable_device(self._h, agent.encode(), state.encode(), var.encode(),
                                              dst.data_ptr(), dst.numel() * dst.element_size()))

    def step(self, n: int = 1):
        _check(self._lib.fgs_step(self._h, n))

    def set_config(self, key: str, value):
        """SimulationConfig() / CUDAConfig() item by name."""
        v = ("true" if value else "false") if isinstance(value, bool) else str(value)
        _check(core().fgs_set_config(self._h, key.encode(), v.encode()))

    def get_config(self, key: str) -> str:
        buf = C.create_string_buffer(4096)
        _check(core().fgs_get_config(self._h, key.encode(), buf, 4096))
        return buf.value.decode()

    def agent_steps(self) -> int:
        """Agents summed over the steps run (each step with the populations that entered it)."""
        v = C.c_uint64()
        _check(core().fgs_agent_steps(self._h, C.byref(v)))
        return v.value

    def simulate(self):
        _check(core().fgs_simulate(self._h))

    def synchronize(self):
        _check(core().fgs_synchronize(self._h))

    def set_env(self, name: str, value, ctype=C.c_float):
        v = ctype(value)
        _check(core().fgs_set_environment(self._h, name.encode(), C.byref(v), C.sizeof(v)))

    def get_env(self, name: str, ctype=C.c_float):
        v = ctype()
        _check(core().fgs_get_environment(self._h, name.encode(), C.byref(v), C.sizeof(v)))
        return v.value

    @property
    def stream(self) -> int:
        p = C.c_void_p()
        _check(core().fgs_stream(self._h, C.byref(p)))
        return p.value or 0

    def stats(self) -> dict:
        g, k, s = C.c_uint64(), C.c_uint32(), C.c_uint32()
        _check(core().fgs_stats(self._h, C.byref(g), C.byref(k), C.byref(s)))
        return {"graph_launches": g.value, "kernels_per_step": k.value, "step_counter": s.value}

    def step_times(self, cap: int = 100000) -> np.ndarray:
        buf = (C.c_double * cap)()
        n = C.c_uint32()
        _check(core().fgs_step_times(self._h, buf, cap, C.byref(n)))
        return np.array(buf[:n.value])

    def set_stage_bytes(self, nbytes: int):
        _check(core().fgs_set_stage_bytes(self._h, nbytes))

    def profile_ops(self, enable: bool = True):
        _check(core().fgs_profile_ops(self._h, int(enable)))

    def export_data(self, path: str):
        _check(core().fgs_export(self._h, str(path).encode()))

    def load_state(self, path: str):
        _check(core().fgs_load_state(self._h, str(path).encode()))

    def set_step_log(self, entries, frequency: int = 1):
        """entries: "count:agent:state", "mean|sd|min|max|sum:agent:state:var", "env:name"."""
        _check(core().fgs_set_log(self._h, 0, ";".join(entries).encode(), frequency))

    def set_exit_log(self, entries):
        _check(core().fgs_set_log(self._h, 1, ";".join(entries).encode(), 1))

    def run_log(self) -> dict:
        import json
        need = C.c_size_t()
        _check(core().fgs_run_log(self._h, None, 0, C.byref(need)))
        buf = C.create_string_buffer(need.value)
        _check(core().fgs_run_log(self._h, buf, need.value, C.byref(need)))
        return json.loads(buf.value.decode())

    def time_ops_in_graphs(self, enable: bool = True):
        _check(core().fgs_time_ops_in_graphs(self._h, int(enable)))

    def time_op_in_graphs(self, label):
        """Time one operation (e.g. "fn:inputdata") by events inside the multi-step graphs (None: off)."""
        _check(core().fgs_time_op_in_graphs(self._h, label.encode() if label else None))

    def harvest_profile(self):
        _check(core().fgs_harvest_profile(self._h))

    def take_profile(self) -> dict:
        """label -> (total_ms, count) of the operations issued since the last call."""
        buf = C.create_string_buffer(1 << 16)
        _check(core().fgs_take_profile(self._h, buf, 1 << 16))
        out = {}
        for rec in buf.value.decode().split(";"):
            if rec:
                label, ms, cnt = rec.rsplit(",", 2)
                out[label] = (float(ms), int(cnt))
        return out


ENSEMBLE_EXPORTS = ["fge_create", "fge_destroy", "fge_configure", "fge_add_run", "fge_set_run_property",
                    "fge_simulate", "fge_get_count", "fge_get_variable", "fge_stats", "fge_step_time",
                    "fge_set_tuning", "fge_tuning"]
_ens_ready = False


def _ens():
    global _ens_ready
    L = core()
    if not _ens_ready:
        vp, u32, i32, sz = C.c_void_p, C.c_uint32, C.c_int32, C.c_size_t
        L.fge_create.argtypes = [C.c_char_p, C.POINTER(C.c_double), i32, i32]
        L.fge_create.restype = vp
        L.fge_destroy.argtypes = [vp]
        L.fge_configure.argtypes = [vp, i32, i32, u32]
        L.fge_set_tuning.argtypes = [vp, i32, C.c_char_p]
        L.fge_tuning.argtypes = [vp, C.c_char_p, sz]
        L.fge_add_run.argtypes = [vp, u32, C.c_uint64, C.c_char_p, u32, i32, C.POINTER(C.c_char_p), C.POINTER(vp),
                                  C.c_char_p, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float]
        L.fge_set_run_property.argtypes = [vp, u32, C.c_char_p, vp, sz]
        L.fge_simulate.argtypes = [vp, C.POINTER(u32)]
        L.fge_get_count.argtypes = [vp, u32, C.c_char_p, C.POINTER(u32)]
        L.fge_get_variable.argtypes = [vp, u32, C.c_char_p, C.c_char_p, vp, sz]
        L.fge_stats.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(i32), C.POINTER(u32), C.POINTER(C.c_uint64)]
        L.fge_step_time.argtypes = [vp, C.POINTER(C.c_double)]
        _ens_ready = True
    return L


# Launch shapes of batched ensemble steps measured on GB300 (CUDAEnsemble's autotuner).
TUNING_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning", "ensemble_shapes.json")


class Ensemble:
    """CUDAEnsemble of a registered model: runs are added, then simulated together."""

    def __init__(self, model: str, params=(), device: int = 0, batched: bool = True, use_graphs: bool = True,
                 stage_bytes: int = 96 * 1024, tuning: str = "off", tuning_cache: str = TUNING_CACHE):
        """tuning: "off" (fixed launch shapes), "cache" (the shape tuning_cache
        holds for this GPU, model and size class) or "measure" (time every
        candidate on the batch and write the fastest to tuning_cache)."""
        L = _ens()
        arr = (C.c_double * max(1, len(params)))(*[float(p) for p in params])
        self._h = L.fge_create(model.encode(), arr, len(params), device)
        if not self._h:
            raise SimError(L.fgs_last_error().decode())
        _check(L.fge_configure(self._h, int(batched), int(use_graphs), stage_bytes))
        mode = {"off": 0, "cache": 1, "measure": 2}[tuning]
        _check(L.fge_set_tuning(self._h, mode, tuning_cache.encode() if tuning_cache else None))
        self.runs = 0

    def tuning(self) -> dict:
        """The launch shape of the last batched simulate() and where it came from."""
        import json
        buf = C.create_string_buffer(1 << 16)
        _check(_ens().fge_tuning(self._h, buf, 1 << 16))
        return json.loads(buf.value.decode())

    def close(self):
        if getattr(self, "_h", None):
            _ens().fge_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_run(self, steps: int, seed: int, agent=None, n: int = 0, columns=None, message=None, mn=None, mx=None,
                radius: float = 0.0) -> int:
        """One run plan; agent None: no initial population (the model's init functions may create one)."""
        columns = columns or {}
        names = list(columns)
        arrs = [np.ascontiguousarray(columns[k]) for k in names]
        cn = (C.c_char_p * max(1, len(names)))(*[k.encode() for k in names])
        cp = (C.c_void_p * max(1, len(names)))(*[a.ctypes.data for a in arrs])
        f3 = lambda v: (C.c_float * 3)(*(list(v) + [0.0] * (3 - len(v)))) if v is not None else None
        _check(_ens().fge_add_run(self._h, steps, seed, agent.encode() if agent else None, n, len(names), cn, cp,
                                  message.encode() if message else None, f3(mn), f3(mx), float(radius)))
        self.runs += 1
        return self.runs - 1

    def set_property(self, run: int, name: str, value, ctype=C.c_float):
        v = ctype(value)
        _check(_ens().fge_set_run_property(self._h, run, name.encode(), C.byref(v), C.sizeof(v)))

    def simulate(self) -> int:
        f = C.c_uint32()
        _check(_ens().fge_simulate(self._h, C.byref(f)))
        return f.value

    def count(self, run: int, agent: str) -> int:
        n = C.c_uint32()
        _check(_ens().fge_get_count(self._h, run, agent.encode(), C.byref(n)))
        return n.value

    def get(self, run: int, agent: str, var: str, dtype) -> np.ndarray:
        out = np.empty(self.count(run, agent), dtype=dtype)
        _check(_ens().fge_get_variable(self._h, run, agent.encode(), var.encode(), out.ctypes.data, out.nbytes))
        return out

    def stats(self) -> dict:
        el, b, k, g = C.c_double(), C.c_int32(), C.c_uint32(), C.c_uint64()
        _check(_ens().fge_stats(self._h, C.byref(el), C.byref(b), C.byref(k), C.byref(g)))
        t = C.c_double()
        _check(_ens().fge_step_time(self._h, C.byref(t)))
        return {"elapsed_s": el.value, "batched": bool(b.value), "kernels_per_step": k.value, "graph_launches": g.value,
                "step_s": t.value}


SERVER_EXPORTS = ["fgv_create", "fgv_destroy", "fgv_submit", "fgv_poll", "fgv_run_until_idle", "fgv_take_completed",
                  "fgv_result_info", "fgv_result_count", "fgv_result_variable", "fgv_release", "fgv_stats",
                  "fgv_counters", "fgv_set_scheduling", "fgv_result_agent_steps"]
_srv_ready = False


def _srv():
    global _srv_ready
    L = core()
    if not _srv_ready:
        vp, u32, i32, sz, u64 = C.c_void_p, C.c_uint32, C.c_int32, C.c_size_t, C.c_uint64
        L.fgv_create.argtypes = [i32, u64, u32, u32, i32]
        L.fgv_create.restype = vp
        L.fgv_destroy.argtypes = [vp]
        L.fgv_submit.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double), i32, u32, u64, i32, C.POINTER(C.c_char_p),
                                 C.POINTER(u32), C.POINTER(i32), C.POINTER(C.c_char_p), C.POINTER(vp), C.POINTER(u64)]
        L.fgv_poll.argtypes = [vp, C.POINTER(u32)]
        L.fgv_run_until_idle.argtypes = [vp]
        L.fgv_take_completed.argtypes = [vp, C.POINTER(u64), u32, C.POINTER(u32)]
        L.fgv_result_info.argtypes = [vp, u64, C.POINTER(C.c_double), C.POINTER(i32), C.c_char_p, sz]
        L.fgv_result_count.argtypes = [vp, u64, C.c_char_p, C.c_char_p, C.POINTER(u32)]
        L.fgv_result_agent_steps.argtypes = [vp, u64, C.POINTER(u64)]
        L.fgv_result_variable.argtypes = [vp, u64, C.c_char_p, C.c_char_p, C.c_char_p, vp, sz]
        L.fgv_release.argtypes = [vp, u64]
        L.fgv_stats.argtypes = [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u64)]
        L.fgv_counters.argtypes = [vp, C.POINTER(u64), C.POINTER(C.c_double), C.POINTER(u64)]
        L.fgv_set_scheduling.argtypes = [vp, C.c_double, C.c_double]
        _srv_ready = True
    return L


class Server:
    """SimulationServer: runs of registered models submitted as requests and
    advanced together (continuous batching) under a device-memory budget."""

    def __init__(self, device: int = 0, memory_budget: int = 150 << 30, max_active: int = 64,
                 steps_per_poll: int = 1, use_graphs: bool = True):
        L = _srv()
        self._h = L.fgv_create(device, memory_budget, max_active, steps_per_poll, int(use_graphs))
        if not self._h:
            raise SimError(L.fgs_last_error().decode())

    def close(self):
        if getattr(self, "_h", None):
            _srv().fgv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, model: str, params, steps: int, seed: int, populations: dict) -> int:
        """populations: {agent: (n, {var: host array})}; returns the run id."""
        agents = list(populations)
        names, cols, keep = [], [], []
        counts, nvars = [], []
        for a in agents:
            n, columns = populations[a]
            counts.append(int(n))
            nvars.append(len(columns))
            for k, v in columns.items():
                arr = np.ascontiguousarray(v)
                keep.append(arr)
                names.append(k.encode())
                cols.append(arr.ctypes.data)
        k = max(1, len(agents))
        m = max(1, len(names))
        arr = (C.c_double * max(1, len(params)))(*[float(p) for p in params])
        rid = C.c_uint64()
        _check(_srv().fgv_submit(self._h, model.encode(), arr, len(params), steps, seed, len(agents),
                                 (C.c_char_p * k)(*[a.encode() for a in agents]), (C.c_uint32 * k)(*counts),
                                 (C.c_int32 * k)(*nvars), (C.c_char_p * m)(*names), (C.c_void_p * m)(*cols),
                                 C.byref(rid)))
        return rid.value

    def poll(self) -> int:
        r = C.c_uint32()
        _check(_srv().fgv_poll(self._h, C.byref(r)))
        return r.value

    def run_until_idle(self):
        _check(_srv().fgv_run_until_idle(self._h))

    def take_completed(self) -> list[int]:
        out = []
        buf = (C.c_uint64 * 256)()
        n = C.c_uint32()
        while True:
            _check(_srv().fgv_take_completed(self._h, buf, 256, C.byref(n)))
            out += list(buf[:n.value])
            if n.value < 256:
                return out

    def info(self, rid: int) -> dict:
        t = (C.c_double * 3)()
        f = C.c_int32()
        err = C.create_string_buffer(1024)
        _check(_srv().fgv_result_info(self._h, rid, t, C.byref(f), err, 1024))
        a = C.c_uint64()
        _check(_srv().fgv_result_agent_steps(self._h, rid, C.byref(a)))
        return {"arrival_s": t[0], "admitted_s": t[1], "completed_s": t[2], "failed": bool(f.value),
                "error": err.value.decode(), "agent_steps": a.value}

    def count(self, rid: int, agent: str, state: str = "default") -> int:
        n = C.c_uint32()
        _check(_srv().fgv_result_count(self._h, rid, agent.encode(), state.encode(), C.byref(n)))
        return n.value

    def get(self, rid: int, agent: str, var: str, dtype, state: str = "default") -> np.ndarray:
        out = np.empty(self.count(rid, agent, state), dtype=dtype)
        _check(_srv().fgv_result_variable(self._h, rid, agent.encode(), state.encode(), var.encode(),
                                          out.ctypes.data, out.nbytes))
        return out

    def release(self, rid: int):
        _check(_srv().fgv_release(self._h, rid))

    def set_scheduling(self, work_in_flight: float = 0.0, total_work_in_flight: float = 0.0):
        _check(_srv().fgv_set_scheduling(self._h, float(work_in_flight), float(total_work_in_flight)))

    def counters(self) -> dict:
        p, t, n = C.c_uint64(), C.c_double(), C.c_uint64()
        _check(_srv().fgv_counters(self._h, C.byref(p), C.byref(t), C.byref(n)))
        return {"polls": p.value, "poll_seconds": t.value, "steps_issued": n.value}

    def stats(self) -> dict:
        q, a, r = C.c_uint32(), C.c_uint32(), C.c_uint64()
        _check(_srv().fgv_stats(self._h, C.byref(q), C.byref(a), C.byref(r)))
        return {"queued": q.value, "active": a.value, "reserved_bytes": r.value}
