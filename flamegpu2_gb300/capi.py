"""ctypes binding of the kernel library's C ABI (include/flamegpu_gb300/fg_capi.h).

This is the binding a Python caller of the drop-in boundary would write; the
tests and the benchmark use it. Device buffers are torch tensors (plumbing:
allocation and streams); every computation runs in libflamegpu2_gb300.so.
There is no fallback: if the library is missing, loading fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(PKG, "lib")
CORE_LIB = os.path.join(LIBDIR, "libflamegpu2_gb300.so")

FG_MAX_RECORD_WORDS = 64
FG_MAX_COLUMNS = 48

FG_OK = 0
FG_ERR_INVALID_ARGUMENT = -1
FG_ERR_WORKSPACE = -2
FG_ERR_CUDA = -3
FG_ERR_DEVICE_TIMEOUT = -4
FG_ERR_CAPACITY = -5
FG_ERR_UNSUPPORTED = -6

# Every symbol include/flamegpu_gb300/fg_capi.h declares.
EXPORTS = [
    "fg_spatial_grid_init", "fg_spatial_build_workspace_size", "fg_spatial_sort_workspace_size",
    "fg_compact_workspace_size", "fg_workspace_init", "fg_workspace_status", "fg_spatial_build",
    "fg_spatial_sort_agents", "fg_compact_agents", "fg_scan_workspace_size", "fg_exclusive_scan_u32",
    "fg_last_cuda_error", "fg_version", "fg_batch_instance_init", "fg_batched_workspace_size",
    "fg_spatial_build_batched", "fg_spatial_sort_agents_batched", "fg_exclusive_scan_u32_noalloc",
    "fg_partition_agents", "fg_append_rows", "fg_workspace_set_wait_limit", "fg_noalloc_scan_status",
    "fg_append_births", "fg_batch_compact_tiles", "fg_compact_batched_workspace_size", "fg_compact_agents_batched",
    "fg_set_thread_tuning",
]
FG_NOALLOC_SCAN_MAX_N = 1 << 25


class FgError(RuntimeError):
    def __init__(self, code, what):
        super().__init__(f"{what} failed with fg_status {code}")
        self.code = code


class SpatialGrid(C.Structure):
    _fields_ = [
        ("dims", C.c_int32), ("min", C.c_float * 3), ("max", C.c_float * 3), ("radius", C.c_float),
        ("width", C.c_float * 3), ("gridDim", C.c_uint32 * 3), ("binCount", C.c_uint32),
        ("wrapCompatible", C.c_int32),
    ]


class BatchInstance(C.Structure):
    _fields_ = [
        ("grid", SpatialGrid), ("row_begin", C.c_uint32), ("row_capacity", C.c_uint32),
        ("bucket_begin", C.c_uint32), ("nbuckets", C.c_uint32), ("sort_width", C.c_float * 3),
        ("sort_gd", C.c_uint32 * 3), ("sort_mask", C.c_uint32), ("pad", C.c_uint32),
    ]


class RecordDesc(C.Structure):
    _fields_ = [
        ("words", C.c_uint32),
        ("src", C.c_void_p * FG_MAX_RECORD_WORDS),
        ("src_stride", C.c_uint32 * FG_MAX_RECORD_WORDS),
        ("src_word", C.c_uint32 * FG_MAX_RECORD_WORDS),
    ]


class Column(C.Structure):
    _fields_ = [("in_", C.c_void_p), ("out", C.c_void_p), ("elem_bytes", C.c_uint32)]


_lock = threading.Lock()
_lib = None


def lib():
    """Load libflamegpu2_gb300.so (built by flamegpu2_gb300.build)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(CORE_LIB):
                raise RuntimeError(f"{CORE_LIB} is missing: run flamegpu2_gb300.build.build() first")
            L = C.CDLL(CORE_LIB)
            vp, u32, sz = C.c_void_p, C.c_uint32, C.c_size_t
            L.fg_spatial_grid_init.argtypes = [C.POINTER(SpatialGrid), C.c_int32, C.POINTER(C.c_float),
                                               C.POINTER(C.c_float), C.c_float]
            L.fg_spatial_build_workspace_size.argtypes = [u32, u32]
            L.fg_spatial_build_workspace_size.restype = sz
            L.fg_spatial_sort_workspace_size.argtypes = [u32, C.POINTER(SpatialGrid)]
            L.fg_spatial_sort_workspace_size.restype = sz
            L.fg_compact_workspace_size.argtypes = [u32]
            L.fg_compact_workspace_size.restype = sz
            L.fg_scan_workspace_size.argtypes = [u32]
            L.fg_scan_workspace_size.restype = sz
            L.fg_workspace_init.argtypes = [vp, sz, vp]
            L.fg_workspace_status.argtypes = [vp, sz, vp, C.c_int32]
            L.fg_spatial_build.argtypes = [C.POINTER(SpatialGrid), u32, vp, vp, vp, vp, vp, C.POINTER(RecordDesc),
                                           vp, vp, vp, sz, vp]
            L.fg_spatial_sort_agents.argtypes = [C.POINTER(SpatialGrid), u32, vp, vp, vp, vp, C.POINTER(Column),
                                                 u32, vp, vp, sz, vp]
            L.fg_compact_agents.argtypes = [u32, vp, vp, vp, C.POINTER(Column), C.POINTER(Column), u32, C.c_int32,
                                            vp, vp, vp, u32, vp, sz, vp]
            L.fg_exclusive_scan_u32.argtypes = [vp, vp, u32, vp, sz, vp]
            L.fg_exclusive_scan_u32_noalloc.argtypes = [vp, vp, u32, vp]
            L.fg_noalloc_scan_status.argtypes = [vp, C.c_int32]
            L.fg_workspace_set_wait_limit.argtypes = [vp, sz, u32, C.c_int32, vp]
            L.fg_partition_agents.argtypes = [u32, vp, vp, C.POINTER(Column), u32, vp, vp, sz, vp]
            L.fg_append_rows.argtypes = [C.POINTER(Column), u32, u32, vp, vp, vp, u32, vp, sz, vp]
            L.fg_batch_compact_tiles.argtypes = [C.POINTER(BatchInstance), u32, C.POINTER(u32)]
            L.fg_batch_compact_tiles.restype = u32
            L.fg_compact_batched_workspace_size.argtypes = [u32, u32]
            L.fg_compact_batched_workspace_size.restype = sz
            L.fg_compact_agents_batched.argtypes = [vp, vp, u32, u32, u32, vp, vp, vp, C.POINTER(Column),
                                                    C.POINTER(Column), u32, C.c_int32, vp, vp, sz, vp]
            L.fg_append_births.argtypes = [u32, vp, vp, C.POINTER(Column), u32, C.c_int32, vp, vp, u32, vp, sz, vp]
            L.fg_version.restype = C.c_char_p
            L.fg_batch_instance_init.argtypes = [C.POINTER(BatchInstance), C.POINTER(SpatialGrid), u32, u32, u32,
                                                 C.c_int32, C.POINTER(u32)]
            L.fg_batched_workspace_size.argtypes = [u32, u32]
            L.fg_batched_workspace_size.restype = sz
            L.fg_spatial_build_batched.argtypes = [vp, vp, u32, u32, u32, vp, vp, vp, C.c_int32, vp,
                                                   C.POINTER(RecordDesc), vp, vp, vp, sz, vp]
            L.fg_spatial_sort_agents_batched.argtypes = [vp, vp, u32, u32, u32, vp, vp, vp, C.c_int32,
                                                         C.POINTER(Column), u32, vp, sz, vp]
            _lib = L
    return _lib


def check(rc, what):
    if rc != FG_OK:
        raise FgError(rc, what)


def grid(dims, mn, mx, radius) -> SpatialGrid:
    g = SpatialGrid()
    mn3 = (C.c_float * 3)(*[float(v) for v in list(mn) + [0.0] * (3 - len(mn))])
    mx3 = (C.c_float * 3)(*[float(v) for v in list(mx) + [0.0] * (3 - len(mx))])
    check(lib().fg_spatial_grid_init(C.byref(g), int(dims), mn3, mx3, float(radius)), "fg_spatial_grid_init")
    return g


def ptr(t) -> int | None:
    return None if t is None else t.data_ptr()


def stream_handle(stream=None) -> int:
    import torch
    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


class Workspace:
    """A caller-owned, zero-initialised scratch buffer for one C-ABI user."""

    def __init__(self, nbytes: int, device="cuda"):
        import torch
        self.nbytes = int(max(nbytes, 256))
        self.buf = torch.zeros(self.nbytes, dtype=torch.uint8, device=device)

    @property
    def ptr(self):
        return self.buf.data_ptr()

    def status(self, clear=True, stream=None) -> int:
        return lib().fg_workspace_status(self.ptr, self.nbytes, stream_handle(stream), int(clear))

    def set_wait_limit(self, spin_limit=0, withhold_first_tile=False, stream=None):
        check(lib().fg_workspace_set_wait_limit(self.ptr, self.nbytes, int(spin_limit), int(bool(withhold_first_tile)),
                                                stream_handle(stream)), "fg_workspace_set_wait_limit")


def record_desc(columns) -> RecordDesc:
    """columns: list of torch tensors (device), each [n] or [n, k] of 4-byte words.
    Record = concatenated words, padded to a multiple of 4 words."""
    rd = RecordDesc()
    w = 0
    for col in columns:
        words = (col.element_size() * (col.shape[1] if col.dim() > 1 else 1)) // 4
        for k in range(words):
            rd.src[w] = col.data_ptr()
            rd.src_stride[w] = words
            rd.src_word[w] = k
            w += 1
    rd.words = (w + 3) // 4 * 4
    return rd


def columns(pairs) -> C.Array:
    arr = (Column * max(1, len(pairs)))()
    for k, (a, b) in enumerate(pairs):
        per = a.element_size() * (a.shape[1] if a.dim() > 1 else 1)
        arr[k] = Column(a.data_ptr(), b.data_ptr(), per)
    return arr
