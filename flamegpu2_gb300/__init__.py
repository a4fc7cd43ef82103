"""flamegpu2_gb300 — GB300-native (sm_103a) implementation of FLAME GPU 2's
per-step core: spatial message build, neighbour iteration, birth/death
compaction and graph-captured layer scheduling.

The product is native: libflamegpu2_gb300.so (CUDA kernels, their C ABI and
the C++ host runtime behind include/flamegpu/) and libfg_models.so (model
sources). This Python package only builds and loads them.
"""
from . import build as _build_mod

__all__ = ["build"]


def build(verbose: bool = False):
    return _build_mod.build(verbose=verbose)
