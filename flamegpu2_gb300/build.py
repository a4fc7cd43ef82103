"""Builds the native libraries in-tree (nvcc, sm_103a only, parallel TUs).

  libflamegpu2_gb300.so  kernels + C ABI (include/flamegpu_gb300/fg_capi.h)
                         + the C++ host runtime (include/flamegpu/...) and its C ABI
  libfg_models.so        the model sources (examples/) compiled against the
                         header-only device API, linked to libflamegpu2_gb300.so

Objects go to flamegpu2_gb300/_build/, libraries to flamegpu2_gb300/lib/.
A TU is recompiled when it or any header under include/ or csrc/ is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
CUDA_HOME = os.path.dirname(os.path.dirname(os.path.realpath(NVCC)))

COMMON = ["-std=c++20", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
          "-Xcompiler", "-fno-strict-aliasing", "-I", os.path.join(ROOT, "include"),
          "-I", os.path.join(PKG, "csrc"), "-Wno-deprecated-gpu-targets"]

CORE_SRCS = sorted(glob.glob(os.path.join(PKG, "csrc", "kernels", "*.cu")) +
                   glob.glob(os.path.join(PKG, "csrc", "runtime", "*.cu")) +
                   glob.glob(os.path.join(PKG, "csrc", "runtime", "*.cpp")))
# Model sources: float arithmetic compiled without FMA contraction so that the
# serial host oracle (compiled with -ffp-contract=off) reproduces it bit for bit.
MODEL_SRCS = sorted(glob.glob(os.path.join(ROOT, "examples", "*", "*.cu")))
MODEL_FLAGS = ["--fmad=false"]

CORE_LIB = os.path.join(LIBDIR, "libflamegpu2_gb300.so")
MODEL_LIB = os.path.join(LIBDIR, "libfg_models.so")


def _headers_mtime() -> float:
    paths = glob.glob(os.path.join(ROOT, "include", "**", "*"), recursive=True)
    paths += glob.glob(os.path.join(PKG, "csrc", "**", "*.cuh"), recursive=True)
    paths += glob.glob(os.path.join(PKG, "csrc", "**", "*.h"), recursive=True)
    return max([os.path.getmtime(p) for p in paths if os.path.isfile(p)] + [0.0])


def _obj_for(src: str) -> str:
    rel = os.path.relpath(src, ROOT).replace(os.sep, "__")
    return os.path.join(BUILD, rel + ".o")


def _compile(src: str, extra: list[str], hdr_mtime: float, verbose: bool) -> str:
    obj = _obj_for(src)
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj
    cmd = [NVCC] + ARCH + COMMON + extra + ["-x", "cu", "-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _link(objs: list[str], out: str, extra: list[str], verbose: bool) -> None:
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(o) for o in objs):
        return
    cmd = [NVCC] + ARCH + ["-shared", "-cudart", "shared", "-o", out] + objs + extra + [
        "-Xlinker", "-rpath", "-Xlinker", os.path.join(CUDA_HOME, "lib64"),
        "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed for {out}:\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False, jobs: int | None = None) -> dict:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hm = _headers_mtime()
    jobs = jobs or max(2, min(16, os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        core = [ex.submit(_compile, s, [], hm, verbose) for s in CORE_SRCS]
        models = [ex.submit(_compile, s, MODEL_FLAGS, hm, verbose) for s in MODEL_SRCS]
        core_objs = [f.result() for f in core]
        model_objs = [f.result() for f in models]
    _link(core_objs, CORE_LIB, [], verbose)
    if model_objs:
        _link(model_objs, MODEL_LIB, ["-L" + LIBDIR, "-lflamegpu2_gb300"], verbose)
    return {"core": CORE_LIB, "models": MODEL_LIB if model_objs else None}


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
