"""Regenerate the golden fixtures in this directory.

  python tests/golden/make_golden.py

1. Compiles gen_golden.cpp (g++) — a restatement of the reference tests'
   population generators and host-side expectations — runs it, and packs its
   raw arrays into reference_tests.npz.
2. When FLAMEGPU2_REFERENCE names a FLAME GPU 2 source tree, builds
   oracle/_ref/numeric_pin from the reference's own
   include/flamegpu/detail/numeric.h (oracle/Makefile `ref`) and stores its
   outputs as wrap_compatible.json.

The fixtures are committed; the tests only read them.
"""
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def main():
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "gen_golden")
        subprocess.run(["g++", "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "gen_golden.cpp")], check=True)
        subprocess.run([exe, td], check=True)
        arrays = {}
        for fn in sorted(os.listdir(td)):
            if "." not in fn or fn == "gen_golden":
                continue
            name, ext = fn.rsplit(".", 1)
            dt = {"f32": np.float32, "u32": np.uint32, "i32": np.int32}[ext]
            arrays[name] = np.fromfile(os.path.join(td, fn), dtype=dt)
        np.savez_compressed(os.path.join(HERE, "reference_tests.npz"), **arrays)
        print("wrote reference_tests.npz:", ", ".join(f"{k}{v.shape}" for k, v in arrays.items()))
    ref = os.environ.get("FLAMEGPU2_REFERENCE", "")
    if ref and os.path.isdir(os.path.join(ref, "include")):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", "REF=" + ref], check=True)
        out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "numeric_pin")], check=True,
                             capture_output=True, text=True).stdout
        rows = json.loads(out)
        with open(os.path.join(HERE, "wrap_compatible.json"), "w") as f:
            json.dump({"source": "reference include/flamegpu/detail/numeric.h:24-31 compiled by oracle/Makefile ref",
                       "rows": rows}, f, indent=0)
        print("wrote wrap_compatible.json:", len(rows), "rows")
    else:
        print("FLAMEGPU2_REFERENCE not set: wrap_compatible.json left as committed", file=sys.stderr)


if __name__ == "__main__":
    main()
