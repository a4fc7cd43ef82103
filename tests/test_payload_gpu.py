"""The large spatial workloads' model (examples/spatial_payload/spatial_payload.cu,
the model behind the spatial2d_large / spatial3d_large bench lines) against
its serial restatement in the oracle (or_payload_run), bit for bit, at reduced
populations of the same shape and density:

  2D: agents uniform in [0, 256)^2, radius 4 (64^2 bins, 16 agents per bin,
      as the 16,777,216-agent workload on 1024^2 bins);
  3D: a 16-component Gaussian mixture (sigma 2, clipped) in [0, 32)^3,
      radius 1 (32^3 bins), as the 8,388,608-agent workload's generator.

20 steps each, with the clamped Moore neighbourhood (the bench lines') and
the wrapped one. Agent order after the automatic spatial sort, ids and the
four payload floats are compared exactly: both sides visit the candidates in
the reference's order (MessageSpatial3DDevice.cuh:693-749,
MessageSpatial2DDevice.cuh:646-698) without FMA contraction.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _population(dims, n, edge, seed):
    from flamegpu2_gb300 import synth, workloads
    if dims == 3:
        pos = workloads.gaussian_mixture_3d(n, edge, 16, 2.0, seed)
    else:
        hi = np.nextafter(np.float32(edge), np.float32(0))
        pos = np.stack([np.minimum(synth.uniform(seed, a, n, 0.0, edge), hi) for a in range(2)], 1)
    cols = {"_id": np.arange(1, n + 1, dtype=np.uint32), "x": pos[:, 0].copy(), "y": pos[:, 1].copy()}
    if dims == 3:
        cols["z"] = pos[:, 2].copy()
    for k in range(4):
        cols[f"p{k}"] = synth.uniform(seed, 20 + k, n, 0.0, 1.0)
    return cols


def _run_gpu(dims, edge, r, wrap, cols, steps):
    from flamegpu2_gb300 import sim
    n = cols["x"].shape[0]
    s = sim.Simulation("spatial_payload", [dims, 0.0, edge, r, 1.0 if wrap else 0.0])
    s.set_population("agent", n, cols)
    s.step(steps)
    keys = ["x", "y"] + (["z"] if dims == 3 else []) + [f"p{k}" for k in range(4)]
    out = {k: s.get("agent", k, np.float32) for k in keys}
    out["_id"] = s.get("agent", "_id", np.uint32)
    s.close()
    return out


@pytest.mark.parametrize("dims,n,edge,r", [(2, 65536, 256.0, 4.0), (3, 32768, 32.0, 1.0)])
@pytest.mark.parametrize("wrap", [False, True])
def test_payload_model_matches_oracle(dims, n, edge, r, wrap):
    steps = 20
    cols = _population(dims, n, edge, seed=2 + dims)
    out = _run_gpu(dims, edge, r, wrap, cols, steps)
    g = O.grid(dims, [0.0] * dims, [edge] * dims, r)
    st = {"id": cols["_id"], **{k: v for k, v in cols.items() if k != "_id"}}
    ref = O.payload_run(g, wrap, st, steps, threads=8)
    np.testing.assert_array_equal(out["_id"], ref["id"])
    for k in ["x", "y"] + (["z"] if dims == 3 else []):
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
    for k in range(4):
        np.testing.assert_array_equal(out[f"p{k}"], ref[f"p{k}"], err_msg=f"p{k}")
    # the payload did mix: 20 steps of averaging move every agent with a neighbour
    assert not np.array_equal(ref["p0"], cols["p0"][ref["id"] - 1])


def test_payload_model_empty_neighbourhoods_keep_payload():
    # agents alone in their neighbourhoods (one per 3x3x3 block of bins) see
    # only their own message: p <- 0.5 p + 0.5 p, unchanged
    dims, edge, r = 3, 30.0, 1.0
    c = np.arange(1.5, 30.0, 3.0, dtype=np.float32)
    gx, gy, gz = np.meshgrid(c, c, c, indexing="ij")
    n = gx.size
    cols = {"_id": np.arange(1, n + 1, dtype=np.uint32), "x": gx.ravel().copy(), "y": gy.ravel().copy(),
            "z": gz.ravel().copy()}
    rng = np.random.default_rng(7)
    for k in range(4):
        cols[f"p{k}"] = rng.random(n, dtype=np.float32)
    out = _run_gpu(dims, edge, r, False, cols, 3)
    g = O.grid(3, [0.0] * 3, [edge] * 3, r)
    ref = O.payload_run(g, False, {"id": cols["_id"], **{k: v for k, v in cols.items() if k != "_id"}}, 3)
    np.testing.assert_array_equal(out["_id"], ref["id"])
    for k in range(4):
        np.testing.assert_array_equal(out[f"p{k}"], ref[f"p{k}"])
        np.testing.assert_array_equal(out[f"p{k}"], cols[f"p{k}"][out["_id"] - 1])


@pytest.mark.parametrize("descent", [None, "group_boundary", "inside_group"])
def test_payload_model_from_rows_in_bin_order(descent):
    # the population starts in message-bin order (then every step's message
    # build and agent sort see rows in key order and write them in place), or
    # with one pair of neighbouring rows in different bins exchanged, at a
    # 32-row group boundary or inside a group: the output launch and the
    # build's scan must find that one descent
    dims, n, edge, r = 2, 40_000, 128.0, 4.0
    cols = _population(dims, n, edge, seed=19)
    g = O.grid(dims, [0.0] * dims, [edge] * dims, r)
    _, perm, bins = O.spatial_build(g, cols["x"], cols["y"])
    cols = {k: v[perm] for k, v in cols.items()}
    if descent:
        bins = bins[perm]
        j = 32 * 601 - 1 if descent == "group_boundary" else 32 * 300 + 5
        while bins[j] == bins[j + 1]:
            j += 32
        for k in cols:
            cols[k][[j, j + 1]] = cols[k][[j + 1, j]]
    out = _run_gpu(dims, edge, r, False, cols, 4)
    ref = O.payload_run(g, False, {"id": cols["_id"], **{k: v for k, v in cols.items() if k != "_id"}}, 4, threads=8)
    np.testing.assert_array_equal(out["_id"], ref["id"])
    for k in ["x", "y", "p0", "p1", "p2", "p3"]:
        np.testing.assert_array_equal(out[k], ref[k], err_msg=k)
