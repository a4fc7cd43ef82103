"""Parity at the benchmark sizes.

* birth/death, 1,048,576 agents x 100 steps: the population entering every
  step equals the oracle's, and the full agent state after 10 steps is
  bit-exact (ids, counters, 8 floats);
* the spatial builds of the large workloads (16,777,216 messages on 1024^2
  bins; 8,388,608 Gaussian-mixture messages on 256^3 bins): the PBM is the
  exclusive scan of the bin histogram computed on the host, and the sorted
  records hold every message once, ordered by bin and, inside a bin, by
  original index (a stable sort by bin, computed with numpy).
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_birth_death_full_size_matches_oracle():
    from flamegpu2_gb300 import sim, synth
    n, seed = 1 << 20, 1
    pop = synth.birth_death_population(n, seed)
    s = sim.Simulation("birth_death", [0.30, 0.20, seed])
    s.set_population("agent", n, pop)
    counts = []
    state10 = None
    for t in range(100):
        counts.append(s.count("agent"))
        if t == 10:
            state10 = (np.stack([s.get("agent", f"f{v}", np.float32) for v in range(8)]),
                       s.get("agent", "counter", np.int32), s.get("agent", "_id", np.uint32))
        s.step(1)
    counts.append(s.count("agent"))
    s.close()
    f0 = np.stack([pop[f"f{v}"] for v in range(8)])
    fo, co, io, _, pops = O.birth_death_run(f0, pop["counter"], pop["_id"], n + 1, 4 * n, 0.30, 0.20, seed, 10)
    np.testing.assert_array_equal(state10[2], io)
    np.testing.assert_array_equal(state10[1], co)
    np.testing.assert_array_equal(state10[0], fo)
    *_, pops100 = O.birth_death_run(f0, pop["counter"], pop["_id"], n + 1, 4 * n, 0.30, 0.20, seed, 100)
    assert counts[:len(pops100)] == [int(p) for p in pops100]


def _build_records(g, pos):
    """fg_spatial_build with records (x, y[, z], original index)."""
    import torch
    from flamegpu2_gb300 import capi
    n, d = pos.shape
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(d)]
    idx = torch.arange(n, dtype=torch.int32, device="cuda")
    rec = capi.record_desc(cols + [idx])
    out = torch.zeros((n, rec.words), dtype=torch.int32, device="cuda")
    pbm = torch.zeros(g.binCount + 1, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(capi.lib().fg_spatial_build_workspace_size(n, g.binCount))
    for _ in range(2):  # the second build reuses the workspace left by the first
        capi.check(capi.lib().fg_spatial_build(C.byref(g), n, None, cols[0].data_ptr(), cols[1].data_ptr(),
                                               cols[2].data_ptr() if d == 3 else None, None, C.byref(rec),
                                               out.data_ptr(), pbm.data_ptr(), ws.ptr, ws.nbytes,
                                               capi.stream_handle()), "fg_spatial_build")
    torch.cuda.synchronize()
    assert ws.status() == 0
    return pbm.cpu().numpy().view(np.uint32), out[:, d].cpu().numpy()


def _host_bins(g, pos):
    """getGridPosition2D/3D + getHash: floor((p - min) / r) clamped, in float32."""
    d = pos.shape[1]
    cell = []
    for a in range(d):
        c = np.floor((pos[:, a] - np.float32(g.min[a])) / np.float32(g.radius)).astype(np.int64)
        cell.append(np.clip(c, 0, g.gridDim[a] - 1))
    if d == 3:
        return (cell[2] * g.gridDim[0] * g.gridDim[1] + cell[1] * g.gridDim[0] + cell[0]).astype(np.int64)
    return (cell[1] * g.gridDim[0] + cell[0]).astype(np.int64)


def _check_build(g, pos):
    pbm, order = _build_records(g, pos)
    bins = _host_bins(g, pos)
    hist = np.bincount(bins, minlength=g.binCount)
    expect_pbm = np.concatenate([[0], np.cumsum(hist)]).astype(np.uint32)
    np.testing.assert_array_equal(pbm, expect_pbm)
    np.testing.assert_array_equal(order, np.argsort(bins, kind="stable").astype(np.int32))


def test_spatial2d_large_build_is_stable_sort_by_bin():
    from flamegpu2_gb300 import capi, synth
    n = 1 << 24
    pos = np.stack([synth.uniform(3, a, n, 0.0, 4096.0) for a in range(2)], 1)
    pos = np.minimum(pos, np.nextafter(np.float32(4096.0), np.float32(0)))
    _check_build(capi.grid(2, (0, 0), (4096, 4096), 4.0), pos)


def test_spatial3d_large_gaussian_mixture_build_is_stable_sort_by_bin():
    from flamegpu2_gb300 import capi, workloads
    pos = workloads.gaussian_mixture_3d(1 << 23, 256.0, 16, 2.0, 2)
    _check_build(capi.grid(3, (0, 0, 0), (256, 256, 256), 1.0), pos)
