"""Parity of the C-ABI kernels (libflamegpu2_gb300.so) with the serial oracle.

GPU tests call the kernels through the C ABI on seeded inputs and require
bit-exact PBMs, stable within-bin order, sorted records, auto-sort
permutations and compaction order/ids. CPU tests check that the library loads,
exports every symbol the header declares, and that the host-side grid set-up
matches the oracle.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _capi():
    from flamegpu2_gb300 import capi
    return capi


def test_header_symbols_exported():
    capi = _capi()
    hdr = open(os.path.join(ROOT, "include", "flamegpu_gb300", "fg_capi.h")).read()
    declared = set(re.findall(r"^(?:int|size_t|uint32_t|const char\*)\s+(fg_\w+)\(", hdr, re.M))
    assert declared == set(capi.EXPORTS)
    L = capi.lib()
    for name in declared:
        assert hasattr(L, name), name
    assert b"sm_103a" in L.fg_version()


def test_sim_header_symbols_exported():
    from flamegpu2_gb300 import sim
    hdr = open(os.path.join(ROOT, "include", "flamegpu_gb300", "fg_sim.h")).read()
    declared = set(re.findall(r"^(?:int|void|const char\*|fg[sev]_\w+\*)\s+(fg[sev]_\w+)\(", hdr, re.M))
    assert declared == set(sim.SIM_EXPORTS + sim.ENSEMBLE_EXPORTS + sim.SERVER_EXPORTS)
    L = sim.core()
    for name in declared:
        assert hasattr(L, name), name


@pytest.mark.parametrize("dims,mn,mx,r", [(3, (0, 0, 0), (64, 64, 64), 2.0), (3, (0, 0, 0), (50.1, 50.1, 50.1), 10.0),
                                          (2, (0, 0), (11, 11), 1.0), (3, (141, -540, 200), (211, -470, 270), 3.5),
                                          (3, (-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), 0.05)])
def test_grid_init_matches_oracle(dims, mn, mx, r):
    capi = _capi()
    g = capi.grid(dims, mn, mx, r)
    o = O.grid(dims, mn, mx, r)
    assert tuple(g.gridDim) == tuple(o.gridDim)
    assert g.binCount == o.binCount
    assert g.wrapCompatible == o.wrapCompatible
    assert list(g.width) == list(o.width)


def test_grid_init_rejects_bad_arguments():
    capi = _capi()
    g = capi.SpatialGrid()
    mn = (C.c_float * 3)(0, 0, 0)
    mx = (C.c_float * 3)(1, 1, 1)
    assert capi.lib().fg_spatial_grid_init(C.byref(g), 3, mn, mx, 0.0) == capi.FG_ERR_INVALID_ARGUMENT
    assert capi.lib().fg_spatial_grid_init(C.byref(g), 4, mn, mx, 1.0) == capi.FG_ERR_INVALID_ARGUMENT
    assert capi.lib().fg_spatial_grid_init(C.byref(g), 3, mx, mn, 1.0) == capi.FG_ERR_INVALID_ARGUMENT


def test_workspace_sizes():
    capi = _capi()
    L = capi.lib()
    assert L.fg_spatial_build_workspace_size(1000, 125) >= 256 + 3 * 4000
    assert L.fg_compact_workspace_size(4 << 20) >= 256 + 2 * 8 * 2048
    g = capi.grid(3, (0, 0, 0), (64, 64, 64), 2.0)
    assert L.fg_spatial_sort_workspace_size(16384, C.byref(g)) > L.fg_spatial_build_workspace_size(16384, 32768)


# ----------------------------------------------------------------------- GPU


def _positions(rng, n, mn, mx, kind):
    mn, mx = np.array(mn, np.float32), np.array(mx, np.float32)
    d = len(mn)
    if kind == "uniform":
        p = rng.uniform(mn, mx, (n, d))
    elif kind == "outside":  # exercise the clamping of out-of-bounds positions
        w = mx - mn
        p = rng.uniform(mn - 0.3 * w, mx + 0.3 * w, (n, d))
    elif kind == "clusters":  # heavy-tailed bins: long-bin path
        centres = rng.uniform(mn, mx, (4, d))
        p = centres[rng.integers(0, 4, n)] + rng.normal(0, 0.02 * (mx - mn).max(), (n, d))
        p = np.clip(p, mn, mx)
    elif kind == "onebin":
        p = np.tile(((mn + mx) / 2)[None, :], (n, 1)) + rng.uniform(0, 1e-3, (n, d))
    return p.astype(np.float32)


def _build(g, pos, valid=None, d_count=None, extra_words=3, ws=None, reps=1):
    import torch
    capi = _capi()
    n = pos.shape[0]
    dev = "cuda"
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).to(dev) for a in range(pos.shape[1])]
    payload = torch.arange(n * extra_words, dtype=torch.int32, device=dev).reshape(n, extra_words) * 7 + 3
    rec = capi.record_desc(cols + [payload])
    sorted_ = torch.zeros((max(n, 1), rec.words), dtype=torch.int32, device=dev)
    pbm = torch.zeros(g.binCount + 1, dtype=torch.int32, device=dev)
    if ws is None:
        ws = capi.Workspace(capi.lib().fg_spatial_build_workspace_size(max(n, 1), g.binCount))
    vt = None if valid is None else torch.from_numpy(valid.astype(np.uint32)).to(dev)
    dn = None if d_count is None else torch.tensor([d_count], dtype=torch.int32, device=dev)
    for _ in range(reps):
        rc = capi.lib().fg_spatial_build(C.byref(g), n, capi.ptr(dn), cols[0].data_ptr(), cols[1].data_ptr(),
                                         cols[2].data_ptr() if len(cols) == 3 else None, capi.ptr(vt), C.byref(rec),
                                         sorted_.data_ptr(), pbm.data_ptr(), ws.ptr, ws.nbytes, capi.stream_handle())
        capi.check(rc, "fg_spatial_build")
    torch.cuda.synchronize()
    assert ws.status() == 0
    return pbm.cpu().numpy().view(np.uint32), sorted_.cpu().numpy().view(np.uint32), payload.cpu().numpy(), rec


def _expect(g, pos, valid=None, d_count=None):
    n = pos.shape[0] if d_count is None else d_count
    keep = np.arange(n) if valid is None else np.nonzero(valid[:n])[0]
    sub = pos[keep]
    og = O.grid(g.dims, list(g.min)[:g.dims], list(g.max)[:g.dims], g.radius)
    pbm, perm, _ = O.spatial_build(og, *[sub[:, a] for a in range(pos.shape[1])])
    return pbm, keep[perm]


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 17, 5000, 100_003])
@pytest.mark.parametrize("kind", ["uniform", "outside", "clusters"])
def test_spatial3d_build_parity(n, kind):
    rng = np.random.default_rng(n + len(kind))
    g = _capi().grid(3, (0, 0, 0), (64, 64, 64), 2.0)
    pos = _positions(rng, n, (0, 0, 0), (64, 64, 64), kind)
    pbm, srt, payload, rec = _build(g, pos)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    m = int(epbm[-1])
    assert m == n
    # sorted records: x,y,z words then the payload, in the oracle's stable order
    np.testing.assert_array_equal(srt[:m, 0:3].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:m, 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3000, 70_000])
def test_spatial2d_build_parity(n):
    rng = np.random.default_rng(7)
    g = _capi().grid(2, (0, 0), (400, 400), 4.0)
    pos = _positions(rng, n, (0, 0), (400, 400), "clusters")
    pbm, srt, payload, _ = _build(g, pos, extra_words=2)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:n, 0:2].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:n, 2:4].view(np.int32), payload[eperm])


@pytest.mark.gpu
def test_build_optional_and_device_count():
    rng = np.random.default_rng(11)
    g = _capi().grid(3, (0, 0, 0), (20, 20, 20), 1.0)
    pos = _positions(rng, 20000, (0, 0, 0), (20, 20, 20), "uniform")
    valid = rng.random(20000) < 0.8
    pbm, srt, payload, _ = _build(g, pos, valid=valid, d_count=15000)
    epbm, eperm = _expect(g, pos, valid=valid, d_count=15000)
    np.testing.assert_array_equal(pbm, epbm)
    m = int(epbm[-1])
    np.testing.assert_array_equal(srt[:m, 0:3].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:m, 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
def test_build_one_heavy_bin_and_reuse():
    # 40k messages in one bin: the long-bin path with 157 chunks; repeated
    # builds on one workspace (histogram kept zero, scan epochs advance).
    rng = np.random.default_rng(3)
    g = _capi().grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    pos = _positions(rng, 40000, (0, 0, 0), (8, 8, 8), "onebin")
    pbm, srt, payload, _ = _build(g, pos, reps=3)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:40000, 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
def test_build_long_bins_sorted_and_ranked():
    # bins of 33 .. 8192 messages are ordered by the shared-memory sort, 8193
    # and more by chunk ranking; messages of all bins interleaved at random
    rng = np.random.default_rng(11)
    g = _capi().grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    sizes = [33, 64, 65, 257, 1000, 4096, 5000, 8191, 8192, 8193, 9000, 1, 2, 31, 32]
    cells = rng.choice(512, len(sizes), replace=False)
    pos = []
    for c, k in zip(cells, sizes):
        cx, cy, cz = c % 8, (c // 8) % 8, c // 64
        pos.append(np.stack([cx + rng.uniform(0.01, 0.99, k), cy + rng.uniform(0.01, 0.99, k),
                             cz + rng.uniform(0.01, 0.99, k)], 1))
    pos = np.concatenate(pos).astype(np.float32)
    pos = pos[rng.permutation(len(pos))]
    pbm, srt, payload, _ = _build(g, pos, reps=2)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:len(pos), 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["bins", "local", "displaced"])
def test_build_long_bins_in_bin_order(order):
    # messages that arrive grouped by bin, as those of spatially sorted agents
    # do: each bin's indices contiguous ("bins"), shuffled within windows of 64
    # ("local"), or 1% of them exchanged at random ("displaced")
    rng = np.random.default_rng(31)
    g = _capi().grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    sizes = [33, 100, 500, 1000, 1024, 1025, 3000, 8192, 8193, 20000, 1, 31, 32]
    cells = rng.choice(512, len(sizes), replace=False)
    pos = []
    for c, k in zip(cells, sizes):
        cx, cy, cz = c % 8, (c // 8) % 8, c // 64
        pos.append(np.stack([cx + rng.uniform(0.01, 0.99, k), cy + rng.uniform(0.01, 0.99, k),
                             cz + rng.uniform(0.01, 0.99, k)], 1))
    pos = np.concatenate(pos).astype(np.float32)
    n = len(pos)
    if order == "local":
        pos = pos[np.argsort(np.arange(n) // 64 + rng.random(n), kind="stable")]
    elif order == "displaced":
        sel = rng.choice(n, n // 100, replace=False)
        pos[sel] = pos[rng.permutation(sel)]
    pbm, srt, payload, _ = _build(g, pos, reps=2)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:n, 0:3].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:n, 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
def test_build_on_256_cubed_bins():
    # 16,777,216 bins: the PBM scan takes four sub-tiles per tile; two builds
    # on one workspace check that the histogram is left cleared
    rng = np.random.default_rng(41)
    g = _capi().grid(3, (0, 0, 0), (256, 256, 256), 1.0)
    pos = _positions(rng, 200_000, (0, 0, 0), (256, 256, 256), "clusters")
    pbm, srt, payload, _ = _build(g, pos, reps=2)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:len(pos), 0:3].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:len(pos), 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
def test_build_mixed_buckets_under_16k():
    # a list of under 16,384 messages with short, warp-sized and long buckets,
    # messages of all buckets interleaved at random
    rng = np.random.default_rng(23)
    g = _capi().grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    sizes = [33, 64, 200, 256, 257, 1000, 4096, 5000, 1, 2, 31, 32]
    cells = rng.choice(512, len(sizes), replace=False)
    pos = []
    for c, k in zip(cells, sizes):
        cx, cy, cz = c % 8, (c // 8) % 8, c // 64
        pos.append(np.stack([cx + rng.uniform(0.01, 0.99, k), cy + rng.uniform(0.01, 0.99, k),
                             cz + rng.uniform(0.01, 0.99, k)], 1))
    pos = np.concatenate(pos).astype(np.float32)
    pos = pos[rng.permutation(len(pos))]
    assert len(pos) <= 16384
    pbm, srt, payload, _ = _build(g, pos, reps=2)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:len(pos), 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [16384, 16385])
def test_build_one_bucket_and_optional_at_16k(n):
    # every message in one bucket, then clustered optional output with a
    # device count, at 16,384 messages and one more
    rng = np.random.default_rng(n)
    g = _capi().grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    pos = _positions(rng, n, (0, 0, 0), (8, 8, 8), "onebin")
    pbm, srt, payload, _ = _build(g, pos)
    epbm, eperm = _expect(g, pos)
    np.testing.assert_array_equal(pbm, epbm)
    np.testing.assert_array_equal(srt[:n, 3:6].view(np.int32), payload[eperm])
    pos = _positions(rng, n, (0, 0, 0), (8, 8, 8), "clusters")
    valid = rng.random(n) < 0.7
    pbm, srt, payload, _ = _build(g, pos, valid=valid, d_count=n - 1000)
    epbm, eperm = _expect(g, pos, valid=valid, d_count=n - 1000)
    np.testing.assert_array_equal(pbm, epbm)
    m = int(epbm[-1])
    np.testing.assert_array_equal(srt[:m, 0:3].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:m, 3:6].view(np.int32), payload[eperm])


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 4095, 4096, 4097, 1_000_000, 4_194_304, 4_194_305, 16_777_217, 17_000_001])
def test_exclusive_scan(n):
    import torch
    capi = _capi()
    rng = np.random.default_rng(n % 1000)
    a = rng.integers(0, 5, n).astype(np.uint32)
    t = torch.from_numpy(a.view(np.int32)).cuda()
    out = torch.empty_like(t)
    ws = capi.Workspace(capi.lib().fg_scan_workspace_size(n))
    for _ in range(2):
        capi.check(capi.lib().fg_exclusive_scan_u32(t.data_ptr(), out.data_ptr(), n, ws.ptr, ws.nbytes,
                                                   capi.stream_handle()), "scan")
    torch.cuda.synchronize()
    expect = (np.cumsum(a.astype(np.uint64)) - a).astype(np.uint32)
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), expect)
    assert ws.status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("dims,n,kind", [(3, 16384, "uniform"), (3, 50000, "outside"), (2, 30000, "clusters"),
                                         (3, 12000, "clusters"), (2, 9000, "outside")])
def test_spatial_sort_agents_parity(dims, n, kind):
    import torch
    capi = _capi()
    rng = np.random.default_rng(n)
    mn, mx = (0,) * dims, (64,) * dims
    g = capi.grid(dims, mn, mx, 2.0)
    pos = _positions(rng, n, mn, mx, kind)
    cols_in = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(dims)]
    extra = torch.arange(n, dtype=torch.int64, device="cuda") * 3 + 1  # an 8-byte column
    tiny = (torch.arange(n, device="cuda") % 251).to(torch.uint8)  # a 1-byte column
    ins = cols_in + [extra, tiny]
    outs = [torch.empty_like(c) for c in ins]
    colarr = capi.columns(list(zip(ins, outs)))
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(capi.lib().fg_spatial_sort_workspace_size(n, C.byref(g)))
    rc = capi.lib().fg_spatial_sort_agents(C.byref(g), n, None, cols_in[0].data_ptr(), cols_in[1].data_ptr(),
                                           cols_in[2].data_ptr() if dims == 3 else None, colarr, len(ins),
                                           perm.data_ptr(), ws.ptr, ws.nbytes, capi.stream_handle())
    capi.check(rc, "fg_spatial_sort_agents")
    torch.cuda.synchronize()
    og = O.grid(dims, mn, mx, 2.0)
    keys = O.sort_keys(og, pos[:, 0], pos[:, 1], pos[:, 2] if dims == 3 else None)
    eperm = O.stable_sort_perm(keys, O.sort_max_bit(og))
    np.testing.assert_array_equal(perm.cpu().numpy().view(np.uint32), eperm)
    for a in range(dims):
        np.testing.assert_array_equal(outs[a].cpu().numpy(), pos[eperm, a])
    np.testing.assert_array_equal(outs[dims].cpu().numpy(), extra.cpu().numpy()[eperm])
    np.testing.assert_array_equal(outs[dims + 1].cpu().numpy(), tiny.cpu().numpy()[eperm])
    assert ws.status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["sorted", "displaced"])
@pytest.mark.parametrize("with_perm", [True, False])
def test_spatial_sort_agents_in_key_order(order, with_perm):
    # a population already in sort-key order (bins of up to thousands of
    # agents, each bin's rows contiguous), or with 1% of its rows exchanged;
    # 4-, 8- and 1-byte columns, with and without the permutation output
    import torch
    capi = _capi()
    rng = np.random.default_rng(5)
    n = 60_000
    g = capi.grid(3, (0, 0, 0), (16, 16, 16), 2.0)
    pos = _positions(rng, n, (0, 0, 0), (16, 16, 16), "clusters")
    og = O.grid(3, (0, 0, 0), (16, 16, 16), 2.0)
    pos = pos[O.stable_sort_perm(O.sort_keys(og, pos[:, 0], pos[:, 1], pos[:, 2]), O.sort_max_bit(og))]
    if order == "displaced":
        sel = rng.choice(n, n // 100, replace=False)
        pos[sel] = pos[rng.permutation(sel)]
    cols_in = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(3)]
    w4 = [torch.arange(n, dtype=torch.int32, device="cuda") * (k + 2) for k in range(3)]
    extra = torch.arange(n, dtype=torch.int64, device="cuda") * 3 + 1
    tiny = (torch.arange(n, device="cuda") % 251).to(torch.uint8)
    ins = cols_in + w4 + [extra, tiny]
    outs = [torch.empty_like(c) for c in ins]
    perm = torch.zeros(n, dtype=torch.int32, device="cuda") if with_perm else None
    ws = capi.Workspace(capi.lib().fg_spatial_sort_workspace_size(n, C.byref(g)))
    capi.check(capi.lib().fg_spatial_sort_agents(C.byref(g), n, None, cols_in[0].data_ptr(), cols_in[1].data_ptr(),
                                                 cols_in[2].data_ptr(), capi.columns(list(zip(ins, outs))), len(ins),
                                                 capi.ptr(perm), ws.ptr, ws.nbytes, capi.stream_handle()), "sort")
    torch.cuda.synchronize()
    eperm = O.stable_sort_perm(O.sort_keys(og, pos[:, 0], pos[:, 1], pos[:, 2]), O.sort_max_bit(og))
    if with_perm:
        np.testing.assert_array_equal(perm.cpu().numpy().view(np.uint32), eperm)
    for a, b in zip(ins, outs):
        np.testing.assert_array_equal(b.cpu().numpy(), a.cpu().numpy()[eperm])
    assert ws.status() == 0


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 2047, 2048, 2049, 300_001])
@pytest.mark.parametrize("with_births", [False, True])
def test_compact_agents_parity(n, with_births):
    import torch
    capi = _capi()
    rng = np.random.default_rng(n + 17 * with_births)
    cap = 2 * n + 8
    alive = (rng.random(n) >= 0.3).astype(np.uint32)
    born = ((rng.random(n) < 0.2) & (alive == 1)).astype(np.uint32) if with_births else None
    f = rng.random((n, 2)).astype(np.float32)
    ids = np.arange(1, n + 1, dtype=np.uint32)
    dev = "cuda"
    f_in = torch.from_numpy(f).to(dev)
    id_in = torch.from_numpy(ids.view(np.int32)).to(dev)
    f_out = torch.zeros((cap, 2), dtype=torch.float32, device=dev)
    id_out = torch.zeros(cap, dtype=torch.int32, device=dev)
    bf_in = (f_in * 10 + 1).contiguous()  # birth staging rows: distinguishable values
    bid_in = torch.zeros(max(n, 1), dtype=torch.int32, device=dev)
    cols = capi.columns([(f_in, f_out), (id_in, id_out)])
    bcols = capi.columns([(bf_in, f_out), (bid_in, id_out)])
    a_t = torch.from_numpy(alive.view(np.int32)).to(dev)
    b_t = None if born is None else torch.from_numpy(born.view(np.int32)).to(dev)
    next_id = torch.tensor([n + 1], dtype=torch.int32, device=dev)
    d_n = torch.tensor([n], dtype=torch.int32, device=dev)
    n_out = torch.zeros(1, dtype=torch.int32, device=dev)
    ws = capi.Workspace(capi.lib().fg_compact_workspace_size(max(n, 1)))
    rc = capi.lib().fg_compact_agents(max(n, 1) if n else 0, d_n.data_ptr(), a_t.data_ptr() if n else None,
                                      capi.ptr(b_t) if n else None, cols, bcols, 2, 1, next_id.data_ptr(), None,
                                      n_out.data_ptr(), cap, ws.ptr, ws.nbytes, capi.stream_handle())
    capi.check(rc, "fg_compact_agents")
    torch.cuda.synchronize()
    surv = O.compact(alive)
    kids = O.compact(born) if born is not None else np.zeros(0, np.uint32)
    m = len(surv) + len(kids)
    assert int(n_out.item()) == m
    np.testing.assert_array_equal(f_out.cpu().numpy()[:len(surv)], f[surv])
    np.testing.assert_array_equal(id_out.cpu().numpy().view(np.uint32)[:len(surv)], ids[surv])
    if len(kids):
        np.testing.assert_array_equal(f_out.cpu().numpy()[len(surv):m], f[kids] * 10 + 1)
        np.testing.assert_array_equal(id_out.cpu().numpy().view(np.uint32)[len(surv):m],
                                      np.arange(n + 1, n + 1 + len(kids), dtype=np.uint32))
    assert int(next_id.item()) == n + 1 + len(kids)
    assert ws.status() == 0


# ------------------------------------------------------------------ batches

def _batch(mode, specs, rows_align=128):
    """specs: list of (grid, count, capacity). Returns (instances array, total rows, total buckets)."""
    capi = _capi()
    arr = (capi.BatchInstance * len(specs))()
    row, bucket = 0, 0
    for k, (g, count, cap) in enumerate(specs):
        nb = C.c_uint32()
        capi.check(capi.lib().fg_batch_instance_init(C.byref(arr[k]), C.byref(g), row, cap, bucket, mode, C.byref(nb)),
                   "fg_batch_instance_init")
        row += cap
        bucket += nb.value
    return arr, row, bucket


@pytest.mark.gpu
@pytest.mark.parametrize("dims", [3, 2])
def test_batched_build_matches_each_instance(dims):
    import torch
    capi = _capi()
    rng = np.random.default_rng(40 + dims)
    specs, pos_list, grids = [], [], []
    for k, (count, r, edge) in enumerate([(1000, 1.0, 10.0), (0, 2.0, 8.0), (5000, 3.0, 33.0), (37, 1.5, 4.5),
                                          (20000, 2.5, 60.0)]):
        cap = (count + 127) // 128 * 128 + 128
        g = capi.grid(dims, (0.0,) * dims, (edge,) * dims, r)
        grids.append(g)
        specs.append((g, count, cap))
        pos_list.append(_positions(rng, count, (0.0,) * dims, (edge,) * dims, "clusters" if k % 2 else "uniform"))
    inst, total_rows, total_buckets = _batch(0, specs)
    pos = np.zeros((total_rows, dims), np.float32)
    for (g, count, cap), p, i in zip(specs, pos_list, inst):
        pos[i.row_begin:i.row_begin + count] = p
    counts = torch.tensor([c for _, c, _ in specs], dtype=torch.int32, device="cuda")
    d_inst = torch.frombuffer(bytearray(bytes(inst)), dtype=torch.uint8).cuda()
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(dims)]
    payload = torch.arange(total_rows, dtype=torch.int32, device="cuda") * 3 + 1
    rec = capi.record_desc(cols + [payload])
    srt = torch.zeros((total_rows, rec.words), dtype=torch.int32, device="cuda")
    pbm = torch.zeros(total_buckets + 1, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(capi.lib().fg_batched_workspace_size(total_rows, total_buckets))
    for _ in range(2):
        capi.check(capi.lib().fg_spatial_build_batched(
            d_inst.data_ptr(), counts.data_ptr(), len(specs), total_rows, total_buckets, cols[0].data_ptr(),
            cols[1].data_ptr(), cols[2].data_ptr() if dims == 3 else None, dims, None, C.byref(rec), srt.data_ptr(),
            pbm.data_ptr(), ws.ptr, ws.nbytes, capi.stream_handle()), "fg_spatial_build_batched")
    torch.cuda.synchronize()
    assert ws.status() == 0
    pbm_h = pbm.cpu().numpy().view(np.uint32)
    srt_h = srt.cpu().numpy().view(np.uint32)
    pay_h = payload.cpu().numpy()
    for (g, count, cap), p, i in zip(specs, pos_list, inst):
        og = O.grid(dims, (0.0,) * dims, list(g.max)[:dims], g.radius)
        epbm, eperm, _ = O.spatial_build(og, *[p[:, a] for a in range(dims)])
        got = pbm_h[i.bucket_begin:i.bucket_begin + g.binCount + 1] - i.row_begin
        np.testing.assert_array_equal(got, epbm)
        rows = i.row_begin + eperm
        np.testing.assert_array_equal(srt_h[i.row_begin:i.row_begin + count, dims].view(np.int32), pay_h[rows])


@pytest.mark.gpu
def test_batched_sort_matches_each_instance():
    import torch
    capi = _capi()
    rng = np.random.default_rng(9)
    specs, pos_list = [], []
    for k, (count, r, edge) in enumerate([(3000, 2.0, 64.0), (10, 1.0, 5.0), (9000, 4.0, 40.0)]):
        cap = (count + 127) // 128 * 128
        g = capi.grid(3, (0.0,) * 3, (edge,) * 3, r)
        specs.append((g, count, cap))
        pos_list.append(_positions(rng, count, (0.0,) * 3, (edge,) * 3, "outside"))
    inst, total_rows, total_buckets = _batch(1, specs)
    pos = np.zeros((total_rows, 3), np.float32)
    for (g, count, cap), p, i in zip(specs, pos_list, inst):
        pos[i.row_begin:i.row_begin + count] = p
    counts = torch.tensor([c for _, c, _ in specs], dtype=torch.int32, device="cuda")
    d_inst = torch.frombuffer(bytearray(bytes(inst)), dtype=torch.uint8).cuda()
    ins = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(3)]
    ids = torch.arange(total_rows, dtype=torch.int32, device="cuda")
    outs = [torch.empty_like(c) for c in ins] + [torch.empty_like(ids)]
    colarr = capi.columns(list(zip(ins + [ids], outs)))
    ws = capi.Workspace(capi.lib().fg_batched_workspace_size(total_rows, total_buckets))
    capi.check(capi.lib().fg_spatial_sort_agents_batched(
        d_inst.data_ptr(), counts.data_ptr(), len(specs), total_rows, total_buckets, ins[0].data_ptr(),
        ins[1].data_ptr(), ins[2].data_ptr(), 3, colarr, 4, ws.ptr, ws.nbytes, capi.stream_handle()), "sort_batched")
    torch.cuda.synchronize()
    got_ids = outs[3].cpu().numpy()
    for (g, count, cap), p, i in zip(specs, pos_list, inst):
        og = O.grid(3, (0.0,) * 3, list(g.max)[:3], g.radius)
        keys = O.sort_keys(og, p[:, 0], p[:, 1], p[:, 2])
        eperm = O.stable_sort_perm(keys, O.sort_max_bit(og))
        np.testing.assert_array_equal(got_ids[i.row_begin:i.row_begin + count], i.row_begin + eperm)


@pytest.mark.gpu
@pytest.mark.parametrize("with_births", [False, True])
def test_batched_compaction_matches_each_instance(with_births):
    # instances of uneven size (empty, one block, several tiles, one with room
    # for few births), each compacted in its own segment; order, ids and
    # counts as a compaction of each instance alone (the oracle's)
    import torch
    capi = _capi()
    L = capi.lib()
    rng = np.random.default_rng(21 + with_births)
    pops = [0, 1, 127, 5000, 2048, 9000, 300, 70_000]
    caps = [128, 128, 256, 12_032, 4096, 9088, 640, 140_032]
    g = capi.grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    arr = (capi.BatchInstance * len(pops))()
    row = 0
    for k, cap in enumerate(caps):
        capi.check(L.fg_batch_instance_init(C.byref(arr[k]), C.byref(g), row, cap, 0, 0, None), "instance")
        row += cap
    total = row
    tb = (C.c_uint32 * (len(pops) + 1))()
    ntiles = L.fg_batch_compact_tiles(arr, len(pops), tb)
    alive = np.zeros(total, np.uint32)
    born = np.zeros(total, np.uint32)
    f = rng.random(total).astype(np.float32)
    ids = np.zeros(total, np.uint32)
    nid = np.zeros(len(pops), np.uint32)
    for k, (n, cap) in enumerate(zip(pops, caps)):
        rb = arr[k].row_begin
        alive[rb:rb + n] = rng.random(n) >= 0.3
        if with_births:
            born[rb:rb + n] = (rng.random(n) < 0.4) * (1 + (rng.random(n) < 0.1))  # some ids claimed (2)
        ids[rb:rb + n] = np.arange(1, n + 1)
        nid[k] = n + 1
        alive[rb + n:rb + cap] = 1  # stale flags past the count must be ignored
        born[rb + n:rb + cap] = 1
    dev = "cuda"
    d_inst = torch.frombuffer(bytearray(bytes(arr)), dtype=torch.uint8).to(dev)
    d_tb = torch.tensor(list(tb), dtype=torch.int32, device=dev)
    counts = torch.tensor(pops, dtype=torch.int32, device=dev)
    next_ids = torch.from_numpy(nid.view(np.int32)).to(dev)
    f_in = torch.from_numpy(f).to(dev)
    id_in = torch.from_numpy(ids.view(np.int32)).to(dev)
    bf_in = f_in * 10 + 1
    bid_in = torch.from_numpy((ids + 100_000).view(np.int32)).to(dev)  # a claimed birth keeps this id
    f_out = torch.zeros(total, dtype=torch.float32, device=dev)
    id_out = torch.zeros(total, dtype=torch.int32, device=dev)
    cols = capi.columns([(f_in, f_out), (id_in, id_out)])
    bcols = capi.columns([(bf_in, f_out), (bid_in, id_out)])
    a_t = torch.from_numpy(alive.view(np.int32)).to(dev)
    b_t = torch.from_numpy(born.view(np.int32)).to(dev) if with_births else None
    ws = capi.Workspace(L.fg_compact_batched_workspace_size(ntiles, len(pops)))
    for _ in range(2):  # the second call reuses the workspace (other status array)
        capi.check(L.fg_compact_agents_batched(d_inst.data_ptr(), d_tb.data_ptr(), len(pops), ntiles, total,
                                               counts.data_ptr(), a_t.data_ptr(), capi.ptr(b_t), cols, bcols, 2, 1,
                                               next_ids.data_ptr(), ws.ptr, ws.nbytes, capi.stream_handle()),
                   "fg_compact_agents_batched")
        torch.cuda.synchronize()
        got_f, got_id = f_out.cpu().numpy(), id_out.cpu().numpy().view(np.uint32)
        got_n, got_nid = counts.cpu().numpy(), next_ids.cpu().numpy().view(np.uint32)
        for k, (n, cap) in enumerate(zip(pops, caps)):
            rb = arr[k].row_begin
            surv = O.compact(alive[rb:rb + n])
            kids = O.compact(born[rb:rb + n]) if with_births else np.zeros(0, np.uint32)
            kids = kids[:max(0, cap - len(surv))]
            m = len(surv) + len(kids)
            assert got_n[k] == m, k
            np.testing.assert_array_equal(got_f[rb:rb + len(surv)], f[rb + surv])
            np.testing.assert_array_equal(got_id[rb:rb + len(surv)], ids[rb + surv])
            if len(kids):
                np.testing.assert_array_equal(got_f[rb + len(surv):rb + m], f[rb + kids] * 10 + 1)
                claimed = born[rb + kids] == 2
                r = np.arange(len(kids), dtype=np.uint32)
                want = np.where(claimed, ids[rb + kids] + 100_000, n + 1 + r)
                np.testing.assert_array_equal(got_id[rb + len(surv):rb + m], want)
            assert got_nid[k] == n + 1 + (len(O.compact(born[rb:rb + n])) if with_births else 0)
        # back to the inputs for the second call
        counts.copy_(torch.tensor(pops, dtype=torch.int32))
        next_ids.copy_(torch.from_numpy(nid.view(np.int32)))
    assert ws.status() == (capi.FG_ERR_CAPACITY if with_births else capi.FG_OK)
