"""Every device-side wait of the kernel library is bounded; these tests make
the look-back waits run out and check that the kernels give up, record
FG_ERR_DEVICE_TIMEOUT in the workspace and return, and that the workspace is
exact again once the defaults are restored.

The failure is injected on the host, through the workspace header
(fg_workspace_set_wait_limit): tile 0 of the next scans and compactions does
not publish its status, and the poll bound is cut to a few dozen polls, so
each wait on tile 0 ends in microseconds. Nothing faults, traps or hangs.
The waits replaced are CUB's unbounded look-back in cub::DeviceScan::ExclusiveSum
(src/flamegpu/runtime/messaging/MessageSpatial3D.cu:134) and the scan of the
death/birth scatter (src/flamegpu/simulation/detail/CUDAScatter.cu:67-88).
"""
import time

import numpy as np
import pytest

import oracle as O

LIMIT = 64  # polls of one predecessor before a look-back gives up


def _capi():
    from flamegpu2_gb300 import capi
    return capi


@pytest.mark.gpu
@pytest.mark.parametrize("n", [3 * 4096 + 5, 5_000_000])
def test_scan_lookback_gives_up_and_recovers(n):
    import torch
    capi = _capi()
    L = capi.lib()
    st = capi.stream_handle()
    a = np.random.default_rng(n).integers(0, 7, n).astype(np.uint32)
    t = torch.from_numpy(a.view(np.int32)).cuda()
    out = torch.empty_like(t)
    ws = capi.Workspace(L.fg_scan_workspace_size(n))
    ws.set_wait_limit(LIMIT, withhold_first_tile=True)
    t0 = time.perf_counter()
    capi.check(L.fg_exclusive_scan_u32(t.data_ptr(), out.data_ptr(), n, ws.ptr, ws.nbytes, st), "scan")
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 5.0
    assert ws.status(clear=True) == capi.FG_ERR_DEVICE_TIMEOUT
    expect = (np.cumsum(a.astype(np.uint64)) - a).astype(np.uint32)
    got = out.cpu().numpy().view(np.uint32)
    # tile 0 needs no look-back; the tiles after it lost tile 0's total
    np.testing.assert_array_equal(got[:4096], expect[:4096])
    assert not np.array_equal(got, expect)
    # defaults back: the same workspace scans exactly, twice, with a clean status
    ws.set_wait_limit(0, withhold_first_tile=False)
    for _ in range(2):
        capi.check(L.fg_exclusive_scan_u32(t.data_ptr(), out.data_ptr(), n, ws.ptr, ws.nbytes, st), "scan")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), expect)
    assert ws.status() == capi.FG_OK


@pytest.mark.gpu
def test_build_scan_gives_up_and_recovers():
    import torch
    capi = _capi()
    L = capi.lib()
    st = capi.stream_handle()
    n = 40_000
    rng = np.random.default_rng(3)
    g = capi.grid(3, (0, 0, 0), (64, 64, 64), 2.0)  # 32^3 bins: 9 scan tiles
    pos = rng.random((n, 3), dtype=np.float32) * 64
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, k])).cuda() for k in range(3)]
    rec = capi.record_desc(cols)
    srt = torch.zeros((n, rec.words), dtype=torch.int32, device="cuda")
    pbm = torch.zeros(g.binCount + 1, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(L.fg_spatial_build_workspace_size(n, g.binCount))

    def build():
        capi.check(L.fg_spatial_build(g, n, None, cols[0].data_ptr(), cols[1].data_ptr(), cols[2].data_ptr(), None,
                                      rec, srt.data_ptr(), pbm.data_ptr(), ws.ptr, ws.nbytes, st), "build")
        torch.cuda.synchronize()

    ws.set_wait_limit(LIMIT, withhold_first_tile=True)
    build()
    assert ws.status(clear=True) == capi.FG_ERR_DEVICE_TIMEOUT
    ws.set_wait_limit(0, withhold_first_tile=False)
    build()
    build()
    og = O.grid(3, [0, 0, 0], [64, 64, 64], 2.0)
    epbm, eperm, _ = O.spatial_build(og, pos[:, 0], pos[:, 1], pos[:, 2])
    np.testing.assert_array_equal(pbm.cpu().numpy().view(np.uint32), epbm)
    np.testing.assert_array_equal(srt.cpu().numpy()[:, :3].view(np.float32), pos[eperm])
    assert ws.status() == capi.FG_OK


@pytest.mark.gpu
@pytest.mark.parametrize("n", [5 * 2048 + 3, 600_000])
def test_compaction_lookback_gives_up_and_recovers(n):
    import torch
    capi = _capi()
    L = capi.lib()
    st = capi.stream_handle()
    rng = np.random.default_rng(n)
    alive = (rng.random(n) >= 0.3).astype(np.uint32)
    f = rng.random(n).astype(np.float32)
    f_in = torch.from_numpy(f).cuda()
    f_out = torch.zeros(n, dtype=torch.float32, device="cuda")
    a_t = torch.from_numpy(alive.view(np.int32)).cuda()
    n_out = torch.zeros(1, dtype=torch.int32, device="cuda")
    cols = capi.columns([(f_in, f_out)])
    ws = capi.Workspace(L.fg_compact_workspace_size(n))

    def compact():
        capi.check(L.fg_compact_agents(n, None, a_t.data_ptr(), None, cols, None, 1, -1, None, None, n_out.data_ptr(),
                                       n, ws.ptr, ws.nbytes, st), "compact")
        torch.cuda.synchronize()

    ws.set_wait_limit(LIMIT, withhold_first_tile=True)
    t0 = time.perf_counter()
    compact()
    assert time.perf_counter() - t0 < 5.0
    assert ws.status(clear=True) == capi.FG_ERR_DEVICE_TIMEOUT
    ws.set_wait_limit(0, withhold_first_tile=False)
    surv = O.compact(alive)
    for _ in range(3):  # both status arrays of the workspace, then the first again
        compact()
        assert int(n_out.item()) == len(surv)
        np.testing.assert_array_equal(f_out.cpu().numpy()[:len(surv)], f[surv])
    assert ws.status() == capi.FG_OK


def test_wait_limit_rejects_bad_workspace():
    capi = _capi()
    L = capi.lib()
    assert L.fg_workspace_set_wait_limit(None, 256, 8, 1, None) == capi.FG_ERR_INVALID_ARGUMENT
    assert L.fg_workspace_set_wait_limit(256, 16, 8, 1, None) == capi.FG_ERR_INVALID_ARGUMENT
    assert L.fg_workspace_set_wait_limit(257, 256, 8, 1, None) == capi.FG_ERR_INVALID_ARGUMENT
