"""fg_exclusive_scan_u32_noalloc: the exclusive scan with its scratch in the
library's static device memory. Compared with fg_exclusive_scan_u32 (caller
scratch) on the same inputs, two calls in a row. The file is collected last so
that it also runs after every other test has used the library; it passes in a
fresh process too."""
import numpy as np
import pytest


def _capi():
    from flamegpu2_gb300 import capi
    return capi


def test_noalloc_scan_declared_and_exported():
    capi = _capi()
    for name in ("fg_exclusive_scan_u32_noalloc", "fg_noalloc_scan_status"):
        assert name in capi.EXPORTS
        assert hasattr(capi.lib(), name)


def test_noalloc_scan_rejects_before_touching_the_device():
    capi = _capi()
    L = capi.lib()
    # too large: refused with FG_ERR_WORKSPACE before any CUDA call
    assert L.fg_exclusive_scan_u32_noalloc(8, 8, capi.FG_NOALLOC_SCAN_MAX_N + 1, None) == capi.FG_ERR_WORKSPACE
    assert L.fg_exclusive_scan_u32_noalloc(None, None, 5, None) == capi.FG_ERR_INVALID_ARGUMENT


@pytest.mark.gpu
@pytest.mark.parametrize("n", [0, 1, 4095, 4097, 1_000_003, 1 << 25])
def test_noalloc_scan_matches_workspace_scan(n):
    import torch
    capi = _capi()
    L = capi.lib()
    st = capi.stream_handle()
    for call in range(2):  # two calls in a row on the same static scratch
        rng = np.random.default_rng(1000 * call + n % 997)
        a = rng.integers(0, 1 << 7, max(n, 1)).astype(np.uint32)[:n]
        t = torch.from_numpy(a.view(np.int32)).cuda()
        got = torch.full_like(t, -1)
        ref = torch.full_like(t, -1)
        ws = capi.Workspace(L.fg_scan_workspace_size(n))
        capi.check(L.fg_exclusive_scan_u32(t.data_ptr(), ref.data_ptr(), n, ws.ptr, ws.nbytes, st), "scan")
        capi.check(L.fg_exclusive_scan_u32_noalloc(t.data_ptr() if n else None, got.data_ptr() if n else None, n,
                                                   st), "noalloc scan")
        torch.cuda.synchronize()
        np.testing.assert_array_equal(got.cpu().numpy(), ref.cpu().numpy())
        expect = (np.cumsum(a.astype(np.uint64)) - a).astype(np.uint32)
        np.testing.assert_array_equal(got.cpu().numpy().view(np.uint32), expect)
        # the device-side status of the static scratch: no bounded wait gave up
        assert L.fg_noalloc_scan_status(st, 1) == capi.FG_OK


@pytest.mark.gpu
@pytest.mark.parametrize("n", [300_000, (1 << 22) + 4097, 1 << 25])
def test_noalloc_scan_in_place(n):
    # n above 2^22 takes the four-sub-tile path, which reads its input again
    # after the look-back: in place, every tile must still see its own input
    import torch
    capi = _capi()
    L = capi.lib()
    a = np.random.default_rng(5).integers(0, 9, n).astype(np.uint32)
    t = torch.from_numpy(a.view(np.int32)).cuda()
    capi.check(L.fg_exclusive_scan_u32_noalloc(t.data_ptr(), t.data_ptr(), n, capi.stream_handle()), "in place")
    torch.cuda.synchronize()
    np.testing.assert_array_equal(t.cpu().numpy().view(np.uint32), (np.cumsum(a.astype(np.uint64)) - a).astype(np.uint32))
    assert L.fg_noalloc_scan_status(capi.stream_handle(), 1) == capi.FG_OK


@pytest.mark.gpu
def test_noalloc_scan_max_size_refused():
    import torch
    capi = _capi()
    L = capi.lib()
    big = torch.zeros(16, dtype=torch.int32, device="cuda")
    assert L.fg_exclusive_scan_u32_noalloc(big.data_ptr(), big.data_ptr(), capi.FG_NOALLOC_SCAN_MAX_N + 1,
                                           capi.stream_handle()) == capi.FG_ERR_WORKSPACE
