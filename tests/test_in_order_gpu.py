"""Builds and agent sorts whose keys are already in row order.

When every row carries a key and the keys never descend over the rows, the
stable counting sort is the identity: the key launch compares neighbouring
rows inside 32-row groups, the scan compares rows 32w - 1 and 32w, and with no
descent found the placement and ranking kernels are skipped and each row is
written in place. These tests put the descents exactly where each of the two
checks has to find them (inside a group, across a group boundary, a row
without a message) and compare every result with the serial oracle, so a
wrong choice of path shows up as a wrong order. The reference's build has no
such path (src/flamegpu/runtime/messaging/MessageSpatial3D.cu:113-146 always
sorts); its result is the same sorted order.
"""
import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _capi():
    from flamegpu2_gb300 import capi
    return capi


def _bin_sorted(rng, n, dims, edge, r):
    """n positions in [0, edge)^dims, rows in message-bin order (each bin's rows in draw order)."""
    pos = rng.uniform(0.0, edge, (n, dims)).astype(np.float32)
    og = O.grid(dims, [0.0] * dims, [edge] * dims, r)
    _, perm, _ = O.spatial_build(og, *[pos[:, a] for a in range(dims)])
    return pos[perm]


def _build(g, pos, valid=None, d_count=None, ws=None):
    import torch
    capi = _capi()
    n = pos.shape[0]
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(pos.shape[1])]
    payload = torch.arange(n * 2, dtype=torch.int32, device="cuda").reshape(n, 2) * 5 + 1
    rec = capi.record_desc(cols + [payload])
    srt = torch.zeros((max(n, 1), rec.words), dtype=torch.int32, device="cuda")
    pbm = torch.zeros(g.binCount + 1, dtype=torch.int32, device="cuda")
    if ws is None:
        ws = capi.Workspace(capi.lib().fg_spatial_build_workspace_size(max(n, 1), g.binCount))
    vt = None if valid is None else torch.from_numpy(valid.astype(np.uint32)).cuda()
    dn = None if d_count is None else torch.tensor([d_count], dtype=torch.int32, device="cuda")
    capi.check(capi.lib().fg_spatial_build(C.byref(g), n, capi.ptr(dn), cols[0].data_ptr(), cols[1].data_ptr(),
                                           cols[2].data_ptr() if len(cols) == 3 else None, capi.ptr(vt), C.byref(rec),
                                           srt.data_ptr(), pbm.data_ptr(), ws.ptr, ws.nbytes, capi.stream_handle()),
               "fg_spatial_build")
    torch.cuda.synchronize()
    assert ws.status() == 0
    return pbm.cpu().numpy().view(np.uint32), srt.cpu().numpy(), payload.cpu().numpy()


def _check_build(g, pos, valid=None, d_count=None, ws=None):
    dims = pos.shape[1]
    pbm, srt, payload = _build(g, pos, valid, d_count, ws)
    n = pos.shape[0] if d_count is None else d_count
    keep = np.arange(n) if valid is None else np.nonzero(valid[:n])[0]
    og = O.grid(dims, list(g.min)[:dims], list(g.max)[:dims], g.radius)
    epbm, perm, _ = O.spatial_build(og, *[pos[keep][:, a] for a in range(dims)])
    eperm = keep[perm]
    np.testing.assert_array_equal(pbm, epbm)
    m = len(eperm)
    np.testing.assert_array_equal(srt[:m, :dims].view(np.float32), pos[eperm])
    np.testing.assert_array_equal(srt[:m, dims:dims + 2], payload[eperm])
    return eperm


def _differing_pair(pos, g, at, step=32):
    """Index j (at, at + step, ...) such that rows j, j + 1 lie in different bins
    (swapping them makes one descent); step keeps the pair's place in its 32-row group."""
    dims = pos.shape[1]
    og = O.grid(dims, list(g.min)[:dims], list(g.max)[:dims], g.radius)
    keys = O.spatial_build(og, *[pos[:, a] for a in range(dims)])[2]
    j = at
    while keys[j] == keys[j + 1]:
        j += step
    return j


@pytest.mark.parametrize("dims,edge,r", [(3, 32.0, 2.0), (2, 256.0, 4.0)])
@pytest.mark.parametrize("n", [1, 31, 32, 33, 64, 65, 5000, 100_003])
def test_build_of_rows_in_bin_order(dims, edge, r, n):
    rng = np.random.default_rng(n + dims)
    g = _capi().grid(dims, (0.0,) * dims, (edge,) * dims, r)
    pos = _bin_sorted(rng, n, dims, edge, r)
    eperm = _check_build(g, pos)
    np.testing.assert_array_equal(eperm, np.arange(n))


@pytest.mark.parametrize("where", ["group_boundary", "inside_group", "last_rows"])
def test_build_one_descent_is_found(where):
    # one pair of neighbouring rows in different bins exchanged: a single
    # descent, at a 32-row group boundary (rows 32w - 1, 32w: found by the
    # scan), inside a group (found by the key launch), or at the end
    rng = np.random.default_rng(7)
    n = 70_000
    g = _capi().grid(3, (0, 0, 0), (32, 32, 32), 2.0)
    pos = _bin_sorted(rng, n, 3, 32.0, 2.0)
    at = {"group_boundary": 32 * 777 - 1, "inside_group": 32 * 500 + 9, "last_rows": n - 2}[where]
    j = _differing_pair(pos, g, at, -32 if where == "last_rows" else 32)
    pos[[j, j + 1]] = pos[[j + 1, j]]
    eperm = _check_build(g, pos)
    assert not np.array_equal(eperm, np.arange(n))


def test_build_in_order_with_optional_messages_and_device_count():
    rng = np.random.default_rng(11)
    n = 20_000
    g = _capi().grid(3, (0, 0, 0), (32, 32, 32), 2.0)
    pos = _bin_sorted(rng, n, 3, 32.0, 2.0)
    valid = np.ones(n, np.uint32)
    valid[12_345] = 0  # a row without a message: its successors move down one place
    _check_build(g, pos, valid=valid)
    # rows past the device count are not looked at, even out of order
    tail = pos.copy()
    tail[15_000:] = tail[15_000:][::-1]
    eperm = _check_build(g, tail, d_count=15_000)
    np.testing.assert_array_equal(eperm, np.arange(15_000))


def test_in_order_and_shuffled_builds_alternate_on_one_workspace():
    rng = np.random.default_rng(13)
    capi = _capi()
    n = 50_000
    g = capi.grid(2, (0, 0), (128, 128), 2.0)
    ws = capi.Workspace(capi.lib().fg_spatial_build_workspace_size(n, g.binCount))
    in_order = _bin_sorted(rng, n, 2, 128.0, 2.0)
    shuffled = in_order[rng.permutation(n)]
    for p in (in_order, shuffled, in_order, in_order, shuffled, shuffled, in_order):
        _check_build(g, p, ws=ws)


@pytest.mark.parametrize("descent", [None, "group_boundary", "inside_group"])
def test_agent_sort_of_rows_in_key_order(descent):
    import torch
    capi = _capi()
    rng = np.random.default_rng(17)
    n = 40_000
    g = capi.grid(3, (0, 0, 0), (16, 16, 16), 1.0)
    og = O.grid(3, (0, 0, 0), (16, 16, 16), 1.0)
    pos = rng.uniform(0, 16, (n, 3)).astype(np.float32)
    keys = O.sort_keys(og, pos[:, 0], pos[:, 1], pos[:, 2])
    pos = pos[O.stable_sort_perm(keys, O.sort_max_bit(og))]
    if descent:
        keys = O.sort_keys(og, pos[:, 0], pos[:, 1], pos[:, 2])
        j = 32 * 333 - 1 if descent == "group_boundary" else 32 * 100 + 17
        while keys[j] == keys[j + 1]:
            j += 32
        pos[[j, j + 1]] = pos[[j + 1, j]]
    cols_in = [torch.from_numpy(np.ascontiguousarray(pos[:, a])).cuda() for a in range(3)]
    ids = torch.arange(1, n + 1, dtype=torch.int32, device="cuda")
    wide = torch.arange(n, dtype=torch.int64, device="cuda") * 7
    ins = cols_in + [ids, wide]
    outs = [torch.empty_like(c) for c in ins]
    perm = torch.zeros(n, dtype=torch.int32, device="cuda")
    ws = capi.Workspace(capi.lib().fg_spatial_sort_workspace_size(n, C.byref(g)))
    for _ in range(2):
        capi.check(capi.lib().fg_spatial_sort_agents(C.byref(g), n, None, cols_in[0].data_ptr(), cols_in[1].data_ptr(),
                                                     cols_in[2].data_ptr(), capi.columns(list(zip(ins, outs))),
                                                     len(ins), perm.data_ptr(), ws.ptr, ws.nbytes,
                                                     capi.stream_handle()), "sort")
    torch.cuda.synchronize()
    eperm = O.stable_sort_perm(O.sort_keys(og, pos[:, 0], pos[:, 1], pos[:, 2]), O.sort_max_bit(og))
    np.testing.assert_array_equal(perm.cpu().numpy().view(np.uint32), eperm)
    for a, b in zip(ins, outs):
        np.testing.assert_array_equal(b.cpu().numpy(), a.cpu().numpy()[eperm])
    assert (descent is None) == np.array_equal(eperm, np.arange(n))
    assert ws.status() == 0
