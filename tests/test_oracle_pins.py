"""Pins the serial oracle against the reference tests' own known answers.

Inputs and expectations come from tests/golden (see make_golden.py): the
reference tests' generators and host-side expectation code, restated, plus the
reference's own approxExactlyDivisible compiled from its source tree.
"""
import json
import os
import struct

import numpy as np
import pytest

import oracle as O

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _f(bits):
    return struct.unpack("<f", struct.pack("<I", bits))[0]


def test_wrap_compatible_matches_reference_numeric():
    rows = json.load(open(os.path.join(GOLDEN, "wrap_compatible.json")))["rows"]
    assert len(rows) > 100
    for r in rows:
        assert O.approx_exactly_divisible(_f(r["x_bits"]), _f(r["y_bits"])) == bool(r["r"]), r


@pytest.mark.parametrize("optional", [False, True])
def test_spatial3d_mandatory_optional_counts(golden, optional):
    # test_spatial_3d.cu Mandatory / Optional: 2049 agents in [0,5)^3, r=1, 5^3 bins.
    pre = "s3d_optional_" if optional else "s3d_mandatory_"
    pos = golden[pre + "pos"].reshape(-1, 3)
    g = O.grid(3, (0, 0, 0), (5, 5, 5), 1.0)
    assert tuple(g.gridDim) == (5, 5, 5) and g.binCount == 125
    r = O.count_model(g, False, pos[:, 0], pos[:, 1], pos[:, 2],
                      do_output=golden[pre + "do_output"] if optional else None)
    order = r["order"]
    expect = golden[pre + "expect"][order]
    np.testing.assert_array_equal(r["count"], expect)
    assert int(r["badCount"].sum()) == 0


@pytest.mark.parametrize("optional", [False, True])
def test_spatial2d_mandatory_optional_counts(golden, optional):
    pre = "s2d_optional_" if optional else "s2d_mandatory_"
    pos = golden[pre + "pos"].reshape(-1, 2)
    g = O.grid(2, (0, 0), (11, 11), 1.0)
    assert g.binCount == 121
    r = O.count_model(g, False, pos[:, 0], pos[:, 1], None,
                      do_output=golden[pre + "do_output"] if optional else None)
    np.testing.assert_array_equal(r["count"], golden[pre + "expect"][r["order"]])
    assert int(r["badCount"].sum()) == 0


@pytest.mark.parametrize("off", [(0.0, 0.0, 0.0), (141.0, -540.0, 200.0), (-1401.5, 5640.3, -2008.8)])
def test_spatial3d_wrapped_lattice(off):
    # test_spatial_3d.cu:855-974: 35^3 lattice spacing 2, r=3.5, width 70.
    i, j, k = np.meshgrid(np.arange(35), np.arange(35), np.arange(35), indexing="ij")
    x = (i.ravel() * np.float32(2.0) + np.float32(off[0])).astype(np.float32)
    y = (j.ravel() * np.float32(2.0) + np.float32(off[1])).astype(np.float32)
    z = (k.ravel() * np.float32(2.0) + np.float32(off[2])).astype(np.float32)
    g = O.grid(3, (0 + off[0], 0 + off[1], 0 + off[2]), (70 + off[0], 70 + off[1], 70 + off[2]), 3.5)
    r = O.count_model(g, True, x, y, z)
    assert np.all(r["count"] == 27)
    assert np.all(r["badCount"] <= 189)
    assert np.all(r["result_x"] == 0.0) and np.all(r["result_y"] == 0.0) and np.all(r["result_z"] == 0.0)


@pytest.mark.parametrize("off", [(0.0, 0.0), (141.0, 0.0), (0.0, 3440.0), (-2342.0, 0.0), (0.0, -7540.0),
                                 (-141.0, 0.0), (141.4, -540.7)])
def test_spatial2d_wrapped_lattice(off):
    # test_spatial_2d.cu:824-906: 15^2 lattice spacing 2, r=3, width 30.
    i, j = np.meshgrid(np.arange(15), np.arange(15), indexing="ij")
    x = (i.ravel() * np.float32(2.0) + np.float32(off[0])).astype(np.float32)
    y = (j.ravel() * np.float32(2.0) + np.float32(off[1])).astype(np.float32)
    g = O.grid(2, (0 + off[0], 0 + off[1]), (30 + off[0], 30 + off[1]), 3.0)
    r = O.count_model(g, True, x, y, None)
    assert np.all(r["count"] == 9)
    assert np.all(r["badCount"] <= 18)
    assert np.all(r["result_x"] == 0.0) and np.all(r["result_y"] == 0.0)


def test_spatial3d_bounds_not_factor_radius():
    # test_spatial_3d.cu:1111-1197 (bug #1157): 6x6x6 grid, last bin 0.1 wide.
    h = np.float32(50.1) / np.float32(2)
    x = np.array([h, h, 0.0, 18.0, h, h], np.float32)
    y = np.array([0.0, 18.0, h, h, 50.0, 50.0], np.float32)
    z = np.array([h, h, 0.5, 0.5, 50.1, np.float32(50.1) - np.float32(10.11)], np.float32)
    g = O.grid(3, (0, 0, 0), (50.1, 50.1, 50.1), 10.0)
    assert tuple(g.gridDim) == (6, 6, 6)
    # count of messages in the Moore neighbourhood (no radius filter), per agent id
    pbm, perm, _ = O.spatial_build(g, x, y, z)
    counts = [len(O.neighbours(g, pbm, float(x[a]), float(y[a]), float(z[a]))) for a in range(6)]
    assert counts == [2, 2, 2, 2, 1, 1]


def test_read_empty():
    # test_spatial_3d.cu:507-540: iterating a list nothing was output to yields nothing.
    g = O.grid(3, (-3, -3, -3), (3, 3, 3), 2.0)
    pbm, perm, _ = O.spatial_build(g, np.zeros(0, np.float32), np.zeros(0, np.float32), np.zeros(0, np.float32))
    assert len(O.neighbours(g, pbm, 0.0, 0.0, 0.0)) == 0


def test_agent_death_order(golden):
    # test_cuda_simulation.cu:406-434: agents with even x die; survivors keep order.
    x = golden["death_x"]
    keep = O.compact((x % 2 != 0).astype(np.uint32))
    np.testing.assert_array_equal(x[keep], golden["death_expect"])


def test_pbm_is_exclusive_scan_and_stable():
    rng = np.random.default_rng(5)
    n = 5000
    x, y, z = (rng.uniform(-1, 9, n).astype(np.float32) for _ in range(3))
    g = O.grid(3, (0, 0, 0), (8, 8, 8), 1.0)
    pbm, perm, bins = O.spatial_build(g, x, y, z)
    hist = np.bincount(bins, minlength=g.binCount + 1)
    np.testing.assert_array_equal(pbm, np.concatenate([[0], np.cumsum(hist)[:-1]]).astype(np.uint32))
    assert pbm[-1] == n
    # stable: within each bin the original indices ascend
    np.testing.assert_array_equal(perm, np.lexsort((np.arange(n), bins)).astype(np.uint32))


def test_sort_key_matches_reference_formula():
    # calculateSpatialHash (CUDASimulation.cu:380-408) in numpy float32 arithmetic
    g = O.grid(3, (0, 0, 0), (64, 64, 64), 2.0)
    rng = np.random.default_rng(1)
    x, y, z = (rng.uniform(-3, 67, 300).astype(np.float32) for _ in range(3))
    w = np.float32(64.0)
    gd = np.float32(32.0)
    gx = np.floor(((x - np.float32(0)) / w) * gd).astype(np.int64)
    gy = np.floor(((y - np.float32(0)) / w) * gd).astype(np.int64)
    gz = np.floor(((z - np.float32(0)) / w) * gd).astype(np.int64)
    expect = ((gz * 32 * 32 + gy * 32 + gx) & 0xFFFFFFFF).astype(np.uint32)
    np.testing.assert_array_equal(O.sort_keys(g, x, y, z), expect)
    assert O.sort_max_bit(g) == 16
