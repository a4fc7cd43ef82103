"""Array messages (MessageArray, MessageArray2D, MessageArray3D): the known
answers of the reference's tests (tests/test_cases/runtime/messaging/
test_array.cu, test_array_2d.cu, test_array_3d.cu), through the models of
examples/array_message_tests/array_message_tests.cu:

* Mandatory / Optional / OptionalNone: every agent outputs index * 3 to the
  cell of a shuffled index (optional: even ones only) and reads its own
  cell: index * 3 (0 where nothing was output).
* DuplicateOutputException: two messages to one cell raise
  ArrayMessageWriteConflict.
* Moore (wrapped and clamped) and von Neumann searches over every small grid
  and radius of the reference's lists: the number of messages read and their
  values against their coordinates; a wrapped search wider than the array is
  a device error.
* ReadEmpty: a list nothing output reads 0.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODELS = {1: "array1d", 2: "array2d", 3: "array3d"}


def _sim():
    from flamegpu2_gb300 import sim
    return sim


def _params(variant, dims, radius=1):
    d = list(dims) + [1] * (3 - len(dims))
    return [variant] + d + [radius]


def _run(D, variant, dims, cols, n, radius=1, use_graphs=True):
    S = _sim()
    s = S.Simulation(MODELS[D], _params(variant, dims, radius), use_graphs=use_graphs, check_each_step=True)
    s.set_population("agent", n, cols)
    s.step(1)
    out = {k: s.get("agent", k, np.uint32) for k in ("index", "message_read", "value_success", "x", "y", "z")}
    s.close()
    return out


def _write_pop(n, seed):
    perm = np.random.default_rng(seed).permutation(n).astype(np.uint32)
    return {"index": np.arange(n, dtype=np.uint32), "message_write": perm}


SHAPES = {1: (156,), 2: (12, 13), 3: (5, 6, 7)}


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("use_graphs", [True, False])
def test_mandatory(D, use_graphs):
    dims = SHAPES[D]
    n = int(np.prod(dims))
    r = _run(D, 0, dims, _write_pop(n, D), n, use_graphs=use_graphs)
    np.testing.assert_array_equal(r["message_read"], r["index"] * 3)


@pytest.mark.parametrize("D", [1, 2, 3])
def test_optional(D):
    dims = SHAPES[D]
    n = int(np.prod(dims))
    r = _run(D, 1, dims, _write_pop(n, 10 + D), n)
    idx = r["index"]
    np.testing.assert_array_equal(r["message_read"], np.where(idx % 2 == 0, idx * 3, 0))


@pytest.mark.parametrize("D", [1, 2, 3])
def test_optional_none(D):
    dims = SHAPES[D]
    n = int(np.prod(dims))
    r = _run(D, 2, dims, _write_pop(n, 20 + D), n)
    np.testing.assert_array_equal(r["message_read"], np.zeros(n, np.uint32))


@pytest.mark.parametrize("D", [1, 2, 3])
def test_duplicate_output_raises(D):
    S = _sim()
    dims = SHAPES[D]
    n = int(np.prod(dims))
    with pytest.raises(S.SimError, match="ArrayMessageWriteConflict"):
        _run(D, 3, dims, {"message_write": np.arange(n, dtype=np.uint32)}, n)


def test_zero_dimension_rejected():
    S = _sim()
    with pytest.raises(S.SimError, match="InvalidArgument"):
        S.Simulation("array2d", _params(0, (0, 12)))


def test_read_empty():
    r = _run(2, 8, (2, 2), {"index": np.zeros(1, np.uint32)}, 1)
    assert r["message_read"].tolist() == [0]


def _grid_pop(dims):
    cells = list(itertools.product(*[range(d) for d in dims]))
    n = len(cells)
    c = np.array(cells, dtype=np.uint32).reshape(n, len(dims))
    cols = {"index": np.arange(n, dtype=np.uint32), "x": c[:, 0].copy()}
    cols["y"] = c[:, 1].copy() if len(dims) > 1 else np.zeros(n, np.uint32)
    cols["z"] = c[:, 2].copy() if len(dims) > 2 else np.zeros(n, np.uint32)
    return cols, n


def _expected(D, dims, loc, r, wrap, vn):
    count = 0
    for off in itertools.product(range(-r, r + 1), repeat=D):
        if not any(off):
            continue
        if vn and sum(abs(o) for o in off) > r:
            continue
        if not wrap and any(not (0 <= loc[a] + off[a] < dims[a]) for a in range(D)):
            continue
        count += 1
    return count


CASES = {
    1: [((1,), 1), ((2,), 1), ((3,), 1), ((4,), 1), ((1,), 2), ((4,), 2), ((5,), 2), ((6,), 2)],
    2: [((1, 1), 1), ((2, 2), 1), ((3, 3), 1), ((4, 4), 1), ((2, 1), 1), ((4, 1), 1),
        ((1, 1), 2), ((3, 3), 2), ((5, 5), 2), ((6, 6), 2), ((5, 1), 2), ((6, 1), 2)],
    3: [((1, 1, 1), 1), ((3, 3, 3), 1), ((4, 4, 4), 1), ((2, 1, 3), 1), ((5, 5, 5), 2), ((6, 5, 7), 2), ((3, 3, 3), 2)],
}


@pytest.mark.parametrize("D", [1, 2, 3])
@pytest.mark.parametrize("kind", ["moore_wrap", "moore", "vn_wrap", "vn"])
def test_neighbourhood_searches(D, kind):
    if D == 1 and kind.startswith("vn"):
        pytest.skip("1D arrays have no von Neumann search (the same cells as Moore)")
    S = _sim()
    variant = {"moore_wrap": 4, "moore": 5, "vn_wrap": 6, "vn": 7}[kind]
    wrap = kind.endswith("wrap")
    for dims, r in CASES[D]:
        cols, n = _grid_pop(dims)
        if wrap and any(2 * r + 1 > d for d in dims):
            # a wrapped search wider than the array would read cells twice
            with pytest.raises(S.SimError, match="DeviceError"):
                _run(D, variant, dims, cols, n, radius=r)
            continue
        out = _run(D, variant, dims, cols, n, radius=r)
        assert (out["value_success"] == 1).all(), (dims, r)
        for i in range(n):
            loc = (int(out["x"][i]), int(out["y"][i]), int(out["z"][i]))
            assert out["message_read"][i] == _expected(D, dims, loc, r, wrap, kind.startswith("vn")), (dims, r, loc)
