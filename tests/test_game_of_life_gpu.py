"""Conway's Game of Life on a wrapped MessageArray2D (the reference's
examples/cpp/game_of_life/src/main.cu), through game_of_life in
examples/game_of_life/game_of_life.cu, against numpy's toroidal update: every
cell's state after each step, exactly."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _life(grid):
    n = sum(np.roll(np.roll(grid, dx, 0), dy, 1) for dx in (-1, 0, 1) for dy in (-1, 0, 1) if dx or dy)
    return ((n == 3) | ((grid == 1) & (n == 2))).astype(np.uint32)


@pytest.mark.parametrize("side,steps,use_graphs", [(64, 30, True), (64, 5, False), (257, 12, True)])
def test_game_of_life_matches_numpy(side, steps, use_graphs):
    from flamegpu2_gb300 import sim
    rng = np.random.default_rng(side)
    grid = (rng.random((side, side)) < 0.35).astype(np.uint32)  # grid[x, y]
    xs, ys = np.meshgrid(np.arange(side), np.arange(side), indexing="ij")
    pos = np.stack([xs.ravel(), ys.ravel()], 1).astype(np.uint32)
    order = rng.permutation(side * side)  # agents in no particular order
    s = sim.Simulation("game_of_life", [side], use_graphs=use_graphs)
    s.set_population("cell", side * side, {"pos": np.ascontiguousarray(pos[order]),
                                           "is_alive": grid.ravel()[order].copy()})
    for _ in range(steps):
        s.step(1)
        grid = _life(grid)
        got_pos = s.get("cell", "pos", np.uint32, elements=2)
        alive = s.get("cell", "is_alive", np.uint32)
        now = np.zeros((side, side), np.uint32)
        now[got_pos[:, 0], got_pos[:, 1]] = alive
        np.testing.assert_array_equal(now, grid)
    s.close()
