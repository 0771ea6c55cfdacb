"""Host-side logic of the batched domains: the tile planner of the C ABI and
the batch validation, on CPU."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from lettuce_gb300 import _lib
from lettuce_gb300._batched import DOMAIN_DTYPE, TILE_DTYPE, plan_tiles


def _domains(sizes):
    d = np.zeros(len(sizes), dtype=DOMAIN_DTYPE)
    for i, s in enumerate(sizes):
        d[i]["res"] = list(s) + [1] * (3 - len(s))
        d[i]["tau"] = 0.6
    return d


@pytest.mark.parametrize("tile_cells", [1, 100, 1000, 4096, 10 ** 6])
def test_tiles_cover_every_row_once(lgb, tile_cells):
    rng = np.random.default_rng(4)
    sizes = [tuple(int(v) for v in rng.integers(1, 300, size=2)) for _ in range(40)]
    tiles = plan_tiles(_lib.D2Q9, _domains(sizes), tile_cells)
    assert tiles.dtype == TILE_DTYPE
    for b, (nx, ny) in enumerate(sizes):
        t = tiles[tiles["domain"] == b]
        assert t["row_begin"][0] == 0 and t["row_end"][-1] == nx
        assert np.all(t["row_begin"][1:] == t["row_end"][:-1])
        rows = t["row_end"] - t["row_begin"]
        assert np.all(rows >= 1)
        per = max(1, tile_cells // ny)
        assert np.all(rows[:-1] == per) and rows[-1] <= per


def test_tiles_3d_rows(lgb):
    tiles = plan_tiles(_lib.D3Q19, _domains([(4, 5, 6), (3, 2, 100)]), 60)
    assert list(tiles[tiles["domain"] == 0]["row_end"]) == [10, 20]
    assert len(tiles[tiles["domain"] == 1]) == 6


def test_plan_errors(lgb):
    with pytest.raises(_lib.LibraryError, match="resolution"):
        plan_tiles(_lib.D2Q9, _domains([(0, 5)]), 10)
    with pytest.raises(_lib.LibraryError, match="tile_cells"):
        plan_tiles(_lib.D2Q9, _domains([(3, 5)]), 0)


def test_batched_config_is_seeded():
    a = np.random.default_rng(0).integers(32, 513, size=(256, 2))
    assert a.min() >= 32 and a.max() <= 512
    cells = int(np.prod(a, axis=1).sum())
    assert 15e6 < cells < 25e6  # about 256 * 272^2


def test_batch_validation_on_cpu():
    ctx = lt.Context("cpu")
    flows = [lt.TaylorGreenVortex(ctx, [8, 8], 100, 0.05, lt.D2Q9)]
    with pytest.raises(RuntimeError, match="CUDA"):
        lt.BatchedSimulation(flows, [lt.TRTCollision(0.6)])
    with pytest.raises(ValueError):
        lt.BatchedSimulation(flows, [])
