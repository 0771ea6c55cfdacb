"""Batched domains on the GPU: every domain of a batch evolves exactly as it
does alone under Simulation (same arithmetic, bit-identical), matches the
CPU oracle, and the CUDA-graph replay equals eager launches."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from lgb_helpers import rel_max, to_np

pytestmark = pytest.mark.gpu


def _batch(storage=None, dtype=torch.float32, n=7, seed=3, lo=9, hi=70):
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    return lt.batched_taylor_green(ctx, n_domains=n, seed=seed, side_min=lo, side_max=hi)


@pytest.mark.parametrize("dtype,storage", [(torch.float64, None), (torch.float32, None),
                                           (torch.float32, "fp16_shifted"),
                                           (torch.float32, "bf16_shifted")])
@pytest.mark.parametrize("persistent", [True, False], ids=["persistent", "block_per_tile"])
def test_batch_equals_single_domain_runs(lgb, dtype, storage, persistent):
    flows, colls = _batch(storage, dtype)
    singles, scolls = _batch(storage, dtype)
    sim = lt.BatchedSimulation(flows, colls, tile_cells=500, threads=128, persistent=persistent)
    assert sim.blocks == (min(sim.n_tiles, sim.sm_count * 16) if persistent else sim.n_tiles)
    sim(13)
    for fl, c, ref in zip(flows, scolls, singles):
        lt.Simulation(ref, c, [], lt.StreamingStrategy.PRE_STREAMING)(13)
        assert torch.equal(fl.f_raw, ref.f_raw)
        assert fl.i == 13


@pytest.mark.parametrize("storage", [None, "fp16_shifted"])
def test_host_rates_equal_kernel_rates(lgb, storage):
    """the per-domain float32 rates formed on the host (lgb_batch_desc.rates)
    and those the kernel forms from tau without the table give the same
    fields bit for bit"""
    a, ca = _batch(storage)
    b, cb = _batch(storage)
    sa = lt.BatchedSimulation(a, ca, tile_cells=500, threads=128)
    sb = lt.BatchedSimulation(b, cb, tile_cells=500, threads=128)
    assert sa._rates_dev is not None
    sb._rates_dev = None
    sa(9, use_graph=False)
    sb(9, use_graph=False)
    for x, y in zip(a, b):
        assert torch.equal(x.f_raw, y.f_raw)


def test_batch_against_oracle(lgb, oracle):
    flows, colls = _batch(None, torch.float64, n=5)
    f0 = [to_np(fl.f) for fl in flows]
    sim = lt.BatchedSimulation(flows, colls, tile_cells=1000, threads=256)
    sim(20)
    for fl, c, f in zip(flows, colls, f0):
        ref = oracle.run("D2Q9", f, 20, collision="trt", tau=c.tau_plus, tau_minus=c.tau_minus,
                         strategy="PRE_STREAMING")
        assert rel_max(to_np(fl.f), ref) < 1e-12


def test_graph_replay_equals_eager(lgb):
    a, ca = _batch()
    b, cb = _batch()
    sa = lt.BatchedSimulation(a, ca, tile_cells=777, threads=256)
    sb = lt.BatchedSimulation(b, cb, tile_cells=777, threads=256)
    sa(11, use_graph=True)
    sb(11, use_graph=False)
    for x, y in zip(a, b):
        assert torch.equal(x.f_raw, y.f_raw)
    sa(6)  # replays the captured graph
    sb(6, use_graph=False)
    for x, y in zip(a, b):
        assert torch.equal(x.f_raw, y.f_raw)


def test_autotune_keeps_state_and_caches(lgb, tmp_path, monkeypatch):
    monkeypatch.setenv("LGB_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    a, ca = _batch()
    b, cb = _batch()
    sa = lt.BatchedSimulation(a, ca)          # tunes, then caches
    assert (tmp_path / "tune.json").exists()
    assert sa.threads in (128, 256, 512) and sa.tile_cells > 0
    sb = lt.BatchedSimulation(b, cb, tile_cells=2048, threads=128)
    sa(5)
    sb(5)
    for x, y in zip(a, b):                    # tuning did not advance the state
        assert torch.equal(x.f_raw, y.f_raw)
    c, cc = _batch()
    sc = lt.BatchedSimulation(c, cc)          # cache hit: same shape, no retune
    assert (sc.threads, sc.tile_cells, sc.persistent) == (sa.threads, sa.tile_cells,
                                                          sa.persistent)
    assert not hasattr(sc, "tuning_results")


def test_invalid_tile_is_skipped_and_flagged(lgb):
    """a tile outside its domain is rejected by the kernel's own bounds
    check (status bit 1), the other tiles still step"""
    flows, colls = _batch(n=2)
    sim = lt.BatchedSimulation(flows, colls, tile_cells=100000, threads=128)
    tiles = sim._tiles_dev.cpu().numpy().view(np.int32).reshape(-1, 4).copy()
    tiles[0, 2] = 10 ** 6  # row_end far beyond the domain
    sim._tiles_dev = torch.from_numpy(tiles.view(np.uint8).reshape(-1)).cuda()
    sim(1, use_graph=False)
    assert sim.status & 2


def test_unpadded_odd_rows_of_16bit_batches_are_refused(lgb):
    """16-bit batches step two cells per 32-bit word: a domain whose odd rows
    are not padded (pitch 0 in place of length + 1) is skipped with status
    bit 1, and the other domains still step exactly as alone"""
    # the first seed whose three domains have odd and even row lengths
    seed = next(s for s in range(100)
                if len({int(z) % 2 for z in
                        np.random.default_rng(s).integers(9, 31, size=(3, 2))[:, 1]}) == 2)
    flows, colls = _batch("fp16_shifted", n=3, seed=seed, lo=9, hi=30)
    singles, scolls = _batch("fp16_shifted", n=3, seed=seed, lo=9, hi=30)
    sim = lt.BatchedSimulation(flows, colls, tile_cells=300, threads=128)
    odd = [b for b, fl in enumerate(flows) if fl.resolution[-1] % 2 == 1]
    even = [b for b, fl in enumerate(flows) if fl.resolution[-1] % 2 == 0]
    assert odd and even, [fl.resolution for fl in flows]
    dom = sim.domains.copy()
    dom["pitch"][odd[0]] = 0
    sim._domains_dev = torch.from_numpy(dom.view(np.uint8).copy()).cuda()
    sim(3, use_graph=False)
    assert sim.status & 2
    for b in even:
        lt.Simulation(singles[b], scolls[b], [], lt.StreamingStrategy.PRE_STREAMING)(3)
        assert torch.equal(flows[b].f_raw, singles[b].f_raw)
