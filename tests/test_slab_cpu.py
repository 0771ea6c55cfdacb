"""Halo indexing of the x-slab decomposition, on the CPU: the lattice is cut
into slabs, each slab is advanced by the oracle over its extended array
(periodic inside the slab), and the halo planes are moved by the product's
exchange routines, by copies within one process and by point-to-point
messages between two gloo ranks. The reassembled interiors must equal the
oracle's run over the whole lattice bit for bit."""
import os
import socket
import sys

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from conftest import ROOT, golden, meta

import lettuce_gb300 as lt
from lettuce_gb300 import _lib

STRATEGY = {_lib.PULL: "PRE_STREAMING", _lib.PUSH: "POST_STREAMING"}


@pytest.mark.parametrize("nx,parts", [(7, 2), (7, 3), (8, 4), (5, 5), (9, 1)])
def test_slab_partition(nx, parts):
    e_x = np.asarray(lt.D3Q19().e)[:, 0]
    slabs = [lt.Slab(nx, parts, i, e_x) for i in range(parts)]
    assert sum(s.nx for s in slabs) == nx
    assert max(s.nx for s in slabs) - min(s.nx for s in slabs) <= 1
    assert [s.x0 for s in slabs] == list(np.cumsum([0] + [s.nx for s in slabs])[:-1])
    for s in slabs:
        assert s.planes[0] == (s.x0 - 1) % nx and s.planes[-1] == (s.x0 + s.nx) % nx
        assert s.planes[1:-1] == list(range(s.x0, s.x0 + s.nx))
        assert len(s.rightward) == len(s.leftward) == 5
        assert all(e_x[q] == 1 for q in s.rightward) and all(e_x[q] == -1 for q in s.leftward)


def test_slab_rejects_bad_splits():
    e_x = np.asarray(lt.D2Q9().e)[:, 0]
    with pytest.raises(ValueError):
        lt.Slab(3, 4, 3, e_x)
    with pytest.raises(ValueError):
        lt.Slab(8, 2, 2, e_x)
    with pytest.raises(ValueError):
        lt.Slab(8, 2, 0, [0, 2, -2])


def _boundaries(res, with_bb):
    if not with_bb:
        return []
    rng = np.random.default_rng(3)
    return [{"kind": "bounce_back", "mask": rng.random(res) < 0.15}]


def _step_slab(oracle, name, slab, ext, pattern, post, tau):
    """one oracle step of the extended slab, its masks cut from the lattice's"""
    post_e = [dict(b, mask=slab.extend(torch.from_numpy(b["mask"]), 0).numpy()) for b in post]
    out = oracle.run(name, ext.numpy(), 1, collision="bgk", tau=tau,
                     strategy=STRATEGY[pattern], post=post_e, nthreads=1)
    return torch.from_numpy(out)


@pytest.mark.parametrize("case", ["random_d3q19_bgk", "random_d2q9_bgk"])
@pytest.mark.parametrize("pattern", [_lib.PULL, _lib.PUSH])
@pytest.mark.parametrize("parts", [2, 3])
@pytest.mark.parametrize("with_bb", [False, True])
def test_exchange_local_matches_whole_lattice(oracle, case, pattern, parts, with_bb):
    z = golden(case)
    name = meta(z)["stencil"]
    f0 = z["f0"]
    res = list(f0.shape[1:])
    tau = float(z["tau"])
    post = _boundaries(res, with_bb)
    steps = 4
    ref = oracle.run(name, f0, steps, collision="bgk", tau=tau,
                     strategy=STRATEGY[pattern], post=post)
    e_x = np.asarray(getattr(lt, name)().e)[:, 0]
    slabs = [lt.Slab(res[0], parts, i, e_x) for i in range(parts)]
    exts = [s.extend(torch.from_numpy(f0), 1) for s in slabs]
    for _ in range(steps):
        if pattern == _lib.PULL:
            lt.exchange_local(slabs, exts, pattern)
        exts = [_step_slab(oracle, name, s, e, pattern, post, tau)
                for s, e in zip(slabs, exts)]
        if pattern == _lib.PUSH:
            lt.exchange_local(slabs, exts, pattern)
    got = torch.cat([s.interior(e) for s, e in zip(slabs, exts)], dim=1).numpy()
    assert np.array_equal(got, ref)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_worker(rank, world, port, out_dir, case, pattern):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    from oracle import oracle as orc
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        z = golden(case)
        name = meta(z)["stencil"]
        f0 = z["f0"]
        res = list(f0.shape[1:])
        post = _boundaries(res, True)
        slab = lt.Slab(res[0], world, rank, np.asarray(getattr(lt, name)().e)[:, 0])
        ext = slab.extend(torch.from_numpy(f0), 1)
        for _ in range(4):
            if pattern == _lib.PULL:
                lt.exchange(slab, ext, pattern)
            ext = _step_slab(orc, name, slab, ext, pattern, post, float(z["tau"]))
            if pattern == _lib.PUSH:
                lt.exchange(slab, ext, pattern)
        np.save(os.path.join(out_dir, f"r{rank}.npy"), slab.interior(ext).numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("pattern", [_lib.PULL, _lib.PUSH])
def test_exchange_two_gloo_ranks(oracle, tmp_path, pattern):
    case = "random_d3q19_bgk"
    mp.start_processes(_rank_worker, args=(2, _free_port(), str(tmp_path), case, pattern),
                       nprocs=2, start_method="spawn")
    z = golden(case)
    name = meta(z)["stencil"]
    post = _boundaries(list(z["f0"].shape[1:]), True)
    ref = oracle.run(name, z["f0"], 4, collision="bgk", tau=float(z["tau"]),
                     strategy=STRATEGY[pattern], post=post)
    got = np.concatenate([np.load(tmp_path / f"r{r}.npy") for r in range(2)], axis=1)
    assert np.array_equal(got, ref)
