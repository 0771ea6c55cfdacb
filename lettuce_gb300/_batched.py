"""Many periodic domains of uneven sizes advanced together.

``BatchedSimulation`` takes a list of flows (same stencil, same context, no
boundaries) with one BGK or TRT collision each, moves their populations into
one pooled pair of fields, cuts every domain into tiles of whole rows
(``lgb_batch_plan``) and advances all of them with one persistent launch per
step (``lgb_batched_step``, lettuce's PRE_STREAMING order). A run of steps is
replayed from a captured CUDA graph. With the 16-bit shifted storages a
domain whose rows have an odd length is stored with one pad element per row,
so that every domain runs the two-cell kernel path; its flow then holds a
copy of its populations, refreshed after each call. Launch shape (threads per block, tile
size) is chosen by measurement on first use and cached on disk
(``lettuce_gb300._autotune``). lettuce itself advances one Flow per
Simulation; the per-domain arithmetic is the same as ``Simulation``'s.
"""
from __future__ import annotations

import ctypes
from timeit import default_timer as timer
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _autotune, _device, _lib
from ._collision import BGKCollision, NoCollision, TRTCollision

__all__ = ["BatchedSimulation", "plan_tiles", "batched_taylor_green"]

DOMAIN_DTYPE = np.dtype([("offset", "<i8"), ("res", "<i4", (3,)), ("pitch", "<i4"),
                         ("tau", "<f8"), ("tau_minus", "<f8")])
POOL_ALIGN = 128  # elements
TILE_DTYPE = np.dtype([("domain", "<i4"), ("row_begin", "<i4"), ("row_end", "<i4"),
                       ("reserved", "<i4")])


class BatchDesc(ctypes.Structure):
    _fields_ = [("abi_version", ctypes.c_int32), ("stencil", ctypes.c_int32),
                ("storage", ctypes.c_int32), ("collision", ctypes.c_int32),
                ("n_domains", ctypes.c_int32), ("n_tiles", ctypes.c_int32),
                ("threads", ctypes.c_int32), ("blocks", ctypes.c_int32),
                ("domains", ctypes.c_void_p), ("tiles", ctypes.c_void_p),
                ("f_in", ctypes.c_void_p), ("f_out", ctypes.c_void_p),
                ("pool_elements", ctypes.c_int64), ("status", ctypes.c_void_p),
                ("rates", ctypes.c_void_p)]


def _bind(L):
    if getattr(L, "_batch_bound", False):
        return
    P, I32 = ctypes.c_void_p, ctypes.c_int32
    L.lgb_batch_plan.argtypes = [I32, I32, P, I32, P, I32, P]
    L.lgb_batch_plan.restype = ctypes.c_int
    L.lgb_batched_step.argtypes = [ctypes.POINTER(BatchDesc), P]
    L.lgb_batched_step.restype = ctypes.c_int
    L._batch_bound = True


def plan_tiles(stencil_id: int, domains: np.ndarray, tile_cells: int) -> np.ndarray:
    """tile table (host) of a domain table, through the library's planner"""
    L = _lib.load()
    _bind(L)
    domains = np.ascontiguousarray(domains, dtype=DOMAIN_DTYPE)
    n = ctypes.c_int32(0)
    _lib.check(L.lgb_batch_plan(stencil_id, len(domains), domains.ctypes.data, int(tile_cells),
                                None, 0, ctypes.byref(n)), "lgb_batch_plan")
    tiles = np.zeros(n.value, dtype=TILE_DTYPE)
    _lib.check(L.lgb_batch_plan(stencil_id, len(domains), domains.ctypes.data, int(tile_cells),
                                tiles.ctypes.data, n.value, ctypes.byref(n)), "lgb_batch_plan")
    return tiles


class BatchedSimulation:
    def __init__(self, flows: Sequence, collisions: Sequence, tile_cells: Optional[int] = None,
                 threads: Optional[int] = None, autotune: bool = True,
                 persistent: Optional[bool] = None):
        if len(flows) == 0 or len(flows) != len(collisions):
            raise ValueError("one collision per flow is required")
        f0 = flows[0]
        self.context = f0.context
        if self.context.device.type != "cuda":
            raise RuntimeError("batched domains run on CUDA devices only; there is no CPU path")
        self.stencil = f0.stencil
        kinds = {type(c) for c in collisions}
        if len(kinds) != 1 or not kinds <= {BGKCollision, TRTCollision, NoCollision}:
            raise NotImplementedError("a batch takes one collision kind: BGK, TRT or none")
        for fl, c in zip(flows, collisions):
            if fl.stencil != self.stencil or fl.context is not self.context and (
                    fl.context.device != self.context.device
                    or fl.context.storage != self.context.storage):
                raise ValueError("all flows of a batch share stencil, device and storage")
            if list(fl.pre_boundaries or []) or list(fl.post_boundaries or []):
                raise NotImplementedError("batched domains are periodic (no boundaries)")
            if getattr(c, "force", None) is not None:
                raise NotImplementedError("no forcing in batched domains")
        self.flows = list(flows)
        self.collisions = list(collisions)
        coll = collisions[0]
        self.collision_id = (_lib.TRT if isinstance(coll, TRTCollision)
                             else _lib.BGK if isinstance(coll, BGKCollision) else _lib.NO_COLLISION)
        q = self.stencil.q
        dom = np.zeros(len(flows), dtype=DOMAIN_DTYPE)
        off = 0
        cells = 0
        # the 16-bit formats step two cells per 32-bit word: a domain with an
        # odd row length is stored with one pad element per row so that its
        # rows are whole words too (the pad is written and never read)
        pad_odd = self.context.storage in (_lib.F16_SHIFTED, _lib.BF16_SHIFTED)
        self._pitch = []
        for b, (fl, c) in enumerate(zip(flows, collisions)):
            res = list(fl.resolution) + [1] * (3 - len(fl.resolution))
            z = int(fl.resolution[-1])
            pitch = z + 1 if (pad_odd and z % 2 == 1) else z
            self._pitch.append(pitch)
            # every domain starts on a 128-element boundary of the pool, so the
            # two-cell kernel of the 16-bit formats reads whole aligned words
            off = -(-off // POOL_ALIGN) * POOL_ALIGN
            dom[b]["offset"] = off
            dom[b]["res"] = res
            dom[b]["pitch"] = pitch
            if isinstance(c, TRTCollision):
                dom[b]["tau"], dom[b]["tau_minus"] = c.tau_plus, c.tau_minus
            elif isinstance(c, BGKCollision):
                dom[b]["tau"], dom[b]["tau_minus"] = c.tau, 1.0
            else:
                dom[b]["tau"], dom[b]["tau_minus"] = 1.0, 1.0
            off += q * self._alloc_cells(fl, pitch)
            cells += int(np.prod(fl.resolution))
        self.domains = dom
        self.pool_elements = off
        self.n_cells = cells
        dev = self.context.device
        sdt = self.context.storage_dtype
        # zero-filled: pad elements start finite
        self._pools = [torch.zeros(off, dtype=sdt, device=dev),
                       torch.zeros(off, dtype=sdt, device=dev)]
        for b, fl in enumerate(flows):
            fl._settle()
            self._domain_view(self._pools[0], b).copy_(fl.f_raw)
        self._cur = 0
        self._domains_dev = torch.from_numpy(dom.view(np.uint8).copy()).to(dev)
        # the float32 rates of every domain, rounded once from the float64
        # quotients (the kernel's float32 and 16-bit collisions use these)
        omega = 1.0 / dom["tau"]
        rates = np.stack([omega, 1.0 - omega, 1.0 / (2.0 * dom["tau"]),
                          1.0 / (2.0 * dom["tau_minus"])], axis=1).astype(np.float32)
        self._rates_dev = torch.from_numpy(np.ascontiguousarray(rates)).to(dev)
        self._status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._graph = None
        self._graph_key = None
        self.sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
        cfg = None
        if tile_cells is None or threads is None:
            cfg = _autotune.lookup(self) if autotune else None
            if cfg is None and autotune:
                cfg = _autotune.tune(self)
            if cfg is None:
                cfg = {"threads": 256, "tile_cells": 4096}
        self.threads = int(threads or cfg["threads"])
        self.tile_cells = int(tile_cells or cfg["tile_cells"])
        if persistent is None:
            persistent = bool((cfg or {}).get("persistent", True))
        self._configure(self.threads, self.tile_cells, persistent)
        self._bind_flows()

    # -- launch configuration ---------------------------------------------
    def _configure(self, threads: int, tile_cells: int, persistent: bool = True):
        """launch shape: threads per block, cells per tile, and the grid --
        persistent (as many blocks as the SMs hold, walking the tile table
        with a grid stride) or one block per tile (the hardware's block
        scheduler hands out the tiles)"""
        tiles = plan_tiles(self.stencil.lgb_id, self.domains, tile_cells)
        self.n_tiles = len(tiles)
        self._tiles_dev = torch.from_numpy(tiles.view(np.uint8).copy()).to(self.context.device)
        self.threads = threads
        self.tile_cells = tile_cells
        self.persistent = bool(persistent)
        if self.persistent:
            self.blocks = max(1, min(self.n_tiles, self.sm_count * max(1, 2048 // threads)))
        else:
            self.blocks = max(1, self.n_tiles)
        self._graph = None

    def _desc(self, src: torch.Tensor, dst: torch.Tensor) -> BatchDesc:
        d = BatchDesc()
        d.abi_version = _lib.ABI_VERSION
        d.stencil = self.stencil.lgb_id
        d.storage = self.context.storage
        d.collision = self.collision_id
        d.n_domains = len(self.domains)
        d.n_tiles = self.n_tiles
        d.threads = self.threads
        d.blocks = self.blocks
        d.domains = self._domains_dev.data_ptr()
        d.tiles = self._tiles_dev.data_ptr()
        d.f_in = src.data_ptr()
        d.f_out = dst.data_ptr()
        d.pool_elements = self.pool_elements
        d.status = self._status.data_ptr()
        d.rates = self._rates_dev.data_ptr() if self._rates_dev is not None else None
        return d

    def _launch(self, src, dst, stream):
        L = _lib.load()
        _bind(L)
        d = self._desc(src, dst)
        _lib.check(L.lgb_batched_step(ctypes.byref(d), stream), "lgb_batched_step")

    def step_once(self):
        """one step of every domain (eager launch)"""
        a, b = self._pools[self._cur], self._pools[1 - self._cur]
        self._launch(a, b, self.context.stream_handle())
        self._cur = 1 - self._cur

    def _capture(self):
        """a CUDA graph of two steps: pool 0 -> 1 -> 0"""
        s = torch.cuda.Stream(self.context.device)
        s.wait_stream(torch.cuda.current_stream(self.context.device))
        with torch.cuda.stream(s):
            self._launch(self._pools[0], self._pools[1], s.cuda_stream)  # warm outside capture
            self._launch(self._pools[1], self._pools[0], s.cuda_stream)
        torch.cuda.current_stream(self.context.device).wait_stream(s)

        def pair(st):
            self._launch(self._pools[0], self._pools[1], st)
            self._launch(self._pools[1], self._pools[0], st)
        self._graph = _device.capture(self.context.device, pair)
        self._graph_key = (self.threads, self.tile_cells, self.persistent)

    def advance(self, num_steps: int, use_graph: bool = True):
        """num_steps steps of every domain, asynchronous on the current stream"""
        if num_steps <= 0:
            return
        if self._cur == 1:
            self.step_once()
            num_steps -= 1
        if use_graph and num_steps >= 2:
            if self._graph is None or self._graph_key != (self.threads, self.tile_cells,
                                                          self.persistent):
                # the capture itself advances the pools by two steps
                self._capture()
                num_steps -= 2
            for _ in range(num_steps // 2):
                self._graph.replay()
            num_steps %= 2
        for _ in range(num_steps):
            self.step_once()

    def __call__(self, num_steps: int, use_graph: bool = True) -> float:
        """advance every domain by num_steps; returns MLUPS over all domains"""
        beg = timer()
        self.advance(num_steps, use_graph)
        self.context.synchronize()
        end = timer()
        for fl in self.flows:
            fl.i += num_steps
        self._bind_flows()
        return num_steps * self.n_cells / 1e6 / (end - beg)

    @staticmethod
    def _alloc_cells(flow, pitch: int) -> int:
        """pool elements per population plane: rows x pitch"""
        return int(np.prod(flow.resolution[:-1])) * int(pitch)

    def _domain_view(self, pool: torch.Tensor, b: int) -> torch.Tensor:
        """domain b's populations [Q, *resolution] inside ``pool`` (strided
        when its rows are padded)"""
        fl = self.flows[b]
        q = self.stencil.q
        pitch = self._pitch[b]
        o = int(self.domains[b]["offset"])
        n = q * self._alloc_cells(fl, pitch)
        v = pool[o:o + n].view([q] + list(fl.resolution[:-1]) + [pitch])
        return v[..., :fl.resolution[-1]]

    def _bind_flows(self):
        """point every flow's population tensor at its slice of the current
        pool; a domain stored with padded rows gets a contiguous copy (the
        flow's kernels read contiguous fields), refreshed after every call"""
        pool = self._pools[self._cur]
        for b, fl in enumerate(self.flows):
            v = self._domain_view(pool, b)
            fl._f = v if v.is_contiguous() else v.contiguous()
            fl._aa_pending = False
            fl._stream_pending = None

    @property
    def status(self) -> int:
        return int(self._status.item())


def batched_taylor_green(context, n_domains: int = 256, seed: int = 0, side_min: int = 32,
                         side_max: int = 512, re_min: float = 100.0, re_max: float = 5000.0,
                         mach_number: float = 0.05, tau_minus: float = 1.0):
    """The batched Taylor-Green configuration: ``n_domains`` periodic D2Q9
    vortices whose sides (n_x, n_y) are drawn independently and uniformly
    from the integers [side_min, side_max] and whose Reynolds numbers are
    drawn uniformly from [re_min, re_max] by ``numpy.random.default_rng(seed)``
    (sides first, then Reynolds numbers); TRT collisions with lettuce's
    default tau_minus = 1. Returns (flows, collisions)."""
    from ._flows import TaylorGreenVortex
    from ._stencil import D2Q9
    rng = np.random.default_rng(seed)
    sides = rng.integers(side_min, side_max + 1, size=(n_domains, 2))
    res = rng.uniform(re_min, re_max, size=n_domains)
    flows, colls = [], []
    for (nx, ny), re in zip(sides, res):
        fl = TaylorGreenVortex(context, [int(nx), int(ny)], float(re), mach_number, D2Q9())
        flows.append(fl)
        colls.append(TRTCollision(fl.units.relaxation_parameter_lu, tau_minus))
    return flows, colls
