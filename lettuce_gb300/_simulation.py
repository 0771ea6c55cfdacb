"""The step engine: lettuce's ``Simulation`` (lettuce/_simulation.py:42-344)
driving the fused GB300 kernels.

``Simulation.__init__`` builds lettuce's no-collision / no-streaming masks
exactly as lettuce does (:100-146), packs them into one flag byte per cell
plus a per-cell no-streaming bit word, and turns the collision and boundary
plugins' ``native_generator`` descriptors into an ``lgb_step_desc``. Each
step is then one (or, for DOUBLE_STREAMING, two) kernel launches on the
current torch stream, with no host synchronisation inside the loop:

* PRE_STREAMING  -> pull pattern (stream then collide, one pass)
* POST_STREAMING -> push pattern, or the in-place AA pattern with
                    ``memory_pattern="aa"`` (half the memory, same traffic)
* NO_STREAMING   -> collide only
* DOUBLE_STREAMING -> pull, then stream only
"""
from __future__ import annotations

import warnings
from abc import ABC, abstractmethod
from enum import Enum
from functools import lru_cache
from timeit import default_timer as timer
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _device, _lib
from ._native import NativeBoundary, NativeCollision

__all__ = ["Reporter", "Simulation", "BreakableSimulation", "StreamingStrategy",
           "apply_local"]


class StreamingStrategy(Enum):
    """same values as lettuce/cuda_native/_default_code_gen.py:13-25"""
    NO_STREAMING = 0b00
    PRE_STREAMING = 0b10
    POST_STREAMING = 0b01
    DOUBLE_STREAMING = 0b11

    @lru_cache
    def pre_streaming(self) -> bool:
        return bool(self.value & StreamingStrategy.PRE_STREAMING.value)

    @lru_cache
    def post_streaming(self) -> bool:
        return bool(self.value & StreamingStrategy.POST_STREAMING.value)


class Reporter(ABC):
    interval: int

    def __init__(self, interval: int):
        self.interval = interval

    @abstractmethod
    def __call__(self, simulation: "Simulation"):
        ...


def _fill_substep(sub: _lib.Substep, native, keep: list, res):
    if isinstance(native, NativeCollision):
        sub.kind = _lib.SUB_COLLISION
        return
    sub.kind = native.kind
    if native.kind == _lib.SUB_EQUILIBRIUM_PU:
        rho, u = native.rho, native.u
        rs = _device.bcast_strides(rho, list(res))
        us = _device.bcast_strides(u, [u.shape[0]] + list(res))
        keep += [rho, u]
        sub.rho = rho.data_ptr()
        sub.u = u.data_ptr()
        for k in range(3):
            sub.rho_stride[k] = rs[k] if k < len(rs) else 0
        for k in range(4):
            sub.u_stride[k] = us[k] if k < len(us) else 0
    elif native.kind in (_lib.SUB_ANTI_BOUNCE_BACK, _lib.SUB_EQUILIBRIUM_OUTLET_P):
        sub.axis = native.axis
        sub.sign = native.sign
    for k, v in enumerate(native.params):
        sub.param[k] = float(v)


def _desc_for(flow, natives, flags, nsb, collision_index, res=None):
    """lgb_step_desc for a list of substep descriptors (collision included);
    ``res`` overrides the flow's resolution (a slab of the grid)"""
    coll = natives[collision_index]
    res = list(flow.resolution if res is None else res)
    d = _device.new_desc(flow.stencil.lgb_id, flow.context.storage, res)
    d.collision = coll.kind
    d.tau = coll.tau
    d.tau_minus = coll.tau_minus
    d.smagorinsky_constant = coll.smagorinsky_constant
    keep = []
    if coll.force is not None:
        d.force = coll.force.kind
        d.force_tau = coll.force.tau
        for k, a in enumerate(coll.force.acceleration):
            d.accel[k] = float(a)
    if coll.mrt_tables is not None:
        # host memory read by lgb_step at each call: kept alive with the desc
        tables = np.ascontiguousarray(coll.mrt_tables, dtype=np.float64)
        keep.append(tables)
        d.mrt_equilibrium = coll.mrt_equilibrium
        d.mrt_tables = tables.ctypes.data
    if flags is not None:
        if len(natives) > _lib.MAX_SUBSTEPS:
            raise ValueError(f"at most {_lib.MAX_SUBSTEPS} substeps (boundaries + collision)")
        d.flags = flags.data_ptr()
        d.no_stream_bits = nsb.data_ptr() if nsb is not None else None
        d.n_sub = len(natives)
        d.collision_index = collision_index
        for k, nat in enumerate(natives):
            _fill_substep(d.sub[k], nat, keep, res)
    return d, keep


def pack_masks(no_collision_mask: torch.Tensor, no_streaming_mask: torch.Tensor,
               e: Optional[Sequence[Sequence[int]]] = None):
    """(flags uint8 [*res], no-stream bits int32 [*res] or None).

    flags = the no-collision index | 0x80 where the cell has any population
    that does not stream; bit q of the word is set where lettuce's torch
    stream keeps population q (``no_streaming_mask[q] == 1``,
    lettuce/_simulation.py:254-255). With the stencil's velocities ``e``,
    0x40 marks the cells x whose neighbour x + e_q keeps population q (the
    cells that must look before they push)."""
    ncm = no_collision_mask.to(torch.uint8)
    if int(ncm.max().item()) > _lib.FLAG_INDEX_MASK:
        raise ValueError("too many substeps for the flag byte")
    keep = no_streaming_mask == 1
    keep[0] = False  # the rest population never streams anyway
    q = keep.shape[0]
    shifts = torch.arange(q, device=keep.device, dtype=torch.int64).view(
        [-1] + [1] * (keep.dim() - 1))
    bits = torch.sum(keep.to(torch.int64) << shifts, dim=0)
    has = bits != 0
    flags = ncm | (has.to(torch.uint8) * _lib.FLAG_NO_STREAM)
    if not bool(has.any().item()):
        return flags.contiguous(), None
    if e is not None:
        d = keep.dim() - 1
        guard = torch.zeros_like(has)
        for qi in range(1, q):
            shift = tuple(-int(v) for v in e[qi])
            guard |= torch.roll(keep[qi], shifts=shift, dims=tuple(range(d)))
        flags |= guard.to(torch.uint8) * _lib.FLAG_PUSH_GUARD
    return flags.contiguous(), bits.to(torch.int32).contiguous()


def apply_local(flow, collision_native: NativeCollision,
                boundary_native: Optional[NativeBoundary] = None,
                flags: Optional[torch.Tensor] = None) -> torch.Tensor:
    """run the collide-only pattern once (out of place) and return the new
    populations in the context dtype; used by direct calls of a collision or
    boundary operator"""
    if flow.context.device.type != "cuda":
        raise RuntimeError("lettuce_gb300 operators run on CUDA devices only; "
                           "there is no CPU path")
    natives = [collision_native] + ([boundary_native] if boundary_native else [])
    flow._settle()
    src = flow.f_raw
    out = torch.empty_like(src)
    d, keep = _desc_for(flow, natives, flags, None, 0)
    d.pattern = _lib.LOCAL
    d.f_in = src.data_ptr()
    d.f_out = out.data_ptr()
    _device.step(d, _device.stream_of(src))
    del keep
    if flow.context.shifted:
        w = flow.torch_stencil.w.to(torch.float32).view([-1] + [1] * flow.stencil.d)
        return out.to(torch.float32) + w
    return out


class Simulation:
    """lettuce's Simulation on the GB300 kernels.

    ``memory_pattern``: "ab" (two fields) or "aa" (in place, POST_STREAMING).
    ``use_graph``: replay pairs of steps from a captured CUDA graph instead of
    launching every step from Python. ``None`` (default) enables it when the
    simulation has no reporters; with reporters and ``use_graph=True`` the
    reporters are called at the steps where one of them is due
    (``flow.i % interval == 0``) instead of after every step.
    ``post_as_pull``: POST_STREAMING with two fields runs as one
    collide-only launch followed by pull steps, the field left
    post-collision with its stream pending until it is read (the
    populations are the same as with the push kernels, bit for bit). None
    (default) chooses it where the pull kernels measured faster: grids
    without boundaries, and KBC. It applies while no reporter has an
    interval below 8."""

    def __init__(self, flow, collision, reporter: List[Reporter],
                 streaming_strategy=StreamingStrategy.POST_STREAMING,
                 memory_pattern: str = "ab", use_graph: Optional[bool] = None,
                 post_as_pull: Optional[bool] = None):
        self.use_graph = use_graph
        self._graph = None
        self.flow = flow
        flow.collision = collision
        self.context = flow.context
        self.collision = collision
        pre = list(flow.pre_boundaries or [])
        post = list(flow.post_boundaries or [])
        self.pre_boundaries = pre
        self.post_boundaries = post
        self.collision_index = len(pre)
        self.transformer = pre + [collision] + post
        self.reporter = reporter
        self.streaming_strategy = streaming_strategy
        if memory_pattern not in ("ab", "aa"):
            raise ValueError("memory_pattern is 'ab' (two fields) or 'aa' (in place)")
        self.memory_pattern = memory_pattern
        collision.bind(flow)

        # masks, exactly as lettuce/_simulation.py:100-146 builds them
        self.no_collision_mask = None
        self.no_streaming_mask = None
        shape_f = [flow.stencil.q, *flow.resolution]
        if len(pre) + len(post) > 0:
            self.no_collision_mask = self.context.full_tensor(
                flow.resolution, self.collision_index, dtype=torch.uint8)
            self.no_streaming_mask = self.context.full_tensor(
                shape_f, self.collision_index, dtype=torch.uint8)
            for i, b in list(enumerate(pre)) + list(enumerate(post, start=self.collision_index + 1)):
                ncm = b.make_no_collision_mask(list(flow.resolution), context=self.context)
                if ncm is not None:
                    self.no_collision_mask[torch.as_tensor(ncm, device=self.context.device).bool()] = i
                nsm = b.make_no_streaming_mask(shape_f, context=self.context)
                if nsm is not None:
                    self.no_streaming_mask |= torch.as_tensor(
                        nsm, device=self.context.device).to(torch.uint8)
        self._extend_masks(shape_f)

        # native descriptors (no fallback: every component must have one)
        missing = [c.__class__.__name__ for c in self.transformer if not c.native_available()]
        if flow.equilibrium is not None and not flow.equilibrium.native_available():
            missing.append(flow.equilibrium.__class__.__name__)
        if missing:
            raise NotImplementedError(
                f"no GB300 kernel for {', '.join(missing)}; lettuce_gb300 has no torch fallback")
        natives = [b.native_generator(i) for i, b in enumerate(pre)]
        natives.append(collision.native_generator(self.collision_index))
        natives += [b.native_generator(i)
                    for i, b in enumerate(post, start=self.collision_index + 1)]
        self._natives = natives

        self._flags = self._nsb = None
        if self.no_collision_mask is not None:
            self._flags, self._nsb = pack_masks(self.no_collision_mask, self.no_streaming_mask,
                                                e=flow.stencil.e)
        self._desc, self._keep = _desc_for(flow, natives, self._flags, self._nsb,
                                           self.collision_index)
        if self._nsb is not None:
            self._desc.options |= _lib.OPT_PUSH_GUARD
        self._extend_desc()
        self._status = None
        if self.context.device.type == "cuda":
            self._status = torch.zeros(1, dtype=torch.int32, device=self.context.device)
            self._desc.status = self._status.data_ptr()

        s = streaming_strategy
        if memory_pattern == "aa":
            if s != StreamingStrategy.POST_STREAMING:
                raise ValueError("the AA pattern implements POST_STREAMING only")
            if self._nsb is not None:
                raise ValueError("the AA pattern does not support no-streaming masks "
                                 "(anti-bounce-back outlets); use memory_pattern='ab'")
        self._pending_fn = self._apply_pending_stream
        if post_as_pull is None:
            # measured: the pull kernels are faster except for masked BGK/TRT
            # runs, where the push kernel is 3 % ahead
            post_as_pull = self._flags is None or self._desc.collision == _lib.KBC
        self._post_pull_ok = (s == StreamingStrategy.POST_STREAMING and memory_pattern == "ab"
                              and bool(post_as_pull))
        self._pull_post = False
        if s == StreamingStrategy.PRE_STREAMING:
            self._patterns = [_lib.PULL]
        elif s == StreamingStrategy.POST_STREAMING:
            self._patterns = [_lib.PUSH]
        elif s == StreamingStrategy.DOUBLE_STREAMING:
            self._patterns = [_lib.PULL, _lib.STREAM_ONLY]
        else:
            self._patterns = [_lib.LOCAL]
        self._choose_pull_post()

    def _extend_masks(self, shape_f):
        """hook: masks of boundaries outside lettuce's pre/post lists"""

    def _extend_desc(self):
        """hook: descriptor fields of boundaries outside the substep list"""

    # ------------------------------------------------------------------
    @property
    def units(self):
        return self.flow.units

    @property
    def status(self) -> int:
        """device status word (bit 0: a non-finite density was seen); reading
        it synchronises with the device"""
        return 0 if self._status is None else int(self._status.item())

    def _require_device(self):
        if self.context.device.type != "cuda":
            raise RuntimeError("lettuce_gb300 steps on CUDA devices only; there is no CPU path")

    def _collide_and_stream(self, *_, stream=None, **__):
        flow = self.flow
        d = self._desc
        if stream is None:
            stream = self.context.stream_handle()
        if self.memory_pattern == "aa":
            if flow._stream_pending is not None:
                flow._settle()
            d.pattern = _lib.AA_ODD if flow._aa_pending else _lib.AA_EVEN
            d.f_in = d.f_out = flow._f.data_ptr()
            _device.step(d, stream)
            flow._aa_pending = not flow._aa_pending
            return
        if self._pull_post:
            # POST_STREAMING as pull steps: (S C)^n = S (C S)^(n-1) C. The
            # field stays post-collision; its stream is applied when read.
            if flow._stream_pending is not self._pending_fn:
                flow._settle()
                self._launch(_lib.LOCAL, stream)
            else:
                self._launch(_lib.PULL, stream)
            flow._stream_pending = self._pending_fn
            return
        if flow._stream_pending is not None:
            flow._settle()
        for pat in self._patterns:
            self._launch(pat, stream)

    def _launch(self, pattern: int, stream: int):
        """one launch of the step kernel, fields A -> B, then swapped"""
        flow = self.flow
        d = self._desc
        src = flow._f
        dst = flow.f_next
        d.pattern = pattern
        d.f_in = src.data_ptr()
        d.f_out = dst.data_ptr()
        _device.step(d, stream)
        flow._f, flow._f_next = dst, src

    def _apply_pending_stream(self):
        """the stream a POST_STREAMING run left pending (one STREAM_ONLY
        launch on the current stream)"""
        self._launch(_lib.STREAM_ONLY, self.context.stream_handle())

    def _choose_pull_post(self):
        """POST_STREAMING runs as pull steps when reporters read the field
        rarely enough (each read applies the pending stream and restarts
        with a collide-only step): no reporters, or none with an interval
        below 8"""
        if not self._post_pull_ok:
            self._pull_post = False
            return
        intervals = [int(getattr(r, "interval", 1) or 1) for r in self.reporter]
        self._pull_post = all(iv >= 8 for iv in intervals)

    # -- the two halves of a step (lettuce/_simulation.py:245-305) ----------
    def _run_pattern(self, pattern: int) -> torch.Tensor:
        self._require_device()
        flow = self.flow
        flow._settle()
        d = self._desc
        d.pattern = pattern
        src, dst = flow._f, flow.f_next
        d.f_in = src.data_ptr()
        d.f_out = dst.data_ptr()
        _device.step(d, self.context.stream_handle())
        flow._f, flow._f_next = dst, src
        return flow.f

    def _stream(self) -> torch.Tensor:
        """lettuce's streaming half alone: f[q](x) <- f[q](x - e_q), keeping
        the populations the no-streaming mask holds (one STREAM_ONLY launch)"""
        return self._run_pattern(_lib.STREAM_ONLY)

    def _collide(self) -> torch.Tensor:
        """lettuce's collide half alone: the masked sequence of
        pre-boundaries, collision and post-boundaries (one LOCAL launch)"""
        return self._run_pattern(_lib.LOCAL)

    # -- CUDA-graph replay -------------------------------------------------
    def _graphs_enabled(self) -> bool:
        if self.use_graph is None:
            return not self.reporter
        return bool(self.use_graph)

    def _state_key(self):
        import ctypes
        d = self._desc
        return (self.flow._f.data_ptr(),
                self.flow._f_next.data_ptr() if self.flow._f_next is not None else 0,
                self.flow._aa_pending, self.flow._stream_pending is not None,
                ctypes.string_at(ctypes.addressof(d), ctypes.sizeof(d)))

    def _advance(self, n: int):
        """n steps without reporters; flow.i is advanced"""
        flow = self.flow
        if not self._graphs_enabled() or n < 4:
            for _ in range(n):
                self._collide_and_stream(self)
                flow.i += 1
            return
        if self.memory_pattern != "aa":
            flow.f_next  # make sure the second field exists before capture
        if self._graph is None:
            self._graph = {}
        g = self._graph.get(self._state_key())
        if g is None:
            # two eager steps (they count), then capture a pair of steps that
            # returns the fields to the same assignment; graphs are kept per
            # field assignment (both parities of A/B, both AA phases). The
            # eager steps may reach a state captured before (a stream that was
            # applied for a reporter is pending again after them).
            for _ in range(2):
                self._collide_and_stream(self)
                flow.i += 1
            n -= 2
            g = self._graph.get(self._state_key())
        if g is None:
            def pair(stream):
                self._collide_and_stream(self, stream=stream)
                self._collide_and_stream(self, stream=stream)
            g = _device.capture(self.context.device, pair)
            if len(self._graph) >= 4:
                self._graph.clear()
            self._graph[self._state_key()] = g
        for _ in range(n // 2):
            g.replay()
        flow.i += 2 * (n // 2)
        for _ in range(n % 2):
            self._collide_and_stream(self)
            flow.i += 1

    def _steps_to_next_report(self) -> int:
        i = self.flow.i
        best = None
        for r in self.reporter:
            iv = int(getattr(r, "interval", 1) or 1)
            k = iv - (i % iv)
            best = k if best is None else min(best, k)
        return best if best is not None else 1 << 62

    def _run(self, target_done, remaining):
        """advance until target_done() holds, reporting like lettuce;
        remaining() bounds the steps taken before the next check"""
        graphs = self._graphs_enabled()
        while not target_done():
            if not graphs:
                self._collide_and_stream(self)
                self.flow.i += 1
                self._report()
                continue
            m = min(self._steps_to_next_report(), remaining())
            self._advance(m)
            self._report()

    def step(self, num_steps: int):
        warnings.warn("Simulation.step() is deprecated; call simulation(num_steps)",
                      DeprecationWarning)
        return self(num_steps)

    def _report(self):
        for reporter in self.reporter:
            reporter(self)

    def __call__(self, num_steps: int) -> float:
        self._require_device()
        self._choose_pull_post()
        beg = timer()
        if self.flow.i == 0:
            self._report()
        stop = self.flow.i + num_steps
        self._run(lambda: self.flow.i >= stop, lambda: stop - self.flow.i)
        self.context.synchronize()
        end = timer()
        return num_steps * self.flow._f[0].numel() / 1e6 / (end - beg)


class BreakableSimulation(Simulation):
    """stops when a reporter pushes flow.i past num_steps
    (lettuce/_simulation.py:325-344)"""

    def __init__(self, flow, collision, reporter: List[Reporter], **kwargs):
        super().__init__(flow, collision, reporter, **kwargs)

    def __call__(self, num_steps: int) -> float:
        self._require_device()
        self._choose_pull_post()
        beg = timer()
        if self.flow.i == 0:
            self._report()
        self._run(lambda: self.flow.i >= num_steps, lambda: max(1, num_steps - self.flow.i))
        self.context.synchronize()
        end = timer()
        return num_steps * self.flow._f[0].numel() / 1e6 / (end - beg)


class EbbSimulation(Simulation):
    """The simulation of lettuce's example project for efficient bounce-back
    (examples/advanced_projects/efficient_bounce_back_obstacle/simulation/
    ebb_simulation.py:11-105): every step collides, streams and then applies
    the flow's post-streaming boundaries (``flow.post_streaming_boundaries``
    when the flow's class defines it), whatever streaming strategy would
    otherwise apply.

    Masks follow ebb_simulation.py:28-57: the post-streaming boundaries'
    cells take the substep indices after the post-collision boundaries (so
    they neither collide nor run a boundary) and do not stream. The bounce
    of ``HalfwayBounceBackBoundary`` runs inside the pull of the step kernel
    (per-cell link bits), so the steps run as one collide-only launch
    followed by pull launches, the last stream and bounce pending until the
    field is read; ``_stream()`` called directly bounces as well. The
    ``LinearInterpolatedBounceBackBoundary`` adds a pass over its links
    before each pulling launch that computes the interpolated values the
    pull then reads; the example's post-streaming
    ``FullwayBounceBackBoundary`` runs as such links of distance 0 on its
    solid cells (the bounced value is the streamed one). One
    post-streaming boundary may compute its force."""

    def __init__(self, flow, collision, reporter: List[Reporter],
                 use_graph: Optional[bool] = None):
        from ._boundary import (FullwayBounceBackBoundary, HalfwayBounceBackBoundary,
                                LinearInterpolatedBounceBackBoundary)
        psb = []
        if hasattr(flow.__class__, "post_streaming_boundaries"):
            psb = list(flow.post_streaming_boundaries or [])
        other = [b.__class__.__name__ for b in psb
                 if not isinstance(b, (HalfwayBounceBackBoundary,
                                       LinearInterpolatedBounceBackBoundary,
                                       FullwayBounceBackBoundary))]
        if other:
            raise NotImplementedError(
                f"no GB300 kernel for the post-streaming boundary {', '.join(other)}")
        if sum(1 for b in psb if b.calc_force) > 1:
            raise NotImplementedError("one post-streaming boundary per simulation may "
                                      "compute its force")
        self.post_streaming_boundaries = psb
        self._link_bits = self._force_links = None
        super().__init__(flow, collision, reporter,
                         streaming_strategy=StreamingStrategy.POST_STREAMING,
                         memory_pattern="ab", use_graph=use_graph, post_as_pull=True)

    def _extend_masks(self, shape_f):
        psb = self.post_streaming_boundaries
        if not psb:
            return
        flow = self.flow
        if self.no_collision_mask is None:
            self.no_collision_mask = self.context.full_tensor(
                flow.resolution, self.collision_index, dtype=torch.uint8)
        if self.no_streaming_mask is None:
            self.no_streaming_mask = self.context.full_tensor(
                shape_f, self.collision_index, dtype=torch.uint8)
        start = self.collision_index + 1 + len(self.post_boundaries)
        for i, b in enumerate(psb, start=start):
            ncm = b.make_no_collision_mask(list(flow.resolution), context=self.context)
            if ncm is not None:
                self.no_collision_mask[torch.as_tensor(ncm, device=self.context.device).bool()] = i
            nsm = b.make_no_streaming_mask(shape_f, context=self.context)
            if nsm is not None:
                self.no_streaming_mask |= torch.as_tensor(
                    nsm, device=self.context.device).to(torch.uint8)

    def _extend_desc(self):
        psb = self.post_streaming_boundaries
        if not psb:
            return
        d = self._desc
        flow = self.flow
        res = list(flow.resolution)
        n_cells = int(np.prod(res))
        opp = np.asarray(flow.stencil.opposite, dtype=np.int64)
        parts = [b.link_rows() for b in psb]
        rows = np.concatenate([r for r, _ in parts]).reshape(-1, len(res) + 1)
        dist = np.concatenate([w for _, w in parts])
        owner = np.concatenate([np.full(len(r), j) for j, (r, _) in enumerate(parts)])
        coords = np.where(rows[:, 1:] < 0, rows[:, 1:] + np.array(res), rows[:, 1:])
        cells = (np.ravel_multi_index(tuple(coords.T), tuple(res)) if len(rows)
                 else np.zeros(0, dtype=np.int64))
        q = rows[:, 0]
        pop = opp[q]  # the population the link sets at its fluid cell
        bits = np.zeros(n_cells, dtype=np.int64)
        np.bitwise_or.at(bits, cells, np.left_shift(1, pop))
        dev = self.context.device
        self._link_bits = torch.as_tensor(bits.astype(np.uint32).view(np.int32).reshape(res),
                                          device=dev).contiguous()
        self._flags |= (self._link_bits != 0).to(torch.uint8) * _lib.FLAG_LINKS
        d.link_bits = self._link_bits.data_ptr()
        pos = np.full(len(rows), 0xFFFFFFFF, dtype=np.int64)
        if np.any(dist >= 0):
            # the value table: links sorted by cell, then by the population
            # they set, so a cell's k-th link bit is its k-th entry
            order = np.lexsort((pop, cells))
            sc, sp = cells[order], pop[order]
            if np.any((sc[1:] == sc[:-1]) & (sp[1:] == sp[:-1])):
                raise ValueError("two links set the same population of one cell")
            first = np.r_[True, sc[1:] != sc[:-1]]
            base = np.zeros(n_cells, dtype=np.int64)
            base[sc[first]] = np.nonzero(first)[0]
            pairs = np.stack([q[order], sc], axis=1).astype(np.uint32)
            vdt = self.context.storage_dtype  # the field's storage format
            self._link_base = torch.as_tensor(base.astype(np.uint32).view(np.int32), device=dev)
            self._link_pairs = torch.as_tensor(pairs.view(np.int32), device=dev).contiguous()
            self._link_d = torch.as_tensor(dist[order], dtype=torch.float64, device=dev)
            self._link_val = torch.zeros(len(order), dtype=vdt, device=dev)
            d.link_base = self._link_base.data_ptr()
            d.link_pairs = self._link_pairs.data_ptr()
            d.link_d = self._link_d.data_ptr()
            d.link_val = self._link_val.data_ptr()
            d.n_links = len(order)
            pos[order] = np.arange(len(order))
        forcing = [j for j, b in enumerate(psb) if b.calc_force]
        if forcing:
            from ._boundary import FullwayBounceBackBoundary
            sel = owner == forcing[0]
            k = np.where(dist[sel] >= 0, pos[sel], 0xFFFFFFFF)
            if isinstance(psb[forcing[0]], FullwayBounceBackBoundary):
                k = k | 0x80000000  # 2 f_q e_q with f_q the streamed value
            trip = np.stack([q[sel], cells[sel], k], axis=1).astype(np.uint32)
            self._force_links = torch.as_tensor(np.ascontiguousarray(trip).view(np.int32),
                                                device=dev)
            d.force_links = self._force_links.data_ptr() if len(trip) else None
            d.n_force_links = len(trip)
            d.force_out = psb[forcing[0]]._force.data_ptr()
            blocks = -(-len(trip) // _lib.LINK_FORCE_BLOCK)
            self._force_scratch = torch.zeros(3 * max(1, blocks), dtype=torch.float64,
                                              device=dev)
            d.force_scratch = self._force_scratch.data_ptr()

    def _choose_pull_post(self):
        if self._link_bits is not None:
            self._pull_post = True  # the bounce is part of the pull
            return
        super()._choose_pull_post()
