"""Slab decomposition of the step along lettuce's first dimension x.

lettuce itself runs one grid on one device; its step
(lettuce/_simulation.py:241-305: periodic roll of every population, then the
masked collide) shards by slabs of x, the slowest axis, so that a slab is one
contiguous block of every population plane. A part holds its slab plus one
halo plane on each side (all stencils move at most one cell per step).

Per step only the populations that cross a face travel between parts:

* pull patterns (PRE_STREAMING, and both halves of DOUBLE_STREAMING): before
  the step, a part's first interior plane sends its populations moving -x to
  the left neighbour's right halo plane, and its last interior plane sends
  the populations moving +x to the right neighbour's left halo plane;
* push pattern (POST_STREAMING): the step scatters the boundary planes'
  populations into the halo planes; after the step each halo plane's crossing
  populations overwrite the neighbour's boundary plane.

Inside a part the step kernel streams periodically over the extended slab.
Interior cells read only the crossing populations of the halo planes, which
the exchange keeps current; what the kernel computes in the halo cells
themselves is never read. Outlet planes (which look one and two planes
inward), the in-place AA pattern, and push steps with populations that do
not stream are not decomposed.

``exchange`` moves the halo planes between processes with point-to-point
``torch.distributed`` messages (any backend); ``exchange_local`` moves them
between parts held by one process (a one-device split)."""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np
import torch

from . import _device, _lib
from ._native import NativeBoundary

__all__ = ["Slab", "exchange", "exchange_local", "SlabSimulation"]

PULL_PATTERNS = (_lib.PULL, _lib.STREAM_ONLY)


class Slab:
    """part ``index`` of ``parts`` equal slabs (sizes differ by at most one
    plane) of a lattice with ``nx`` planes along x; ``e_x`` is the x
    component of the stencil's velocities"""

    def __init__(self, nx: int, parts: int, index: int, e_x: Sequence[int]):
        if parts < 1 or not 0 <= index < parts:
            raise ValueError(f"part {index} of {parts}")
        base, extra = divmod(int(nx), parts)
        self.parts, self.index, self.nx_global = parts, index, int(nx)
        self.x0 = index * base + min(index, extra)
        self.nx = base + (1 if index < extra else 0)
        if self.nx < 1:
            raise ValueError(f"{nx} planes cannot be split into {parts} slabs")
        self.left = (index - 1) % parts
        self.right = (index + 1) % parts
        e_x = [int(v) for v in e_x]
        if max(abs(v) for v in e_x) > 1:
            raise ValueError("stencils with velocities longer than one cell need wider halos")
        self.rightward = [q for q, v in enumerate(e_x) if v > 0]
        self.leftward = [q for q, v in enumerate(e_x) if v < 0]
        if len(self.rightward) != len(self.leftward):
            raise ValueError("the stencil is not symmetric in x")
        # global x of each plane of the extended slab: left halo, interior, right halo
        self.planes = [(self.x0 - 1 + k) % self.nx_global for k in range(self.nx + 2)]

    # -- global <-> extended slab -------------------------------------------
    def extend(self, t: torch.Tensor, axis: int) -> torch.Tensor:
        """the extended slab (halo planes included) of a global tensor whose
        dimension ``axis`` is x; a dimension of size 1 (broadcast) is kept"""
        if t.shape[axis] == 1:
            return t.contiguous()
        if t.shape[axis] != self.nx_global:
            raise ValueError(f"dimension {axis} of {tuple(t.shape)} is not x ({self.nx_global})")
        idx = torch.as_tensor(self.planes, dtype=torch.long, device=t.device)
        return t.index_select(axis, idx).contiguous()

    def interior(self, ext: torch.Tensor, axis: int = 1) -> torch.Tensor:
        return ext.narrow(axis, 1, self.nx)

    # -- halo planes ---------------------------------------------------------
    def outgoing(self, ext: torch.Tensor, pattern: int):
        """(to_left, to_right): copies of the crossing populations this part
        sends; ``ext`` is [Q, nx + 2, ...]"""
        if pattern in PULL_PATTERNS:
            to_left = ext[self.leftward, 1]
            to_right = ext[self.rightward, self.nx]
        elif pattern == _lib.PUSH:
            to_left = ext[self.leftward, 0]
            to_right = ext[self.rightward, self.nx + 1]
        else:
            raise ValueError(f"pattern {pattern} exchanges no halo")
        return to_left.contiguous(), to_right.contiguous()

    def incoming(self, ext: torch.Tensor, pattern: int, from_left: torch.Tensor,
                 from_right: torch.Tensor):
        """write what the neighbours sent: from_left is the left neighbour's
        to_right, from_right the right neighbour's to_left"""
        if pattern in PULL_PATTERNS:
            ext[self.rightward, 0] = from_left
            ext[self.leftward, self.nx + 1] = from_right
        elif pattern == _lib.PUSH:
            ext[self.rightward, 1] = from_left
            ext[self.leftward, self.nx] = from_right
        else:
            raise ValueError(f"pattern {pattern} exchanges no halo")


def exchange(slab: Slab, ext: torch.Tensor, pattern: int, group=None):
    """halo exchange of one part per process; the part index is the rank in
    ``group``. Messages to the right carry tag 0, to the left tag 1, so two
    parts (left neighbour == right neighbour) stay apart."""
    import torch.distributed as dist
    to_left, to_right = slab.outgoing(ext, pattern)
    if slab.parts == 1:
        slab.incoming(ext, pattern, to_right, to_left)
        return
    peer = (lambda i: dist.get_global_rank(group, i)) if group is not None else (lambda i: i)
    from_left = torch.empty_like(to_right)
    from_right = torch.empty_like(to_left)
    ops = [dist.P2POp(dist.isend, to_right, peer(slab.right), group, 0),
           dist.P2POp(dist.irecv, from_left, peer(slab.left), group, 0),
           dist.P2POp(dist.isend, to_left, peer(slab.left), group, 1),
           dist.P2POp(dist.irecv, from_right, peer(slab.right), group, 1)]
    for req in dist.batch_isend_irecv(ops):
        req.wait()
    slab.incoming(ext, pattern, from_left, from_right)


def exchange_local(slabs: List[Slab], exts: List[torch.Tensor], pattern: int):
    """halo exchange between all parts of one lattice held by one process"""
    if sorted(s.index for s in slabs) != list(range(slabs[0].parts)):
        raise ValueError("exchange_local needs every part of the lattice")
    by_index = {s.index: k for k, s in enumerate(slabs)}
    outs = [s.outgoing(e, pattern) for s, e in zip(slabs, exts)]
    for s, e in zip(slabs, exts):
        from_left = outs[by_index[s.left]][1]
        from_right = outs[by_index[s.right]][0]
        s.incoming(e, pattern, from_left, from_right)


class SlabSimulation:
    """the step of a ``Simulation`` run over x-slabs of its grid.

    ``simulation`` supplies the flow, the masks and the operators (it may be
    built on a CPU context: set-up only). ``parts`` is the number of slabs;
    ``indices`` the slabs this process holds: all of them (one-device split,
    halos moved by ``exchange_local``) or one (one part per rank, halos moved
    by ``exchange`` over ``group``). Populations stay in the storage format
    of the flow's context."""

    def __init__(self, simulation, parts: int, indices: Optional[Sequence[int]] = None,
                 device=None, group=None):
        from ._simulation import _desc_for
        sim = simulation
        flow = sim.flow
        if sim.memory_pattern == "aa":
            raise ValueError("the AA pattern is not decomposed into slabs")
        for nat in sim._natives:
            if isinstance(nat, NativeBoundary) and nat.kind in (_lib.SUB_ANTI_BOUNCE_BACK,
                                                                _lib.SUB_EQUILIBRIUM_OUTLET_P):
                raise ValueError("outlet planes are not decomposed into slabs")
        if getattr(sim, "_link_bits", None) is not None:
            raise ValueError("halfway bounce-back links are not decomposed into slabs")
        if _lib.PUSH in sim._patterns and sim._nsb is not None:
            raise ValueError("push steps with populations that do not stream are "
                             "not decomposed into slabs")
        self.simulation = sim
        self.flow = flow
        self.patterns = list(sim._patterns)
        self.group = group
        self.device = torch.device(device) if device is not None else flow.context.device
        if self.device.type != "cuda":
            raise RuntimeError("lettuce_gb300 steps on CUDA devices only; there is no CPU path")
        indices = list(range(parts)) if indices is None else list(indices)
        e_x = np.asarray(flow.stencil.e)[:, 0]
        self.slabs = [Slab(flow.resolution[0], parts, i, e_x) for i in indices]
        if len(self.slabs) > 1 and len(self.slabs) != parts:
            raise ValueError("a process holds one part or all of them")
        flow._settle()
        f = flow.f_raw
        self.f = [s.extend(f, 1).to(self.device) for s in self.slabs]
        self.f_next = [torch.empty_like(t) for t in self.f]
        self._keep = []
        self._descs = []
        self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        for s, fe in zip(self.slabs, self.f):
            res = [s.nx + 2] + list(flow.resolution[1:])
            flags = nsb = None
            if sim._flags is not None:
                flags = s.extend(sim._flags, 0).to(self.device)
                nsb = s.extend(sim._nsb, 0).to(self.device) if sim._nsb is not None else None
            natives = [self._slab_native(n, s) for n in sim._natives]
            d, keep = _desc_for(flow, natives, flags, nsb, sim.collision_index, res=res)
            d.collision = sim._desc.collision
            d.tau = sim._desc.tau
            d.tau_minus = sim._desc.tau_minus
            d.status = self._status.data_ptr()
            d.options = sim._desc.options
            self._keep += [flags, nsb, natives, keep]
            self._descs.append(d)
        self.i = flow.i

    def _slab_native(self, nat, slab: Slab):
        """a substep descriptor with its per-cell tensors cut to the slab"""
        import copy
        if not isinstance(nat, NativeBoundary) or nat.kind != _lib.SUB_EQUILIBRIUM_PU:
            return nat
        nat = copy.copy(nat)
        nat.rho = slab.extend(nat.rho, 0).to(self.device)
        nat.u = slab.extend(nat.u, 1).to(self.device)
        return nat

    def _exchange(self, pattern: int):
        if len(self.slabs) == self.slabs[0].parts:
            exchange_local(self.slabs, self.f, pattern)
        else:
            exchange(self.slabs[0], self.f[0], pattern, self.group)

    def step(self):
        stream = torch.cuda.current_stream(self.device).cuda_stream
        for pat in self.patterns:
            if pat in PULL_PATTERNS:
                self._exchange(pat)
            for k, d in enumerate(self._descs):
                d.pattern = pat
                d.f_in = self.f[k].data_ptr()
                d.f_out = self.f_next[k].data_ptr()
                _device.step(d, stream)
            self.f, self.f_next = self.f_next, self.f
            if pat == _lib.PUSH:
                self._exchange(pat)
        self.i += 1

    def __call__(self, num_steps: int):
        for _ in range(num_steps):
            self.step()

    @property
    def status(self) -> int:
        return int(self._status.item())

    def interiors(self) -> List[torch.Tensor]:
        """this process's slabs without halo planes, [Q, nx_part, ...]"""
        return [s.interior(fe) for s, fe in zip(self.slabs, self.f)]

    def gather(self) -> torch.Tensor:
        """the whole lattice (one-device split only), in storage format"""
        if len(self.slabs) != self.slabs[0].parts:
            raise ValueError("gather needs every part of the lattice")
        order = sorted(range(len(self.slabs)), key=lambda k: self.slabs[k].index)
        return torch.cat([self.interiors()[k] for k in order], dim=1)
