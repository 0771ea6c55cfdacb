"""Differentiable rollout of the BGK step with a hand-written adjoint.

``rollout(f0, stencil, tau, steps)`` advances populations by ``steps``
pull-pattern BGK steps (lettuce's PRE_STREAMING order) on the GPU and is a
``torch.autograd.Function``: its backward pass runs the adjoint step kernel
(``lgb_adjoint_step``) from the last step to the first. The forward pass
keeps a copy of the field every ``checkpoint_every`` steps; the backward pass
recomputes the states of one segment at a time from its checkpoint, so
memory holds ``steps / k`` checkpoints plus ``k`` states instead of all
``steps`` states. Per forward step the reverse pass moves 5 Q values per cell
(recompute: read Q, write Q; adjoint: read f Q, read lambda Q, write
lambda Q) on top of the forward's 2 Q.

Full segments (k forward steps; k - 1 recomputed states and k adjoint steps)
are replayed from CUDA graphs captured once per configuration; their
buffers live in a workspace kept between calls (``release_workspaces()``
frees them), so a rollout issues a few launches per segment instead of
several per step.

Everything before and after the rollout (the initial equilibrium from a
velocity field, moments and a loss) stays ordinary differentiable torch code,
so ``loss.backward()`` delivers gradients with respect to, e.g., the initial
velocity. torch autograd through lettuce's own step computes the same
gradient; the tests compare the two.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import torch

from . import _device, _lib

__all__ = ["rollout", "moments_torch", "release_workspaces"]


def _res3(res):
    return _lib.i32x3(list(res))


class _Workspace:
    """Buffers and captured graphs of one rollout configuration (stencil,
    tau, checkpoint interval k, field shape, dtype, device), kept between
    calls: two fields for the forward steps, k states of a segment and two
    adjoint fields for the reverse pass. A full segment of k steps (forward)
    or of k - 1 recomputed states plus k adjoint steps (reverse) is one
    CUDA-graph replay; a shorter last segment runs eagerly. Graphs are
    captured per parity of the field that holds the current state (both
    parities occur when k is odd). A workspace serves one rollout at a time."""

    def __init__(self, stencil_id, tau, k, like: torch.Tensor):
        self.stencil_id, self.tau, self.k = stencil_id, float(tau), int(k)
        self.res = list(like.shape[1:])
        self.r3 = _res3(self.res)
        self.storage = _device.storage_of(like.dtype)
        self.device = like.device
        self.fields = [torch.empty_like(like), torch.empty_like(like)]
        self.states = torch.empty([self.k] + list(like.shape), dtype=like.dtype,
                                  device=like.device)
        self.lams = [torch.empty_like(like), torch.empty_like(like)]
        self.desc = _device.new_desc(stencil_id, self.storage, self.res)
        self.desc.collision = _lib.BGK
        self.desc.tau = self.tau
        self.desc.pattern = _lib.PULL
        self.fwd_graphs = {}
        self.bwd_graphs = {}

    # -- launches ---------------------------------------------------------
    def _step(self, src: torch.Tensor, dst: torch.Tensor, stream: int):
        self.desc.f_in = src.data_ptr()
        self.desc.f_out = dst.data_ptr()
        _device.step(self.desc, stream)

    def _adjoint(self, state: torch.Tensor, lam: torch.Tensor, out: torch.Tensor, stream: int):
        L = _lib.load()
        _lib.check(L.lgb_adjoint_step(self.stencil_id, self.storage,
                                      ctypes.cast(self.r3, ctypes.c_void_p), self.tau,
                                      state.data_ptr(), lam.data_ptr(), out.data_ptr(), stream),
                   "lgb_adjoint_step")

    def _forward_segment(self, parity: int, n: int, stream: int) -> int:
        """n steps from fields[parity]; returns the parity holding the result"""
        for _ in range(n):
            self._step(self.fields[parity], self.fields[1 - parity], stream)
            parity = 1 - parity
        return parity

    def _reverse_segment(self, parity: int, n: int, stream: int) -> int:
        """states[1..n-1] recomputed from states[0], then n adjoint steps from
        lams[parity]; returns the parity holding the adjoint"""
        for i in range(n - 1):
            self._step(self.states[i], self.states[i + 1], stream)
        for i in reversed(range(n)):
            self._adjoint(self.states[i], self.lams[parity], self.lams[1 - parity], stream)
            parity = 1 - parity
        return parity

    def _graph(self, table, key, fn):
        g = table.get(key)
        if g is None:
            g = _device.capture(self.device, fn)
            table[key] = g
        return g

    # -- passes -----------------------------------------------------------
    def forward(self, f0: torch.Tensor, steps: int):
        """(f_T, checkpoints [n_seg, Q, ...]): checkpoint s is the state
        after s k steps"""
        k = self.k
        n_seg = (steps + k - 1) // k
        ckpts = torch.empty([n_seg] + list(f0.shape), dtype=f0.dtype, device=f0.device)
        stream = torch.cuda.current_stream(self.device).cuda_stream
        parity = 0
        self.fields[0].copy_(f0)
        for seg in range(n_seg):
            ckpts[seg].copy_(self.fields[parity])
            n = min(k, steps - seg * k)
            if n == k and k > 1:
                # (a fresh capture records the steps without running them)
                self._graph(self.fwd_graphs, parity,
                            lambda st, p=parity: self._forward_segment(p, k, st)).replay()
                parity = parity ^ (k & 1)
            else:
                parity = self._forward_segment(parity, n, stream)
        return self.fields[parity].clone(), ckpts

    def backward(self, grad: torch.Tensor, ckpts: torch.Tensor, steps: int) -> torch.Tensor:
        k = self.k
        n_seg = ckpts.shape[0]
        stream = torch.cuda.current_stream(self.device).cuda_stream
        parity = 0
        self.lams[0].copy_(grad)
        for seg in reversed(range(n_seg)):
            n = min(k, steps - seg * k)
            self.states[0].copy_(ckpts[seg])
            if n == k and k > 1:
                self._graph(self.bwd_graphs, parity,
                            lambda st, p=parity: self._reverse_segment(p, k, st)).replay()
                parity = parity ^ (k & 1)
            else:
                parity = self._reverse_segment(parity, n, stream)
        return self.lams[parity].clone()


_WORKSPACES = {}


def _workspace(stencil_id, tau, k, like: torch.Tensor) -> _Workspace:
    key = (stencil_id, float(tau), int(k), tuple(like.shape), like.dtype, like.device)
    ws = _WORKSPACES.get(key)
    if ws is None:
        ws = _Workspace(stencil_id, tau, k, like)
        _WORKSPACES[key] = ws
    return ws


def release_workspaces():
    """free the buffers and graphs kept between rollouts"""
    _WORKSPACES.clear()


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, stencil_id, tau, steps, checkpoint_every):
        if not f0.is_cuda:
            raise RuntimeError("rollout runs on CUDA tensors only; there is no CPU path")
        k = max(1, min(int(checkpoint_every), max(1, int(steps))))
        f0 = f0.detach().contiguous()
        if steps == 0:
            ctx.ckpts = None
            ctx.meta = (stencil_id, float(tau), 0, k)
            return f0.clone()
        ws = _workspace(stencil_id, tau, k, f0)
        fT, ckpts = ws.forward(f0, int(steps))
        ctx.ckpts = ckpts
        ctx.meta = (stencil_id, float(tau), int(steps), k)
        return fT

    @staticmethod
    def backward(ctx, grad_fT):
        stencil_id, tau, steps, k = ctx.meta
        grad = grad_fT.contiguous()
        if steps == 0:
            return grad.clone(), None, None, None, None
        ws = _workspace(stencil_id, tau, k, grad)
        lam = ws.backward(grad, ctx.ckpts, steps)
        ctx.ckpts = None
        return lam, None, None, None, None


def rollout(f0: torch.Tensor, stencil, tau: float, steps: int,
            checkpoint_every: int = 20) -> torch.Tensor:
    """populations after ``steps`` BGK steps (PRE_STREAMING), differentiable
    with respect to ``f0`` through the hand-written adjoint"""
    return _Rollout.apply(f0, stencil.lgb_id, float(tau), int(steps), int(checkpoint_every))


def moments_torch(f: torch.Tensor, stencil):
    """(rho [1, *res], u [D, *res]) with torch operations (differentiable)"""
    e = torch.tensor(stencil.e, dtype=f.dtype, device=f.device)
    rho = f.sum(0, keepdim=True)
    j = torch.einsum("qd,q...->d...", e, f)
    return rho, j / rho
