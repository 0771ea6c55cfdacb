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

__all__ = ["rollout", "moments_torch"]


def _res3(res):
    return _lib.i32x3(list(res))


def _forward_steps(f: torch.Tensor, stencil_id: int, tau: float, steps: int,
                   keep_every: Optional[int] = None):
    """advance f by steps; returns (f_T, checkpoints every keep_every steps)"""
    storage = _device.storage_of(f.dtype)
    res = list(f.shape[1:])
    d = _device.new_desc(stencil_id, storage, res)
    d.collision = _lib.BGK
    d.tau = float(tau)
    d.pattern = _lib.PULL
    cur = f.contiguous().clone()
    nxt = torch.empty_like(cur)
    stream = _device.stream_of(cur)
    ckpts = []
    for n in range(steps):
        if keep_every and n % keep_every == 0:
            ckpts.append(cur.clone())
        d.f_in = cur.data_ptr()
        d.f_out = nxt.data_ptr()
        _device.step(d, stream)
        cur, nxt = nxt, cur
    return cur, ckpts


class _Rollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, f0, stencil_id, tau, steps, checkpoint_every):
        if not f0.is_cuda:
            raise RuntimeError("rollout runs on CUDA tensors only; there is no CPU path")
        k = max(1, int(checkpoint_every))
        fT, ckpts = _forward_steps(f0.detach(), stencil_id, tau, steps, keep_every=k)
        ctx.ckpts = ckpts
        ctx.meta = (stencil_id, float(tau), int(steps), k, list(f0.shape[1:]))
        return fT

    @staticmethod
    def backward(ctx, grad_fT):
        stencil_id, tau, steps, k, res = ctx.meta
        L = _lib.load()
        lam = grad_fT.contiguous().clone()
        if steps == 0:
            return lam, None, None, None, None
        storage = _device.storage_of(lam.dtype)
        buf = torch.empty_like(lam)
        r3 = _res3(res)
        stream = _device.stream_of(lam)
        n_seg = (steps + k - 1) // k
        for seg in reversed(range(n_seg)):
            start = seg * k
            end = min(start + k, steps)
            # states f_start .. f_{end-1} recomputed from the checkpoint
            states = [ctx.ckpts[seg]]
            for _ in range(start, end - 1):
                nxt, _ = _forward_steps(states[-1], stencil_id, tau, 1)
                states.append(nxt)
            for n in reversed(range(start, end)):
                _lib.check(L.lgb_adjoint_step(stencil_id, storage,
                                              ctypes.cast(r3, ctypes.c_void_p), tau,
                                              states[n - start].data_ptr(), lam.data_ptr(),
                                              buf.data_ptr(), stream), "lgb_adjoint_step")
                lam, buf = buf, lam
            del states
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
