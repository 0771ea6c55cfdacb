"""Body forces with lettuce's constructors and interface
(lettuce/ext/_force/_force.py, guo.py, shan_chen.py).

A force is a constant acceleration in lattice units. Passed to
``BGKCollision(tau, force=...)`` or ``SmagorinskyCollision(..., force=...)``
it runs inside the step kernel: the equilibrium is evaluated at
u = j / rho + s a / rho (s = 1/2 for Guo, the force's tau for Shan-Chen) and
Guo adds the source term (1 - 1/(2 tau)) w_q [(e_q - u)/cs^2 + (e_q.u) e_q/cs^4].a.
``u_eq`` and ``source_term`` restate those terms on torch tensors for
callers that evaluate them outside the step (lettuce's Force interface).
"""
from __future__ import annotations

from abc import ABC, abstractmethod

import torch

from . import _lib
from ._native import NativeForce

__all__ = ["Force", "Guo", "ShanChen"]


def _append_axes(t: torch.Tensor, d: int) -> torch.Tensor:
    return t[(...,) + (None,) * d]


class Force(ABC):
    @abstractmethod
    def __init__(self, flow, tau, acceleration):
        ...

    @abstractmethod
    def source_term(self, u):
        ...

    @abstractmethod
    def u_eq(self, flow=None):
        ...

    @property
    @abstractmethod
    def ueq_scaling_factor(self):
        ...

    def native_available(self) -> bool:
        return True

    def _accel_tuple(self):
        a = self.acceleration
        return tuple(float(v) for v in (a.reshape(-1).tolist() if torch.is_tensor(a) else a))


class Guo(Force):
    """Guo forcing (lettuce/ext/_force/guo.py)"""

    def __init__(self, flow, tau, acceleration):
        self.flow = flow
        self.tau = tau
        self.acceleration = flow.context.convert_to_tensor(acceleration)

    def source_term(self, u):
        ts = self.flow.torch_stencil
        e = ts.e.to(u.dtype)
        w = ts.w.to(u.dtype)
        a = self.acceleration.to(u.dtype)
        d = self.flow.stencil.d
        emu = _append_axes(e, d) - u                       # [Q, D, ...]
        eu = torch.einsum("ib,b...->i...", e, u)           # [Q, ...]
        eeu = torch.einsum("ia,i...->ia...", e, eu)        # [Q, D, ...]
        emu_eeu = emu / ts.cs ** 2 + eeu / ts.cs ** 4
        emu_eeuF = torch.einsum("ia...,a->i...", emu_eeu, a)
        return (1 - 1 / (2 * self.tau)) * _append_axes(w, d) * emu_eeuF

    def u_eq(self, flow=None):
        flow = self.flow if flow is None else flow
        return (self.ueq_scaling_factor * _append_axes(self.acceleration, flow.stencil.d)
                / flow.rho())

    @property
    def ueq_scaling_factor(self):
        return 0.5

    def native_generator(self) -> NativeForce:
        return NativeForce(_lib.FORCE_GUO, float(self.tau), self._accel_tuple())


class ShanChen(Force):
    """Shan-Chen forcing (lettuce/ext/_force/shan_chen.py): the equilibrium
    velocity is shifted by tau a / rho, no source term"""

    def __init__(self, flow, tau, acceleration):
        self.flow = flow
        self.tau = tau
        self.acceleration = flow.context.convert_to_tensor(acceleration)

    def source_term(self, u):
        return 0

    def u_eq(self, flow=None):
        flow = self.flow if flow is None else flow
        return (self.ueq_scaling_factor * _append_axes(self.acceleration, flow.stencil.d)
                / flow.rho())

    @property
    def ueq_scaling_factor(self):
        return self.tau * 1

    def native_generator(self) -> NativeForce:
        return NativeForce(_lib.FORCE_SHAN_CHEN, float(self.tau), self._accel_tuple())
