"""Collision operators with lettuce's constructors and plugin hooks
(lettuce/_simulation.py:17-28, lettuce/ext/_collision/*.py). The arithmetic
runs inside the fused step kernel; calling a collision directly
(``collision(flow)``) runs the kernel's collide-only pattern on a copy of
the populations and returns the result, like lettuce's torch operators."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

import torch

from . import _lib
from ._native import NativeCollision

__all__ = ["Collision", "BGKCollision", "TRTCollision", "KBCCollision", "NoCollision"]


class Collision(ABC):
    @abstractmethod
    def __call__(self, flow) -> torch.Tensor:
        ...

    @abstractmethod
    def native_available(self) -> bool:
        ...

    @abstractmethod
    def native_generator(self, index: int) -> NativeCollision:
        ...

    def bind(self, flow):
        """called once by Simulation with the flow it will advance"""

    def _apply_standalone(self, flow) -> torch.Tensor:
        from ._simulation import apply_local
        self.bind(flow)
        return apply_local(flow, self.native_generator(0), None)


class BGKCollision(Collision):
    """f - (f - feq) / tau (lettuce/ext/_collision/bgk_collision.py:17-22)"""

    def __init__(self, tau, force: Optional[object] = None):
        self.tau = tau
        self.force = force

    def __call__(self, flow) -> torch.Tensor:
        return self._apply_standalone(flow)

    def name(self) -> str:
        if self.force is not None:
            return f"{self.__class__.__name__}_{self.force.__class__.__name__}"
        return self.__class__.__name__

    def native_available(self) -> bool:
        # forcing terms (Guo, Shan-Chen) are not part of the fused kernels
        return self.force is None

    def native_generator(self, index: int) -> NativeCollision:
        return NativeCollision(_lib.BGK, index, tau=float(self.tau))


class TRTCollision(Collision):
    """two-relaxation-time collision (lettuce/ext/_collision/trt_collision.py:16-27):
    symmetric part relaxed with tau_plus, antisymmetric with tau_minus"""

    def __init__(self, tau, tau_minus=1.0):
        self.tau_plus = tau
        self.tau_minus = tau_minus

    def __call__(self, flow) -> torch.Tensor:
        return self._apply_standalone(flow)

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeCollision:
        return NativeCollision(_lib.TRT, index, tau=float(self.tau_plus),
                               tau_minus=float(self.tau_minus))


class KBCCollision(Collision):
    """entropic KBC collision (lettuce/ext/_collision/kbc_collision.py:11-160).
    Like lettuce, it relaxes with the flow's ``units.relaxation_parameter_lu``
    (the constructor argument is overwritten when bound to a flow) and is
    defined for D2Q9 and D3Q27."""

    def __init__(self, tau: float = None):
        self.tau = tau
        self.beta = None

    def bind(self, flow):
        if flow.stencil.d == 3 and flow.stencil.q != 27:
            raise AssertionError("KBC Collision is only implemented for D3Q27!")
        if flow.stencil.d == 2 and flow.stencil.q != 9:
            raise AssertionError("KBC Collision is only implemented for D2Q9!")
        if flow.stencil.d == 1:
            raise NotImplementedError("KBC Collision is only implemented for 2d and 3d!")
        self.tau = flow.units.relaxation_parameter_lu
        self.beta = 1.0 / (2 * self.tau)

    def __call__(self, flow) -> torch.Tensor:
        return self._apply_standalone(flow)

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeCollision:
        if self.tau is None:
            raise RuntimeError("KBCCollision needs a flow (Simulation binds it) before use")
        return NativeCollision(_lib.KBC, index, tau=float(self.tau))


class NoCollision(Collision):
    def __call__(self, flow) -> torch.Tensor:
        return flow.f

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeCollision:
        return NativeCollision(_lib.NO_COLLISION, index)
