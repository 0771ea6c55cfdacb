"""Collision operators with lettuce's constructors and plugin hooks
(lettuce/_simulation.py:17-28, lettuce/ext/_collision/*.py). The arithmetic
runs inside the fused step kernel; calling a collision directly
(``collision(flow)``) runs the kernel's collide-only pattern on a copy of
the populations and returns the result, like lettuce's torch operators."""
from __future__ import annotations

from abc import ABC, abstractmethod
from typing import Optional

import numpy as np
import torch

from . import _lib
from ._native import NativeCollision

__all__ = ["Collision", "BGKCollision", "TRTCollision", "KBCCollision", "NoCollision",
           "RegularizedCollision", "SmagorinskyCollision", "MRTCollision"]


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
        return self.force is None or self.force.native_available()

    def native_generator(self, index: int) -> NativeCollision:
        force = self.force.native_generator() if self.force is not None else None
        return NativeCollision(_lib.BGK, index, tau=float(self.tau), force=force)


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


class RegularizedCollision(Collision):
    """regularized BGK (Latt & Chopard 2006,
    lettuce/ext/_collision/regularized_collision.py:8-47): the non-equilibrium
    part is replaced by its projection on the second moments,
    f = feq + (1 - 1/tau) w_q Q_q : Pi_neq / (2 cs^4). Like lettuce, it
    relaxes with the flow's ``units.relaxation_parameter_lu`` (the
    constructor argument is overwritten when bound to a flow)."""

    def __init__(self, tau: float = None):
        self.tau = tau

    def bind(self, flow):
        self.tau = flow.units.relaxation_parameter_lu

    def __call__(self, flow) -> torch.Tensor:
        return self._apply_standalone(flow)

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeCollision:
        if self.tau is None:
            raise RuntimeError("RegularizedCollision needs a flow (Simulation binds it) before use")
        return NativeCollision(_lib.REGULARIZED, index, tau=float(self.tau))


class SmagorinskyCollision(Collision):
    """Smagorinsky large-eddy BGK
    (lettuce/ext/_collision/smagorinsky_collision.py:8-41): per cell,
    tau_eff from two fixed-point iterations of
    nu_eff = (tau - 1/2)/3 + C^2 S:S with S = Pi_neq / (2 rho cs^2 tau_eff),
    optionally with a body force"""

    def __init__(self, tau, smagorinsky_constant=0.17, force: Optional[object] = None):
        self.force = force
        self.tau = tau
        self.iterations = 2
        self.tau_eff = tau
        self.constant = smagorinsky_constant

    def __call__(self, flow) -> torch.Tensor:
        return self._apply_standalone(flow)

    def native_available(self) -> bool:
        return self.force is None or self.force.native_available()

    def native_generator(self, index: int) -> NativeCollision:
        force = self.force.native_generator() if self.force is not None else None
        return NativeCollision(_lib.SMAGORINSKY, index, tau=float(self.tau), force=force,
                               smagorinsky_constant=float(self.constant))


class MRTCollision(Collision):
    """multiple-relaxation-time collision
    (lettuce/ext/_collision/mrt_collision.py:8-30): m = M f,
    m <- m - (m - meq) / s, f = M^-1 m, with the moment basis and equilibrium
    of ``transform`` (``lettuce_gb300._moments``) and one relaxation time per
    moment"""

    def __init__(self, transform, relaxation_parameters: list, context):
        self.transform = transform
        self.relaxation_parameters = context.convert_to_tensor(relaxation_parameters)

    def __call__(self, flow) -> torch.Tensor:
        return self._apply_standalone(flow)

    def _equilibrium_kind(self):
        """the kernel's equilibrium for the transform: that of the class of
        this package defining the transform's ``equilibrium``, or None"""
        from . import _moments
        owner = next((k for k in type(self.transform).__mro__ if "equilibrium" in k.__dict__),
                     None)
        if owner is None or owner.__module__ != _moments.__name__:
            return None
        return owner.__dict__.get("equilibrium_kind", _lib.MRT_EQ_GENERIC)

    def native_available(self) -> bool:
        return self._equilibrium_kind() is not None

    def native_generator(self, index: int) -> NativeCollision:
        kind = self._equilibrium_kind()
        if kind is None:
            raise NotImplementedError(f"no kernel for the transform {type(self.transform).__name__}")
        s = self.relaxation_parameters.detach().to("cpu", torch.float64).numpy().reshape(-1)
        tables = np.concatenate([self.transform.matrix_np.reshape(-1),
                                 self.transform.inverse_np.reshape(-1), s])
        return NativeCollision(_lib.MRT, index, mrt_equilibrium=kind, mrt_tables=tables)


class NoCollision(Collision):
    def __call__(self, flow) -> torch.Tensor:
        return flow.f

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeCollision:
        return NativeCollision(_lib.NO_COLLISION, index)
