"""Boundary conditions with lettuce's constructors, masks and plugin hooks.

* BounceBackBoundary  -- lettuce/ext/_boundary/bounce_back_boundary.py:10-32
* EquilibriumBoundaryPU -- lettuce/ext/_boundary/equilibrium_boundary_pu.py:15-98
* AntiBounceBackOutlet -- lettuce/ext/_boundary/anti_bounce_back_outlet.py:13-109
* EquilibriumOutletP -- lettuce/ext/_boundary/equilibrium_outlet_p.py:12-91
* PartiallySaturatedBC -- lettuce/ext/_boundary/partially_saturated_boundary.py:6-51

The masks are built exactly as lettuce builds them (they are combined by
``Simulation`` into the per-cell flag byte); the operators themselves run
inside the step kernel. Calling a boundary directly runs that operator
through the kernel's collide-only pattern.
"""
from __future__ import annotations

import numbers
from typing import List, Optional, Union

import numpy as np
import torch

from . import _lib
from ._flow import Boundary
from ._native import NativeBoundary, NativeCollision

__all__ = ["BounceBackBoundary", "EquilibriumBoundaryPU", "AntiBounceBackOutlet",
           "EquilibriumOutletP", "PartiallySaturatedBC"]


def _apply_alone(flow, native: NativeBoundary, flags_value):
    """run one boundary operator over the whole field (flags = its index)"""
    from ._simulation import apply_local
    native.index = 1
    flags = torch.full(flow.resolution, flags_value, dtype=torch.uint8,
                       device=flow.context.device)
    return apply_local(flow, NativeCollision(_lib.NO_COLLISION, 0), native, flags)


class BounceBackBoundary(Boundary):
    """full-way bounce-back: f <- f[opposite] on the mask"""

    def __init__(self, mask: torch.Tensor):
        self._mask = mask

    def __call__(self, flow):
        return _apply_alone(flow, self.native_generator(1), 1)

    def make_no_streaming_mask(self, shape: List[int], context) -> Optional[torch.Tensor]:
        return None

    def make_no_collision_mask(self, shape: List[int], context) -> Optional[torch.Tensor]:
        return self._mask

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        return NativeBoundary(_lib.SUB_BOUNCE_BACK, index)


class EquilibriumBoundaryPU(Boundary):
    """f <- feq(rho(pressure), velocity) on the mask; velocity and pressure in
    physical units, broadcastable over the grid"""

    @staticmethod
    def checked_tensor(t, context, flow) -> torch.Tensor:
        # same accepted shapes as equilibrium_boundary_pu.py:23-69
        if not torch.is_tensor(t):
            if isinstance(t, numbers.Number):
                t = torch.tensor(t)
            elif isinstance(t, (np.ndarray, list, tuple)):
                t = torch.as_tensor(t)
            else:
                raise TypeError(f"Cannot convert {type(t)} to tensor")
        d = flow.stencil.d
        spatial = list(flow.resolution)
        full_ndim = 1 + len(spatial)
        if t.ndim == 0:
            t = t.reshape([1] * full_ndim)
        elif t.ndim == 1 and t.shape[0] == d:
            t = t.reshape([d] + [1] * len(spatial))
        elif t.ndim == len(spatial) and list(t.shape) == spatial:
            t = t.unsqueeze(0)
        elif t.ndim != full_ndim:
            raise ValueError(f"Tensor has wrong rank: expected {full_ndim}, got {t.ndim}")
        for i in range(full_ndim):
            size = t.shape[i]
            if i == 0:
                if size not in (1, d):
                    raise ValueError(f"Component dim must be 1 or {d}, got {size}")
            elif size not in (1, spatial[i - 1]):
                raise ValueError(f"Spatial dim {i} must be 1 or {spatial[i - 1]}, got {size}")
        return context.convert_to_tensor(t)

    def __init__(self, context, flow, mask, velocity, pressure=0):
        self.velocity = self.checked_tensor(velocity, context, flow)
        self.pressure = self.checked_tensor(pressure, context, flow)
        self._mask = mask
        self._units = flow.units

    def __call__(self, flow):
        return _apply_alone(flow, self.native_generator(1), 1)

    def make_no_collision_mask(self, shape: List[int], context) -> Optional[torch.Tensor]:
        return self._mask

    def make_no_streaming_mask(self, shape: List[int], context) -> Optional[torch.Tensor]:
        return None

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        rho = self._units.convert_pressure_pu_to_density_lu(self.pressure)[0]
        u = self._units.convert_velocity_to_lu(self.velocity)
        return NativeBoundary(_lib.SUB_EQUILIBRIUM_PU, index,
                              rho=rho.contiguous(), u=u.contiguous())


class AntiBounceBackOutlet(Boundary):
    """outflow: f[opp(v)] = -f[v] + w_v rho (2 + (e_v.u_w)^2/cs^4 - |u_w|^2/cs^2)
    on the outlet plane with u_w = u + (u - u_neighbour)/2, for the velocities
    v pointing out of the domain (Krueger et al. 2016, p. 195)"""

    def __init__(self, direction: List[int], flow, collision=None):
        assert len(direction) in [1, 2, 3], \
            f"Invalid direction parameter. Expected length 1, 2 or 3 but got {len(direction)}."
        assert ((direction.count(0) == (len(direction) - 1))
                and ((1 in direction) ^ (-1 in direction))), \
            (f"Invalid direction parameter. Expected direction with all entries 0 "
             f"except one 1 or -1 but got {direction}.")
        self.direction = list(direction)
        self.stencil = flow.torch_stencil
        e = np.array(flow.stencil.e)
        self.velocities = np.concatenate(
            np.argwhere(e @ np.array(direction) > 1 - 1e-6), axis=0)
        self.index = []
        for i in direction:
            if i == 0:
                self.index.append(slice(None))
            elif i == 1:
                self.index.append(-1)
            else:
                self.index.append(0)
        self._opposite = np.array(flow.stencil.opposite)

    def __call__(self, flow):
        # the outlet mutates the field in place and returns it
        out = _apply_alone(flow, self.native_generator(1), 0)
        flow.f = out
        return flow.f

    def make_no_streaming_mask(self, f_shape, context):
        m = torch.zeros(size=list(f_shape), dtype=torch.bool, device=context.device)
        m[tuple([self._opposite[self.velocities]] + self.index)] = True
        return m

    def make_no_collision_mask(self, shape: List[int], context):
        m = torch.zeros(list(shape), dtype=torch.bool, device=context.device)
        m[tuple(self.index)] = True
        return m

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        axis = [i for i, v in enumerate(self.direction) if v != 0][0]
        return NativeBoundary(_lib.SUB_ANTI_BOUNCE_BACK, index, axis=axis,
                              sign=int(self.direction[axis]))


class EquilibriumOutletP(AntiBounceBackOutlet):
    """pressure outlet: the outlet plane takes feq(rho_outlet, u of the plane
    one cell inside); only the populations leaving the domain stream into
    the plane, the others keep the boundary values"""

    def __init__(self, direction: List[int], flow, rho_outlet: float = 1.0):
        super().__init__(direction, flow)
        self.context = flow.context
        self.rho_outlet = self.context.convert_to_tensor(rho_outlet)

    def make_no_streaming_mask(self, shape, context):
        m = torch.zeros(list(shape), dtype=torch.bool, device=context.device)
        others = np.setdiff1d(np.arange(shape[0]), self.velocities)
        m[tuple([others] + self.index)] = True
        return m

    def native_generator(self, index: int) -> NativeBoundary:
        axis = [i for i, v in enumerate(self.direction) if v != 0][0]
        return NativeBoundary(_lib.SUB_EQUILIBRIUM_OUTLET_P, index, axis=axis,
                              sign=int(self.direction[axis]),
                              params=(float(self.rho_outlet.item()), 0.0))


class PartiallySaturatedBC(Boundary):
    """partially saturated cells (Noble & Torczynski 1998, Krueger et al.
    p. 448): a blend of BGK and bounce-back weighted by
    B = eps (tau - 1/2) / ((1 - eps) + (tau - 1/2)) on the mask"""

    def __init__(self, mask: torch.Tensor, tau: float, saturation: float):
        self._mask = mask
        self.tau = tau
        self.B = saturation * (tau - 0.5) / ((1 - saturation) + (tau - 0.5))

    def __call__(self, flow):
        return _apply_alone(flow, self.native_generator(1), 1)

    def make_no_collision_mask(self, shape: List[int], context) -> torch.Tensor:
        return self._mask

    def make_no_streaming_mask(self, shape: List[int], context):
        return None

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        return NativeBoundary(_lib.SUB_PARTIALLY_SATURATED, index,
                              params=(float(self.tau), float(self.B)))
