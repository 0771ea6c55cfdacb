"""Problem set-ups: lettuce's ExtFlow, TaylorGreenVortex, Obstacle and
PoiseuilleFlow2D (lettuce/ext/_flows/_ext_flow.py, taylorgreen.py,
obstacle.py, poiseuille.py) with the same
constructors, unit conventions, initial fields and boundary lists."""
from __future__ import annotations

import warnings
from abc import ABC, abstractmethod
from typing import List, Optional, Union

import numpy as np
import torch

from ._boundary import AntiBounceBackOutlet, BounceBackBoundary, EquilibriumBoundaryPU
from ._flow import Flow, QuadraticEquilibrium
from ._stencil import D1Q3, D2Q9, D3Q19
from ._unit import UnitConversion

__all__ = ["ExtFlow", "TaylorGreenVortex", "Obstacle", "PoiseuilleFlow2D"]


class ExtFlow(Flow, ABC):
    """common constructor: default stencil by dimension (D1Q3/D2Q9/D3Q19)
    and the quadratic equilibrium"""

    def __init__(self, context, resolution: Union[int, List[int]], reynolds_number,
                 mach_number, stencil=None, equilibrium=None):
        resolution = self.make_resolution(resolution, stencil)
        assert len(resolution) in [1, 2, 3], \
            f"flow supports dimensions 1, 2 and 3 but {len(resolution)} were requested."
        defaults = [D1Q3(), D2Q9(), D3Q19()]
        stencil = stencil or defaults[len(resolution) - 1]
        stencil = stencil() if callable(stencil) else stencil
        equilibrium = equilibrium or QuadraticEquilibrium()
        Flow.__init__(self, context, resolution,
                      self.make_units(reynolds_number, mach_number, resolution),
                      stencil, equilibrium)

    @abstractmethod
    def make_resolution(self, resolution, stencil=None) -> List[int]:
        ...

    @abstractmethod
    def make_units(self, reynolds_number, mach_number, resolution) -> UnitConversion:
        ...


class TaylorGreenVortex(ExtFlow):
    """2-D / 3-D Taylor-Green vortex on [0, 2 pi)^D, L_lu = N / (2 pi); the
    2-D field is u = (cos x sin y, -sin x cos y) e^{-2 nu t}
    (taylorgreen.py:63-94). ``initialize_fneq`` (default True) adds the
    first-order non-equilibrium part."""

    def __init__(self, context, resolution, reynolds_number, mach_number,
                 stencil=None, equilibrium=None, initialize_fneq: bool = True):
        self.initialize_fneq = initialize_fneq
        if stencil is None and not isinstance(resolution, list):
            warnings.warn("Requiring information about dimensionality! Either via stencil "
                          "or resolution. Setting dimension to 2.", UserWarning)
            self.stencil = D2Q9()
        else:
            self.stencil = stencil() if callable(stencil) else stencil
        ExtFlow.__init__(self, context, resolution, reynolds_number, mach_number,
                         stencil, equilibrium)

    def make_resolution(self, resolution, stencil=None) -> List[int]:
        if isinstance(resolution, int):
            return [resolution] * self.stencil.d
        assert len(resolution) in [2, 3], \
            "the resolution of a taylor-green-vortex must be 2- or 3-dimensional!"
        return list(resolution)

    def make_units(self, reynolds_number, mach_number, resolution) -> UnitConversion:
        return UnitConversion(reynolds_number=reynolds_number, mach_number=mach_number,
                              characteristic_length_lu=resolution[0] / (2 * torch.pi),
                              characteristic_length_pu=1, characteristic_velocity_pu=1)

    @property
    def grid(self):
        ends = [2 * torch.pi * (1 - 1 / n) for n in self.resolution]
        xyz = tuple(torch.linspace(0, ends[n], steps=self.resolution[n],
                                   device=self.context.device, dtype=self.context.dtype)
                    for n in range(self.stencil.d))
        return torch.meshgrid(*xyz, indexing="ij")

    def initial_pu(self):
        return self.analytic_solution(t=0)

    def analytic_solution(self, t: float):
        if t > 0 and self.stencil.d > 2:
            warnings.warn("The analytic solution is only true for the 2D TGV!")
        g = self.grid
        nu = self.context.convert_to_tensor(self.units.viscosity_pu)
        if len(self.resolution) == 2:
            u = torch.stack([torch.cos(g[0]) * torch.sin(g[1]) * torch.exp(-2 * nu * t),
                             -torch.sin(g[0]) * torch.cos(g[1]) * torch.exp(-2 * nu * t)])
            p = -torch.stack([0.25 * (torch.cos(2 * g[0]) + torch.cos(2 * g[1]))
                              * torch.exp(-4 * nu * t)])
        else:
            u = torch.stack([torch.sin(g[0]) * torch.cos(g[1]) * torch.cos(g[2]),
                             -torch.cos(g[0]) * torch.sin(g[1]) * torch.cos(g[2]),
                             torch.zeros_like(g[0])])
            p = torch.stack([1 / 16. * (torch.cos(2 * g[0]) + torch.cos(2 * g[1]))
                             * (torch.cos(2 * g[2]) + 2)])
        return p, u

    @property
    def post_boundaries(self):
        return []


class Obstacle(ExtFlow):
    """flow in +x around a boolean obstacle ``mask`` (bounce-back) with an
    equilibrium velocity inlet at x = 0 and an anti-bounce-back outlet at
    x = -1; the other directions are periodic (obstacle.py:15-122)"""

    def __init__(self, context, resolution, reynolds_number, mach_number,
                 domain_length_x, char_length=1, char_velocity=1, stencil=None,
                 equilibrium=None):
        self.char_length_lu = resolution[0] / domain_length_x * char_length
        self.char_length = char_length
        self.char_velocity = char_velocity
        self.resolution = self.make_resolution(resolution, stencil)
        self._mask = torch.zeros(self.resolution, dtype=torch.bool)
        ExtFlow.__init__(self, context, resolution, reynolds_number, mach_number,
                         stencil, equilibrium)

    def make_units(self, reynolds_number, mach_number, resolution) -> UnitConversion:
        return UnitConversion(reynolds_number=reynolds_number, mach_number=mach_number,
                              characteristic_length_lu=self.char_length_lu,
                              characteristic_length_pu=self.char_length,
                              characteristic_velocity_pu=self.char_velocity)

    def make_resolution(self, resolution, stencil=None) -> List[int]:
        if isinstance(resolution, int):
            return [resolution] * (stencil.d or self.stencil.d)
        return list(resolution)

    @property
    def mask(self):
        return self._mask

    @mask.setter
    def mask(self, m):
        assert (isinstance(m, (np.ndarray, torch.Tensor))
                and all(m.shape[d] == self.resolution[d] for d in range(self.stencil.d)))
        self._mask = self.context.convert_to_tensor(m, dtype=torch.bool)

    def initial_pu(self):
        p = np.zeros_like(self.grid[0], dtype=float)[None, ...]
        u_char = self.units.characteristic_velocity_pu * self._unit_vector()
        u_char = u_char[(...,) + (None,) * self.stencil.d]
        mask = self.mask.cpu() if isinstance(self.mask, torch.Tensor) else self.mask
        u = ~mask * u_char
        return p, u

    @property
    def grid(self):
        xyz = tuple(self.units.convert_length_to_pu(torch.arange(n)) for n in self.resolution)
        return torch.meshgrid(*xyz, indexing="ij")

    @property
    def post_boundaries(self):
        x = self.grid[0]
        return [
            EquilibriumBoundaryPU(flow=self, context=self.context,
                                  mask=(torch.abs(x) < 1e-6).to(self.context.device),
                                  velocity=self.units.characteristic_velocity_pu
                                  * self._unit_vector()),
            AntiBounceBackOutlet(self._unit_vector().tolist(), self),
            BounceBackBoundary(self.mask),
        ]

    def _unit_vector(self, i=0):
        return torch.eye(self.stencil.d)[i]


class PoiseuilleFlow2D(ExtFlow):
    """plane Poiseuille channel driven by a body force a = (0.001, 0)
    (physical units) between bounce-back walls at y = 0 and y = 1,
    periodic in x (lettuce/ext/_flows/poiseuille.py:16-95); starts at rest by
    default"""

    def __init__(self, context, resolution: Union[int, List[int]], reynolds_number,
                 mach_number, stencil=None, equilibrium=None, initialize_with_zeros=True):
        self.stencil = D2Q9() if stencil is None else (stencil() if callable(stencil) else stencil)
        self.initialize_with_zeros = initialize_with_zeros
        ExtFlow.__init__(self, context, resolution, reynolds_number, mach_number,
                         self.stencil, equilibrium)

    def analytic_solution(self, t=0):
        half_lattice_spacing = 0.5 / self.resolution[0]
        x, y = self.grid
        nu = self.units.viscosity_pu
        rho = 1
        ux = (self.acceleration[0] / (2 * rho * nu)
              * ((y - half_lattice_spacing) * (1 - half_lattice_spacing - y)))
        uy = self.context.zero_tensor(self.resolution)
        u = torch.stack([ux, uy], dim=0)
        p = y * 0 + self.units.convert_density_lu_to_pressure_pu(rho)
        return p, u

    def initial_pu(self):
        if self.initialize_with_zeros:
            zeros = self.context.zero_tensor(self.resolution)
            return zeros[None, ...], torch.stack(2 * [zeros], dim=0)
        return self.analytic_solution()

    def make_units(self, reynolds_number, mach_number, resolution) -> UnitConversion:
        return UnitConversion(reynolds_number=reynolds_number, mach_number=mach_number,
                              characteristic_length_lu=resolution[0] - 1,
                              characteristic_length_pu=1, characteristic_velocity_pu=1)

    def make_resolution(self, resolution, stencil=None) -> List[int]:
        if isinstance(resolution, list):
            assert len(resolution) == self.stencil.d
            return list(resolution)
        return [resolution] * self.stencil.d

    @property
    def grid(self):
        xyz = tuple(torch.linspace(0, 1, steps=n, device=self.context.device,
                                   dtype=self.context.dtype) for n in self.resolution)
        return torch.meshgrid(*xyz, indexing="ij")

    @property
    def post_boundaries(self):
        mask = self.context.zero_tensor(self.resolution, dtype=bool)
        mask[:, [0, -1]] = True
        return [BounceBackBoundary(mask=mask)]

    @property
    def acceleration(self):
        return self.context.convert_to_tensor([0.001, 0])
