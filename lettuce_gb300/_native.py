"""Descriptors returned by the plugin hooks ``native_generator``.

lettuce's hooks (lettuce/_simulation.py:17-28, lettuce/_flow.py:17-52) return
code-emitting objects that the cuda_native generator turns into CUDA source
at run time. Here the kernels are compiled ahead of time, so the same hooks
return small descriptors: which operator, which substep index, and its
scalar/tensor parameters. ``Simulation`` packs them into ``lgb_step_desc``.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import torch

from . import _lib

__all__ = ["NativeEquilibrium", "NativeQuadraticEquilibrium", "NativeCollision",
           "NativeBoundary", "NativeForce"]


@dataclass
class NativeEquilibrium:
    name: str


def NativeQuadraticEquilibrium() -> NativeEquilibrium:
    return NativeEquilibrium("quadratic")


@dataclass
class NativeForce:
    kind: int                  # _lib.FORCE_GUO / FORCE_SHAN_CHEN
    tau: float
    acceleration: tuple        # lattice units, one entry per dimension


@dataclass
class NativeCollision:
    kind: int                  # _lib.NO_COLLISION / BGK / TRT / KBC / REGULARIZED / SMAGORINSKY
    index: int
    tau: float = 1.0
    tau_minus: float = 1.0
    force: Optional[NativeForce] = None
    smagorinsky_constant: float = 0.0
    mrt_equilibrium: int = 0
    mrt_tables: Optional[object] = None  # float64 numpy [M, M^-1, relaxation times]


@dataclass
class NativeBoundary:
    kind: int                  # _lib.SUB_BOUNCE_BACK / SUB_EQUILIBRIUM_PU / ...
    index: int
    rho: Optional[torch.Tensor] = None   # equilibrium BC, [1|N1, 1|N2, ...]
    u: Optional[torch.Tensor] = None     # equilibrium BC, [1|D, 1|N1, ...]
    axis: int = 0                        # outlet-plane substeps
    sign: int = 1
    params: tuple = (0.0, 0.0)           # pressure outlet (rho,), partially saturated (tau, B)
    keep: list = field(default_factory=list)
