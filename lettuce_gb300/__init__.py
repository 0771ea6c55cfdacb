"""lettuce_gb300 -- a GB300-native (sm_103a) lattice Boltzmann step behind
lettuce's plugin surface.

The public names mirror lettuce's (``Context``, stencils, ``UnitConversion``,
``Flow``, collisions, boundaries, ``Simulation``, reporters, flows), so a
script written against lettuce's native path runs unchanged. The stepping
is done by hand-written CUDA kernels in ``liblettuce_gb300.so``, reached
through its C ABI (include/lettuce_gb300.h); there is no CPU or torch
fallback for the step. ``native_invoke`` / ``install`` put the same kernels
behind lettuce's own ``Simulation`` objects (lettuce/_simulation.py:229).
"""
from ._context import Context
from ._stencil import D1Q3, D2Q9, D3Q15, D3Q19, D3Q27, Stencil, TorchStencil
from ._unit import UnitConversion
from ._flow import (Boundary, Equilibrium, Flow, QuadraticEquilibrium,
                    QuadraticEquilibriumLessMemory,
                    initialize_f_neq, torch_gradient)
from ._collision import (BGKCollision, Collision, KBCCollision, MRTCollision, NoCollision,
                         RegularizedCollision, SmagorinskyCollision, TRTCollision)
from ._moments import D1Q3Transform, D2Q9Dellar, D2Q9Lallemand, D3Q27Hermite, Transform
from ._force import Force, Guo, ShanChen
from ._boundary import (AntiBounceBackOutlet, BounceBackBoundary, EquilibriumBoundaryPU,
                        EquilibriumOutletP, FullwayBounceBackBoundary,
                        HalfwayBounceBackBoundary, LinearInterpolatedBounceBackBoundary,
                        PartiallySaturatedBC, SolidBoundaryData, fwbb_links, hwbb_links)
from ._simulation import (BreakableSimulation, EbbSimulation, Reporter, Simulation,
                          StreamingStrategy)
from ._reporter import (EnergySpectrum, Enstrophy, ErrorReporter, FailureReporterBase,
                        HighMaReporter, IncompressibleKineticEnergy, Mass,
                        DragCoefficient, LiftCoefficient,
                        MaximumVelocity, NaNReporter, Observable, ObservableReporter)
from ._flows import ExtFlow, Obstacle, PoiseuilleFlow2D, TaylorGreenVortex
from ._native import NativeBoundary, NativeCollision, NativeEquilibrium
from ._batched import BatchedSimulation, batched_taylor_green
from ._adjoint import moments_torch, rollout
from ._slab import Slab, SlabSimulation, exchange, exchange_local
from ._lettuce_native import NativeStep, install, native_invoke, native_step

__version__ = "0.1.0"

__all__ = [
    "Context", "Stencil", "TorchStencil", "D1Q3", "D2Q9", "D3Q15", "D3Q19", "D3Q27",
    "UnitConversion", "Flow", "Equilibrium", "QuadraticEquilibrium",
    "QuadraticEquilibriumLessMemory", "Boundary",
    "initialize_f_neq", "torch_gradient", "Collision", "BGKCollision",
    "TRTCollision", "KBCCollision", "NoCollision", "BounceBackBoundary",
    "EquilibriumBoundaryPU", "AntiBounceBackOutlet", "EquilibriumOutletP",
    "PartiallySaturatedBC", "HalfwayBounceBackBoundary", "LinearInterpolatedBounceBackBoundary",
    "FullwayBounceBackBoundary", "SolidBoundaryData", "hwbb_links", "fwbb_links",
    "Simulation", "EbbSimulation",
    "BreakableSimulation", "StreamingStrategy", "Reporter", "Observable",
    "ObservableReporter", "MaximumVelocity", "IncompressibleKineticEnergy",
    "Enstrophy", "EnergySpectrum", "Mass", "DragCoefficient", "LiftCoefficient",
    "ErrorReporter", "FailureReporterBase",
    "NaNReporter", "HighMaReporter", "ExtFlow", "TaylorGreenVortex", "Obstacle",
    "NativeBoundary", "NativeCollision", "NativeEquilibrium", "BatchedSimulation",
    "batched_taylor_green", "rollout", "moments_torch", "Slab", "SlabSimulation",
    "exchange", "exchange_local", "RegularizedCollision", "SmagorinskyCollision", "Force",
    "Guo", "ShanChen", "PoiseuilleFlow2D", "MRTCollision", "Transform", "D1Q3Transform",
    "D2Q9Dellar", "D2Q9Lallemand", "D3Q27Hermite", "native_invoke", "native_step", "install",
    "NativeStep",
]
