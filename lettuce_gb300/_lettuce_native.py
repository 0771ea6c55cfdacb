"""The GB300 step for lettuce's own ``Simulation`` objects.

lettuce swaps its step at lettuce/_simulation.py:172-229: with
``Context(use_native=True)`` it asks the equilibrium, the collision and each
boundary for a ``native_generator``, generates CUDA source from them, builds
it as a torch extension and assigns ``self._collide_and_stream =
native_kernel``. The generated ``invoke(simulation)``
(lettuce/cuda_native/_template.py:35-40) calls ``cuda_native.lettuce(f,
f_next, ...)`` and swaps ``flow.f`` / ``flow.f_next``.

``native_invoke(simulation)`` returns that ``invoke`` for the same
simulation, built from lettuce's objects as they stand -- no code generation
and no compiler at run time:

* the stencil, resolution and population dtype of ``simulation.flow``;
* the collision (``BGKCollision`` with its optional ``Guo`` / ``ShanChen``
  force, ``TRTCollision``, ``KBCCollision``, ``NoCollision``,
  ``RegularizedCollision``, ``SmagorinskyCollision``, ``MRTCollision``) and
  the boundaries of ``simulation.pre_boundaries`` / ``post_boundaries``
  (``BounceBackBoundary``, ``EquilibriumBoundaryPU``,
  ``AntiBounceBackOutlet``, ``EquilibriumOutletP``, ``PartiallySaturatedBC``),
  read from their attributes; a component of another kind raises
  ``NotImplementedError`` (there is no torch fallback);
* lettuce's own ``no_collision_mask`` / ``no_streaming_mask`` as the
  simulation built them (lettuce/_simulation.py:100-146), packed into the
  flag byte and no-streaming word of ``lgb_step_desc``;
* ``simulation.streaming_strategy``: PRE -> one pull launch, POST -> one push
  launch, DOUBLE -> pull then stream-only, NO -> collide only.

Each call launches on the current torch stream, does not synchronise, and
swaps the fields exactly as lettuce's ``invoke`` does. ``install(simulation)``
assigns it the way lettuce/_simulation.py:229 does. lettuce itself is not
imported: components are recognised by their class names (the first known
name along the class's MRO) and the attributes lettuce gives them.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from types import SimpleNamespace
from typing import List, Optional

import numpy as np
import torch

from . import _device, _lib
from ._native import NativeBoundary, NativeCollision, NativeForce
from ._simulation import _desc_for, pack_masks
from ._stencil import D1Q3, D2Q9, D3Q15, D3Q19, D3Q27

__all__ = ["native_step", "native_invoke", "install", "NativeStep"]

_STENCILS = {"D1Q3": D1Q3, "D2Q9": D2Q9, "D3Q15": D3Q15, "D3Q19": D3Q19, "D3Q27": D3Q27}
_MRT_EQUILIBRIA = {"D2Q9Dellar": _lib.MRT_EQ_DELLAR, "D2Q9Lallemand": _lib.MRT_EQ_LALLEMAND,
                   "D3Q27Hermite": _lib.MRT_EQ_HERMITE}


def _kind(obj, known) -> Optional[str]:
    """the first class name along obj's MRO that is in ``known``"""
    for k in type(obj).__mro__:
        if k.__name__ in known:
            return k.__name__
    return None


def _as_np(t) -> np.ndarray:
    if isinstance(t, torch.Tensor):
        return t.detach().cpu().numpy()
    return np.asarray(t)


def _stencil_id(stencil) -> int:
    name = _kind(stencil, _STENCILS)
    if name is None:
        raise NotImplementedError(f"no GB300 kernels for the stencil {type(stencil).__name__}")
    ours = _STENCILS[name]()
    if not np.array_equal(np.asarray(_as_np(stencil.e), dtype=np.int64),
                          np.asarray(ours.e, dtype=np.int64)):
        raise ValueError(f"stencil {name}: velocity set differs from lettuce's {name} table")
    return ours.lgb_id


def _force_native(force) -> Optional[NativeForce]:
    if force is None:
        return None
    name = _kind(force, ("Guo", "ShanChen"))
    if name is None:
        raise NotImplementedError(f"no GB300 kernel for the force {type(force).__name__}")
    acc = tuple(float(v) for v in _as_np(force.acceleration).reshape(-1))
    return NativeForce(_lib.FORCE_GUO if name == "Guo" else _lib.FORCE_SHAN_CHEN,
                       float(force.tau), acc)


def _collision_native(coll, flow, index: int) -> NativeCollision:
    """lettuce/ext/_collision/*.py: the operator and its parameters"""
    known = ("KBCCollision", "TRTCollision", "RegularizedCollision", "SmagorinskyCollision",
             "MRTCollision", "BGKCollision", "NoCollision")
    name = _kind(coll, known)
    tau_flow = float(flow.units.relaxation_parameter_lu)
    if name == "KBCCollision":
        # relaxes with the flow's tau (kbc_collision.py:97-99)
        q, d = int(flow.stencil.q), int(flow.stencil.d)
        if (d, q) not in ((2, 9), (3, 27)):
            raise AssertionError("KBC Collision is only implemented for D2Q9 and D3Q27")
        return NativeCollision(_lib.KBC, index, tau=tau_flow)
    if name == "TRTCollision":
        return NativeCollision(_lib.TRT, index, tau=float(coll.tau_plus),
                               tau_minus=float(coll.tau_minus))
    if name == "RegularizedCollision":
        # relaxes with the flow's tau (regularized_collision.py:17-20)
        return NativeCollision(_lib.REGULARIZED, index, tau=tau_flow)
    if name == "SmagorinskyCollision":
        return NativeCollision(_lib.SMAGORINSKY, index, tau=float(coll.tau),
                               force=_force_native(getattr(coll, "force", None)),
                               smagorinsky_constant=float(coll.constant))
    if name == "MRTCollision":
        tr = coll.transform
        kind = _kind(tr, _MRT_EQUILIBRIA)
        if kind is not None:
            eq = _MRT_EQUILIBRIA[kind]
        elif any("equilibrium" in k.__dict__ for k in type(tr).__mro__
                 if k.__name__ not in ("Transform", "object")):
            raise NotImplementedError(f"no GB300 kernel for the moment equilibrium of "
                                      f"{type(tr).__name__}")
        else:
            eq = _lib.MRT_EQ_GENERIC
        s = _as_np(coll.relaxation_parameters).astype(np.float64).reshape(-1)
        tables = np.concatenate([_as_np(tr.matrix).astype(np.float64).reshape(-1),
                                 _as_np(tr.inverse).astype(np.float64).reshape(-1), s])
        return NativeCollision(_lib.MRT, index, mrt_equilibrium=eq, mrt_tables=tables)
    if name == "BGKCollision":
        return NativeCollision(_lib.BGK, index, tau=float(coll.tau),
                               force=_force_native(getattr(coll, "force", None)))
    if name == "NoCollision":
        return NativeCollision(_lib.NO_COLLISION, index)
    raise NotImplementedError(f"no GB300 kernel for the collision {type(coll).__name__}")


def _outlet_axis(boundary):
    """(axis, sign) of an outlet from lettuce's plane index: -1 on the
    normal's axis for +1, 0 for -1, a full slice elsewhere
    (anti_bounce_back_outlet.py:46-57)"""
    idx = list(boundary.index)
    axes = [i for i, v in enumerate(idx) if not isinstance(v, slice)]
    if len(axes) != 1:
        raise ValueError(f"outlet index {idx} names no single plane")
    a = axes[0]
    return a, (1 if int(idx[a]) == -1 else -1)


def _boundary_native(b, flow, index: int, device, dtype) -> NativeBoundary:
    """lettuce/ext/_boundary/*.py: the operator and its parameters"""
    known = ("BounceBackBoundary", "EquilibriumBoundaryPU", "EquilibriumOutletP",
             "AntiBounceBackOutlet", "PartiallySaturatedBC")
    name = _kind(b, known)
    if name == "BounceBackBoundary":
        return NativeBoundary(_lib.SUB_BOUNCE_BACK, index)
    if name == "EquilibriumBoundaryPU":
        # equilibrium_boundary_pu.py:79-84: density from the pressure, both
        # converted to lattice units, broadcast over the mask
        rho = flow.units.convert_pressure_pu_to_density_lu(b.pressure)[0]
        u = flow.units.convert_velocity_to_lu(b.velocity)
        rho = torch.as_tensor(rho).to(device=device, dtype=dtype).contiguous()
        u = torch.as_tensor(u).to(device=device, dtype=dtype).contiguous()
        return NativeBoundary(_lib.SUB_EQUILIBRIUM_PU, index, rho=rho, u=u)
    if name == "EquilibriumOutletP":
        axis, sign = _outlet_axis(b)
        return NativeBoundary(_lib.SUB_EQUILIBRIUM_OUTLET_P, index, axis=axis, sign=sign,
                              params=(float(_as_np(b.rho_outlet).reshape(-1)[0]), 0.0))
    if name == "AntiBounceBackOutlet":
        axis, sign = _outlet_axis(b)
        return NativeBoundary(_lib.SUB_ANTI_BOUNCE_BACK, index, axis=axis, sign=sign)
    if name == "PartiallySaturatedBC":
        return NativeBoundary(_lib.SUB_PARTIALLY_SATURATED, index,
                              params=(float(b.tau), float(b.B)))
    raise NotImplementedError(f"no GB300 kernel for the boundary {type(b).__name__}")


def _patterns(strategy) -> List[int]:
    """lettuce's StreamingStrategy (lettuce/cuda_native/_default_code_gen.py:
    13-25) as launch patterns"""
    pre = bool(strategy.pre_streaming())
    post = bool(strategy.post_streaming())
    if pre and post:
        return [_lib.PULL, _lib.STREAM_ONLY]
    if post:
        return [_lib.PUSH]
    if pre:
        return [_lib.PULL]
    return [_lib.LOCAL]


@dataclass
class NativeStep:
    """the launch description of one lettuce step: the descriptor, its
    patterns, and the device tensors it points into (kept alive here)"""
    desc: _lib.StepDesc
    patterns: List[int]
    storage: int
    shape: tuple
    dtype: torch.dtype
    device: torch.device
    flags: Optional[torch.Tensor]
    no_stream_bits: Optional[torch.Tensor]
    natives: list
    keep: list = field(default_factory=list)
    status: Optional[torch.Tensor] = None


def native_step(simulation) -> NativeStep:
    """The descriptor of lettuce's step for ``simulation`` (a lettuce
    ``Simulation``, or any object with its attributes). Works on any
    device; launching needs CUDA (``native_invoke``)."""
    flow = simulation.flow
    f = flow.f
    if f.dtype == torch.float64:
        storage = _lib.F64
    elif f.dtype == torch.float32:
        storage = _lib.F32
    else:
        raise NotImplementedError(f"the GB300 kernels keep lettuce's populations in float32 or "
                                  f"float64; got {f.dtype} (16-bit storage is this package's "
                                  "shifted format, lettuce_gb300.Context(storage=...))")
    eq = getattr(flow, "equilibrium", None)
    if eq is not None and _kind(eq, ("QuadraticEquilibrium",
                                     "QuadraticEquilibriumLessMemory")) is None:
        raise NotImplementedError(f"no GB300 kernel for the equilibrium {type(eq).__name__}")
    sid = _stencil_id(flow.stencil)
    res = [int(n) for n in flow.resolution]
    device, dtype = f.device, f.dtype
    pre = list(simulation.pre_boundaries or [])
    post = list(simulation.post_boundaries or [])
    ci = int(simulation.collision_index)
    if ci != len(pre):
        raise ValueError(f"collision_index {ci} is not the number of pre-boundaries {len(pre)}")
    natives = [_boundary_native(b, flow, i, device, dtype) for i, b in enumerate(pre)]
    natives.append(_collision_native(simulation.collision, flow, ci))
    natives += [_boundary_native(b, flow, i, device, dtype)
                for i, b in enumerate(post, start=ci + 1)]
    flags = nsb = None
    ncm = getattr(simulation, "no_collision_mask", None)
    if ncm is not None:
        flags, nsb = pack_masks(torch.as_tensor(ncm), torch.as_tensor(simulation.no_streaming_mask),
                                e=_STENCILS[_kind(flow.stencil, _STENCILS)]().e)
    view = SimpleNamespace(stencil=SimpleNamespace(lgb_id=sid),
                           context=SimpleNamespace(storage=storage), resolution=res)
    desc, keep = _desc_for(view, natives, flags, nsb, ci)
    if nsb is not None:
        desc.options |= _lib.OPT_PUSH_GUARD
    keep += [n.rho for n in natives if isinstance(n, NativeBoundary) and n.rho is not None]
    keep += [n.u for n in natives if isinstance(n, NativeBoundary) and n.u is not None]
    step = NativeStep(desc=desc, patterns=_patterns(simulation.streaming_strategy),
                      storage=storage, shape=tuple([int(flow.stencil.q)] + res), dtype=dtype,
                      device=device, flags=flags, no_stream_bits=nsb, natives=natives, keep=keep)
    if device.type == "cuda":
        step.status = torch.zeros(1, dtype=torch.int32, device=device)
        desc.status = step.status.data_ptr()
    return step


def native_invoke(simulation):
    """lettuce's ``invoke(simulation)`` for this simulation on the GB300
    kernels: each call advances ``simulation.flow`` by one step on the
    current torch stream and swaps ``flow.f`` / ``flow.f_next``
    (lettuce/cuda_native/_template.py:35-40). ``invoke.status`` is the
    device status word (bit 0: a non-finite density was seen)."""
    step = native_step(simulation)
    if step.device.type != "cuda":
        raise RuntimeError("lettuce_gb300 steps on CUDA devices only; there is no CPU path "
                           "(the flow's populations are on the CPU)")
    _lib.load()
    desc = step.desc

    def invoke(sim, *_, **__):
        flow = sim.flow
        stream = torch.cuda.current_stream(step.device).cuda_stream
        for pattern in step.patterns:
            f, f_next = flow.f, flow.f_next
            for t in (f, f_next):
                if (t.dtype != step.dtype or t.device != step.device
                        or tuple(t.shape) != step.shape or not t.is_contiguous()):
                    raise RuntimeError(f"flow populations changed to {tuple(t.shape)} "
                                       f"{t.dtype} on {t.device}; rebuild the step with "
                                       "native_invoke(simulation)")
            desc.pattern = pattern
            desc.f_in = f.data_ptr()
            desc.f_out = f_next.data_ptr()
            _device.step(desc, stream)
            flow.f, flow.f_next = flow.f_next, flow.f

    invoke.step = step
    invoke.status = step.status
    return invoke


def install(simulation):
    """Replace the simulation's step by the GB300 kernels, as
    lettuce/_simulation.py:229 installs its generated kernel; returns the
    installed ``invoke``"""
    invoke = native_invoke(simulation)
    simulation._collide_and_stream = invoke
    return invoke
