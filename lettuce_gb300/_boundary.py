"""Boundary conditions with lettuce's constructors, masks and plugin hooks.

* BounceBackBoundary  -- lettuce/ext/_boundary/bounce_back_boundary.py:10-32
* EquilibriumBoundaryPU -- lettuce/ext/_boundary/equilibrium_boundary_pu.py:15-98
* AntiBounceBackOutlet -- lettuce/ext/_boundary/anti_bounce_back_outlet.py:13-109
* EquilibriumOutletP -- lettuce/ext/_boundary/equilibrium_outlet_p.py:12-91
* PartiallySaturatedBC -- lettuce/ext/_boundary/partially_saturated_boundary.py:6-51
* HalfwayBounceBackBoundary, LinearInterpolatedBounceBackBoundary,
  FullwayBounceBackBoundary, SolidBoundaryData -- lettuce's example project
  examples/advanced_projects/efficient_bounce_back_obstacle/boundary/
  halfway_bounce_back_boundary.py:10-254,
  linear_interpolated_bounce_back_boundary.py:9-212,
  fullway_bounce_back_boundary.py:9-185 and solid_boundary_data.py:7-14;
  post-streaming boundaries, run by ``EbbSimulation``

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
           "EquilibriumOutletP", "PartiallySaturatedBC", "SolidBoundaryData",
           "HalfwayBounceBackBoundary", "LinearInterpolatedBounceBackBoundary",
           "FullwayBounceBackBoundary", "hwbb_links", "fwbb_links"]


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


class SolidBoundaryData(dict):
    """The solid description of the example project's bounce-back boundaries
    (solid_boundary_data.py:7-14): ``solid_mask`` and, optionally, the link
    lists ``f_index_lt`` / ``f_index_gt`` (rows q, x, y[, z]; q points from
    the fluid cell into the solid) with their wall distances ``d_lt`` /
    ``d_gt``. Attributes are set by the caller."""


def _to_numpy_bool(m) -> np.ndarray:
    if isinstance(m, torch.Tensor):
        return m.detach().cpu().numpy().astype(bool)
    return np.asarray(m, dtype=bool)


def hwbb_links(e, opposite, mask, global_solid_mask=None, periodicity=None) -> np.ndarray:
    """The link list of the halfway bounce-back's neighbour search
    (halfway_bounce_back_boundary.py:70-161), rows (q, x, y[, z]) in its
    order: for every solid cell p of ``mask`` (``np.where`` order) and every
    velocity i, the neighbour c = p + e_i. Along an axis marked periodic c
    wraps around; along the others a c past the upper end drops the link,
    and c = -1 is kept as written (Python indexing reads the last cell
    there, so the link acts on that cell). A neighbour that is solid neither
    in ``mask`` nor in ``global_solid_mask`` (default: ``mask``) gives the
    link (opposite[i], c)."""
    mask = _to_numpy_bool(mask)
    gmask = mask if global_solid_mask is None else _to_numpy_bool(global_solid_mask)
    return _neighbour_links(e, opposite, mask, gmask, periodicity, at_solid=False)


def fwbb_links(e, opposite, mask, global_solid_mask=None, periodicity=None) -> np.ndarray:
    """The link list of the post-streaming full-way bounce-back's search
    (fullway_bounce_back_boundary.py:47-131), rows (q, x, y[, z]) in its
    order: the same neighbours c = p + e_i of the solid cells p as
    ``hwbb_links``; a neighbour that is neither in ``mask`` nor in the
    other solids of ``global_solid_mask`` (default: none) gives the link
    (opposite[i], p), the population that streamed into the solid cell."""
    mask = _to_numpy_bool(mask)
    other = np.zeros_like(mask) if global_solid_mask is None else \
        (_to_numpy_bool(global_solid_mask) & ~mask)
    return _neighbour_links(e, opposite, mask, mask | other, periodicity, at_solid=True)


def _neighbour_links(e, opposite, mask, gmask, periodicity, at_solid):
    e = np.asarray(e, dtype=np.int64)
    opp = np.asarray(opposite, dtype=np.int64)
    dims = mask.ndim
    if periodicity is None:
        periodicity = (False,) * dims
    shape = np.array(mask.shape, dtype=np.int64)
    p = np.stack(np.nonzero(mask), axis=1).astype(np.int64)          # [P, D]
    c = p[:, None, :] + e[None, :, :dims]                            # [P, Q, D]
    ok = np.ones(c.shape[:2], dtype=bool)
    for k in range(dims):
        if periodicity[k]:
            # the search's border shift: only -1 and n occur (|e| <= 1)
            c[..., k] = np.where(c[..., k] < 0, c[..., k] + shape[k],
                                 np.where(c[..., k] >= shape[k], c[..., k] - shape[k], c[..., k]))
        else:
            ok &= c[..., k] < shape[k]
    wrapped = np.where(c < 0, c + shape, c)
    wrapped = np.where(ok[..., None], wrapped, 0)
    idx = tuple(wrapped[..., k] for k in range(dims))
    ok &= ~mask[idx] & ~gmask[idx]
    q = np.broadcast_to(opp[None, :], ok.shape)
    at = np.broadcast_to(p[:, None, :], c.shape) if at_solid else c
    rows = np.concatenate([q[..., None], at], axis=-1)[ok]
    return rows.reshape(-1, dims + 1).astype(np.int64)


class HalfwayBounceBackBoundary(Boundary):
    """Halfway bounce-back with momentum exchange (the example project's
    HWBB, halfway_bounce_back_boundary.py:10-254). The solid cells neither
    collide nor stream; after each step's stream, every fluid cell x next to
    the solid takes for population opp(q) its own post-collision value of
    population q, for each link q pointing into the solid. With
    ``calc_force`` the momentum exchange 2 sum f*_q(x) e_q of the step's
    links (lattice units) is kept as ``force_sum``.

    The bounce runs inside the step kernel's pull (``EbbSimulation``); the
    links are those of ``solid_boundary_data.f_index_lt`` /
    ``f_index_gt`` when given, else of the neighbour search of
    ``hwbb_links``."""

    def __init__(self, context, flow, solid_boundary_data, global_solid_mask=None,
                 periodicity=None, calc_force: bool = False):
        self.context = context
        self.flow = flow
        self.mask = _to_numpy_bool(solid_boundary_data.solid_mask)
        st = flow.stencil
        if periodicity is None:
            periodicity = (False, False, False if st.d == 3 else None)
        lists = [np.asarray(getattr(solid_boundary_data, a)) for a in ("f_index_lt", "f_index_gt")
                 if hasattr(solid_boundary_data, a)]
        lists = [a.reshape(-1, st.d + 1) for a in lists if a.size]
        if lists:
            links = np.concatenate(lists, axis=0).astype(np.int64)
        else:
            links = hwbb_links(st.e, st.opposite, self.mask, global_solid_mask,
                               tuple(periodicity)[:st.d])
        self.f_index = torch.as_tensor(links, dtype=torch.int64, device=context.device)
        self.calc_force = bool(calc_force)
        self._force = None
        if self.calc_force:
            self._force = torch.zeros(3, dtype=torch.float64, device=context.device)

    @property
    def force_sum(self) -> torch.Tensor:
        """momentum-exchange force of the last step's links, [D], context
        dtype (lattice units); reading it applies a pending stream"""
        if self._force is None:
            raise AttributeError("force_sum needs calc_force=True")
        self.flow._settle()
        return self._force[:self.flow.stencil.d].to(self.context.dtype)

    def link_rows(self):
        """(link rows q, x, y[, z] as int64 [K, 1 + D], wall distances
        float64 [K]: -1, the halfway links)"""
        rows = self.f_index.detach().cpu().numpy().astype(np.int64)
        return rows, np.full(len(rows), -1.0)

    def __call__(self, flow):
        raise RuntimeError("the halfway bounce-back runs inside the step of an EbbSimulation")

    def make_no_collision_mask(self, shape: List[int], context) -> torch.Tensor:
        return torch.as_tensor(self.mask, device=context.device)

    def make_no_streaming_mask(self, shape: List[int], context) -> torch.Tensor:
        return torch.as_tensor(self.mask, device=context.device)

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        # the solid cells run no substep; the links travel as bits
        return NativeBoundary(_lib.SUB_NONE, index)


class LinearInterpolatedBounceBackBoundary(Boundary):
    """Linear interpolated bounce-back (Bouzidi et al. 2001; the example
    project's IBB1, linear_interpolated_bounce_back_boundary.py:9-212) with
    momentum exchange. The links and wall distances come from the solid
    boundary data: ``f_index_lt`` / ``d_lt`` (d < 1/2) and ``f_index_gt`` /
    ``d_gt``, rows q, x, y[, z] with q pointing from the fluid cell into the
    solid. After each step's stream the fluid cell x takes for population
    opp(q)
      d < 1/2:  2 d f*_q(x) + (1 - 2 d) f_q(x)   (f_q(x) the streamed value)
      d >= 1/2: f*_q(x) / (2 d) + (1 - 1 / (2 d)) f*_{opp(q)}(x),
    f* the post-collision populations. With ``calc_force`` the momentum
    exchange sum (f*_q(x) + f_opp(q)(x)) e_q over the links is kept as
    ``force_sum``. The solid cells neither collide nor stream. The
    interpolation runs as a pass over the links before each pulling step
    kernel, which reads the bounced values (``EbbSimulation``)."""

    def __init__(self, context, flow, solid_boundary_data, calc_force: bool = False):
        self.context = context
        self.flow = flow
        self.mask = _to_numpy_bool(solid_boundary_data.solid_mask)
        d1 = flow.stencil.d + 1
        self.f_index_lt = torch.as_tensor(
            np.asarray(solid_boundary_data.f_index_lt, dtype=np.int64).reshape(-1, d1),
            device=context.device)
        self.f_index_gt = torch.as_tensor(
            np.asarray(solid_boundary_data.f_index_gt, dtype=np.int64).reshape(-1, d1),
            device=context.device)
        self.d_lt = context.convert_to_tensor(np.asarray(solid_boundary_data.d_lt).ravel())
        self.d_gt = context.convert_to_tensor(np.asarray(solid_boundary_data.d_gt).ravel())
        if len(self.d_lt) != len(self.f_index_lt) or len(self.d_gt) != len(self.f_index_gt):
            raise ValueError("one wall distance per link")
        self.calc_force = bool(calc_force)
        self._force = None
        if self.calc_force:
            self._force = torch.zeros(3, dtype=torch.float64, device=context.device)

    @property
    def force_sum(self) -> torch.Tensor:
        """momentum-exchange force of the last step's links, [D], context
        dtype (lattice units); reading it applies a pending stream"""
        if self._force is None:
            raise AttributeError("force_sum needs calc_force=True")
        self.flow._settle()
        return self._force[:self.flow.stencil.d].to(self.context.dtype)

    def link_rows(self):
        """(link rows q, x, y[, z] as int64 [K, 1 + D], wall distances
        float64 [K]) in the order lt, gt; the distances as the context
        dtype holds them"""
        rows = np.concatenate([self.f_index_lt.detach().cpu().numpy(),
                               self.f_index_gt.detach().cpu().numpy()]).astype(np.int64)
        dist = np.concatenate([self.d_lt.detach().cpu().double().numpy(),
                               self.d_gt.detach().cpu().double().numpy()])
        if np.any(dist < 0):
            raise ValueError("wall distances must be >= 0")
        return rows, dist

    def __call__(self, flow):
        raise RuntimeError("the interpolated bounce-back runs inside the step of an "
                           "EbbSimulation")

    def make_no_collision_mask(self, shape: List[int], context) -> torch.Tensor:
        return torch.as_tensor(self.mask, device=context.device)

    def make_no_streaming_mask(self, shape: List[int], context) -> torch.Tensor:
        return torch.as_tensor(self.mask, device=context.device)

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        return NativeBoundary(_lib.SUB_NONE, index)


class FullwayBounceBackBoundary(Boundary):
    """The example project's post-streaming full-way bounce-back
    (fullway_bounce_back_boundary.py:9-185), with momentum exchange. Its
    solid cells do not collide but do stream; after each step's stream the
    solid cell p sets population opp(q) to the population q that streamed
    in from a fluid neighbour, for each link (q, p) of ``fwbb_links``. With
    ``calc_force`` the momentum exchange 2 sum f_q(p) e_q over the links
    (f_q(p) the streamed value) is kept as ``force_sum``. Runs inside the
    step kernel's pull (``EbbSimulation``), as links of distance 0 of the
    interpolated bounce-back's table, whose value is the streamed one. Not
    lettuce's own ``BounceBackBoundary``, which replaces the collision."""

    def __init__(self, context, flow, mask, global_solid_mask=None, periodicity=None,
                 calc_force: bool = False):
        self.context = context
        self.flow = flow
        self.mask = _to_numpy_bool(mask)
        st = flow.stencil
        if periodicity is None:
            periodicity = (False, False, False if st.d == 3 else None)
        rows = fwbb_links(st.e, st.opposite, self.mask, global_solid_mask,
                          tuple(periodicity)[:st.d])
        self.f_index_fwbb = torch.as_tensor(rows, dtype=torch.int64, device=context.device)
        self.calc_force = bool(calc_force)
        self._force = None
        if self.calc_force:
            self._force = torch.zeros(3, dtype=torch.float64, device=context.device)

    @property
    def force_sum(self) -> torch.Tensor:
        """momentum-exchange force of the last step's links, [D], context
        dtype (lattice units); reading it applies a pending stream"""
        if self._force is None:
            raise AttributeError("force_sum needs calc_force=True")
        self.flow._settle()
        return self._force[:self.flow.stencil.d].to(self.context.dtype)

    def link_rows(self):
        """(link rows q, x, y[, z] at the solid cells as int64 [K, 1 + D],
        wall distances 0: the bounced value is the streamed one)"""
        rows = self.f_index_fwbb.detach().cpu().numpy().astype(np.int64)
        return rows, np.zeros(len(rows))

    def __call__(self, flow):
        raise RuntimeError("the post-streaming full-way bounce-back runs inside the step of "
                           "an EbbSimulation")

    def make_no_collision_mask(self, shape: List[int], context) -> torch.Tensor:
        return torch.as_tensor(self.mask, device=context.device)

    def make_no_streaming_mask(self, shape: List[int], context):
        return None

    def native_available(self) -> bool:
        return True

    def native_generator(self, index: int) -> NativeBoundary:
        return NativeBoundary(_lib.SUB_NONE, index)
