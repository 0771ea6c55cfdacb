"""Flow state, equilibrium and the plugin ABCs.

Mirrors lettuce/_flow.py: ``Flow`` owns the population field ``f`` of shape
[Q, *resolution] (lettuce/_flow.py:81-95), its moments (:157-204), the
equilibrium/fneq initialisation (:127-143, :341-367) and the pickle
checkpoint (:258-268). The moments of a flow on a CUDA device come from the
library's moment kernel; the field itself lives in the context's population
storage (float32/float64, or shifted 16-bit).
"""
from __future__ import annotations

import pickle
import warnings
from abc import ABC, abstractmethod
from typing import List, Optional

import numpy as np
import torch

from . import _device, _lib
from ._native import NativeQuadraticEquilibrium
from ._stencil import TorchStencil

__all__ = ["Equilibrium", "QuadraticEquilibrium", "QuadraticEquilibriumLessMemory", "Boundary", "Flow",
           "torch_gradient", "initialize_f_neq"]


class Equilibrium(ABC):
    @abstractmethod
    def __call__(self, flow: "Flow", rho=None, u=None) -> torch.Tensor:
        ...

    @abstractmethod
    def native_available(self) -> bool:
        ...

    @abstractmethod
    def native_generator(self):
        ...


class QuadraticEquilibrium(Equilibrium):
    """w_q rho (1 + (2 e.u - u.u) / (2 cs^2) + (e.u)^2 / (2 cs^4))
    (lettuce/ext/_equilibrium/quadratic_equilibrium.py:11-24); evaluated with
    torch for initial and boundary fields, inlined in the step kernels."""

    def __call__(self, flow: "Flow", rho=None, u=None):
        rho = flow.rho() if rho is None else rho
        u = flow.u() if u is None else u
        e = flow.torch_stencil.e.to(u.dtype)
        w = flow.torch_stencil.w.to(u.dtype)
        cs2 = flow.torch_stencil.cs ** 2
        exu = torch.tensordot(e, u, dims=1)
        uxu = torch.einsum("d...,d...->...", u, u)
        inner = rho * ((2 * exu - uxu) / (2 * cs2) + 0.5 * (exu / cs2) ** 2 + 1)
        return torch.einsum("q,q...->q...", w, inner)

    def native_available(self) -> bool:
        return True

    def native_generator(self):
        return NativeQuadraticEquilibrium()


class QuadraticEquilibriumLessMemory(QuadraticEquilibrium):
    """lettuce's lower-memory form of the same quadratic equilibrium
    (lettuce/ext/_equilibrium/quadratic_equilibrium_less_memory.py:8-30,
    "does the same as the normal equilibrium"): here the same torch
    expression and the same step kernels."""


class Boundary(ABC):
    @abstractmethod
    def __call__(self, flow: "Flow"):
        ...

    @abstractmethod
    def make_no_collision_mask(self, shape: List[int], context) -> Optional[torch.Tensor]:
        ...

    @abstractmethod
    def make_no_streaming_mask(self, shape: List[int], context) -> Optional[torch.Tensor]:
        ...

    @abstractmethod
    def native_available(self) -> bool:
        ...

    @abstractmethod
    def native_generator(self, index: int):
        ...


def _weights_view(flow: "Flow", dtype) -> torch.Tensor:
    return flow.torch_stencil.w.to(dtype).view([-1] + [1] * flow.stencil.d)


class Flow(ABC):
    """Physical configuration and state of a simulation."""

    initialize_pressure: bool = False
    initialize_fneq: bool = False

    def __init__(self, context, resolution: List[int], units, stencil, equilibrium):
        self.context = context
        self.resolution = list(resolution)
        self.units = units
        self.stencil = stencil
        self.torch_stencil = TorchStencil(stencil, context)
        self.equilibrium = equilibrium
        self.i = 0
        self._f = torch.empty([stencil.q, *self.resolution], device=context.device,
                              dtype=context.storage_dtype)
        self._f_next = None
        self._aa_pending = False
        # a Simulation running POST_STREAMING as pull steps leaves the field
        # post-collision with its stream still to apply: this is then the
        # callable that applies it (see Simulation)
        self._stream_pending = None
        self.initialize()

    # -- boundaries ------------------------------------------------------
    @property
    def pre_boundaries(self) -> List["Boundary"]:
        return []

    @property
    def post_boundaries(self) -> List["Boundary"]:
        return self.boundaries

    @property
    def boundaries(self) -> List["Boundary"]:
        return []

    @abstractmethod
    def initial_pu(self):
        """initial solution in physical units"""

    def initialize(self):
        """equilibrium initialisation, plus the non-equilibrium part if
        ``initialize_fneq`` (lettuce/_flow.py:127-143). On a CUDA device with
        the quadratic equilibrium the populations come from the library's
        initialisation kernels (the equilibrium, then the non-equilibrium
        part from 6th-order differences of its velocity); elsewhere from the
        torch expressions."""
        initial_p, initial_u = self.initial_pu()
        initial_rho = self.context.convert_to_tensor(
            self.units.convert_pressure_pu_to_density_lu(initial_p))
        initial_u = self.context.convert_to_tensor(
            self.units.convert_velocity_to_lu(initial_u))
        if self._initialize_on_device(initial_rho, initial_u):
            return
        self.f = self.equilibrium(self, rho=initial_rho, u=initial_u)
        if self.initialize_fneq:
            self.f = initialize_f_neq(self)

    def _device_equilibrium(self) -> bool:
        """the flow's equilibrium is the one the kernels evaluate"""
        return (self.context.device.type == "cuda"
                and type(self.equilibrium) in (QuadraticEquilibrium,
                                               QuadraticEquilibriumLessMemory))

    def _initialize_on_device(self, rho: torch.Tensor, u: torch.Tensor) -> bool:
        if not self._device_equilibrium() or (self.initialize_fneq and self.stencil.d < 2):
            return False
        ctx = self.context
        res = list(self.resolution)
        rho = rho.to(device=ctx.device, dtype=ctx.dtype)
        u = u.to(device=ctx.device, dtype=ctx.dtype)
        out = torch.empty([self.stencil.q] + res, dtype=ctx.storage_dtype, device=ctx.device)
        sid = self.stencil.lgb_id
        if not self.initialize_fneq:
            _device.equilibrium(sid, ctx.storage, res, rho, u, f=out)
        else:
            # lettuce reads rho and u back from the equilibrium it has just
            # set, then adds the non-equilibrium part (lettuce/_flow.py:341-367)
            r1 = torch.empty(res, dtype=ctx.dtype, device=ctx.device)
            u1 = torch.empty([self.stencil.d] + res, dtype=ctx.dtype, device=ctx.device)
            _device.equilibrium(sid, ctx.storage, res, rho, u, moments=(r1, u1))
            _device.init_fneq(sid, ctx.storage, res, r1, u1,
                              self.units.relaxation_parameter_lu, out)
        self._f = out
        self._aa_pending = False
        self._stream_pending = None
        return True

    # -- the population field ---------------------------------------------
    @property
    def f(self) -> torch.Tensor:
        """populations [Q, *resolution] in the context dtype. For float32 /
        float64 storage this is the stored tensor itself; for the shifted
        16-bit formats it is a decoded float32 copy (assign ``flow.f = ...``
        to write)."""
        self._settle()
        if self.context.shifted:
            return self._f.to(torch.float32) + _weights_view(self, torch.float32)
        return self._f

    @f.setter
    def f(self, value: torch.Tensor):
        value = torch.as_tensor(value)
        self._aa_pending = False
        self._stream_pending = None
        if self._upload_pinned(value):
            return
        if self.context.shifted:
            v = value.to(device=self.context.device, dtype=torch.float32)
            self._f = (v - _weights_view(self, torch.float32)).to(
                self.context.storage_dtype).contiguous()
        else:
            if value.dtype != self.context.dtype or value.device != self.context.device:
                value = value.to(device=self.context.device, dtype=self.context.dtype)
            self._f = value if value.is_contiguous() else value.contiguous()

    # -- host transfers ----------------------------------------------------
    def _host_transfer_ok(self, t: torch.Tensor) -> bool:
        return (self.context.device.type == "cuda" and t.device.type == "cpu"
                and t.dtype == self.context.dtype and t.is_contiguous()
                and list(t.shape) == [self.stencil.q] + list(self.resolution))

    def _upload_pinned(self, value: torch.Tensor) -> bool:
        """a page-locked host field in the context dtype goes to the device
        through one conversion kernel reading host memory (storage format
        applied on the way); False when that path does not apply"""
        if not self._host_transfer_ok(value):
            return False
        ptr = _device.host_device_pointer(value)
        if ptr is None:
            return False
        shape = [self.stencil.q] + list(self.resolution)
        spare = self._f_next
        if (spare is not None and list(spare.shape) == shape
                and spare.dtype == self.context.storage_dtype
                and spare.data_ptr() != self._f.data_ptr()):
            # the second field is scratch between steps: upload into it and
            # keep the pair of buffers (captured step graphs stay valid)
            out, self._f_next = spare, self._f
        else:
            out = torch.empty(shape, dtype=self.context.storage_dtype,
                              device=self.context.device)
        _device.convert_ptr(self.stencil.lgb_id, ptr, _device.storage_of(value.dtype),
                            out.data_ptr(), self.context.storage, out[0].numel(),
                            torch.cuda.current_stream(self.context.device).cuda_stream)
        self._f = out
        return True

    def download(self, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """The populations in the context dtype, written into ``out`` (a host
        tensor; allocated page-locked when None). Into page-locked host memory
        one conversion kernel writes them over the host link, asynchronously
        on the current stream (synchronise before reading ``out``); any other
        ``out`` takes a torch copy."""
        shape = [self.stencil.q] + list(self.resolution)
        if out is None:
            out = torch.empty(shape, dtype=self.context.dtype,
                              pin_memory=self.context.device.type == "cuda")
        if self._host_transfer_ok(out):
            ptr = _device.host_device_pointer(out)
            if ptr is not None:
                self._settle()
                _device.convert_ptr(self.stencil.lgb_id, self._f.data_ptr(), self.context.storage,
                                    ptr, _device.storage_of(out.dtype), out[0].numel(),
                                    torch.cuda.current_stream(self.context.device).cuda_stream)
                return out
        out.copy_(self.f, non_blocking=True)
        return out

    @property
    def f_raw(self) -> torch.Tensor:
        """the stored population tensor (storage dtype, possibly AA-pending)"""
        return self._f

    @property
    def f_next(self) -> torch.Tensor:
        if self._f_next is None or self._f_next.shape != self._f.shape \
                or self._f_next.dtype != self._f.dtype:
            self._f_next = torch.empty_like(self._f)
        return self._f_next

    @f_next.setter
    def f_next(self, value):
        self._f_next = value

    def _unpack_aa(self):
        """materialise the natural layout of a field left by an AA even step"""
        out = torch.empty_like(self._f)
        d = _device.new_desc(self.stencil.lgb_id, self.context.storage, self.resolution)
        d.pattern = _lib.AA_UNPACK
        d.collision = _lib.NO_COLLISION
        d.f_in = self._f.data_ptr()
        d.f_out = out.data_ptr()
        _device.step(d, _device.stream_of(self._f))
        self._f = out
        self._aa_pending = False

    def _settle(self):
        """bring the stored field to lettuce's layout and time level: apply
        a pending stream, or unpack an AA layout"""
        if self._stream_pending is not None:
            apply, self._stream_pending = self._stream_pending, None
            apply()
        if self._aa_pending:
            self._unpack_aa()

    # -- moments (lettuce/_flow.py:157-204) ---------------------------------
    def _own_moments(self):
        if self._stream_pending is not None:
            self._settle()
        return _device.moments(self.stencil.lgb_id, self.context.storage, self.resolution,
                               self._f, self._aa_pending, self.context.dtype)

    def _moments_of(self, f: torch.Tensor):
        if f.is_cuda and f.dtype in (torch.float32, torch.float64):
            return _device.moments(self.stencil.lgb_id, _device.storage_of(f.dtype),
                                   self.resolution, f.contiguous(), False, f.dtype)
        # host-side tensors (set-up on a CPU context)
        e = self.torch_stencil.e.to(device=f.device, dtype=f.dtype)
        rho = torch.sum(f, dim=0)[None, ...]
        j = torch.einsum("qd,q...->d...", e, f)
        return rho, j / rho

    def rho(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        """density [1, *resolution]"""
        if f is None and self.context.device.type == "cuda":
            return self._own_moments()[0]
        return self._moments_of(self.f if f is None else f)[0]

    def j(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        """momentum [D, *resolution]"""
        rho, u = (self._own_moments() if f is None and self.context.device.type == "cuda"
                  else self._moments_of(self.f if f is None else f))
        return rho * u

    def u(self, f: Optional[torch.Tensor] = None, rho=None, acceleration=None) -> torch.Tensor:
        """velocity [D, *resolution]; ``acceleration`` adds the forcing
        correction a / (2 rho) (lettuce/_flow.py:178-193)"""
        if f is None and self.context.device.type == "cuda":
            r, v = self._own_moments()
        else:
            r, v = self._moments_of(self.f if f is None else f)
        if rho is not None:
            v = v * r / rho
            r = rho
        if acceleration is not None:
            if len(acceleration.shape) == 1:
                acceleration = acceleration[(...,) + (None,) * self.stencil.d]
            v = v + acceleration / (2 * r)
        return v

    @property
    def velocity(self):
        return self.u()

    @property
    def rho_pu(self):
        return self.units.convert_density_to_pu(self.rho())

    @property
    def p_pu(self):
        return self.units.convert_density_lu_to_pressure_pu(self.rho())

    @property
    def u_pu(self):
        return self.units.convert_velocity_to_pu(self.u())

    def incompressible_energy(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        """0.5 |u|^2 per cell"""
        u = self.u(f)
        return 0.5 * torch.einsum("d...,d...->...", u, u)

    def entropy(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        f = self.f if f is None else f
        w = self.torch_stencil.w.to(f.dtype)
        f_log = -torch.log(torch.einsum("q...,q->q...", f, 1 / w))
        return torch.einsum("q...,q...->...", f, f_log)

    def pseudo_entropy_global(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        f = self.f if f is None else f
        w = self.torch_stencil.w.to(f.dtype)
        f_w = torch.einsum("q...,q->q...", f, 1 / w)
        return self.rho(f) - torch.einsum("q...,q...->...", f, f_w)

    def pseudo_entropy_local(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        f = self.f if f is None else f
        f_feq = f / self.equilibrium(self, self.rho(f), self.u(f))
        return self.rho(f) - torch.einsum("q...,q...->...", f, f_feq)

    def shear_tensor(self, f: Optional[torch.Tensor] = None) -> torch.Tensor:
        f = self.f if f is None else f
        e = self.torch_stencil.e.to(f.dtype)
        shear = torch.einsum("qa,qb->qab", e, e)
        return torch.einsum("q...,qab->ab...", f, shear)

    # -- checkpoint (lettuce/_flow.py:258-268) ----------------------------
    def dump(self, filename):
        with open(filename, "wb") as fh:
            pickle.dump(self.context.convert_to_ndarray(self.f), fh)

    def load(self, filename):
        with open(filename, "rb") as fh:
            self.f = self.context.convert_to_tensor(pickle.load(fh), dtype=self.context.dtype)
        self._f_next = None


def torch_gradient(f: torch.Tensor, dx=1, order=2) -> torch.Tensor:
    """First derivatives of a periodic field by central finite differences of
    order 2, 4 or 6 (Fornberg 1988 weights; the same operator as
    lettuce/util/utility.py:37-99). Returns [ndim, *f.shape]."""
    weights = {2: [-1 / 2, 1 / 2],
               4: [1 / 12, -2 / 3, 2 / 3, -1 / 12],
               6: [-1 / 60, 3 / 20, -3 / 4, 3 / 4, -3 / 20, 1 / 60]}
    shifts = {2: [1, -1], 4: [2, 1, -1, -2], 6: [3, 2, 1, -1, -2, -3]}
    if order not in weights:
        raise ValueError(f"order {order} not in (2, 4, 6)")
    dim = f.ndim
    if dim not in (2, 3):
        raise ValueError("torch_gradient works on 2-D and 3-D fields")
    out = torch.empty([dim] + list(f.shape), dtype=f.dtype, device=f.device)
    with torch.no_grad():
        for i in range(dim):
            acc = torch.zeros_like(f)
            for wgt, s in zip(weights[order], shifts[order]):
                acc = acc + wgt * torch.roll(f, shifts=s, dims=i)
            out[i] = acc * (1.0 / dx)
    return out


def initialize_f_neq(flow: Flow) -> torch.Tensor:
    """feq - fneq with the first-order non-equilibrium part
    fneq_i = w_i tau rho S_ab Q_iab / cs^2, Q_iab = e_ia e_ib - cs^2 delta_ab,
    S_ab = d_b u_a by 6th-order differences (Krueger et al. 2017; the same
    initialisation as lettuce/_flow.py:341-367). On a CUDA device with the
    quadratic equilibrium: the moment kernel and the library's fneq kernel."""
    if flow._device_equilibrium() and flow.stencil.d >= 2:
        rho, u = flow._own_moments()
        out = flow.context.empty_tensor([flow.stencil.q] + list(flow.resolution))
        _device.init_fneq(flow.stencil.lgb_id, _device.storage_of(out.dtype), flow.resolution,
                          rho.contiguous(), u.contiguous(), flow.units.relaxation_parameter_lu,
                          out)
        return out
    f = flow.f
    rho = flow.rho(f)
    u = flow.u(f)
    grads = [torch_gradient(u[a], dx=1, order=6)[None, ...] for a in range(flow.stencil.d)]
    S = torch.cat(grads)
    cs = flow.torch_stencil.cs
    e = flow.torch_stencil.e.to(u.dtype)
    w = flow.torch_stencil.w.to(u.dtype)
    pi1 = 1.0 * flow.units.relaxation_parameter_lu * rho * S / cs ** 2
    # the identity term is formed in torch's default dtype (float32), so
    # cs^2 enters rounded to float32 exactly as in lettuce/_flow.py:358-360
    Q = (torch.einsum("ia,ib->iab", e, e)
         - torch.eye(flow.stencil.d, device=e.device) * cs ** 2)
    pi1_q = torch.einsum("ab...,iab->i...", pi1, Q)
    fneq = torch.einsum("i,i...->i...", w, pi1_q)
    feq = flow.equilibrium(flow, rho, u)
    return feq - fneq
