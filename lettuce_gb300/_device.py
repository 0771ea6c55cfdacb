"""Thin wrappers that call the C ABI on torch tensors (device memory and the
current torch stream are PyTorch's; the arithmetic is the library's)."""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib

_scratch = {}


def _require_cuda(t: torch.Tensor, what: str):
    if not t.is_cuda:
        raise RuntimeError(f"{what}: lettuce_gb300 runs on CUDA tensors only "
                           f"(got a tensor on {t.device}); there is no CPU path")
    if not t.is_contiguous():
        raise RuntimeError(f"{what}: tensor must be contiguous")


def storage_of(dtype: torch.dtype) -> int:
    if dtype == torch.float64:
        return _lib.F64
    if dtype == torch.float32:
        return _lib.F32
    raise TypeError(f"no natural population storage for {dtype}")


def stream_of(t: torch.Tensor) -> int:
    return torch.cuda.current_stream(t.device).cuda_stream


def moments(stencil_id: int, storage: int, res: Sequence[int], f: torch.Tensor,
            aa_pending: bool, compute_dtype: torch.dtype):
    """(rho [1, *res], u [D, *res]) of a population field on the device"""
    _require_cuda(f, "moments")
    L = _lib.load()
    d = len(res)
    rho = torch.empty([1] + list(res), device=f.device, dtype=compute_dtype)
    u = torch.empty([d] + list(res), device=f.device, dtype=compute_dtype)
    r3 = _lib.i32x3(res)
    _lib.check(L.lgb_moments(stencil_id, storage, ctypes.cast(r3, ctypes.c_void_p),
                             f.data_ptr(), int(bool(aa_pending)), rho.data_ptr(),
                             u.data_ptr(), stream_of(f)), "lgb_moments")
    return rho, u


def scratch_for(device: torch.device) -> torch.Tensor:
    key = (device.type, device.index)
    buf = _scratch.get(key)
    if buf is None:
        n = _lib.load().lgb_reduce_scratch_bytes()
        buf = torch.empty(int(n), dtype=torch.uint8, device=device)
        _scratch[key] = buf
    return buf


def reduce(stencil_id: int, storage: int, res: Sequence[int], f: torch.Tensor,
           aa_pending: bool, lo: Optional[Sequence[int]] = None,
           hi: Optional[Sequence[int]] = None,
           mask: Optional[torch.Tensor] = None, out: Optional[torch.Tensor] = None
           ) -> torch.Tensor:
    """float64 [mass, 0.5*sum|u|^2, max|u|^2, non-finite cells, masked mass]
    as a device tensor (no host synchronisation)"""
    _require_cuda(f, "reduce")
    L = _lib.load()
    if out is None:
        out = torch.empty(_lib.REDUCE_FIELDS, dtype=torch.float64, device=f.device)
    r3 = _lib.i32x3(res)
    lo3 = _lib.i32x3(lo) if lo is not None else None
    hi3 = _lib.i32x3(hi) if hi is not None else None
    mptr = None
    if mask is not None:
        _require_cuda(mask, "reduce mask")
        assert mask.dtype == torch.uint8
        mptr = mask.data_ptr()
    scratch = scratch_for(f.device)
    _lib.check(L.lgb_reduce(stencil_id, storage, ctypes.cast(r3, ctypes.c_void_p),
                            f.data_ptr(), int(bool(aa_pending)),
                            ctypes.cast(lo3, ctypes.c_void_p) if lo3 is not None else None,
                            ctypes.cast(hi3, ctypes.c_void_p) if hi3 is not None else None,
                            mptr, out.data_ptr(), scratch.data_ptr(), stream_of(f)),
               "lgb_reduce")
    return out


def _broadcast_view(t: torch.Tensor, lead: int, res: Sequence[int]) -> torch.Tensor:
    """``t`` viewed as [lead, *res] with stride 0 on broadcast dimensions (a
    tensor without the leading dimension gets one)"""
    full = [lead] + list(res)
    if t.dim() < len(full):
        t = t.reshape([1] * (len(full) - t.dim()) + list(t.shape))
    return t.expand(full)


def equilibrium(stencil_id: int, storage: int, res: Sequence[int], rho: torch.Tensor,
                u: torch.Tensor, f: Optional[torch.Tensor] = None,
                moments: Optional[tuple] = None):
    """feq(rho, u) into ``f`` (storage format) and/or its moments into
    ``moments`` = (rho_out [*res], u_out [D, *res]) in the compute dtype;
    rho broadcastable to [1, *res], u to [D, *res], both on the device in
    the compute dtype"""
    L = _lib.load()
    d = len(res)
    rv = _broadcast_view(rho, 1, res)
    uv = _broadcast_view(u, d, res)
    for t, what in ((rv, "equilibrium density"), (uv, "equilibrium velocity")):
        if not t.is_cuda:
            raise RuntimeError(f"{what}: lettuce_gb300 runs on CUDA tensors only")
    rs = (ctypes.c_int64 * 3)(*(list(rv.stride()[1:]) + [0] * (3 - d)))
    us = (ctypes.c_int64 * 4)(*(list(uv.stride()) + [0] * (3 - d)))
    r3 = _lib.i32x3(res)
    fptr = None
    if f is not None:
        _require_cuda(f, "equilibrium output")
        fptr = f.data_ptr()
    rptr = uptr = None
    if moments is not None:
        for t in moments:
            _require_cuda(t, "equilibrium moments")
        rptr, uptr = moments[0].data_ptr(), moments[1].data_ptr()
    _lib.check(L.lgb_equilibrium(stencil_id, storage, ctypes.cast(r3, ctypes.c_void_p),
                                 rv.data_ptr(), ctypes.cast(rs, ctypes.c_void_p), uv.data_ptr(),
                                 ctypes.cast(us, ctypes.c_void_p), fptr, rptr, uptr,
                                 stream_of(rv)), "lgb_equilibrium")


def init_fneq(stencil_id: int, storage: int, res: Sequence[int], rho: torch.Tensor,
              u: torch.Tensor, tau: float, f: torch.Tensor):
    """f = feq(rho, u) - fneq (lettuce's initialize_f_neq) from contiguous
    rho [*res] / u [D, *res] in the compute dtype, into ``f`` (storage format)"""
    for t, what in ((rho, "density"), (u, "velocity"), (f, "population field")):
        _require_cuda(t, f"init_fneq {what}")
    L = _lib.load()
    r3 = _lib.i32x3(res)
    _lib.check(L.lgb_init_fneq(stencil_id, storage, ctypes.cast(r3, ctypes.c_void_p),
                               rho.data_ptr(), u.data_ptr(), float(tau), f.data_ptr(),
                               stream_of(f)), "lgb_init_fneq")


def enstrophy_lu(u: torch.Tensor) -> torch.Tensor:
    """float64 device tensor [1]: sum over cells of |curl u|^2 of a velocity
    field [D, *res] (D = 2 or 3, lattice units, dx = 1)"""
    _require_cuda(u, "enstrophy")
    if u.dtype not in (torch.float32, torch.float64):
        raise TypeError(f"enstrophy: velocity in float32 or float64, not {u.dtype}")
    L = _lib.load()
    d = u.shape[0]
    out = torch.empty(1, dtype=torch.float64, device=u.device)
    r3 = _lib.i32x3(list(u.shape[1:]))
    prec = _lib.F64 if u.dtype == torch.float64 else _lib.F32
    _lib.check(L.lgb_enstrophy(int(d), prec, ctypes.cast(r3, ctypes.c_void_p), u.data_ptr(),
                               out.data_ptr(), scratch_for(u.device).data_ptr(), stream_of(u)),
               "lgb_enstrophy")
    return out


def convert(stencil_id: int, src: torch.Tensor, src_storage: int, dst: torch.Tensor,
            dst_storage: int, n_cells: int):
    _require_cuda(src, "convert")
    _require_cuda(dst, "convert")
    L = _lib.load()
    _lib.check(L.lgb_convert(stencil_id, src_storage, src.data_ptr(), dst_storage,
                             dst.data_ptr(), int(n_cells), stream_of(src)), "lgb_convert")


def host_device_pointer(t: torch.Tensor) -> Optional[int]:
    """The device address of a page-locked host tensor's data, or None when
    ``t`` is not in page-locked, mapped host memory."""
    if t.device.type != "cpu" or not t.is_pinned():
        return None
    L = _lib.load()
    base = t.untyped_storage().data_ptr()
    out = ctypes.c_void_p()
    if L.lgb_host_pointer(ctypes.c_void_p(base), ctypes.byref(out)) != 0 or not out.value:
        return None
    return out.value + (t.data_ptr() - base)


def convert_ptr(stencil_id: int, src_ptr: int, src_storage: int, dst_ptr: int, dst_storage: int,
                n_cells: int, stream: int):
    """lgb_convert on raw addresses (device memory, or host memory through
    host_device_pointer)"""
    L = _lib.load()
    _lib.check(L.lgb_convert(stencil_id, src_storage, ctypes.c_void_p(src_ptr), dst_storage,
                             ctypes.c_void_p(dst_ptr), int(n_cells), stream), "lgb_convert")


def step(desc: _lib.StepDesc, stream: int):
    L = _lib.load()
    _lib.check(L.lgb_step(ctypes.byref(desc), stream), "lgb_step")


def new_desc(stencil_id: int, storage: int, res: Sequence[int]) -> _lib.StepDesc:
    d = _lib.StepDesc()
    d.abi_version = _lib.ABI_VERSION
    d.stencil = stencil_id
    d.storage = storage
    for k, v in enumerate(list(res) + [1] * (3 - len(res))):
        d.res[k] = int(v)
    d.tau = 1.0
    d.tau_minus = 1.0
    return d


def bcast_strides(t: torch.Tensor, full_shape: Sequence[int]) -> list:
    """element strides of ``t`` broadcast to ``full_shape`` (0 where t has
    size 1)"""
    assert t.dim() == len(full_shape), (tuple(t.shape), tuple(full_shape))
    out = []
    for i, n in enumerate(full_shape):
        if t.shape[i] == 1:
            out.append(0)
        elif t.shape[i] == n:
            out.append(int(t.stride(i)))
        else:
            raise ValueError(f"shape {tuple(t.shape)} does not broadcast to {tuple(full_shape)}")
    return out


def as_numpy_f64(t: torch.Tensor) -> np.ndarray:
    return t.detach().to(torch.float64).cpu().numpy()


def capture(device: torch.device, launch) -> "torch.cuda.CUDAGraph":
    """A CUDA graph of the launches ``launch(stream_handle)`` makes, captured
    on a side stream ordered after the current one. Unlike the
    ``torch.cuda.graph`` context manager this neither synchronises the
    device nor empties torch's allocator cache nor runs the garbage
    collector, so a re-capture (new field pointers) costs about as much as
    the launches themselves. The launches must not allocate memory."""
    g = torch.cuda.CUDAGraph()
    cur = torch.cuda.current_stream(device)
    side = torch.cuda.Stream(device)
    side.wait_stream(cur)
    with torch.cuda.device(device), torch.cuda.stream(side):
        g.capture_begin(capture_error_mode="thread_local")
        try:
            launch(side.cuda_stream)
        finally:
            g.capture_end()
    cur.wait_stream(side)
    return g
