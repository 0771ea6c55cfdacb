"""Device, dtype and population storage of a simulation.

Mirrors lettuce's ``Context`` (lettuce/_context.py:9-122): the same
constructor arguments and tensor factories, and the same placements (a
contradictory device / use_native pair raises AssertionError, as in lettuce). One addition: ``storage``
selects the population storage format of the GB300 kernels:

* ``None`` -- the population field is stored in ``dtype`` (float32/float64);
* ``"fp16_shifted"`` / ``"bf16_shifted"`` -- 16-bit storage of ``f - w`` with
  float32 collision arithmetic. ``dtype=torch.float16`` selects
  ``"fp16_shifted"`` (lettuce's float16 context computes in float16; this
  library keeps float16 for storage only and computes in float32).

A CPU context is accepted for host-side set-up (flows, masks, unit
conversion); stepping requires a CUDA device -- there is no CPU path.
"""
from __future__ import annotations

from typing import List, Optional, Union

import numpy as np
import torch

from . import _lib

__all__ = ["Context"]

_STORAGE = {
    None: None,
    "fp16_shifted": _lib.F16_SHIFTED,
    "bf16_shifted": _lib.BF16_SHIFTED,
}


def _need(ok: bool, message: str):
    """lettuce signals a contradictory context with AssertionError; raise
    the same type (explicitly, so that ``python -O`` keeps the check)"""
    if not ok:
        raise AssertionError(message)


def _placement(device, use_native):
    """(torch.device, use_native) for the constructor's arguments.

    ============  ==========  =========================================
    device        use_native  result
    ============  ==========  =========================================
    None          None        cuda:0 and native if torch sees a GPU,
                              else cpu without native
    None          True/False  cuda:0; True needs a visible GPU
    cuda[:k]      any         needs a visible GPU; native unless False
    cpu           None/False  cpu, not native
    cpu           True        refused
    other         any         refused
    ============  ==========  =========================================
    """
    gpu = torch.cuda.is_available()
    if device is None:
        if use_native is None:
            return torch.device("cuda:0" if gpu else "cpu"), gpu
        _need(gpu or not use_native,
              "use_native=True asks for the GPU kernels, but torch sees no CUDA device")
        return torch.device("cuda:0"), bool(use_native)
    kind = str(device)
    if "cuda" in kind:
        _need(gpu, f"device {kind!r} was requested, but torch sees no CUDA device")
        return torch.device(device), True if use_native is None else bool(use_native)
    _need("cpu" in kind, f"device {kind!r}: lettuce_gb300 places flows on 'cpu' (set-up "
                         "only) or on a 'cuda' device")
    _need(not use_native, "use_native=True runs the GPU kernels and cannot be combined "
                          "with a cpu device")
    return torch.device(device), False


def _is_mask_dtype(array) -> bool:
    """boolean and uint8 arrays / tensors keep an integer type when they are
    converted (lettuce turns masks into uint8, not into the float dtype)"""
    dt = getattr(array, "dtype", None)
    if dt is None:
        return False
    if isinstance(dt, torch.dtype):
        return dt in (torch.bool, torch.uint8)
    try:
        return np.dtype(dt) in (np.dtype(np.bool_), np.dtype(np.uint8))
    except TypeError:
        return False


class Context:
    def __init__(self, device: Optional[Union[torch.device, str]] = None,
                 dtype: Optional[torch.dtype] = None,
                 use_native: Optional[bool] = None,
                 storage: Optional[str] = None):
        self.device, self.use_native = _placement(device, use_native)
        dtype = dtype or torch.float32
        _need(dtype in (torch.float16, torch.bfloat16, torch.float32, torch.float64),
              f"populations are float16, bfloat16, float32 or float64, not {dtype}")
        if storage not in _STORAGE:
            raise ValueError(f"unknown population storage {storage!r}; "
                             f"choose one of {[k for k in _STORAGE if k]}")
        # a 16-bit dtype means 16-bit storage with float32 arithmetic
        storage = storage or {torch.float16: "fp16_shifted",
                              torch.bfloat16: "bf16_shifted"}.get(dtype)
        self.storage_name = storage
        if storage is None:
            self.dtype = dtype
            self.storage = _lib.F64 if dtype == torch.float64 else _lib.F32
        else:
            self.dtype = torch.float32
            self.storage = _STORAGE[storage]

    @property
    def storage_dtype(self) -> torch.dtype:
        return {_lib.F64: torch.float64, _lib.F32: torch.float32,
                _lib.F16_SHIFTED: torch.float16,
                _lib.BF16_SHIFTED: torch.bfloat16}[self.storage]

    @property
    def shifted(self) -> bool:
        return self.storage in (_lib.F16_SHIFTED, _lib.BF16_SHIFTED)

    def synchronize(self):
        if self.device.type == "cuda":
            torch.cuda.synchronize(self.device)

    def empty_tensor(self, size: Union[List[int], torch.Size], *args,
                     dtype=None, **kwargs) -> torch.Tensor:
        return torch.empty(size, *args, **kwargs, device=self.device,
                           dtype=(dtype or self.dtype))

    def zero_tensor(self, size, *args, dtype=None, **kwargs) -> torch.Tensor:
        return torch.zeros(size, *args, **kwargs, device=self.device,
                           dtype=(dtype or self.dtype))

    def full_tensor(self, size, value, *args, dtype=None, **kwargs) -> torch.Tensor:
        return torch.full(size, value, *args, **kwargs, device=self.device,
                          dtype=(dtype or self.dtype))

    def one_tensor(self, size, *args, dtype=None, **kwargs) -> torch.Tensor:
        return torch.ones(size, *args, **kwargs, device=self.device,
                          dtype=(dtype or self.dtype))

    def convert_to_tensor(self, array, *args, dtype: Optional[torch.dtype] = None,
                          **kwargs) -> torch.Tensor:
        """``array`` (tensor, ndarray, list or number) on this context's
        device; in ``dtype`` if given, else uint8 for boolean / uint8 input
        and the context dtype for everything else"""
        target = dtype or (torch.uint8 if _is_mask_dtype(array) else self.dtype)
        if not isinstance(array, torch.Tensor):
            array = torch.from_numpy(np.ascontiguousarray(np.asarray(array)))
        return array.to(*args, **kwargs, device=self.device, dtype=target)

    @staticmethod
    def convert_to_ndarray(tensor) -> np.ndarray:
        if isinstance(tensor, torch.Tensor):
            return tensor.detach().cpu().numpy()
        return np.array(tensor)

    def stream_handle(self) -> int:
        """the current torch CUDA stream of this device, as a cudaStream_t"""
        return torch.cuda.current_stream(self.device).cuda_stream
