"""Device, dtype and population storage of a simulation.

Mirrors lettuce's ``Context`` (lettuce/_context.py:9-122): same constructor
arguments, same validation and tensor factories. One addition: ``storage``
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


class Context:
    def __init__(self, device: Optional[Union[torch.device, str]] = None,
                 dtype: Optional[torch.dtype] = None,
                 use_native: Optional[bool] = None,
                 storage: Optional[str] = None):
        if device is None and use_native is None:
            device = torch.device("cuda:0" if torch.cuda.is_available() else "cpu")
            use_native = torch.cuda.is_available()
        elif device is None:
            assert not use_native or torch.cuda.is_available(), \
                "native CUDA path requested but CUDA is not available!"
            device = torch.device("cuda:0")
        elif use_native is None:
            if "cuda" in str(device):
                assert torch.cuda.is_available(), \
                    "cuda device explicitly requested but cuda is not available!"
                use_native = True
            else:
                assert "cpu" in str(device), \
                    f"lettuce_gb300 works on cpu (set-up) or cuda devices, not {device}"
                use_native = False
        else:
            if "cuda" in str(device):
                assert torch.cuda.is_available(), \
                    "cuda device explicitly requested but cuda is not available!"
            else:
                assert "cpu" in str(device), \
                    f"lettuce_gb300 works on cpu (set-up) or cuda devices, not {device}"
                assert not use_native, \
                    "can not use the native CUDA path on an explicitly requested cpu device!"

        dtype = dtype or torch.float32
        assert dtype in [torch.float16, torch.bfloat16, torch.float32, torch.float64], \
            f"unsupported dtype {dtype}"
        if storage not in _STORAGE:
            raise ValueError(f"unknown population storage {storage!r}; "
                             f"choose one of {[k for k in _STORAGE if k]}")
        if dtype == torch.float16:
            storage = storage or "fp16_shifted"
        if dtype == torch.bfloat16:
            storage = storage or "bf16_shifted"

        self.device = torch.device(device)
        self.use_native = bool(use_native)
        self.storage_name = storage
        if storage is None:
            self.dtype = dtype
            self.storage = _lib.F64 if dtype == torch.float64 else _lib.F32
        else:
            # compute (and moment) type of the 16-bit formats is float32
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
        new_dtype = dtype
        if dtype is None:
            bool_types = [bool, torch.bool, torch.uint8, np.uint8]
            if hasattr(array, "dtype") and array.dtype in bool_types:
                new_dtype = torch.uint8
            else:
                new_dtype = self.dtype
        if isinstance(array, torch.Tensor):
            return array.to(*args, **kwargs, device=self.device, dtype=new_dtype)
        array = np.ascontiguousarray(np.array(array))
        return torch.from_numpy(array).to(*args, **kwargs, device=self.device,
                                          dtype=new_dtype)

    @staticmethod
    def convert_to_ndarray(tensor) -> np.ndarray:
        if isinstance(tensor, torch.Tensor):
            return tensor.detach().cpu().numpy()
        return np.array(tensor)

    def stream_handle(self) -> int:
        """the current torch CUDA stream of this device, as a cudaStream_t"""
        return torch.cuda.current_stream(self.device).cuda_stream
