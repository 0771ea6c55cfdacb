"""lgb_reduce_static: the reductions of lgb_reduce for callers that cannot
allocate device memory (an application whose device memory belongs to
another allocator, or a loop that must not take cudaMalloc's implicit
device synchronisation). Its scratch is a device array inside the library,
so the caller passes only the field and the output.

Checked through the C ABI against lgb_reduce (which uses caller-provided
scratch), on two calls in a row with different fields, box and mask: both
fold the same partial sums in the same order, and the tests hold float64
reductions to 1e-12 relative. This file is collected last."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _field(lt, seed):
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", torch.float32), [24, 20, 18], 1600, 0.05,
                                lt.D3Q19)
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = 1 + 0.01 * torch.randn(tuple(flow.f.shape), generator=g)
    flow.f = flow.f * noise.to("cuda:0")
    return flow


def _static(L, _lib, flow, lo, hi, mask):
    out = torch.full((_lib.REDUCE_FIELDS,), float("nan"), dtype=torch.float64, device="cuda:0")
    r3 = _lib.i32x3(flow.resolution)
    lo3 = _lib.i32x3(lo) if lo is not None else None
    hi3 = _lib.i32x3(hi) if hi is not None else None
    rc = L.lgb_reduce_static(_lib.D3Q19, _lib.F32, ctypes.cast(r3, ctypes.c_void_p),
                             flow.f_raw.data_ptr(), 0,
                             ctypes.cast(lo3, ctypes.c_void_p) if lo3 is not None else None,
                             ctypes.cast(hi3, ctypes.c_void_p) if hi3 is not None else None,
                             mask.data_ptr() if mask is not None else None, out.data_ptr(),
                             torch.cuda.current_stream().cuda_stream)
    assert rc == 0, L.lgb_last_error().decode()
    return out


def test_reduce_static_matches_reduce(lgb):
    from lettuce_gb300 import _device, _lib
    lt = lgb
    L = _lib.load()
    cases = [(_field(lt, 1), None, None, None),
             (_field(lt, 2), [2, 1, 3], [20, 19, 15],
              (torch.rand(24, 20, 18, generator=torch.Generator().manual_seed(3)) < 0.3)
              .to(torch.uint8).cuda())]
    for flow, lo, hi, mask in cases:  # two calls in a row share the static array
        got = _static(L, _lib, flow, lo, hi, mask)
        ref = _device.reduce(_lib.D3Q19, _lib.F32, flow.resolution, flow.f_raw, False, lo, hi,
                             mask)
        torch.cuda.synchronize()
        g, r = got.cpu().numpy(), ref.cpu().numpy()
        assert np.all(np.isfinite(g))
        assert np.allclose(g, r, rtol=1e-12, atol=0), (g, r)
    # the static path allocates nothing and rejects bad arguments cleanly
    assert _lib.REDUCE_STATIC_SCRATCH_BYTES >= L.lgb_reduce_scratch_bytes()
    bad_hi = _lib.i32x3([25, 20, 18])
    r3 = _lib.i32x3([24, 20, 18])
    rc = L.lgb_reduce_static(_lib.D3Q19, _lib.F32, ctypes.cast(r3, ctypes.c_void_p),
                             cases[0][0].f_raw.data_ptr(), 0, None,
                             ctypes.cast(bad_hi, ctypes.c_void_p), None,
                             torch.empty(5, dtype=torch.float64, device="cuda:0").data_ptr(), None)
    assert rc != 0 and "box" in L.lgb_last_error().decode()
