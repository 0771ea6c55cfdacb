"""lgb_reduce_static: the reductions of lgb_reduce for callers that cannot
allocate device memory (an application whose device memory belongs to
another allocator, or a loop that must not take cudaMalloc's implicit
device synchronisation). Its scratch is a device array inside the library,
so the caller passes only the field and the output.

Checked through the C ABI against lgb_reduce (which uses caller-provided
scratch): both run the same kernels and fold the same partial sums in the
same order, so the results must be equal bit for bit. Two calls are issued
back to back on one stream into separate outputs before one synchronise
(the ordering the header promises is safe for the shared array); the cases
cover D3Q19 float32 with a box and mask, and D2Q9 float64 with the field in
the AA layout (aa_pending = 1). A warm call must leave the device's free
memory unchanged. This file is collected last."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

HERE = os.path.dirname(os.path.abspath(__file__))


def _field_d3q19(lt, seed):
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", torch.float32), [24, 20, 18], 1600, 0.05,
                                lt.D3Q19)
    g = torch.Generator(device="cpu").manual_seed(seed)
    noise = 1 + 0.01 * torch.randn(tuple(flow.f.shape), generator=g)
    flow.f = flow.f * noise.to("cuda:0")
    return flow


def _field_d2q9_aa(lt):
    """a float64 D2Q9 field left by one AA even step (populations in their
    opposite slots, stream pending)"""
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", torch.float64), [30, 22], 1000, 0.05,
                                lt.D2Q9)
    sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [],
                        memory_pattern="aa", use_graph=False)
    sim._collide_and_stream()
    assert flow._aa_pending
    return flow


def _ptr(arr):
    return ctypes.cast(arr, ctypes.c_void_p) if arr is not None else None


def _static(L, _lib, stencil, storage, flow, aa, lo, hi, mask, out, stream):
    r3 = _lib.i32x3(flow.resolution)
    lo3 = _lib.i32x3(lo) if lo is not None else None
    hi3 = _lib.i32x3(hi) if hi is not None else None
    rc = L.lgb_reduce_static(stencil, storage, ctypes.cast(r3, ctypes.c_void_p),
                             flow.f_raw.data_ptr(), int(aa), _ptr(lo3), _ptr(hi3),
                             mask.data_ptr() if mask is not None else None, out.data_ptr(),
                             stream)
    assert rc == 0, L.lgb_last_error().decode()


@pytest.mark.gpu
def test_reduce_static_matches_reduce(lgb):
    from lettuce_gb300 import _device, _lib
    lt = lgb
    L = _lib.load()
    mask = (torch.rand(24, 20, 18, generator=torch.Generator().manual_seed(3)) < 0.3) \
        .to(torch.uint8).cuda()
    cases = [(_lib.D3Q19, _lib.F32, _field_d3q19(lt, 1), False, None, None, None),
             (_lib.D3Q19, _lib.F32, _field_d3q19(lt, 2), False, [2, 1, 3], [20, 19, 15], mask),
             (_lib.D2Q9, _lib.F64, _field_d2q9_aa(lt), True, [3, 0], [27, 22], None)]
    stream = torch.cuda.current_stream().cuda_stream
    for first in range(0, len(cases), 2):
        pair = cases[first:first + 2]
        outs = [torch.full((_lib.REDUCE_FIELDS,), float("nan"), dtype=torch.float64,
                           device="cuda:0") for _ in pair]
        # back to back on one stream, no synchronisation in between: the
        # second call's partial sums overwrite the first's only after the
        # first call's final fold has read them
        for (st, sto, flow, aa, lo, hi, m), out in zip(pair, outs):
            _static(L, _lib, st, sto, flow, aa, lo, hi, m, out, stream)
        refs = [_device.reduce(st, sto, flow.resolution, flow.f_raw, aa, lo, hi, m)
                for st, sto, flow, aa, lo, hi, m in pair]
        torch.cuda.synchronize()
        for out, ref in zip(outs, refs):
            g, r = out.cpu().numpy(), ref.cpu().numpy()
            assert np.all(np.isfinite(g)), g
            assert np.array_equal(g.view(np.int64), r.view(np.int64)), (g, r)


@pytest.mark.gpu
def test_reduce_static_allocates_nothing(lgb):
    from lettuce_gb300 import _lib
    lt = lgb
    L = _lib.load()
    flow = _field_d3q19(lt, 4)
    out = torch.empty(_lib.REDUCE_FIELDS, dtype=torch.float64, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream
    _static(L, _lib, _lib.D3Q19, _lib.F32, flow, False, None, None, None, out, stream)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _static(L, _lib, _lib.D3Q19, _lib.F32, flow, False, None, None, None, out, stream)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    # a device allocation takes at least one 2 MiB page
    assert free1 == free0, (free0, free1)
    # bad arguments are refused before any launch
    bad_hi = _lib.i32x3([25, 20, 18])
    r3 = _lib.i32x3([24, 20, 18])
    rc = L.lgb_reduce_static(_lib.D3Q19, _lib.F32, ctypes.cast(r3, ctypes.c_void_p),
                             flow.f_raw.data_ptr(), 0, None,
                             ctypes.cast(bad_hi, ctypes.c_void_p), None, out.data_ptr(), None)
    assert rc != 0 and "box" in L.lgb_last_error().decode()
    huge = _lib.i32x3([1 << 16, 1 << 16, 2])
    rc = L.lgb_reduce_static(_lib.D3Q19, _lib.F32, ctypes.cast(huge, ctypes.c_void_p),
                             flow.f_raw.data_ptr(), 0, None, None, None, out.data_ptr(), None)
    assert rc != 0 and "2^32" in L.lgb_last_error().decode()


def test_reduce_static_source_allocates_nothing():
    """the entry point's body names no allocating call (CPU check of the
    source; the GPU test above checks the device's free memory)"""
    src = open(os.path.join(HERE, "..", "lettuce_gb300", "csrc", "lgb_abi.cu")).read()
    start = src.index("int lgb_reduce_static(")
    body = src[start:src.index("\n}\n", start)]
    lookup = src[src.index("int static_scratch_address("):]
    lookup = lookup[:lookup.index("\n}\n")]
    for text in (body, lookup):
        assert not re.search(r"cudaMalloc|cudaFree|cudaMallocAsync|\bnew\b|malloc\(|torch",
                             text), text
    assert "cudaGetSymbolAddress(&p, g_reduce_scratch)" in lookup
