"""Host transfers of the population field: a page-locked host tensor goes
up (``flow.f = host``) and comes back (``flow.download(out)``) through one
conversion kernel on mapped host memory; the results equal the torch copies
bit for bit, for every storage format and for a field left in the AA
layout. Host memory that is not page-locked takes the torch path."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from lettuce_gb300 import _device, _lib

pytestmark = pytest.mark.gpu


def tgv(dtype, storage=None):
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    return lt.TaylorGreenVortex(ctx, [16, 12, 10], 400, 0.05, lt.D3Q19)


@pytest.mark.parametrize("dtype,storage", [(torch.float64, None), (torch.float32, None),
                                           (torch.float32, "fp16_shifted"),
                                           (torch.float32, "bf16_shifted")])
def test_pinned_upload_and_download_equal_torch_copies(lgb, dtype, storage):
    ref = tgv(dtype, storage)
    host = ref.f.cpu() * (1 + 0.01 * torch.rand(ref.f.shape, dtype=dtype,
                                                generator=torch.Generator().manual_seed(1)))
    pinned = host.pin_memory()
    assert _device.host_device_pointer(pinned) is not None
    assert _device.host_device_pointer(host) is None
    a, b = tgv(dtype, storage), tgv(dtype, storage)
    a.f = pinned                 # conversion kernel on mapped host memory
    b.f = host.to("cuda:0")      # torch copy, then the setter's conversion
    assert torch.equal(a.f_raw, b.f_raw)
    out = a.download()
    torch.cuda.synchronize()
    assert out.is_pinned() and torch.equal(out, b.f.cpu())
    plain = torch.empty_like(host)
    a.download(plain)            # not page-locked: torch copy
    torch.cuda.synchronize()
    assert torch.equal(plain, out)


def test_download_of_aa_pending_field(lgb):
    flow = tgv(torch.float32)
    sim = lt.Simulation(flow, lt.BGKCollision(0.6), [], memory_pattern="aa")
    sim(3)
    assert flow._aa_pending
    out = flow.download()
    torch.cuda.synchronize()
    assert torch.equal(out, flow.f.cpu())


def test_host_pointer_on_pageable_memory(lgb):
    """pageable memory: the query fails where the device cannot address it,
    and on hosts whose GPU reads pageable memory through the host page
    tables (a Grace host) it returns an address; either way the package
    moves only page-locked tensors with the kernel"""
    import ctypes
    L = _lib.load()
    arr = np.zeros(1024, dtype=np.float32)
    out = ctypes.c_void_p()
    rc = L.lgb_host_pointer(ctypes.c_void_p(arr.ctypes.data), ctypes.byref(out))
    if rc != 0:
        assert b"not page-locked" in L.lgb_last_error()
    else:
        assert out.value
    assert _device.host_device_pointer(torch.from_numpy(arr)) is None
    # the query leaves no error behind: a step still runs
    flow = tgv(torch.float32)
    lt.Simulation(flow, lt.BGKCollision(0.6), [])(2)
    torch.cuda.synchronize()


def test_pinned_upload_reuses_the_second_field(lgb):
    """after steps, an upload goes into the scratch field: the simulation
    keeps its two buffers (and its captured graphs) and continues exactly
    as after a torch upload"""
    a, b = tgv(torch.float32), tgv(torch.float32)
    sa = lt.Simulation(a, lt.BGKCollision(0.6), [])
    sb = lt.Simulation(b, lt.BGKCollision(0.6), [])
    sa(6)
    sb(6)
    bufs = {a._f.data_ptr(), a._f_next.data_ptr()}
    host = (a.f.cpu() * 1.001).pin_memory()
    a.f = host
    b.f = host.to("cuda:0")
    assert {a._f.data_ptr(), a._f_next.data_ptr()} == bufs
    sa(6)
    sb(6)
    assert torch.equal(a.f, b.f)
