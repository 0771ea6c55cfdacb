"""Initial populations and the enstrophy observable from the library's kernels
(lgb_equilibrium, lgb_init_fneq, lgb_enstrophy) against lettuce's torch
expressions: the golden Taylor-Green fields lettuce wrote (float64, 1e-13;
the TGV parity tests hold them too), this package's CPU set-up of the same
flows (the torch restatement of lettuce/_flow.py:127-143, 341-367) for every
stencil and storage, and the enstrophy lettuce computed
(observable_reporter.py:45-67)."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden
from lgb_helpers import rel_max, to_np

pytestmark = pytest.mark.gpu
F64, F32 = torch.float64, torch.float32


def _pair(make, dtype, storage=None):
    """(flow initialised on the GPU, same flow initialised on the CPU)"""
    dev = make(lt.Context("cuda:0", dtype, storage=storage))
    cpu = make(lt.Context("cpu", dtype))
    return dev, cpu


@pytest.mark.parametrize("dtype", [F64, F32])
@pytest.mark.parametrize("S,res", [(lt.D2Q9, [24, 20]), (lt.D3Q19, [12, 10, 14]),
                                   (lt.D3Q27, [10, 12, 8]), (lt.D3Q15, [8, 8, 8])])
def test_taylor_green_initialisation_matches_torch(lgb, S, res, dtype):
    dev, cpu = _pair(lambda c: lt.TaylorGreenVortex(c, res, 1600, 0.05, S), dtype)
    err = rel_max(to_np(dev.f), to_np(cpu.f))
    assert err < (1e-14 if dtype == F64 else 5e-7), err


@pytest.mark.parametrize("storage", ["fp16_shifted", "bf16_shifted"])
def test_taylor_green_initialisation_shifted(lgb, storage):
    """16-bit storage: the device field equals the torch float32 field stored
    in the format, up to one rounding of the stored deviation"""
    dev, cpu = _pair(lambda c: lt.TaylorGreenVortex(c, [16, 12, 10], 1600, 0.05, lt.D3Q19),
                     F32, storage)
    w = cpu.torch_stencil.w.view(-1, 1, 1, 1)
    h_ref = (cpu.f - w).to(torch.float64)
    h_dev = dev.f_raw.to(torch.float64).cpu()
    # half an ulp of the format relative to |h| (doubled for the float32
    # differences of the two set-ups), plus a few float32 ulps of f ~ w
    # (both set-ups form f in float32 before subtracting w, so an h near 0
    # carries that absolute rounding)
    rel = 2.0 ** (-10 if storage == "fp16_shifted" else -7)
    floor = 2.0 ** -22
    assert torch.all(torch.abs(h_dev - h_ref) <= rel * torch.abs(h_ref) + floor)


def test_obstacle_initialisation_matches_torch(lgb):
    """equilibrium without the non-equilibrium part (lettuce's Obstacle),
    velocity field with a masked sphere, float64"""
    def make(c):
        flow = lt.Obstacle(c, [32, 16, 16], 100, 0.1, 32 / 6, stencil=lt.D3Q27)
        grid = np.meshgrid(*[np.arange(n) for n in flow.resolution], indexing="ij")
        flow.mask = sum((g - m) ** 2 for g, m in zip(grid, [8, 8, 8])) < 9
        flow.initialize()
        return flow
    dev, cpu = _pair(make, F64)
    assert rel_max(to_np(dev.f), to_np(cpu.f)) < 1e-14


def test_golden_taylor_green_fields(lgb):
    for name in ("tgv2d_d2q9_bgk", "tgv3d_d3q19_bgk", "tgv3d_d3q27_kbc"):
        z = golden(name)
        import json
        m = json.loads(str(z["meta"]))
        flow = lt.TaylorGreenVortex(lt.Context("cuda:0", F64), m["res"], m["re"], m["ma"],
                                    getattr(lt, m["stencil"]))
        assert rel_max(to_np(flow.f), z["f0"]) < 1e-13, name


@pytest.mark.parametrize("dtype", [F64, F32])
def test_initialize_f_neq_function(lgb, dtype):
    """lettuce_gb300.initialize_f_neq on a CUDA flow (moment kernel + fneq
    kernel) equals the torch restatement on the same populations"""
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", dtype), [20, 16], 1000, 0.05, lt.D2Q9,
                                initialize_fneq=False)
    g = torch.Generator().manual_seed(5)
    f = flow.f.cpu() * (1 + 0.01 * torch.rand(tuple(flow.f.shape), generator=g, dtype=dtype))
    flow.f = f
    got = lt.initialize_f_neq(flow)
    ref_flow = lt.TaylorGreenVortex(lt.Context("cpu", dtype), [20, 16], 1000, 0.05, lt.D2Q9,
                                    initialize_fneq=False)
    ref_flow.f = f
    ref = lt.initialize_f_neq(ref_flow)
    assert rel_max(to_np(got), to_np(ref)) < (1e-14 if dtype == F64 else 2e-6)


@pytest.mark.parametrize("dtype", [F64, F32])
def test_enstrophy_kernel(lgb, dtype):
    z = golden("observables")
    for tag, S, n in [("2d", lt.D2Q9, 16), ("3d", lt.D3Q19, 8)]:
        flow = lt.TaylorGreenVortex(lt.Context("cuda:0", dtype), n, 1000, 0.05, S)
        got = lt.Enstrophy(flow)().item()
        # float32: the velocity itself carries ~1e-7 relative rounding, which
        # the differences of a smooth field amplify
        assert abs(got / z[f"{tag}_enstrophy"] - 1) < (1e-12 if dtype == F64 else 1e-5), tag
    # a non-square, random velocity field against the torch expression
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", F64), [14, 9, 11], 1000, 0.05, lt.D3Q19)
    g = torch.Generator().manual_seed(2)
    flow.f = flow.f.cpu() * (1 + 0.02 * torch.rand(tuple(flow.f.shape), generator=g,
                                                    dtype=F64))
    got = lt.Enstrophy(flow)().item()
    cpu = lt.TaylorGreenVortex(lt.Context("cpu", F64), [14, 9, 11], 1000, 0.05, lt.D3Q19)
    cpu.f = flow.f.cpu()
    ref = lt.Enstrophy(cpu)().item()
    assert abs(got / ref - 1) < 1e-12


def test_initialisation_launches_no_torch_stencil_kernels(lgb):
    """the Taylor-Green set-up on the GPU runs the library's kernels for the
    equilibrium and the non-equilibrium part (no torch roll / einsum passes
    over the population field)"""
    from torch.profiler import ProfilerActivity, profile
    torch.cuda.synchronize()
    with profile(activities=[ProfilerActivity.CUDA]) as prof:
        lt.TaylorGreenVortex(lt.Context("cuda:0", F32), [32, 32, 32], 1600, 0.05, lt.D3Q19)
        torch.cuda.synchronize()
    names = [e.name for e in prof.events() if e.device_type.name == "CUDA"]
    if not names:
        pytest.skip("the profiler recorded no device activity")
    assert any("init_fneq_kernel" in n for n in names), names
    assert any("equilibrium_kernel" in n for n in names), names
    assert not any("roll" in n for n in names), names
