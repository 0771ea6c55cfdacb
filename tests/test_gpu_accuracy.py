"""Accuracy of the shifted 16-bit population storage on the benchmark
workload itself: D3Q19 BGK Taylor-Green vortex, 256^3, Re 1600, Ma 0.05,
1000 PRE_STREAMING steps, against the float64 oracle.

The oracle (the C restatement of lettuce's step, pinned to lettuce-generated
vectors) ran this workload once; tests/golden/make_accuracy_pin.py stored
its velocity at 8192 cells, its per-plane sums over every cell and its
totals in tests/golden/accuracy_pin_d3q19_256_f64_1000.npz. Here the
float64 kernels run the same 1000 steps and must reproduce those summaries
(which pins the whole float64 field to the oracle), and then:

* fp16-shifted storage: relative L2 velocity error over the whole field
  <= 1e-3 (the target), and the same bound at the oracle's own 8192 cells;
* float32: <= 1e-4;
* bf16-shifted misses the 1e-3 target (8 mantissa bits); its error is held
  below 2e-2 so that a regression still shows."""
import os

import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import GOLDEN

pytestmark = pytest.mark.gpu
PIN = os.path.join(GOLDEN, "accuracy_pin_d3q19_256_f64_1000.npz")
RES, RE, MA, STEPS = [256, 256, 256], 1600, 0.05, 1000


def _run(storage, dtype=torch.float32):
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", dtype, storage=storage), RES, RE, MA,
                                lt.D3Q19)
    sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [],
                        streaming_strategy=lt.StreamingStrategy.PRE_STREAMING)
    sim(STEPS)
    assert sim.status == 0
    u = flow.u().to(torch.float64)
    del sim, flow
    torch.cuda.empty_cache()
    return u


@pytest.fixture(scope="module")
def reference(lgb):
    pin = np.load(PIN)
    assert int(pin["grid"]) == 256 and int(pin["steps"]) == STEPS
    u = _run(None, torch.float64)
    return pin, u


def test_float64_kernels_reproduce_the_oracle(reference):
    pin, u = reference
    cells = torch.as_tensor(pin["cells"], device=u.device)
    got = u.reshape(3, -1)[:, cells].cpu().numpy()
    umax = np.max(np.abs(pin["u_samples"]))
    assert np.max(np.abs(got - pin["u_samples"])) <= 1e-11 * umax

    def plane_sums(a):
        return np.stack([a.sum(dim=(1, 2)).cpu().numpy(), a.sum(dim=(0, 2)).cpu().numpy(),
                         a.sum(dim=(0, 1)).cpu().numpy()])
    # sums of u_c over planes vanish by symmetry (rounding noise of the
    # 65536 terms): absolute bound; sums of u_c^2 over planes: relative
    sums = np.stack([plane_sums(u[c]) for c in range(3)])
    assert np.max(np.abs(sums - pin["u_plane_sums"])) <= 1e-9 * umax
    # (planes of symmetry carry nearly no u_z: scale by the largest plane
    # sum of the same component and axis)
    sq = np.stack([plane_sums(u[c] * u[c]) for c in range(3)])
    ref = pin["u_sq_plane_sums"]
    scale = np.max(np.abs(ref), axis=2, keepdims=True)
    assert np.max(np.abs(sq - ref) / scale) <= 1e-10
    usq = np.array([torch.sum(u[c] * u[c]).item() for c in range(3)])
    assert np.max(np.abs(usq / pin["u_sq_sums"] - 1)) <= 1e-10


def _errors(u, reference):
    pin, u_ref = reference
    full = (torch.linalg.vector_norm(u - u_ref) / torch.linalg.vector_norm(u_ref)).item()
    cells = torch.as_tensor(pin["cells"], device=u.device)
    us = u.reshape(3, -1)[:, cells].cpu().numpy()
    samples = float(np.linalg.norm(us - pin["u_samples"]) / np.linalg.norm(pin["u_samples"]))
    return full, samples


def test_fp16_shifted_meets_the_target(reference):
    full, samples = _errors(_run("fp16_shifted"), reference)
    print(f"fp16-shifted u rel L2 after 1000 steps: {full:.4e} (oracle cells {samples:.4e})")
    assert full <= 1e-3, full
    assert samples <= 1e-3, samples


def test_float32_and_bf16_errors(reference):
    f32, _ = _errors(_run(None), reference)
    assert f32 <= 1e-4, f32
    bf16, _ = _errors(_run("bf16_shifted"), reference)
    print(f"float32 {f32:.3e}, bf16-shifted {bf16:.3e} (misses the 1e-3 target)")
    assert bf16 <= 2e-2, bf16
