"""The hand-written adjoint (lgb_adjoint_step behind lettuce_gb300.rollout):

* gradient of MSE(u(T), target) w.r.t. the initial velocity equals torch
  autograd through lettuce's own step (golden, float64, 32^2, 10 steps);
* the adjoint kernel equals torch's vector-Jacobian product of a one-step
  torch restatement for every stencil;
* the checkpoint interval does not change the gradient (bit-identical);
* the differentiable D2Q9 BGK 512^2 configuration (float32, 200 steps,
  checkpoint every 20) passes a central finite-difference check.

Tolerances: float64 gradients 1e-9 relative; float32 adjoint against a
float64 finite difference 2e-3 relative (float32 accumulation over 400
kernel applications)."""
import math

import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden

pytestmark = pytest.mark.gpu


def _carrier(n, dtype, S=lt.D2Q9):
    """a flow used only for its stencil tables (equilibrium of given moments)"""
    return lt.TaylorGreenVortex(lt.Context("cuda:0", dtype), n, 1000, 0.05, S)


def _loss(u0, target, tau, steps, dtype, k=20, S=lt.D2Q9):
    fl = _carrier(list(u0.shape[1:]), dtype, S)
    rho0 = torch.ones([1] + list(u0.shape[1:]), dtype=dtype, device="cuda")
    f0 = lt.QuadraticEquilibrium()(fl, rho0, u0)
    fT = lt.rollout(f0, fl.stencil, tau, steps, checkpoint_every=k)
    _, u = lt.moments_torch(fT, fl.stencil)
    return torch.mean((u - target) ** 2)


def test_gradient_matches_lettuce_autograd(lgb):
    z = golden("adjoint_d2q9_32")
    u0 = torch.tensor(z["u0"], device="cuda", requires_grad=True)
    target = torch.tensor(z["target"], device="cuda")
    loss = _loss(u0, target, float(z["tau"]), int(z["steps"]), torch.float64, k=3)
    loss.backward()
    assert abs(loss.item() / float(z["loss"]) - 1) < 1e-12
    g = u0.grad.cpu().numpy()
    ref = z["grad_u0"]
    assert np.max(np.abs(g - ref)) / np.max(np.abs(ref)) < 1e-9


def _torch_step(f, S, tau):
    """one pull-pattern BGK step in torch (lettuce's stream then collide)"""
    s = S()
    e = torch.tensor(s.e, dtype=f.dtype, device=f.device)
    w = torch.tensor(s.w, dtype=f.dtype, device=f.device)
    d = s.d
    g = torch.stack([torch.roll(f[q], shifts=tuple(s.e[q]), dims=tuple(range(d)))
                     for q in range(s.q)])
    rho = g.sum(0)
    u = torch.einsum("qd,q...->d...", e, g) / rho
    eu = torch.einsum("qd,d...->q...", e, u)
    uu = (u * u).sum(0)
    feq = w.view([-1] + [1] * d) * rho * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * uu)
    return g - (g - feq) / tau


@pytest.mark.parametrize("S,res", [(lt.D1Q3, [23]), (lt.D2Q9, [12, 9]), (lt.D3Q15, [5, 6, 7]),
                                   (lt.D3Q19, [6, 5, 7]), (lt.D3Q27, [5, 7, 6])])
def test_adjoint_kernel_equals_torch_vjp(lgb, S, res):
    import ctypes
    from lettuce_gb300 import _device, _lib
    s = S()
    rng = np.random.default_rng(11)
    w = np.array(s.w).reshape([-1] + [1] * len(res))
    f = torch.tensor(w * (1 + 0.05 * rng.standard_normal([s.q] + res)), device="cuda",
                     requires_grad=True)
    lam_next = torch.tensor(rng.standard_normal([s.q] + res), device="cuda")
    tau = 0.61
    (_torch_step(f, S, tau) * lam_next).sum().backward()
    lam = torch.empty_like(lam_next)
    L = _lib.load()
    r3 = _lib.i32x3(res)
    _lib.check(L.lgb_adjoint_step(s.lgb_id, _lib.F64, ctypes.cast(r3, ctypes.c_void_p), tau,
                                  f.detach().contiguous().data_ptr(), lam_next.data_ptr(),
                                  lam.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "adjoint")
    ref = f.grad
    assert torch.max(torch.abs(lam - ref)).item() / torch.max(torch.abs(ref)).item() < 1e-12


def test_checkpoint_interval_does_not_change_gradient(lgb):
    """k = 1 runs eagerly, 7 (odd: both field parities, a 2-step remainder)
    and 20 replay captured segments, 1000 is one segment; repeated k replay
    the graphs kept in the workspace"""
    gen = torch.Generator().manual_seed(2)
    u0 = (0.02 * torch.randn(2, 40, 36, generator=gen)).cuda()
    target = (0.02 * torch.randn(2, 40, 36, generator=gen)).cuda()
    grads = []
    for k in (1, 7, 7, 20, 20, 1000):
        x = u0.clone().requires_grad_(True)
        _loss(x, target, 0.57, 30, torch.float32, k=k).backward()
        grads.append(x.grad.clone())
    for g in grads[1:]:
        assert torch.equal(g, grads[0])


def _config5_fields(n=512, dtype=torch.float32):
    """TGV velocity (Re 1000, Ma 0.05, lattice units) plus 1e-3 N(0,1)
    (seed 0), and an independent target field (seed 1)"""
    ulu = 0.05 / math.sqrt(3)
    x = torch.arange(n, dtype=torch.float64) * 2 * math.pi / n
    X, Y = torch.meshgrid(x, x, indexing="ij")
    u0 = torch.stack([torch.cos(X) * torch.sin(Y), -torch.sin(X) * torch.cos(Y)]) * ulu
    u0 = u0 + 1e-3 * torch.randn(u0.shape, generator=torch.Generator().manual_seed(0),
                                 dtype=torch.float64)
    target = ulu * torch.randn(u0.shape, generator=torch.Generator().manual_seed(1),
                               dtype=torch.float64)
    nu = (n / (2 * math.pi)) * ulu / 1000
    tau = 3 * nu + 0.5
    return u0.to(dtype).cuda(), target.to(dtype).cuda(), tau


def test_config5_finite_difference(lgb):
    """D2Q9 BGK 512^2, float32, 200 steps, checkpoint every 20: the adjoint
    directional derivative against a central difference of float64 runs"""
    u0, target, tau = _config5_fields()
    x = u0.clone().requires_grad_(True)
    loss = _loss(x, target, tau, 200, torch.float32, k=20)
    loss.backward()
    v = torch.randn(u0.shape, generator=torch.Generator().manual_seed(7)).cuda()
    dd_adj = float((x.grad.double() * v.double()).sum())
    eps = 1e-6
    u64, t64 = u0.double(), target.double()
    with torch.no_grad():
        lp = _loss(u64 + eps * v.double(), t64, tau, 200, torch.float64).item()
        lm = _loss(u64 - eps * v.double(), t64, tau, 200, torch.float64).item()
    dd_fd = (lp - lm) / (2 * eps)
    print(f"config 5: adjoint {dd_adj:.8e}  finite difference {dd_fd:.8e}")
    assert abs(dd_adj / dd_fd - 1) < 2e-3
    # float64 adjoint against the same difference
    x64 = u64.clone().requires_grad_(True)
    _loss(x64, t64, tau, 200, torch.float64, k=20).backward()
    dd64 = float((x64.grad * v.double()).sum())
    assert abs(dd64 / dd_fd - 1) < 1e-6
