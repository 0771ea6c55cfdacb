"""Physics and reporter behaviour on the GPU: the 2-D Taylor-Green energy
decay against lettuce's series and the analytic rate, lettuce's collision
property tests, the failure reporters, observables, and the accuracy of the
shifted 16-bit population storage against a float64 run."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden
from lgb_helpers import GivenFlow, rel_l2, rel_max, to_np

pytestmark = pytest.mark.gpu
F64, F32 = torch.float64, torch.float32


def ctx(dtype=F64, storage=None):
    return lt.Context("cuda:0", dtype, storage=storage)


def test_energy_decay_matches_lettuce_and_analytic(lgb):
    """D2Q9 BGK Taylor-Green 256^2, Re 1000, Ma 0.05, float64, 1000 steps
    (POST_STREAMING). lettuce's energy series to 1e-10 relative; the decay
    ratio E(t)/E(0) against exp(-4 nu t) to 1e-4 relative."""
    z = golden("tgv2d_energy_256")
    flow = lt.TaylorGreenVortex(ctx(), 256, 1000, 0.05, lt.D2Q9)
    energy = lt.IncompressibleKineticEnergy(flow)
    sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [])
    e = [energy().item()]
    for _ in range(10):
        sim(100)
        e.append(energy().item())
    e = np.array(e)
    assert np.max(np.abs(e / z["energy"] - 1)) < 1e-10
    ratio = e / e[0]
    assert np.max(np.abs(ratio / z["analytic_ratio"] - 1)) < 1e-4
    assert rel_max(to_np(flow.u()), z["u_final"]) < 1e-6


def test_observables_match_lettuce(lgb):
    z = golden("observables")
    for tag, S, n in [("2d", lt.D2Q9, 16), ("3d", lt.D3Q19, 8)]:
        flow = lt.TaylorGreenVortex(ctx(), n, 1000, 0.05, S)
        assert abs(lt.IncompressibleKineticEnergy(flow)().item() / z[f"{tag}_energy"] - 1) < 1e-13
        assert abs(lt.MaximumVelocity(flow)().item() / z[f"{tag}_umax"] - 1) < 1e-13
        assert abs(lt.Enstrophy(flow)().item() / z[f"{tag}_enstrophy"] - 1) < 1e-12


def test_mass_observable(lgb):
    f0 = golden("random_d2q9_bgk")["f0"]
    flow = GivenFlow(ctx(), lt.D2Q9(), f0)
    ref = f0[..., 1:-1, 1:-1].sum()
    assert abs(lt.Mass(flow)().item() - ref) < 1e-12
    mask = np.zeros(f0.shape[1:], dtype=bool)
    mask[2, 3] = mask[4, 1] = True
    ref2 = ref - (f0 * mask).sum()
    assert abs(lt.Mass(flow, no_mass_mask=mask)().item() - ref2) < 1e-12


@pytest.mark.parametrize("coll", ["bgk", "trt", "kbc"])
@pytest.mark.parametrize("S", [lt.D2Q9, lt.D3Q27])
def test_collisions_conserve_mass_and_momentum(lgb, coll, S):
    """lettuce tests/collision/test_collision_conserves_mass.py / _momentum.py
    (on a perturbed field: see test_gpu_parity for the ill-conditioned KBC
    case of a freshly initialised Taylor-Green vortex)"""
    flow = lt.TaylorGreenVortex(ctx(), 16 if S is lt.D2Q9 else 8, 100, 0.05, S)
    rng = np.random.default_rng(5)
    flow.f = flow.f * torch.as_tensor(1 + 0.01 * rng.standard_normal(tuple(flow.f.shape)),
                                      device="cuda")
    tau = flow.units.relaxation_parameter_lu
    c = {"bgk": lt.BGKCollision(tau), "trt": lt.TRTCollision(tau), "kbc": lt.KBCCollision()}[coll]
    f_new = c(flow)
    assert rel_max(to_np(flow.rho(f_new)), to_np(flow.rho())) < 1e-13
    j_old, j_new = to_np(flow.j()), to_np(flow.j(f_new))
    assert np.max(np.abs(j_new - j_old)) < 1e-14


def test_bgk_fixpoint_twice(lgb):
    """lettuce tests/collision/test_collision_fixpoint_2x.py: BGK with
    tau = 0.5 applied twice is the identity"""
    flow = lt.TaylorGreenVortex(ctx(), 16, 100, 0.05, lt.D2Q9)
    f0 = flow.f.clone()
    c = lt.BGKCollision(0.5)
    flow.f = c(flow)
    flow.f = c(flow)
    assert rel_max(to_np(flow.f), to_np(f0)) < 1e-14


def test_anti_bounce_back_operator_formula(lgb):
    """lettuce tests/boundary/test_antibounceback_outlet_bc.py: the operator
    equals the Krueger p. 195 formula on the outlet plane"""
    for S, res in [(lt.D2Q9, [16, 16]), (lt.D3Q19, [8, 6, 5]), (lt.D3Q27, [8, 6, 5])]:
        rng = np.random.default_rng(1)
        s = S()
        w = np.array(s.w).reshape([-1] + [1] * len(res))
        f0 = w * (1 + 0.1 * rng.standard_normal([s.q] + res))
        flow = GivenFlow(ctx(), s, f0)
        direction = [1] + [0] * (len(res) - 1)
        rho = to_np(flow.rho())[0]
        u = to_np(flow.u())
        uw = u[:, -1] + 0.5 * (u[:, -1] - u[:, -2])
        ref = f0.copy()
        e = np.array(s.e)
        for v in np.where(e @ np.array(direction) == 1)[0]:
            eu = np.einsum("c,c...->...", e[v], uw)
            ref[s.opposite[v], -1] = -f0[v, -1] + s.w[v] * rho[-1] * (
                2 + eu ** 2 / s.cs ** 4 - (np.linalg.norm(uw, axis=0) / s.cs) ** 2)
        out = lt.AntiBounceBackOutlet(direction, flow)(flow)
        assert rel_max(to_np(out), ref) < 1e-13


def test_bounce_back_and_equilibrium_operators(lgb):
    f0 = golden("random_d3q19_bgk")["f0"]
    flow = GivenFlow(ctx(), lt.D3Q19(), f0)
    out = lt.BounceBackBoundary(torch.ones(f0.shape[1:], dtype=torch.bool).cuda())(flow)
    assert np.array_equal(to_np(out), f0[lt.D3Q19().opposite])
    b = lt.EquilibriumBoundaryPU(flow.context, flow, torch.ones(f0.shape[1:], dtype=torch.bool),
                                 [0.1, 0.0, -0.05], 0.01)
    out = to_np(b(flow))
    # numbers and lists become float32 tensors in checked_tensor, as in lettuce
    rho = flow.units.convert_pressure_pu_to_density_lu(torch.tensor(0.01).to(F64)).item()
    u = torch.as_tensor([0.1, 0.0, -0.05]).to(F64).view(3, 1, 1, 1) \
        * flow.units.characteristic_velocity_lu
    feq = lt.QuadraticEquilibrium()(flow, rho * torch.ones([1] + list(f0.shape[1:]),
                                                          dtype=F64, device="cuda"),
                                   u.cuda().expand(3, *f0.shape[1:]))
    assert rel_max(out, to_np(feq)) < 1e-14


def test_nan_reporter_stops_breakable_simulation(lgb, tmp_path):
    """lettuce tests/reporter/test_nan_reporter.py: TGV 16^2 at Re 1e12,
    Ma 1 diverges; the reporter (interval 10) stops the run at 70 or 80"""
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0"), [16, 16], 1e12, 1)
    rep = lt.NaNReporter(10, outdir=str(tmp_path))
    sim = lt.BreakableSimulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [rep])
    sim(100)
    assert (tmp_path / "NaN_reporter.log").exists()
    assert flow.i > 100
    assert rep.failed_iteration in [70, 80]
    assert sim.status & 1


def test_high_ma_reporter(lgb, tmp_path):
    """lettuce tests/reporter/test_high_ma_reporter.py: stops at step 13"""
    flow = lt.Obstacle(lt.Context("cuda:0"), [16, 16], 10, 0.2, 16)
    g = flow.grid
    flow.mask = ((2 < g[0]) & (g[0] < 10) & (2 < g[1]) & (g[1] < 10))
    rep = lt.HighMaReporter(1, outdir=str(tmp_path))
    sim = lt.BreakableSimulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [rep])
    sim(100)
    assert (tmp_path / "HighMa_reporter.log").exists()
    assert flow.i > 100
    assert rep.failed_iteration == 13


def test_observable_reporter_collects(lgb):
    flow = lt.TaylorGreenVortex(ctx(F32), 32, 1000, 0.05, lt.D2Q9)
    rep = lt.ObservableReporter(lt.IncompressibleKineticEnergy(flow), interval=5, out=None)
    lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [rep])(20)
    assert [r[0] for r in rep.out] == [0, 5, 10, 15, 20]
    e = [r[2] for r in rep.out]
    assert all(a > b for a, b in zip(e, e[1:]))


@pytest.mark.parametrize("storage,bound", [("fp16_shifted", 2e-3), ("bf16_shifted", 2e-2)])
def test_shifted_storage_accuracy(lgb, storage, bound):
    """3-D Taylor-Green D3Q19 BGK 64^3, Re 1600: relative L2 velocity error
    of 16-bit shifted storage after 200 steps against a float64 run (the
    float64 kernels are pinned to lettuce above)"""
    ref = lt.TaylorGreenVortex(ctx(F64), 64, 1600, 0.05, lt.D3Q19)
    low = lt.TaylorGreenVortex(ctx(F32, storage), 64, 1600, 0.05, lt.D3Q19)
    tau = ref.units.relaxation_parameter_lu
    lt.Simulation(ref, lt.BGKCollision(tau), [], lt.StreamingStrategy.PRE_STREAMING)(200)
    lt.Simulation(low, lt.BGKCollision(tau), [], lt.StreamingStrategy.PRE_STREAMING)(200)
    err = rel_l2(to_np(low.u()), to_np(ref.u()))
    print(f"{storage}: rel L2 u error after 200 steps = {err:.3e}")
    assert err < bound
