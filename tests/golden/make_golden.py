"""Generate golden vectors from lettuce itself (its CPU torch path, float64).

Run in a container where the lettuce sources are available:

    PYTHONDONTWRITEBYTECODE=1 \
    PYTHONPATH=tests/golden/_stubs:<lettuce checkout> \
        python tests/golden/make_golden.py

Options: ``--no-energy`` skips the long 256^2 energy-decay series;
``--only-hwbb``, ``--only-ibb`` and ``--only-fwbb`` write only the cases of
the efficient-bounce-back example's halfway, interpolated or full-way
boundary (their modules are imported from the example's directory, found
next to the imported lettuce package).

``_stubs/`` holds empty stand-ins for lettuce's optional imports (mmh3,
h5py, pyevtk, matplotlib) -- none of them is on the arithmetic path. The
outputs (``*.npz`` next to this script) are what the CPU oracle and the CUDA
path are checked against; lettuce itself never runs in the test-suite.
"""
import json
import os
import sys
import warnings

import numpy as np
import torch

warnings.filterwarnings("ignore")
import lettuce as lt  # noqa: E402
from lettuce import (Context, Simulation, StreamingStrategy,  # noqa: E402
                     UnitConversion)
from lettuce.ext._boundary.partially_saturated_boundary import PartiallySaturatedBC  # noqa: E402
from lettuce.ext import (D1Q3, D2Q9, D3Q15, D3Q19, D3Q27,  # noqa: E402
                         AntiBounceBackOutlet, BGKCollision, EquilibriumOutletP,
                         BounceBackBoundary, EquilibriumBoundaryPU, ExtFlow,
                         IncompressibleKineticEnergy, KBCCollision,
                         MaximumVelocity, NoCollision, Obstacle,
                         TaylorGreenVortex, TRTCollision, Enstrophy)

OUT = os.path.dirname(os.path.abspath(__file__))
CTX = Context(device="cpu", dtype=torch.float64, use_native=False)
STRATS = {"PRE_STREAMING": StreamingStrategy.PRE_STREAMING,
          "POST_STREAMING": StreamingStrategy.POST_STREAMING}


def npf(t):
    return t.detach().cpu().numpy().copy()


class GivenFlow(ExtFlow):
    """A flow whose populations are given directly (like the DummyFlow of
    lettuce's tests/conftest.py)."""
    f_init = None
    bnds = []

    def __init__(self, stencil, f0, boundaries=()):
        GivenFlow.f_init = f0
        self.bnds = list(boundaries)
        ExtFlow.__init__(self, CTX, list(f0.shape[1:]), 100.0, 0.05,
                         stencil=stencil)

    def make_resolution(self, resolution, stencil=None):
        return list(resolution)

    def make_units(self, reynolds_number, mach_number, resolution):
        return UnitConversion(reynolds_number=reynolds_number,
                              mach_number=mach_number)

    def initial_pu(self):
        ...

    def initialize(self):
        self.f = torch.tensor(GivenFlow.f_init, dtype=torch.float64)

    @property
    def post_boundaries(self):
        return self.bnds


def collision_of(kind, tau):
    if kind == "bgk":
        return BGKCollision(tau=tau)
    if kind == "trt":
        return TRTCollision(tau=tau, tau_minus=1.0)
    if kind == "kbc":
        return KBCCollision(tau=tau)
    return NoCollision()


def case_tgv(name, stencil, res, re, coll, steps):
    out = {}
    for sname, strat in STRATS.items():
        flow = TaylorGreenVortex(CTX, resolution=res, reynolds_number=re,
                                 mach_number=0.05, stencil=stencil)
        f0 = npf(flow.f)
        tau = flow.units.relaxation_parameter_lu
        sim = Simulation(flow, collision_of(coll, tau), [],
                         streaming_strategy=strat)
        sim(steps)
        out["f0"] = f0
        out[f"f_{sname}"] = npf(flow.f)
        out["tau"] = np.float64(tau)
    out["steps"] = np.int64(steps)
    out["meta"] = json.dumps({"flow": "TaylorGreenVortex", "res": res,
                              "re": re, "ma": 0.05, "collision": coll,
                              "stencil": stencil.__name__})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_random(name, stencil, res, coll, steps, seed):
    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.2 * rng.standard_normal([st.q] + res))
    tau = 0.73
    out = {"f0": f0, "tau": np.float64(tau), "steps": np.int64(steps)}
    for sname, strat in STRATS.items():
        flow = GivenFlow(st, f0)
        sim = Simulation(flow, collision_of(coll, tau), [],
                         streaming_strategy=strat)
        sim(steps)
        out[f"f_{sname}"] = npf(flow.f)
        if coll == "kbc":
            # KBCCollision relaxes with flow.units.relaxation_parameter_lu,
            # not with its constructor argument (kbc_collision.py:97-99)
            out["tau"] = np.float64(flow.units.relaxation_parameter_lu)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res,
                              "collision": coll})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_obstacle(name, stencil, res, radius, coll, steps):
    out = {}
    for sname, strat in STRATS.items():
        flow = Obstacle(CTX, resolution=res, reynolds_number=100,
                        mach_number=0.1, domain_length_x=res[0] / 4.0,
                        stencil=stencil)
        grid = np.meshgrid(*[np.arange(n) for n in res], indexing="ij")
        centre = [res[0] / 3.0] + [n / 2.0 - 0.5 for n in res[1:]]
        r2 = sum((g - c) ** 2 for g, c in zip(grid, centre))
        mask = r2 < radius ** 2
        flow.mask = mask
        flow.initialize()
        f0 = npf(flow.f)
        tau = flow.units.relaxation_parameter_lu
        sim = Simulation(flow, collision_of(coll, tau), [],
                         streaming_strategy=strat)
        out["ncm"] = npf(sim.no_collision_mask).astype(np.uint8)
        out["nsm"] = npf(sim.no_streaming_mask).astype(np.uint8)
        sim(steps)
        out["f0"] = f0
        out["mask"] = mask
        out[f"f_{sname}"] = npf(flow.f)
        out["tau"] = np.float64(tau)
        inlet = flow.post_boundaries[0]
        out["inlet_u_lu"] = npf(flow.units.convert_velocity_to_lu(
            inlet.velocity))
        out["inlet_rho_lu"] = npf(flow.units.convert_pressure_pu_to_density_lu(
            inlet.pressure))
    out["steps"] = np.int64(steps)
    out["meta"] = json.dumps({"flow": "Obstacle", "res": res,
                              "radius": radius, "collision": coll,
                              "stencil": stencil.__name__, "re": 100,
                              "ma": 0.1, "domain_length_x": res[0] / 4.0})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_outlet_p(name, stencil, res, radius, rho_outlet, steps):
    """an obstacle flow whose outlet is lettuce's pressure outlet
    (EquilibriumOutletP, left commented out in obstacle.py:119-120)"""
    class ObstacleP(Obstacle):
        @property
        def post_boundaries(self):
            b = Obstacle.post_boundaries.fget(self)
            return [b[0], EquilibriumOutletP(self._unit_vector().tolist(), self,
                                             rho_outlet=rho_outlet), b[2]]
    out = {}
    for sname, strat in STRATS.items():
        flow = ObstacleP(CTX, resolution=res, reynolds_number=100, mach_number=0.1,
                         domain_length_x=res[0] / 4.0, stencil=stencil)
        grid = np.meshgrid(*[np.arange(n) for n in res], indexing="ij")
        centre = [res[0] / 3.0] + [n / 2.0 - 0.5 for n in res[1:]]
        mask = sum((g - c) ** 2 for g, c in zip(grid, centre)) < radius ** 2
        flow.mask = mask
        flow.initialize()
        out["f0"] = npf(flow.f)
        tau = flow.units.relaxation_parameter_lu
        sim = Simulation(flow, BGKCollision(tau), [], streaming_strategy=strat)
        out["ncm"] = npf(sim.no_collision_mask).astype(np.uint8)
        out["nsm"] = npf(sim.no_streaming_mask).astype(np.uint8)
        sim(steps)
        out["mask"] = mask
        out[f"f_{sname}"] = npf(flow.f)
        out["tau"] = np.float64(tau)
        inlet = flow.post_boundaries[0]
        out["inlet_u_lu"] = npf(flow.units.convert_velocity_to_lu(inlet.velocity))
        out["inlet_rho_lu"] = npf(flow.units.convert_pressure_pu_to_density_lu(
            inlet.pressure))
    out["steps"] = np.int64(steps)
    out["meta"] = json.dumps({"flow": "ObstacleP", "res": res, "radius": radius,
                              "collision": "bgk", "stencil": stencil.__name__, "re": 100,
                              "ma": 0.1, "domain_length_x": res[0] / 4.0,
                              "rho_outlet": rho_outlet})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_psm(name, stencil, res, saturation, steps, seed):
    """partially saturated cells (Noble-Torczynski) on a block of cells"""
    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.05 * rng.standard_normal([st.q] + res))
    mask = np.zeros(res, dtype=bool)
    mask[tuple(slice(n // 4, n // 4 + max(2, n // 3)) for n in res)] = True
    tau = 0.7
    out = {"f0": f0, "mask": mask, "tau": np.float64(tau), "steps": np.int64(steps),
           "saturation": np.float64(saturation)}
    for sname, strat in STRATS.items():
        flow = GivenFlow(st, f0)
        b = PartiallySaturatedBC(torch.tensor(mask), tau, saturation)
        flow.bnds = [b]
        out["B"] = np.float64(b.B)
        sim = Simulation(flow, BGKCollision(tau), [], streaming_strategy=strat)
        sim(steps)
        out[f"f_{sname}"] = npf(flow.f)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res, "collision": "bgk"})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_eqpu_field(name):
    """equilibrium boundary with a per-cell velocity field and a scalar
    pressure (lettuce tests/boundary/test_equilibrium_bc_pu.py style)"""
    st = D2Q9()
    res = [12, 10]
    rng = np.random.default_rng(7)
    w = np.array(st.w).reshape([-1, 1, 1])
    f0 = w * (1.0 + 0.1 * rng.standard_normal([st.q] + res))
    mask = np.zeros(res, dtype=bool)
    mask[3:6, 2:8] = True
    vel = 0.1 * rng.standard_normal([2] + res)
    out = {"f0": f0, "mask": mask, "velocity_pu": vel, "pressure_pu": 0.02}
    for sname, strat in STRATS.items():
        flow = GivenFlow(st, f0)
        b = EquilibriumBoundaryPU(CTX, flow, torch.tensor(mask),
                                  torch.tensor(vel), 0.02)
        flow.bnds = [b]
        sim = Simulation(flow, BGKCollision(tau=0.8), [],
                         streaming_strategy=strat)
        out["u_lu"] = npf(flow.units.convert_velocity_to_lu(b.velocity))
        out["rho_lu"] = npf(flow.units.convert_pressure_pu_to_density_lu(
            b.pressure))
        sim(3)
        out[f"f_{sname}"] = npf(flow.f)
    out["tau"] = np.float64(0.8)
    out["steps"] = np.int64(3)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_native_kats():
    """known-answer cases of lettuce's tests/native/test_native_streaming.py
    (impulse per direction) and test_native_bounce_back.py"""
    st = D2Q9()
    f0 = np.zeros([9, 16, 16])
    for i in range(9):
        f0[i, i + 1, i + 1] = float(i + 1)
    flow = GivenFlow(st, f0)
    Simulation(flow, NoCollision(), [])(1)
    out = {"stream_f0": f0, "stream_f1": npf(flow.f)}
    f0 = np.zeros([9, 16, 16])
    f0[:, 1, 1] = 1.0
    mask = np.zeros([16, 16], dtype=bool)
    mask[0, :] = True
    mask[:, 0] = True
    mask[2:, :] = True
    mask[:, 2:] = True
    flow = GivenFlow(st, f0, [BounceBackBoundary(torch.tensor(mask))])
    Simulation(flow, NoCollision(), [])(1)
    out.update({"bb_f0": f0, "bb_mask": mask, "bb_f1": npf(flow.f)})
    flow = GivenFlow(st, f0, [BounceBackBoundary(torch.tensor(mask))])
    Simulation(flow, NoCollision(), [])(2)
    out["bb_f2"] = npf(flow.f)
    np.savez_compressed(os.path.join(OUT, "native_kats.npz"), **out)


def case_observables():
    out = {}
    for tag, stencil, res in [("2d", D2Q9, 16), ("3d", D3Q19, 8)]:
        flow = TaylorGreenVortex(CTX, resolution=res, reynolds_number=1000,
                                 mach_number=0.05, stencil=stencil)
        out[f"{tag}_f"] = npf(flow.f)
        out[f"{tag}_energy"] = np.float64(
            IncompressibleKineticEnergy(flow)().item())
        out[f"{tag}_umax"] = np.float64(MaximumVelocity(flow)().item())
        out[f"{tag}_enstrophy"] = np.float64(Enstrophy(flow)().item())
        out[f"{tag}_rho"] = npf(flow.rho())
        out[f"{tag}_u"] = npf(flow.u())
        out[f"{tag}_units"] = json.dumps({
            "relaxation_parameter_lu": flow.units.relaxation_parameter_lu,
            "viscosity_lu": flow.units.viscosity_lu,
            "characteristic_velocity_lu":
                flow.units.characteristic_velocity_lu,
            "characteristic_length_lu": flow.units.characteristic_length_lu,
            "time_pu_100": flow.units.convert_time_to_pu(100)})
    np.savez_compressed(os.path.join(OUT, "observables.npz"), **out)


def case_tgv_energy_decay():
    """the 2-D Taylor-Green energy decay: D2Q9 BGK 256^2, Re 1000, Ma 0.05,
    float64, 1000 steps (POST_STREAMING, lettuce's default)"""
    flow = TaylorGreenVortex(CTX, resolution=256, reynolds_number=1000,
                             mach_number=0.05, stencil=D2Q9)
    energy = IncompressibleKineticEnergy(flow)
    sim = Simulation(flow, BGKCollision(flow.units.relaxation_parameter_lu),
                     [])
    e = [energy().item()]
    t = [0.0]
    for _ in range(10):
        sim(100)
        e.append(energy().item())
        t.append(flow.units.convert_time_to_pu(flow.i))
    nu = flow.units.viscosity_pu
    out = {"energy": np.array(e), "time_pu": np.array(t),
           "analytic_ratio": np.exp(-4 * nu * np.array(t)),
           "u_final": npf(flow.u()).astype(np.float32)}
    np.savez_compressed(os.path.join(OUT, "tgv2d_energy_256.npz"), **out)


def case_adjoint():
    """gradient of MSE(u(T), target) w.r.t. the initial velocity through
    lettuce's torch step (torch autograd, float64) -- D2Q9 BGK 32^2,
    PRE_STREAMING, 10 steps, f0 = feq(rho=1, u0)"""
    n, steps, tau = 32, 10, 0.56
    st = D2Q9()
    gen = torch.Generator().manual_seed(0)
    x = torch.arange(n, dtype=torch.float64) * 2 * np.pi / n
    X, Y = torch.meshgrid(x, x, indexing="ij")
    ulu = 0.05 / np.sqrt(3)
    u0 = torch.stack([torch.cos(X) * torch.sin(Y),
                      -torch.sin(X) * torch.cos(Y)]) * ulu
    u0 = u0 + 1e-3 * torch.randn(u0.shape, generator=gen, dtype=torch.float64)
    gen1 = torch.Generator().manual_seed(1)
    target = ulu * torch.randn(u0.shape, generator=gen1, dtype=torch.float64)
    u0 = u0.clone().requires_grad_(True)
    flow = GivenFlow(st, np.zeros([9, n, n]))
    rho0 = torch.ones([1, n, n], dtype=torch.float64)
    flow.f = flow.equilibrium(flow, rho=rho0, u=u0)
    sim = Simulation(flow, BGKCollision(tau=tau), [],
                     streaming_strategy=StreamingStrategy.PRE_STREAMING)
    sim(steps)
    loss = torch.mean((flow.u() - target) ** 2)
    loss.backward()
    out = {"u0": npf(u0), "target": npf(target), "loss": np.float64(loss.item()),
           "grad_u0": npf(u0.grad), "tau": np.float64(tau),
           "steps": np.int64(steps)}
    np.savez_compressed(os.path.join(OUT, "adjoint_d2q9_32.npz"), **out)


def case_collision_ext(name, stencil, res, kind, steps, seed):
    """random populations under the regularized / Smagorinsky collisions and
    BGK with a Guo or Shan-Chen body force (PRE and POST streaming)"""
    from lettuce.ext import Guo, ShanChen, RegularizedCollision, SmagorinskyCollision
    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.2 * rng.standard_normal([st.q] + res))
    tau, force_tau = 0.73, 0.81
    accel = [1e-3, -4e-4, 6e-4][:len(res)]
    out = {"f0": f0, "tau": np.float64(tau), "steps": np.int64(steps),
           "force_tau": np.float64(force_tau), "accel": np.array(accel)}
    for sname, strat in STRATS.items():
        flow = GivenFlow(st, f0)
        if kind == "regularized":
            coll = RegularizedCollision(tau)
            out["tau"] = np.float64(flow.units.relaxation_parameter_lu)
        elif kind == "smagorinsky":
            coll = SmagorinskyCollision(tau, smagorinsky_constant=0.3)
        elif kind == "smagorinsky_guo":
            coll = SmagorinskyCollision(tau, smagorinsky_constant=0.3,
                                        force=Guo(flow, force_tau, accel))
        elif kind == "bgk_guo":
            coll = BGKCollision(tau, force=Guo(flow, force_tau, accel))
        elif kind == "bgk_shanchen":
            coll = BGKCollision(tau, force=ShanChen(flow, force_tau, accel))
        sim = Simulation(flow, coll, [], streaming_strategy=strat)
        sim(steps)
        out[f"f_{sname}"] = npf(flow.f)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res, "kind": kind,
                              "smagorinsky_constant": 0.3})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_poiseuille(name, force_kind, steps):
    """lettuce's forced Poiseuille channel (tests/collision/test_force.py set-up:
    PoiseuilleFlow2D 17^2, Re 1, Ma 0.02, BGK with Guo or Shan-Chen)"""
    from lettuce.ext import Guo, ShanChen, PoiseuilleFlow2D
    flow = PoiseuilleFlow2D(context=CTX, resolution=17, reynolds_number=1,
                            mach_number=0.02, initialize_with_zeros=True)
    a_lu = flow.units.convert_acceleration_to_lu(flow.acceleration)
    tau = flow.units.relaxation_parameter_lu
    F = Guo if force_kind == "guo" else ShanChen
    force = F(flow=flow, tau=tau, acceleration=a_lu)
    sim = Simulation(flow=flow, collision=BGKCollision(tau=tau, force=force), reporter=[])
    f0 = npf(flow.f)
    sim(steps)
    out = {"f0": f0, "f_final": npf(flow.f), "tau": np.float64(tau),
           "accel": npf(a_lu), "steps": np.int64(steps),
           "u_final": npf(flow.u(acceleration=a_lu)),
           "ncm": npf(sim.no_collision_mask).astype(np.uint8)}
    out["meta"] = json.dumps({"force": force_kind, "res": [17, 17]})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_mrt(name, stencil, transform, res, steps, seed):
    """random populations under lettuce's MRT collision with one of its
    moment transforms and per-moment relaxation times (PRE and POST)"""
    from lettuce.ext import MRTCollision
    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.2 * rng.standard_normal([st.q] + res))
    srel = 0.55 + 0.6 * rng.random(st.q)
    srel[0] = 1.0
    out = {"f0": f0, "steps": np.int64(steps), "relaxation": srel}
    for sname, strat in STRATS.items():
        flow = GivenFlow(st, f0)
        t = transform(st, CTX)
        sim = Simulation(flow, MRTCollision(t, srel.tolist(), CTX), [], streaming_strategy=strat)
        sim(steps)
        out[f"f_{sname}"] = npf(flow.f)
        out["matrix"] = npf(t.matrix)
        out["inverse"] = npf(t.inverse)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res,
                              "transform": transform.__name__})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_dump():
    """lettuce's own checkpoint file (Flow.dump, lettuce/_flow.py:258-260) of a
    D2Q9 Taylor-Green field, written by lettuce"""
    flow = TaylorGreenVortex(CTX, resolution=12, reynolds_number=100, mach_number=0.05,
                             stencil=D2Q9)
    flow.dump(os.path.join(OUT, "lettuce_dump_d2q9_12.pkl"))
    np.savez_compressed(os.path.join(OUT, "lettuce_dump_d2q9_12.npz"), f=npf(flow.f),
                        meta=json.dumps({"res": [12, 12], "re": 100, "ma": 0.05}))


EBB = os.path.join("examples", "advanced_projects", "efficient_bounce_back_obstacle")


def case_hwbb(name, stencil, res, coll, steps, seed, solid, periodicity=None,
              inlet=False, global_extra=None):
    """lettuce's example halfway bounce-back boundary
    (examples/advanced_projects/efficient_bounce_back_obstacle/boundary/
    halfway_bounce_back_boundary.py) under the example's EbbSimulation
    (simulation/ebb_simulation.py: collide, stream, then the post-streaming
    boundaries), with its momentum-exchange force after every step. The
    link list comes from the boundary's own neighbour search (no solid
    boundary data given). ``inlet`` adds an equilibrium boundary on the x = 0
    plane as an ordinary post-collision boundary; ``global_extra`` is a
    second solid region given as part of ``global_solid_mask``."""
    import lettuce
    root = os.path.dirname(os.path.dirname(os.path.abspath(lettuce.__file__)))
    for sub in ("boundary", "simulation"):
        d = os.path.join(root, EBB, sub)
        if d not in sys.path:
            sys.path.insert(0, d)
    from halfway_bounce_back_boundary import HalfwayBounceBackBoundary
    from solid_boundary_data import SolidBoundaryData
    from ebb_simulation import EbbSimulation

    class HwbbFlow(GivenFlow):
        psb = []

        @property
        def post_streaming_boundaries(self):
            return self.psb

    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.2 * rng.standard_normal([st.q] + res))
    flow = HwbbFlow(st, f0)
    if inlet:
        m = np.zeros(res, dtype=bool)
        m[0] = True
        flow.bnds = [EquilibriumBoundaryPU(CTX, flow, torch.tensor(m),
                                           torch.tensor([0.02] + [0.0] * (len(res) - 1),
                                                        dtype=torch.float64))]
    # the example's neighbour search sizes its periodic-border offsets by
    # flow.context.d, an attribute lettuce's Context does not have: give it
    flow.context.d = st.d
    sbd = SolidBoundaryData()
    sbd.solid_mask = solid
    gmask = None if global_extra is None else (solid | global_extra)
    hw = HalfwayBounceBackBoundary(CTX, flow, sbd, global_solid_mask=gmask,
                                   periodicity=periodicity, calc_force=True)
    flow.psb = [hw]
    tau = 0.8
    sim = EbbSimulation(flow, collision_of(coll, tau), [])
    out = {"f0": f0, "solid": solid, "tau": np.float64(tau), "steps": np.int64(steps),
           "f_index": npf(hw.f_index).astype(np.int64),
           "ncm": npf(sim.no_collision_mask).astype(np.uint8),
           "nsm": npf(sim.no_streaming_mask).astype(np.uint8)}
    if global_extra is not None:
        out["global_extra"] = global_extra
    if inlet:
        b = flow.bnds[0]
        out["inlet_u_lu"] = npf(flow.units.convert_velocity_to_lu(b.velocity))
        out["inlet_rho_lu"] = npf(flow.units.convert_pressure_pu_to_density_lu(b.pressure))
    forces = []
    for _ in range(steps):
        sim(1)
        forces.append(npf(hw.force_sum))
    out["force"] = np.array(forces)
    out["f"] = npf(flow.f)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res, "collision": coll,
                              "periodicity": None if periodicity is None else list(periodicity),
                              "inlet": bool(inlet)})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def case_ibb(name, stencil, res, coll, steps, seed, solid, periodicity=None):
    """lettuce's example linear interpolated bounce-back (Bouzidi et al.;
    examples/advanced_projects/efficient_bounce_back_obstacle/boundary/
    linear_interpolated_bounce_back_boundary.py) under the example's
    EbbSimulation, with the momentum-exchange force after every step. The
    links are the halfway bounce-back's neighbour search of the same solid;
    each gets a wall distance drawn uniformly from [0.05, 0.95] by
    numpy.random.default_rng(seed) after the populations, links with
    d < 0.5 going to f_index_lt / d_lt and the others to f_index_gt / d_gt."""
    import lettuce
    root = os.path.dirname(os.path.dirname(os.path.abspath(lettuce.__file__)))
    for sub in ("boundary", "simulation"):
        d = os.path.join(root, EBB, sub)
        if d not in sys.path:
            sys.path.insert(0, d)
    from halfway_bounce_back_boundary import HalfwayBounceBackBoundary
    from linear_interpolated_bounce_back_boundary import LinearInterpolatedBounceBackBoundary
    from solid_boundary_data import SolidBoundaryData
    from ebb_simulation import EbbSimulation

    class IbbFlow(GivenFlow):
        psb = []

        @property
        def post_streaming_boundaries(self):
            return self.psb

    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.2 * rng.standard_normal([st.q] + res))
    flow = IbbFlow(st, f0)
    flow.context.d = st.d  # see case_hwbb
    sbd = SolidBoundaryData()
    sbd.solid_mask = solid
    links = npf(HalfwayBounceBackBoundary(CTX, flow, sbd, periodicity=periodicity).f_index)
    dist = rng.uniform(0.05, 0.95, size=len(links))
    lt_ = dist < 0.5
    sbd = SolidBoundaryData()
    sbd.solid_mask = solid
    sbd.f_index_lt, sbd.f_index_gt = links[lt_], links[~lt_]
    sbd.d_lt, sbd.d_gt = dist[lt_], dist[~lt_]
    ibb = LinearInterpolatedBounceBackBoundary(CTX, flow, sbd, calc_force=True)
    flow.psb = [ibb]
    tau = 0.8
    sim = EbbSimulation(flow, collision_of(coll, tau), [])
    out = {"f0": f0, "solid": solid, "tau": np.float64(tau), "steps": np.int64(steps),
           "f_index_lt": sbd.f_index_lt.astype(np.int64), "f_index_gt": sbd.f_index_gt.astype(np.int64),
           "d_lt": sbd.d_lt, "d_gt": sbd.d_gt,
           "ncm": npf(sim.no_collision_mask).astype(np.uint8),
           "nsm": npf(sim.no_streaming_mask).astype(np.uint8)}
    forces = []
    for _ in range(steps):
        sim(1)
        forces.append(npf(ibb.force_sum))
    out["force"] = np.array(forces)
    out["f"] = npf(flow.f)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res, "collision": coll,
                              "periodicity": None if periodicity is None else list(periodicity),
                              "inlet": False})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def ibb_cases():
    g = np.meshgrid(np.arange(20), np.arange(12), indexing="ij")
    solid = (g[0] - 8.0) ** 2 + (g[1] - 5.5) ** 2 < 3.1 ** 2
    case_ibb("ibb_d2q9_bgk", D2Q9, [20, 12], "bgk", 6, 90, solid)
    g = np.meshgrid(np.arange(10), np.arange(8), np.arange(6), indexing="ij")
    solid = (g[0] - 4.5) ** 2 + (g[1] - 3.5) ** 2 + (g[2] - 2.5) ** 2 < 2.3 ** 2
    case_ibb("ibb_d3q19_trt", D3Q19, [10, 8, 6], "trt", 4, 91, solid,
             periodicity=(False, True, True))


def case_fwbb(name, stencil, res, coll, steps, seed, solid, periodicity=None,
              global_extra=None):
    """lettuce's example post-streaming full-way bounce-back
    (examples/advanced_projects/efficient_bounce_back_obstacle/boundary/
    fullway_bounce_back_boundary.py) under the example's EbbSimulation, with
    its momentum-exchange force after every step; ``global_extra`` is a
    second solid region given through ``global_solid_mask``."""
    import lettuce
    root = os.path.dirname(os.path.dirname(os.path.abspath(lettuce.__file__)))
    for sub in ("boundary", "simulation"):
        d = os.path.join(root, EBB, sub)
        if d not in sys.path:
            sys.path.insert(0, d)
    from fullway_bounce_back_boundary import FullwayBounceBackBoundary
    from ebb_simulation import EbbSimulation

    class FwbbFlow(GivenFlow):
        psb = []

        @property
        def post_streaming_boundaries(self):
            return self.psb

    st = stencil()
    rng = np.random.default_rng(seed)
    w = np.array(st.w).reshape([-1] + [1] * len(res))
    f0 = w * (1.0 + 0.2 * rng.standard_normal([st.q] + res))
    flow = FwbbFlow(st, f0)
    gmask = None if global_extra is None else (solid | global_extra)
    fw = FullwayBounceBackBoundary(CTX, flow, solid, global_solid_mask=gmask,
                                   periodicity=periodicity, calc_force=True)
    flow.psb = [fw]
    tau = 0.8
    sim = EbbSimulation(flow, collision_of(coll, tau), [])
    out = {"f0": f0, "solid": solid, "tau": np.float64(tau), "steps": np.int64(steps),
           "f_index": npf(fw.f_index_fwbb).astype(np.int64),
           "ncm": npf(sim.no_collision_mask).astype(np.uint8),
           "nsm": npf(sim.no_streaming_mask).astype(np.uint8)}
    if global_extra is not None:
        out["global_extra"] = global_extra
    forces = []
    for _ in range(steps):
        sim(1)
        forces.append(npf(fw.force_sum))
    out["force"] = np.array(forces)
    out["f"] = npf(flow.f)
    out["meta"] = json.dumps({"stencil": stencil.__name__, "res": res, "collision": coll,
                              "periodicity": None if periodicity is None else list(periodicity),
                              "inlet": False})
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)


def fwbb_cases():
    g = np.meshgrid(np.arange(22), np.arange(12), indexing="ij")
    solid = (g[0] - 9.0) ** 2 + (g[1] - 5.5) ** 2 < 3.3 ** 2
    solid[0, 2:4] = True
    solid[21, 7:9] = True
    case_fwbb("fwbb_d2q9_bgk", D2Q9, [22, 12], "bgk", 6, 95, solid)
    solid = np.zeros([9, 7, 6], dtype=bool)
    solid[2:5, 2:5, 1:4] = True
    extra = np.zeros_like(solid)
    extra[5:7, 2:4, 1:3] = True
    case_fwbb("fwbb_d3q19_trt", D3Q19, [9, 7, 6], "trt", 4, 96, solid,
              periodicity=(False, True, True), global_extra=extra)


def hwbb_cases():
    # a disc inside a non-periodic 2-D box, and two blocks on the x = 0 and
    # x = 23 columns: the neighbour search wraps negative indices (Python
    # indexing) and drops those past the end
    g = np.meshgrid(np.arange(24), np.arange(14), indexing="ij")
    solid = (g[0] - 10.0) ** 2 + (g[1] - 6.5) ** 2 < 3.2 ** 2
    solid[0, 3:6] = True
    solid[23, 8:10] = True
    case_hwbb("hwbb_d2q9_bgk", D2Q9, [24, 14], "bgk", 6, 80, solid)
    # a sphere, periodic along z, behind an equilibrium inlet (mask index of
    # the post-streaming boundary after the ordinary boundaries)
    g = np.meshgrid(np.arange(12), np.arange(8), np.arange(6), indexing="ij")
    solid = (g[0] - 5.0) ** 2 + (g[1] - 3.5) ** 2 + (g[2] - 2.5) ** 2 < 2.2 ** 2
    case_hwbb("hwbb_d3q19_trt", D3Q19, [12, 8, 6], "trt", 4, 81, solid,
              periodicity=(False, False, True), inlet=True)
    # a cube touching y = 0 with y periodic, next to a second solid region
    # given only through global_solid_mask
    solid = np.zeros([8, 6, 5], dtype=bool)
    solid[2:5, 0:2, 1:4] = True
    extra = np.zeros_like(solid)
    extra[5:7, 0:2, 1:3] = True
    case_hwbb("hwbb_d3q27_bgk", D3Q27, [8, 6, 5], "bgk", 3, 82, solid,
              periodicity=(True, True, False), global_extra=extra)


def main():
    torch.set_num_threads(os.cpu_count() or 1)
    if "--only-hwbb" in sys.argv:
        hwbb_cases()
        return
    if "--only-ibb" in sys.argv:
        ibb_cases()
        return
    if "--only-fwbb" in sys.argv:
        fwbb_cases()
        return
    case_tgv("tgv2d_d2q9_bgk", D2Q9, 16, 1000, "bgk", 5)
    case_tgv("tgv2d_d2q9_trt", D2Q9, [16, 12], 300, "trt", 5)
    case_tgv("tgv2d_d2q9_kbc", D2Q9, 16, 1000, "kbc", 5)
    case_tgv("tgv3d_d3q19_bgk", D3Q19, 8, 1600, "bgk", 3)
    case_tgv("tgv3d_d3q27_kbc", D3Q27, 8, 1600, "kbc", 3)
    seed = 0
    for stencil, res in [(D1Q3, [13]), (D2Q9, [7, 5]), (D3Q15, [5, 4, 3]),
                         (D3Q19, [5, 4, 3]), (D3Q27, [5, 4, 3])]:
        colls = ["bgk", "trt", "none"]
        if stencil in (D2Q9, D3Q27):
            colls.append("kbc")
        for coll in colls:
            case_random(f"random_{stencil.__name__.lower()}_{coll}", stencil,
                        res, coll, 2, seed)
            seed += 1
    case_obstacle("obstacle2d_d2q9_bgk", D2Q9, [32, 16], 3.0, "bgk", 10)
    case_obstacle("obstacle3d_d3q27_kbc", D3Q27, [24, 8, 8], 2.0, "kbc", 3)
    case_eqpu_field("eqpu_field_d2q9")
    case_outlet_p("outletp_d2q9_bgk", D2Q9, [32, 16], 3.0, 1.0, 10)
    case_outlet_p("outletp_d3q19_bgk", D3Q19, [20, 8, 8], 2.0, 1.01, 4)
    case_psm("psm_d2q9_bgk", D2Q9, [20, 16], 0.4, 5, 21)
    case_psm("psm_d3q19_bgk", D3Q19, [9, 8, 7], 0.7, 3, 22)
    for stencil, res, seed0 in [(D2Q9, [7, 6], 40), (D3Q19, [5, 4, 4], 50),
                                (D3Q27, [4, 4, 3], 60)]:
        for k, kind in enumerate(["regularized", "smagorinsky", "smagorinsky_guo", "bgk_guo",
                                  "bgk_shanchen"]):
            case_collision_ext(f"ext_{stencil.__name__.lower()}_{kind}", stencil, res, kind, 3,
                               seed0 + k)
    from lettuce.util.moments import D2Q9Dellar, D2Q9Lallemand, D3Q27Hermite
    case_mrt("mrt_d2q9_lallemand", D2Q9, D2Q9Lallemand, [7, 6], 3, 70)
    case_mrt("mrt_d2q9_dellar", D2Q9, D2Q9Dellar, [7, 6], 3, 71)
    case_mrt("mrt_d3q27_hermite", D3Q27, D3Q27Hermite, [4, 4, 3], 3, 72)
    case_poiseuille("poiseuille_guo", "guo", 300)
    case_poiseuille("poiseuille_shanchen", "shan_chen", 300)
    case_dump()
    hwbb_cases()
    ibb_cases()
    fwbb_cases()
    case_native_kats()
    case_observables()
    case_adjoint()
    if "--no-energy" not in sys.argv:
        case_tgv_energy_decay()
    print("golden vectors written to", OUT)


if __name__ == "__main__":
    main()
