"""Parity of the CUDA step with lettuce (golden vectors) and with the CPU
oracle, through the public API and the C ABI.

Tolerances (``tol`` below): float64 kernels against lettuce's float64 step,
max relative error <= 1e-12 (round-off of a different summation order);
float32 kernels against float64 references, max relative error <= 2e-6 per
10 steps of accumulated float32 rounding, 1e-5 per 10 steps for KBC, whose
stabiliser gamma divides two small sums and amplifies the rounding.

KBC on a field whose non-shear non-equilibrium part is zero (the first
collision after lettuce's fneq initialisation of a Taylor-Green vortex) is
not compared: there delta_h is pure round-off (|delta_h| ~ 1e-17,
sum(delta_h^2/feq) ~ 1e-33), so gamma is a ratio of rounding noise in
lettuce's formula (kbc_collision.py:149-158) and any two implementations
differ at the size of delta_s."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden, golden_names, meta
from lgb_helpers import (GivenFlow, collision_of, obstacle_flow, obstacle_oracle_boundaries,
                         rel_l2, rel_max, to_np)

pytestmark = pytest.mark.gpu

STRATS = {"PRE_STREAMING": lt.StreamingStrategy.PRE_STREAMING,
          "POST_STREAMING": lt.StreamingStrategy.POST_STREAMING}
F64 = torch.float64
F32 = torch.float32


def ctx(dtype=F64, storage=None):
    return lt.Context("cuda:0", dtype, storage=storage)


def tol(dtype, collision, steps):
    if dtype == F64:
        return 1e-12
    return (1e-5 if collision == "kbc" else 2e-6) * max(1.0, steps / 10)


@pytest.mark.parametrize("name", golden_names("random_"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_random_fields_match_lettuce(lgb, name, strategy, dtype):
    z = golden(name)
    m = meta(z)
    S = getattr(lt, m["stencil"])
    flow = GivenFlow(ctx(dtype), S(), z["f0"])
    coll = collision_of(m["collision"], float(z["tau"]))
    if m["collision"] == "kbc":
        coll.bind = lambda fl, c=coll: setattr(c, "tau", float(z["tau"]))
    sim = lt.Simulation(flow, coll, [], streaming_strategy=STRATS[strategy])
    sim(int(z["steps"]))
    err = rel_max(to_np(flow.f), z[f"f_{strategy}"])
    assert err < tol(dtype, m["collision"], int(z["steps"])), err


@pytest.mark.parametrize("name", golden_names("tgv"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_taylor_green_matches_lettuce(lgb, name, strategy, dtype):
    if "energy" in name:
        pytest.skip("energy series is checked in test_energy_decay")
    z = golden(name)
    m = meta(z)
    if m["collision"] == "kbc" and strategy == "POST_STREAMING":
        pytest.skip("first KBC collision on the fneq-initialised TGV is ill-conditioned")
    S = getattr(lt, m["stencil"])
    res = m["res"]
    flow = lt.TaylorGreenVortex(ctx(dtype), res, m["re"], m["ma"], S)
    assert rel_max(to_np(flow.f), z["f0"]) < (1e-13 if dtype == F64 else 1e-6)
    flow.f = torch.as_tensor(z["f0"])
    coll = collision_of(m["collision"], float(z["tau"]))
    sim = lt.Simulation(flow, coll, [], streaming_strategy=STRATS[strategy])
    sim(int(z["steps"]))
    err = rel_max(to_np(flow.f), z[f"f_{strategy}"])
    assert err < tol(dtype, m["collision"], int(z["steps"])), err


@pytest.mark.parametrize("name", golden_names("obstacle"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_obstacle_matches_lettuce(lgb, name, strategy, dtype):
    z = golden(name)
    m = meta(z)
    flow = obstacle_flow(ctx(dtype), z, m)
    coll = lt.KBCCollision() if m["collision"] == "kbc" else \
        lt.BGKCollision(flow.units.relaxation_parameter_lu)
    sim = lt.Simulation(flow, coll, [], streaming_strategy=STRATS[strategy])
    assert np.array_equal(to_np(sim.no_collision_mask), z["ncm"])
    sim(int(z["steps"]))
    err = rel_max(to_np(flow.f), z[f"f_{strategy}"])
    assert err < tol(dtype, m["collision"], int(z["steps"])), err


@pytest.mark.parametrize("strategy", list(STRATS))
def test_equilibrium_boundary_field(lgb, strategy):
    z = golden("eqpu_field_d2q9")
    c = ctx()
    flow = GivenFlow(c, lt.D2Q9(), z["f0"])
    b = lt.EquilibriumBoundaryPU(c, flow, torch.tensor(z["mask"]).cuda(),
                                 torch.tensor(z["velocity_pu"]), float(z["pressure_pu"]))
    flow._bnds = [b]
    sim = lt.Simulation(flow, lt.BGKCollision(float(z["tau"])), [],
                        streaming_strategy=STRATS[strategy])
    sim(int(z["steps"]))
    assert rel_max(to_np(flow.f), z[f"f_{strategy}"]) < 1e-12


def test_native_known_answers(lgb):
    """lettuce tests/native/test_native_streaming.py and
    test_native_bounce_back.py: bit-exact (NoCollision moves values only)"""
    z = golden("native_kats")
    for dtype in (F64, F32):
        flow = GivenFlow(ctx(dtype), lt.D2Q9(), z["stream_f0"])
        lt.Simulation(flow, lt.NoCollision(), [])(1)
        assert np.array_equal(to_np(flow.f), z["stream_f1"])
        for steps, key in [(1, "bb_f1"), (2, "bb_f2")]:
            flow = GivenFlow(ctx(dtype), lt.D2Q9(), z["bb_f0"])
            flow._bnds = [lt.BounceBackBoundary(torch.tensor(z["bb_mask"]).cuda())]
            lt.Simulation(flow, lt.NoCollision(), [])(steps)
            assert np.array_equal(to_np(flow.f), z[key])


# -- differential tests against the CPU oracle at larger, odd-sized grids ----

ORACLE_CASES = [
    # stencil, resolution, collision, strategy, steps
    ("D3Q19", [24, 20, 18], "bgk", "PRE_STREAMING", 60),
    ("D3Q19", [17, 9, 33], "trt", "POST_STREAMING", 40),
    ("D3Q27", [12, 10, 14], "kbc", "PRE_STREAMING", 30),
    ("D3Q15", [9, 11, 7], "bgk", "POST_STREAMING", 30),
    ("D2Q9", [70, 51], "trt", "PRE_STREAMING", 80),
    ("D2Q9", [33, 40], "kbc", "POST_STREAMING", 50),
    ("D1Q3", [129], "bgk", "PRE_STREAMING", 50),
    ("D2Q9", [30, 20], "bgk", "DOUBLE_STREAMING", 20),
    ("D3Q19", [8, 9, 10], "bgk", "NO_STREAMING", 10),
    # degenerate extents: a dimension of one or two cells wraps onto itself
    ("D3Q19", [1, 5, 7], "bgk", "PRE_STREAMING", 6),
    ("D3Q19", [4, 1, 2], "trt", "POST_STREAMING", 6),
    ("D3Q27", [2, 3, 1], "kbc", "PRE_STREAMING", 4),
    ("D2Q9", [1, 1], "bgk", "POST_STREAMING", 5),
    ("D2Q9", [2, 3], "trt", "PRE_STREAMING", 5),
    ("D1Q3", [1], "bgk", "PRE_STREAMING", 5),
    ("D1Q3", [2], "trt", "POST_STREAMING", 5),
]


def _tgv_like(name, res, seed):
    e, w, _ = __import__("oracle.oracle", fromlist=["x"]).stencil_tables(name)
    rng = np.random.default_rng(seed)
    d = len(res)
    grids = np.meshgrid(*[np.arange(n) * 2 * np.pi / n for n in res], indexing="ij")
    u = np.stack([0.04 * np.sin(grids[(i + 1) % d] + i) for i in range(d)])
    u += 0.005 * rng.standard_normal(u.shape)
    rho = 1 + 0.01 * rng.standard_normal(res)
    eu = np.einsum("qd,d...->q...", e, u)
    uu = np.sum(u * u, axis=0)
    return w.reshape([-1] + [1] * d) * rho * (1 + 3 * eu + 4.5 * eu ** 2 - 1.5 * uu)


@pytest.mark.parametrize("case", ORACLE_CASES, ids=lambda c: f"{c[0]}-{c[2]}-{c[3]}")
@pytest.mark.parametrize("dtype", [F64, F32])
def test_against_oracle(lgb, oracle, case, dtype):
    name, res, coll, strategy, steps = case
    f0 = _tgv_like(name, res, 3)
    tau = 0.55
    flow = GivenFlow(ctx(dtype), getattr(lt, name)(), f0)
    c = collision_of(coll, tau)
    if coll == "kbc":
        c.bind = lambda fl, c=c: setattr(c, "tau", tau)
    sim = lt.Simulation(flow, c, [], streaming_strategy=getattr(lt.StreamingStrategy, strategy))
    sim(steps)
    ref = oracle.run(name, f0, steps, collision=coll, tau=tau, tau_minus=1.0, strategy=strategy)
    err = rel_max(to_np(flow.f), ref)
    assert err < tol(dtype, coll, steps), err


def test_obstacle_3d_kbc_against_oracle(lgb, oracle):
    """config-3 physics at reduced size: D3Q27 KBC, sphere bounce-back,
    equilibrium inlet, anti-bounce-back outlet, float32, 40 steps"""
    res = [48, 16, 16]
    for strategy in STRATS:
        flow = lt.Obstacle(ctx(F32), res, 300, 0.0866, res[0] / 6.0, stencil=lt.D3Q27)
        g = np.meshgrid(*[np.arange(n) for n in res], indexing="ij")
        mask = ((g[0] - 12) ** 2 + (g[1] - 7.5) ** 2 + (g[2] - 7.5) ** 2) < 9
        flow.mask = mask
        flow.initialize()
        f0 = to_np(flow.f)
        sim = lt.Simulation(flow, lt.KBCCollision(), [], streaming_strategy=STRATS[strategy])
        inlet = sim._natives[1]
        sim(40)
        z = {"inlet_rho_lu": to_np(inlet.rho), "inlet_u_lu": to_np(inlet.u), "mask": mask}
        post = obstacle_oracle_boundaries(z, {"res": res})
        ref = oracle.run("D3Q27", f0, 40, collision="kbc",
                         tau=flow.units.relaxation_parameter_lu, strategy=strategy, post=post)
        assert rel_max(to_np(flow.f), ref) < tol(F32, "kbc", 40)


@pytest.mark.parametrize("dtype,storage", [(F64, None), (F32, None), (F32, "fp16_shifted"),
                                           (F32, "bf16_shifted")])
def test_aa_pattern_equals_push(lgb, dtype, storage):
    """the in-place AA pattern (even/odd pair) is bit-identical to two
    push (POST_STREAMING) steps, for an even and an odd step count"""
    for steps in (6, 7):
        fa = lt.TaylorGreenVortex(ctx(dtype, storage), [20, 18, 16], 1600, 0.05, lt.D3Q19)
        fb = lt.TaylorGreenVortex(ctx(dtype, storage), [20, 18, 16], 1600, 0.05, lt.D3Q19)
        tau = fa.units.relaxation_parameter_lu
        lt.Simulation(fa, lt.BGKCollision(tau), [], memory_pattern="aa")(steps)
        lt.Simulation(fb, lt.BGKCollision(tau), [])(steps)
        assert fa._aa_pending == (steps % 2 == 1)
        # moments read the AA-pending layout directly
        assert torch.equal(fa.rho(), fb.rho()) and torch.equal(fa.u(), fb.u())
        assert torch.equal(fa.f, fb.f)


def test_aa_pattern_with_bounce_back(lgb):
    z = golden("native_kats")
    mask = torch.tensor(z["bb_mask"]).cuda()
    f0 = golden("random_d2q9_bgk")["f0"]
    f0 = np.tile(f0, (1, 3, 4))[:, :16, :16]
    fa = GivenFlow(ctx(), lt.D2Q9(), f0, [lt.BounceBackBoundary(mask)])
    fb = GivenFlow(ctx(), lt.D2Q9(), f0, [lt.BounceBackBoundary(mask)])
    lt.Simulation(fa, lt.BGKCollision(0.7), [], memory_pattern="aa")(9)
    lt.Simulation(fb, lt.BGKCollision(0.7), [])(9)
    assert torch.equal(fa.f, fb.f)


def test_moments_match_lettuce(lgb):
    z = golden("observables")
    for tag, S in [("2d", lt.D2Q9), ("3d", lt.D3Q19)]:
        flow = GivenFlow(ctx(), S(), z[f"{tag}_f"])
        assert rel_max(to_np(flow.rho()), z[f"{tag}_rho"]) < 1e-14
        assert rel_max(to_np(flow.u()), z[f"{tag}_u"]) < 1e-12


def test_status_word_flags_non_finite(lgb):
    f0 = golden("random_d2q9_bgk")["f0"].copy()
    f0[3, 2, 1] = np.nan
    flow = GivenFlow(ctx(), lt.D2Q9(), f0)
    sim = lt.Simulation(flow, lt.BGKCollision(0.7), [])
    sim(1)
    assert sim.status & 1
    flow2 = GivenFlow(ctx(), lt.D2Q9(), golden("random_d2q9_bgk")["f0"])
    sim2 = lt.Simulation(flow2, lt.BGKCollision(0.7), [])
    sim2(3)
    assert sim2.status == 0


def test_convert_round_trip(lgb):
    from lettuce_gb300 import _device, _lib
    f = torch.as_tensor(golden("tgv3d_d3q19_bgk")["f0"], dtype=F32).cuda().contiguous()
    n = f[0].numel()
    h = torch.empty(f.shape, dtype=torch.float16, device="cuda")
    _device.convert(_lib.D3Q19, f, _lib.F32, h, _lib.F16_SHIFTED, n)
    w = torch.tensor(lt.D3Q19().w, dtype=F32, device="cuda").view(-1, 1, 1, 1)
    assert torch.equal(h, (f - w).to(torch.float16))
    back = torch.empty_like(f)
    _device.convert(_lib.D3Q19, h, _lib.F16_SHIFTED, back, _lib.F32, n)
    assert torch.equal(back, h.to(F32) + w)


def test_invalid_configuration_raises_through_abi(lgb):
    from lettuce_gb300 import _lib
    flow = lt.TaylorGreenVortex(ctx(), [8, 8, 8], 100, 0.05, lt.D3Q19)
    sim = lt.Simulation(flow, lt.BGKCollision(0.6), [])
    sim._desc.tau = -1.0
    with pytest.raises(_lib.LibraryError, match="relaxation time"):
        sim(1)
    sim._desc.tau = 0.6
    sim(1)  # the context is still usable
    assert torch.isfinite(flow.f).all()


@pytest.mark.parametrize("storage", ["fp16_shifted", "bf16_shifted"])
@pytest.mark.parametrize("S,res,coll", [(lt.D3Q19, [12, 10, 16], "bgk"),
                                        (lt.D2Q9, [30, 24], "trt"),
                                        (lt.D3Q27, [6, 8, 10], "bgk")])
@pytest.mark.parametrize("pattern", ["pull", "push", "aa"])
def test_two_cell_kernel_bit_identical(lgb, storage, S, res, coll, pattern):
    """the two-cells-per-thread kernel of the 16-bit formats (packed f32x2
    arithmetic) gives exactly the one-cell kernel's populations"""
    from lettuce_gb300 import _lib
    out = []
    for options in (0, _lib.OPT_ONE_CELL):
        flow = lt.TaylorGreenVortex(ctx(F32, storage), res, 300, 0.05, S)
        tau = flow.units.relaxation_parameter_lu
        c = lt.BGKCollision(tau) if coll == "bgk" else lt.TRTCollision(tau, 0.8)
        kw = {"memory_pattern": "aa"} if pattern == "aa" else {
            "streaming_strategy": lt.StreamingStrategy.PRE_STREAMING if pattern == "pull"
            else lt.StreamingStrategy.POST_STREAMING, "post_as_pull": False}
        sim = lt.Simulation(flow, c, [], **kw)
        sim._desc.options = options
        sim(7)
        out.append(flow.f.clone())
    assert torch.equal(out[0], out[1])


@pytest.mark.parametrize("res", [[3, 1, 2], [1, 1, 2], [2, 2, 2]])
@pytest.mark.parametrize("pattern", ["pull", "push", "aa"])
def test_two_cell_kernel_tiny_rows(lgb, res, pattern):
    """rows of two cells (one pair per row: the shifted pair wraps onto
    itself) give the same populations in the two-cell and one-cell kernels"""
    from lettuce_gb300 import _lib
    f0 = _tgv_like("D3Q19", res, 5)
    outs = []
    for one_cell in (False, True):
        c = lt.Context("cuda:0", F32, storage="fp16_shifted")
        flow = GivenFlow(c, lt.D3Q19(), f0)
        kw = ({"memory_pattern": "aa"} if pattern == "aa" else
              {"streaming_strategy": STRATS["PRE_STREAMING" if pattern == "pull"
                                            else "POST_STREAMING"], "post_as_pull": False})
        sim = lt.Simulation(flow, lt.BGKCollision(0.6), [], use_graph=False, **kw)
        if one_cell:
            sim._desc.options |= _lib.OPT_ONE_CELL
        sim(5)
        outs.append(flow.f_raw.clone())
    assert torch.equal(outs[0], outs[1])


def test_shifted_storage_matches_f32_closely(lgb, oracle):
    """fp16-shifted D2Q9 TRT against the float64 oracle: within the fp16
    storage precision (2^-11 of the largest deviation per step)"""
    f0 = _tgv_like("D2Q9", [64, 48], 4)
    flow = GivenFlow(ctx(F32, "fp16_shifted"), lt.D2Q9(), f0)
    lt.Simulation(flow, lt.TRTCollision(0.6, 0.9), [], lt.StreamingStrategy.PRE_STREAMING)(20)
    ref = oracle.run("D2Q9", f0, 20, collision="trt", tau=0.6, tau_minus=0.9,
                     strategy="PRE_STREAMING")
    w = np.array(lt.D2Q9().w).reshape(-1, 1, 1)
    hmax = np.max(np.abs(ref - w))
    assert np.max(np.abs(to_np(flow.f) - ref)) < 20 * hmax * 2.0 ** -11


class _ObstacleP(lt.Obstacle):
    """an obstacle flow with lettuce's pressure outlet instead of the
    anti-bounce-back outlet"""
    rho_outlet = 1.0

    @property
    def post_boundaries(self):
        b = lt.Obstacle.post_boundaries.fget(self)
        return [b[0], lt.EquilibriumOutletP(self._unit_vector().tolist(), self,
                                            rho_outlet=self.rho_outlet), b[2]]


@pytest.mark.parametrize("name", golden_names("outletp"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_pressure_outlet_matches_lettuce(lgb, name, strategy, dtype):
    z = golden(name)
    m = meta(z)
    S = getattr(lt, m["stencil"])
    _ObstacleP.rho_outlet = m["rho_outlet"]
    flow = _ObstacleP(ctx(dtype), m["res"], m["re"], m["ma"], m["domain_length_x"], stencil=S)
    flow.mask = z["mask"]
    flow.initialize()
    sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [],
                        streaming_strategy=STRATS[strategy])
    assert np.array_equal(to_np(sim.no_collision_mask), z["ncm"])
    assert np.array_equal(to_np(sim.no_streaming_mask), z["nsm"])
    sim(int(z["steps"]))
    assert rel_max(to_np(flow.f), z[f"f_{strategy}"]) < tol(dtype, "bgk", int(z["steps"]))


@pytest.mark.parametrize("name", golden_names("psm"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_partially_saturated_matches_lettuce(lgb, name, strategy, dtype):
    z = golden(name)
    m = meta(z)
    S = getattr(lt, m["stencil"])
    flow = GivenFlow(ctx(dtype), S(), z["f0"])
    b = lt.PartiallySaturatedBC(torch.tensor(z["mask"]).cuda(), float(z["tau"]),
                                float(z["saturation"]))
    assert abs(b.B - float(z["B"])) < 1e-15
    flow._bnds = [b]
    sim = lt.Simulation(flow, lt.BGKCollision(float(z["tau"])), [],
                        streaming_strategy=STRATS[strategy])
    sim(int(z["steps"]))
    assert rel_max(to_np(flow.f), z[f"f_{strategy}"]) < tol(dtype, "bgk", int(z["steps"]))


@pytest.mark.parametrize("name", golden_names("obstacle") + golden_names("outletp"))
def test_push_guard_bit_identical(lgb, name):
    """the push-guard flag bit (only cells next to a non-streaming population
    look at their destinations' bits) changes no result"""
    z = golden(name)
    m = meta(z)
    outs = []
    for guard in (True, False):
        if name.startswith("outletp"):
            _ObstacleP.rho_outlet = m["rho_outlet"]
            flow = _ObstacleP(ctx(F64), m["res"], m["re"], m["ma"], m["domain_length_x"],
                              stencil=getattr(lt, m["stencil"]))
            flow.mask = z["mask"]
            flow.initialize()
        else:
            flow = obstacle_flow(ctx(F64), z, m)
        coll = lt.KBCCollision() if m["collision"] == "kbc" else \
            lt.BGKCollision(flow.units.relaxation_parameter_lu)
        sim = lt.Simulation(flow, coll, [], streaming_strategy=lt.StreamingStrategy.POST_STREAMING,
                            post_as_pull=False)
        from lettuce_gb300 import _lib
        assert sim._desc.options & _lib.OPT_PUSH_GUARD
        if not guard:
            sim._desc.options &= ~_lib.OPT_PUSH_GUARD
        sim(7)
        outs.append(flow.f_raw.clone())
    assert torch.equal(outs[0], outs[1])


def _ext_collision(kind, flow, z, m):
    tau = float(z["tau"])
    ftau = float(z["force_tau"])
    accel = z["accel"].tolist()
    c = m["smagorinsky_constant"]
    if kind == "regularized":
        return lt.RegularizedCollision(tau)
    if kind == "smagorinsky":
        return lt.SmagorinskyCollision(tau, smagorinsky_constant=c)
    if kind == "smagorinsky_guo":
        return lt.SmagorinskyCollision(tau, smagorinsky_constant=c,
                                       force=lt.Guo(flow, ftau, accel))
    if kind == "bgk_guo":
        return lt.BGKCollision(tau, force=lt.Guo(flow, ftau, accel))
    return lt.BGKCollision(tau, force=lt.ShanChen(flow, ftau, accel))


@pytest.mark.parametrize("name", golden_names("ext_"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_forces_and_collisions_match_lettuce(lgb, name, strategy, dtype):
    """regularized, Smagorinsky, and forced BGK / Smagorinsky kernels against
    lettuce (float64 golden, random populations, 3 steps)"""
    z = golden(name)
    m = meta(z)
    S = getattr(lt, m["stencil"])
    flow = GivenFlow(ctx(dtype), S(), z["f0"])
    sim = lt.Simulation(flow, _ext_collision(m["kind"], flow, z, m), [],
                        streaming_strategy=STRATS[strategy])
    sim(int(z["steps"]))
    err = rel_max(to_np(flow.f), z[f"f_{strategy}"])
    assert err < (1e-12 if dtype == F64 else 2e-6), err


@pytest.mark.parametrize("name", golden_names("poiseuille"))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_poiseuille_force_matches_lettuce(lgb, name, dtype):
    """lettuce's forced Poiseuille channel (tests/collision/test_force.py
    set-up) for 300 steps: populations against lettuce's float64 run"""
    z = golden(name)
    m = meta(z)
    flow = lt.PoiseuilleFlow2D(ctx(dtype), 17, 1, 0.02, initialize_with_zeros=True)
    a = flow.units.convert_acceleration_to_lu(flow.acceleration)
    tau = flow.units.relaxation_parameter_lu
    F = lt.Guo if m["force"] == "guo" else lt.ShanChen
    sim = lt.Simulation(flow, lt.BGKCollision(tau, force=F(flow, tau, a)), [])
    assert np.array_equal(to_np(sim.no_collision_mask), z["ncm"])
    sim(int(z["steps"]))
    err = rel_max(to_np(flow.f), z["f_final"])
    assert err < (1e-11 if dtype == F64 else 1e-5), err
    if dtype == F64:
        # in float32 the per-step forcing (~1e-9 against populations ~0.4)
        # is below the storage's resolution, for lettuce as here: only the
        # float64 velocity is compared
        u = to_np(flow.u(acceleration=a))
        assert rel_max(u, z["u_final"]) < 1e-9


@pytest.mark.parametrize("force", ["guo", "shan_chen"])
def test_poiseuille_force_reaches_analytic_profile(lgb, force):
    """lettuce tests/collision/test_force.py: after 1000 steps the forced
    channel's velocity matches the analytic parabola within 1 % of its
    maximum on the fluid cells"""
    flow = lt.PoiseuilleFlow2D(ctx(F64), 17, 1, 0.02, initialize_with_zeros=True)
    a = flow.units.convert_acceleration_to_lu(flow.acceleration)
    tau = flow.units.relaxation_parameter_lu
    F = lt.Guo if force == "guo" else lt.ShanChen
    sim = lt.Simulation(flow, lt.BGKCollision(tau, force=F(flow, tau, a)), [])
    sim(1000)
    u_sim = flow.units.convert_velocity_to_pu(flow.u(acceleration=a))
    _, u_ref = flow.analytic_solution()
    fluid = to_np(sim.no_collision_mask) == 0
    for d in range(2):
        us, ur = to_np(u_sim[d])[fluid], to_np(u_ref[d])[fluid]
        assert us.max() == pytest.approx(ur.max(), rel=0.01)
        assert np.max(np.abs(us - ur)) <= 0.01 * to_np(u_ref[0]).max()


def test_forced_fp16_storage(lgb):
    """a forced Taylor-Green run in fp16-shifted storage stays within the
    storage's rounding of the float32 run"""
    outs = []
    for storage in (None, "fp16_shifted"):
        flow = lt.TaylorGreenVortex(lt.Context("cuda:0", F32, storage=storage), [32, 32, 16],
                                    400, 0.05, lt.D3Q19)
        tau = flow.units.relaxation_parameter_lu
        sim = lt.Simulation(flow, lt.BGKCollision(tau, force=lt.Guo(flow, tau, [1e-5, 0, 0])), [])
        sim(50)
        outs.append(to_np(flow.u()))
    assert rel_l2(outs[1], outs[0]) < 5e-3


@pytest.mark.parametrize("name", golden_names("mrt_"))
@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [F64, F32])
def test_mrt_matches_lettuce(lgb, name, strategy, dtype):
    """MRT kernels (Lallemand, Dellar, Hermite bases) against lettuce"""
    z = golden(name)
    m = meta(z)
    S = getattr(lt, m["stencil"])
    c = ctx(dtype)
    flow = GivenFlow(c, S(), z["f0"])
    T = getattr(lt, m["transform"])
    coll = lt.MRTCollision(T(S(), c), z["relaxation"].tolist(), c)
    sim = lt.Simulation(flow, coll, [], streaming_strategy=STRATS[strategy])
    sim(int(z["steps"]))
    err = rel_max(to_np(flow.f), z[f"f_{strategy}"])
    assert err < (1e-12 if dtype == F64 else 5e-6), err


def test_mrt_generic_equilibrium_d1q3(lgb):
    """the generic MRT equilibrium (moments of feq(rho, u)) with the D1Q3
    basis: one kernel collision against its torch restatement. (lettuce's
    own Transform.equilibrium raises a TypeError at moments.py:101, so there
    is no lettuce vector for it.)"""
    c = ctx(F64)
    rng = np.random.default_rng(9)
    w = np.array(lt.D1Q3().w).reshape(-1, 1)
    f0 = w * (1 + 0.2 * rng.standard_normal([3, 11]))
    flow = GivenFlow(c, lt.D1Q3(), f0)
    t = lt.D1Q3Transform(lt.D1Q3(), c)
    srel = [1.0, 0.7, 0.9]
    got = to_np(lt.MRTCollision(t, srel, c)(flow))
    f = torch.tensor(f0, dtype=F64, device="cuda")
    mm = t.transform(f)
    meq = t.equilibrium(mm, flow)
    s = torch.tensor(srel, dtype=F64, device="cuda")[:, None]
    ref = to_np(t.inverse_transform(mm - (mm - meq) / s))
    assert np.max(np.abs(got - ref)) < 1e-14


@pytest.mark.parametrize("name", golden_names("obstacle") + golden_names("outletp"))
def test_collide_and_stream_halves(lgb, name):
    """Simulation._collide() then _stream() (lettuce/_simulation.py:245-305)
    equals a POST_STREAMING step, _stream() then _collide() a PRE_STREAMING
    step, bit for bit, with every boundary of the flow"""
    z = golden(name)
    m = meta(z)

    def make():
        if name.startswith("outletp"):
            _ObstacleP.rho_outlet = m["rho_outlet"]
            flow = _ObstacleP(ctx(F64), m["res"], m["re"], m["ma"], m["domain_length_x"],
                              stencil=getattr(lt, m["stencil"]))
            flow.mask = z["mask"]
            flow.initialize()
            return flow
        return obstacle_flow(ctx(F64), z, m)

    for strategy, halves in [("POST_STREAMING", ("_collide", "_stream")),
                             ("PRE_STREAMING", ("_stream", "_collide"))]:
        a, b = make(), make()
        coll = (lambda fl: lt.KBCCollision()) if m.get("collision") == "kbc" else \
            (lambda fl: lt.BGKCollision(fl.units.relaxation_parameter_lu))
        sa = lt.Simulation(a, coll(a), [], streaming_strategy=STRATS[strategy], use_graph=False)
        sb = lt.Simulation(b, coll(b), [], streaming_strategy=STRATS[strategy])
        sa(3)
        for _ in range(3):
            for h in halves:
                getattr(sb, h)()
        assert torch.equal(a.f, b.f), strategy


@pytest.mark.parametrize("name", golden_names("obstacle") + golden_names("outletp"))
def test_post_as_pull_bit_identical(lgb, name):
    """POST_STREAMING run as a collide-only launch plus pull steps (the
    stream applied when the field is read) equals the push kernels bit for
    bit, with every boundary of the flow; reporters with short intervals
    switch it off, long ones keep it"""
    z = golden(name)
    m = meta(z)

    def make():
        if name.startswith("outletp"):
            _ObstacleP.rho_outlet = m["rho_outlet"]
            flow = _ObstacleP(ctx(F32), m["res"], m["re"], m["ma"], m["domain_length_x"],
                              stencil=getattr(lt, m["stencil"]))
            flow.mask = z["mask"]
            flow.initialize()
            return flow
        return obstacle_flow(ctx(F32), z, m)

    def coll(fl):
        return lt.KBCCollision() if m.get("collision") == "kbc" else \
            lt.BGKCollision(fl.units.relaxation_parameter_lu)

    post = lt.StreamingStrategy.POST_STREAMING
    a, b = make(), make()
    sa = lt.Simulation(a, coll(a), [], streaming_strategy=post, post_as_pull=False)
    sb = lt.Simulation(b, coll(b), [], streaming_strategy=post, post_as_pull=True)
    assert sb._pull_post and not sa._pull_post
    # the automatic choice: pull for KBC, push for masked BGK
    auto = lt.Simulation(make(), coll(b), [], streaming_strategy=post)
    assert auto._pull_post == (m.get("collision") == "kbc")
    sa(9)
    sb(9)
    assert b._stream_pending is not None
    assert torch.equal(a.f, b.f) and b._stream_pending is None
    # observables read through the pending stream
    sa(5)
    sb(5)
    assert torch.equal(lt.IncompressibleKineticEnergy(b)(), lt.IncompressibleKineticEnergy(a)())
    # a reporter every step switches the mode off; every 10 steps keeps it
    for iv, expect in ((1, False), (10, True)):
        c = make()
        rep = lt.ObservableReporter(lt.MaximumVelocity(c), interval=iv, out=None)
        sc = lt.Simulation(c, coll(c), [rep], streaming_strategy=post, post_as_pull=True)
        assert sc._pull_post == expect
        sc(20)
        d = make()
        lt.Simulation(d, coll(d), [], streaming_strategy=post, post_as_pull=False)(20)
        assert torch.equal(c.f, d.f)


@pytest.mark.parametrize("storage", [None, "fp16_shifted"])
def test_post_as_pull_periodic(lgb, storage):
    """the same on a periodic Taylor-Green vortex (two-cell kernel for fp16)"""
    outs = []
    for pap in (False, True):
        flow = lt.TaylorGreenVortex(ctx(F32, storage), [24, 20, 16], 400, 0.05, lt.D3Q19)
        lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [],
                      streaming_strategy=lt.StreamingStrategy.POST_STREAMING,
                      post_as_pull=pap)(11)
        outs.append(flow.f.clone())
    assert torch.equal(outs[0], outs[1])


def test_double_streaming_with_force(lgb, oracle):
    """DOUBLE_STREAMING (pull, then a collision-free stream) with a forced
    collision: the stream launch runs as a plain stream"""
    z = golden("ext_d2q9_bgk_guo")
    m = meta(z)
    flow = GivenFlow(ctx(F64), lt.D2Q9(), z["f0"])
    coll = _ext_collision("bgk_guo", flow, z, m)
    lt.Simulation(flow, coll, [], streaming_strategy=lt.StreamingStrategy.DOUBLE_STREAMING)(3)
    ref = oracle.run("D2Q9", z["f0"], 3, collision="bgk", tau=float(z["tau"]),
                     strategy="DOUBLE_STREAMING", force="guo", force_tau=float(z["force_tau"]),
                     accel=z["accel"])
    assert rel_max(to_np(flow.f), ref) < 1e-12
