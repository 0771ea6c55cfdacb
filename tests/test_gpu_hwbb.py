"""Halfway bounce-back (the post-streaming boundary of lettuce's example
project, run by ``EbbSimulation``) through the step kernel's pull: the
populations after every step and the momentum-exchange force of each step
against the golden vectors of the example itself (float64), against the
oracle in float32 and 16-bit storage, graph replay against eager steps, and
a reporter that reads the force while the stream is pending."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden, golden_names, meta
from lgb_helpers import hwbb_case, rel_max, to_np

pytestmark = pytest.mark.gpu

CASES = golden_names("hwbb_")


def _sim(z, m, dtype=torch.float64, storage=None, use_graph=False, f0=None):
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    flow, hw = hwbb_case(ctx, z, m, f0=f0)
    coll = lt.TRTCollision(float(z["tau"]), 1.0) if m["collision"] == "trt" else \
        lt.BGKCollision(float(z["tau"]))
    return lt.EbbSimulation(flow, coll, [], use_graph=use_graph), flow, hw


@pytest.mark.parametrize("name", CASES)
def test_f64_matches_example_step_by_step(lgb, name):
    z = golden(name)
    m = meta(z)
    sim, flow, hw = _sim(z, m)
    forces = []
    for _ in range(int(z["steps"])):
        sim(1)
        forces.append(to_np(hw.force_sum))
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.array(forces), z["force"], rtol=0, atol=1e-12)
    assert sim.status == 0


@pytest.mark.parametrize("name", CASES)
def test_f64_graph_run_matches_example(lgb, name):
    """all steps in one call (collide-only launch, pull launches from a
    captured graph, the last stream pending until read)"""
    z = golden(name)
    m = meta(z)
    sim, flow, hw = _sim(z, m, use_graph=True)
    sim(int(z["steps"]))
    assert flow._stream_pending is not None
    np.testing.assert_allclose(to_np(hw.force_sum), z["force"][-1], rtol=0, atol=1e-12)
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("storage,tol", [(None, 2e-6), ("fp16_shifted", 2e-3),
                                         ("bf16_shifted", 1.5e-2)])
def test_reduced_precision_against_oracle(lgb, oracle, storage, tol):
    z = golden("hwbb_d3q19_trt")
    m = meta(z)
    steps = 12
    forces = np.zeros((steps, 3))
    from test_hwbb_cpu import _post
    ref = oracle.run(m["stencil"], z["f0"].astype(np.float32), steps, collision="trt",
                     tau=float(z["tau"]), tau_minus=1.0, post=_post(z, m),
                     post_streaming=[dict(solid=z["solid"], f_index=z["f_index"])],
                     forces=forces)
    sim, flow, hw = _sim(z, m, torch.float32, storage, use_graph=True,
                         f0=z["f0"].astype(np.float32))
    sim(steps)
    assert rel_max(to_np(flow.f), ref) < tol
    assert rel_max(to_np(hw.force_sum), forces[-1]) < 20 * tol


def test_eager_and_graph_runs_identical(lgb):
    z = golden("hwbb_d3q27_bgk")
    m = meta(z)
    a, fa, ha = _sim(z, m, torch.float32, use_graph=False, f0=z["f0"].astype(np.float32))
    b, fb, hb = _sim(z, m, torch.float32, use_graph=True, f0=z["f0"].astype(np.float32))
    a(11)
    b(11)
    assert torch.equal(fa.f, fb.f)
    assert torch.equal(ha.force_sum, hb.force_sum)


def test_force_reporter_reads_each_step(lgb):
    """a reporter reading the force every 3 steps sees the example's force of
    that step (the read applies the pending stream and bounce)"""
    z = golden("hwbb_d2q9_bgk")
    m = meta(z)
    seen = {}

    class ForceReporter(lt.Reporter):
        def __call__(self, simulation):
            if simulation.flow.i % self.interval == 0 and simulation.flow.i > 0:
                seen[simulation.flow.i] = to_np(hw.force_sum)

    ctx = lt.Context("cuda:0", torch.float64)
    flow, hw = hwbb_case(ctx, z, m)
    sim = lt.EbbSimulation(flow, lt.BGKCollision(float(z["tau"])), [ForceReporter(3)],
                           use_graph=True)
    sim(6)
    assert sorted(seen) == [3, 6]
    for i, F in seen.items():
        np.testing.assert_allclose(F, z["force"][i - 1], rtol=0, atol=1e-12)
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)


def test_stream_half_alone_bounces(lgb):
    """lettuce's collide and stream halves called directly reproduce the
    step (the stream half carries the bounce)"""
    z = golden("hwbb_d2q9_bgk")
    m = meta(z)
    sim, flow, hw = _sim(z, m)
    for _ in range(int(z["steps"])):
        sim._collide()
        sim._stream()
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(to_np(hw.force_sum), z["force"][-1], rtol=0, atol=1e-12)


# -- the linear interpolated bounce-back of the same project ----------------

IBB_CASES = golden_names("ibb_")


def _ibb_sim(z, m, dtype=torch.float64, storage=None, use_graph=False, f0=None):
    from lgb_helpers import ibb_case
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    flow, b = ibb_case(ctx, z, m, f0=f0)
    coll = lt.TRTCollision(float(z["tau"]), 1.0) if m["collision"] == "trt" else \
        lt.BGKCollision(float(z["tau"]))
    return lt.EbbSimulation(flow, coll, [], use_graph=use_graph), flow, b


@pytest.mark.parametrize("name", IBB_CASES)
def test_ibb_f64_matches_example_step_by_step(lgb, name):
    z = golden(name)
    m = meta(z)
    sim, flow, b = _ibb_sim(z, m)
    forces = []
    for _ in range(int(z["steps"])):
        sim(1)
        forces.append(to_np(b.force_sum))
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.array(forces), z["force"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("name", IBB_CASES)
def test_ibb_f64_graph_run_matches_example(lgb, name):
    z = golden(name)
    m = meta(z)
    sim, flow, b = _ibb_sim(z, m, use_graph=True)
    sim(int(z["steps"]))
    np.testing.assert_allclose(to_np(b.force_sum), z["force"][-1], rtol=0, atol=1e-12)
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("storage,tol", [(None, 2e-6), ("fp16_shifted", 2e-3)])
def test_ibb_reduced_precision_against_oracle(lgb, oracle, storage, tol):
    z = golden("ibb_d3q19_trt")
    m = meta(z)
    steps = 10
    forces = np.zeros((steps, 3))
    rows = np.concatenate([z["f_index_lt"], z["f_index_gt"]])
    dist = np.concatenate([z["d_lt"], z["d_gt"]]).astype(np.float32)
    ref = oracle.run(m["stencil"], z["f0"].astype(np.float32), steps, collision="trt",
                     tau=float(z["tau"]), tau_minus=1.0,
                     post_streaming=[dict(solid=z["solid"], f_index=rows, d=dist)],
                     forces=forces)
    sim, flow, b = _ibb_sim(z, m, torch.float32, storage, use_graph=True,
                            f0=z["f0"].astype(np.float32))
    sim(steps)
    assert rel_max(to_np(flow.f), ref) < tol
    assert rel_max(to_np(b.force_sum), forces[-1]) < 50 * tol


def test_halfway_and_interpolated_together(lgb, oracle):
    """two post-streaming boundaries on separate solids, a halfway one and
    an interpolated one that computes the force, against the oracle"""
    zh = golden("hwbb_d2q9_bgk")
    st = lt.D2Q9()
    g = np.meshgrid(np.arange(24), np.arange(14), indexing="ij")
    solid_i = (g[0] - 18.0) ** 2 + (g[1] - 6.5) ** 2 < 2.2 ** 2
    assert not np.any(solid_i & zh["solid"])
    both = zh["solid"] | solid_i
    rows_i = lt.hwbb_links(st.e, st.opposite, solid_i, both)
    d_i = np.random.default_rng(3).uniform(0.05, 0.95, len(rows_i))
    small = d_i < 0.5
    ctx = lt.Context("cuda:0", torch.float64)
    from lgb_helpers import HwbbFlow
    flow = HwbbFlow(ctx, st, zh["f0"])
    sh = lt.SolidBoundaryData()
    sh.solid_mask = zh["solid"]
    hw = lt.HalfwayBounceBackBoundary(ctx, flow, sh, global_solid_mask=both)
    si = lt.SolidBoundaryData()
    si.solid_mask = solid_i
    si.f_index_lt, si.f_index_gt = rows_i[small], rows_i[~small]
    si.d_lt, si.d_gt = d_i[small], d_i[~small]
    ib = lt.LinearInterpolatedBounceBackBoundary(ctx, flow, si, calc_force=True)
    flow.psb = [hw, ib]
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.8), [], use_graph=True)
    steps = 7
    sim(steps)
    forces = np.zeros((steps, 3))
    ref = oracle.run("D2Q9", zh["f0"], steps, collision="bgk", tau=0.8,
                     post_streaming=[dict(solid=zh["solid"], f_index=hw.f_index.cpu().numpy(),
                                          force=False),
                                     dict(solid=solid_i,
                                          f_index=np.concatenate([rows_i[small], rows_i[~small]]),
                                          d=np.concatenate([d_i[small], d_i[~small]]))],
                     forces=forces)
    np.testing.assert_allclose(to_np(flow.f), ref, rtol=0, atol=1e-13)
    np.testing.assert_allclose(to_np(ib.force_sum), forces[-1, :2], rtol=0, atol=1e-12)
    assert sim.status == 0


# -- the post-streaming full-way bounce-back of the same project -------------

FWBB_CASES = golden_names("fwbb_")


def _fwbb_sim(z, m, dtype=torch.float64, storage=None, use_graph=False, f0=None):
    from lgb_helpers import fwbb_case
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    flow, b = fwbb_case(ctx, z, m, f0=f0)
    coll = lt.TRTCollision(float(z["tau"]), 1.0) if m["collision"] == "trt" else \
        lt.BGKCollision(float(z["tau"]))
    return lt.EbbSimulation(flow, coll, [], use_graph=use_graph), flow, b


@pytest.mark.parametrize("name", FWBB_CASES)
def test_fwbb_f64_matches_example(lgb, name):
    z = golden(name)
    m = meta(z)
    sim, flow, b = _fwbb_sim(z, m)
    forces = []
    for _ in range(int(z["steps"])):
        sim(1)
        forces.append(to_np(b.force_sum))
    np.testing.assert_allclose(to_np(flow.f), z["f"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(np.array(forces), z["force"], rtol=0, atol=1e-12)
    sim2, flow2, b2 = _fwbb_sim(z, m, use_graph=True)
    sim2(int(z["steps"]))
    np.testing.assert_allclose(to_np(flow2.f), z["f"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(to_np(b2.force_sum), z["force"][-1], rtol=0, atol=1e-12)


@pytest.mark.parametrize("storage,tol", [(None, 2e-6), ("fp16_shifted", 2e-3)])
def test_fwbb_reduced_precision_against_oracle(lgb, oracle, storage, tol):
    z = golden("fwbb_d3q19_trt")
    m = meta(z)
    steps = 10
    forces = np.zeros((steps, 3))
    ref = oracle.run(m["stencil"], z["f0"].astype(np.float32), steps, collision="trt",
                     tau=float(z["tau"]), tau_minus=1.0,
                     post_streaming=[dict(solid=z["solid"], f_index=z["f_index"],
                                          d=np.zeros(len(z["f_index"])), fullway=True)],
                     forces=forces)
    sim, flow, b = _fwbb_sim(z, m, torch.float32, storage, use_graph=True,
                             f0=z["f0"].astype(np.float32))
    sim(steps)
    assert rel_max(to_np(flow.f), ref) < tol
    assert rel_max(to_np(b.force_sum), forces[-1]) < 50 * tol


# -- links next to the anti-bounce-back outlet --------------------------------

@pytest.mark.parametrize("stencil,res,coll", [("D2Q9", [20, 10], "bgk"),
                                              ("D3Q27", [14, 6, 6], "kbc")])
def test_links_beside_the_outlet_against_oracle(lgb, oracle, stencil, res, coll):
    """an equilibrium inlet, an anti-bounce-back outlet and a halfway
    solid whose links sit on the outlet's neighbour plane and on the outlet
    plane itself (the outlet's velocity extrapolation reads bounced cells;
    the outlet-plane launch carries links), float64, against the oracle"""
    from lgb_helpers import HwbbFlow
    st = getattr(lt, stencil)()
    d = len(res)
    rng = np.random.default_rng(11)
    w = np.asarray(st.w).reshape([-1] + [1] * d)
    f0 = w * (1.0 + 0.05 * rng.standard_normal([st.q] + res))
    X = res[0]
    solid = np.zeros(res, dtype=bool)
    solid[X - 4:X - 2, 2:4] = True      # its links reach x = X - 2
    solid[X - 2, res[1] - 2] = True     # a solid cell on the neighbour plane
    inlet = np.zeros(res, dtype=bool)
    inlet[0] = True
    ctx = lt.Context("cuda:0", torch.float64)
    flow = HwbbFlow(ctx, st, f0)
    vel = torch.tensor([0.02] + [0.0] * (d - 1), dtype=torch.float64)
    eq = lt.EquilibriumBoundaryPU(ctx, flow, torch.as_tensor(inlet), vel)
    flow._bnds = [eq, lt.AntiBounceBackOutlet([1] + [0] * (d - 1), flow)]
    sbd = lt.SolidBoundaryData()
    sbd.solid_mask = solid
    hw = lt.HalfwayBounceBackBoundary(ctx, flow, sbd, calc_force=True)
    assert np.any(hw.f_index.cpu().numpy()[:, 1] == X - 1)   # links on the outlet plane
    flow.psb = [hw]
    coll_obj = lt.KBCCollision(flow.units.relaxation_parameter_lu) if coll == "kbc" \
        else lt.BGKCollision(0.7)
    tau = flow.units.relaxation_parameter_lu if coll == "kbc" else 0.7
    sim = lt.EbbSimulation(flow, coll_obj, [], use_graph=True)
    steps = 7
    sim(steps)
    nat = eq.native_generator(1)
    post = [{"kind": "equilibrium_pu", "mask": inlet,
             "rho": nat.rho.cpu().numpy().reshape([1] * d),
             "u": nat.u.cpu().numpy().reshape([d] + [1] * d)},
            {"kind": "anti_bounce_back", "direction": [1] + [0] * (d - 1)}]
    forces = np.zeros((steps, 3))
    ref = oracle.run(stencil, f0, steps, collision=coll, tau=tau, post=post,
                     post_streaming=[dict(solid=solid, f_index=hw.f_index.cpu().numpy())],
                     forces=forces)
    assert rel_max(to_np(flow.f), ref) < 1e-12
    np.testing.assert_allclose(to_np(hw.force_sum), forces[-1, :d], rtol=1e-10, atol=1e-13)


def test_drag_and_lift_coefficients(lgb):
    """the example's force coefficients from the halfway boundary's force
    and the mean fluid density, against the same formula on the example's
    own populations and force"""
    z = golden("hwbb_d2q9_bgk")
    m = meta(z)
    sim, flow, hw = _sim(z, m, use_graph=True)
    area_pu = 0.7
    cd = lt.DragCoefficient(flow, hw, z["solid"], area_pu)
    cl = lt.LiftCoefficient(flow, hw, z["solid"], area_pu)
    sim(int(z["steps"]))
    st = lt.D2Q9()
    rho = z["f"].sum(axis=0)
    rho_mean = rho[~z["solid"]].mean()
    u = flow.units
    area_lu = area_pu * (u.characteristic_length_lu / u.characteristic_length_pu)
    denom = 0.5 * rho_mean * u.characteristic_velocity_lu ** 2 * area_lu
    assert abs(cd().item() - z["force"][-1][0] / denom) < 1e-10 * abs(z["force"][-1][0] / denom)
    assert abs(cl().item() - z["force"][-1][1] / denom) < 1e-9 * abs(z["force"][-1][1] / denom) + 1e-14
    # as a reporter's observable
    rep = lt.ObservableReporter(cd, interval=2, out=None)
    sim.reporter.append(rep)
    sim(2)
    assert len(rep.out) >= 1 and np.isfinite(np.asarray(rep.out[-1][-1], dtype=float)).all()


@pytest.mark.parametrize("kind", ["halfway", "interpolated"])
def test_momentum_balance_periodic_box(lgb, kind):
    """periodic D3Q19 Taylor-Green 64^3 around a sphere, float64 BGK: the
    collision conserves momentum and the solid cells keep theirs, so over n
    steps the total momentum changes by minus the sum of the boundary's
    momentum-exchange forces"""
    from lgb_helpers import HwbbFlow
    res = [64, 64, 64]
    ctx = lt.Context("cuda:0", torch.float64)
    tgv = lt.TaylorGreenVortex(ctx, res, 400, 0.05, lt.D3Q19)
    f0 = tgv.f.cpu().numpy()
    st = lt.D3Q19()
    g = np.meshgrid(*[np.arange(k) for k in res], indexing="ij", sparse=True)
    centre = [30.3, 33.1, 31.7]
    solid = sum((gi - ci) ** 2 for gi, ci in zip(g, centre)) < 8.0 ** 2
    flow = HwbbFlow(ctx, st, f0)
    sbd = lt.SolidBoundaryData()
    sbd.solid_mask = solid
    if kind == "halfway":
        b = lt.HalfwayBounceBackBoundary(ctx, flow, sbd, periodicity=(True, True, True),
                                         calc_force=True)
    else:
        rows = lt.hwbb_links(st.e, st.opposite, solid, None, (True, True, True))
        d = np.random.default_rng(2).uniform(0.05, 0.95, len(rows))
        small = d < 0.5
        sbd.f_index_lt, sbd.f_index_gt = rows[small], rows[~small]
        sbd.d_lt, sbd.d_gt = d[small], d[~small]
        b = lt.LinearInterpolatedBounceBackBoundary(ctx, flow, sbd, calc_force=True)
    flow.psb = [b]
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.62), [])

    def total_momentum():
        return flow.j().sum(dim=(1, 2, 3)).cpu().numpy()

    j0 = total_momentum()
    fsum = np.zeros(3)
    for _ in range(20):
        sim(1)
        fsum += to_np(b.force_sum)
    dj = total_momentum() - j0
    assert np.linalg.norm(fsum) > 1e-6
    np.testing.assert_allclose(dj, -fsum, rtol=0, atol=1e-9 * np.abs(fsum).max() + 1e-12)
