"""The D3Q27 KBC channel flow past a sphere (lettuce's Obstacle with
EquilibriumBoundaryPU inlet, AntiBounceBackOutlet and BounceBackBoundary,
lettuce/ext/_flows/obstacle.py:54-122) at the sizes its parity contract
names, float32 on the GPU against the float64 oracle:

* a 128x32x32 channel with a sphere of diameter 6 (the 512x128x128 case
  scaled by 1/4), 50 steps, PRE and POST streaming;
* the full 512x128x128 channel with the sphere of diameter 24, 5 steps.

Both check lettuce's masks bit for bit first: the no-collision index field
and the no-streaming mask the Simulation assembled (as
lettuce/_simulation.py:100-146 does) against the oracle's restatement, and
the packed flag byte / no-streaming word against them. Populations are held
to the float32 KBC tolerance of the parity suite (1e-5 relative per 10
steps, at least 1e-5)."""
import math

import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from lgb_helpers import obstacle_oracle_boundaries, rel_max, to_np

pytestmark = pytest.mark.gpu


def channel_with_sphere(context, g):
    """the KBC sphere channel scaled by g/256: [2g, g/2, g/2] cells, sphere of
    diameter 24 g/256 centred at x = g/2 on the channel axis, Re 300 on the
    diameter, inlet velocity 0.05 in lattice units"""
    res = [2 * g, g // 2, g // 2]
    flow = lt.Obstacle(context, res, 300, 0.05 * math.sqrt(3), res[0] / (24 * g / 256),
                       stencil=lt.D3Q27)
    grid = np.meshgrid(*[np.arange(n) for n in res], indexing="ij", sparse=True)
    r = 12.0 * g / 256
    centre = [g / 2, (res[1] - 1) / 2, (res[2] - 1) / 2]
    mask = sum((x - c) ** 2 for x, c in zip(grid, centre)) < r * r
    flow.mask = mask
    flow.initialize()
    return flow, mask


def _check_masks(oracle, sim, mask, res):
    inlet = sim._natives[1]
    z = {"inlet_rho_lu": to_np(inlet.rho), "inlet_u_lu": to_np(inlet.u), "mask": mask}
    post = obstacle_oracle_boundaries(z, {"res": res})
    ncm, nsm = oracle.assemble_masks(res, 27, "D3Q27", [], post)
    assert np.array_equal(sim.no_collision_mask.cpu().numpy(), ncm)
    assert np.array_equal(sim.no_streaming_mask.cpu().numpy(), nsm)
    flags = sim._flags.cpu().numpy()
    assert np.array_equal(flags & lt._lib.FLAG_INDEX_MASK, ncm)
    keep = nsm == 1
    keep[0] = False
    has = keep.any(axis=0)
    assert np.array_equal((flags & lt._lib.FLAG_NO_STREAM) != 0, has)
    bits = sim._nsb.cpu().numpy().view(np.uint32)
    want = np.zeros(res, dtype=np.uint32)
    for q in range(1, 27):
        want |= keep[q].astype(np.uint32) << np.uint32(q)
    assert np.array_equal(bits, want)
    return post


@pytest.mark.parametrize("strategy", ["PRE_STREAMING", "POST_STREAMING"])
def test_quarter_scale_channel_50_steps(lgb, oracle, strategy):
    flow, mask = channel_with_sphere(lt.Context("cuda:0", torch.float32), 64)
    assert flow.resolution == [128, 32, 32] and int(mask.sum()) > 0
    f0 = to_np(flow.f).astype(np.float64)
    sim = lt.Simulation(flow, lt.KBCCollision(), [],
                        streaming_strategy=getattr(lt.StreamingStrategy, strategy))
    post = _check_masks(oracle, sim, mask, flow.resolution)
    sim(50)
    ref = oracle.run("D3Q27", f0, 50, collision="kbc", tau=flow.units.relaxation_parameter_lu,
                     strategy=strategy, post=post)
    assert sim.status == 0
    err = rel_max(to_np(flow.f), ref)
    assert err < 5e-5, err


def test_full_channel_5_steps(lgb, oracle):
    flow, mask = channel_with_sphere(lt.Context("cuda:0", torch.float32), 256)
    assert flow.resolution == [512, 128, 128]
    f0 = to_np(flow.f).astype(np.float64)
    sim = lt.Simulation(flow, lt.KBCCollision(), [],
                        streaming_strategy=lt.StreamingStrategy.PRE_STREAMING)
    post = _check_masks(oracle, sim, mask, flow.resolution)
    sim(5)
    ref = oracle.run("D3Q27", f0, 5, collision="kbc", tau=flow.units.relaxation_parameter_lu,
                     strategy="PRE_STREAMING", post=post)
    assert sim.status == 0
    err = rel_max(to_np(flow.f), ref)
    assert err < 1e-5, err


def test_anti_bounce_back_outlet_onset_is_lettuces(lgb, oracle):
    """With lettuce's anti-bounce-back outlet this channel does not stay
    finite: lettuce's algorithm (the float64 oracle) grows a disturbance next
    to the outlet plane from about step 400 and overflows within 600 steps
    at this size. The float64 kernels follow the oracle through the onset
    (450 steps: the largest velocity, one plane inside the outlet, already
    above 1.5 times the inlet's), so the divergence the 5000-step run reports
    is the configuration's, not the kernels'."""
    flow, mask = channel_with_sphere(lt.Context("cuda:0", torch.float64), 64)
    f0 = to_np(flow.f)
    sim = lt.Simulation(flow, lt.KBCCollision(), [],
                        streaming_strategy=lt.StreamingStrategy.PRE_STREAMING)
    inlet = sim._natives[1]
    z = {"inlet_rho_lu": to_np(inlet.rho), "inlet_u_lu": to_np(inlet.u), "mask": mask}
    post = obstacle_oracle_boundaries(z, {"res": flow.resolution})
    sim(450)
    ref = oracle.run("D3Q27", f0, 450, collision="kbc", tau=flow.units.relaxation_parameter_lu,
                     strategy="PRE_STREAMING", post=post)
    got = to_np(flow.f)
    assert rel_max(got, ref) < 1e-8
    _, u = oracle.moments("D3Q27", ref)
    speed = np.sqrt((u * u).sum(axis=0))
    at = np.unravel_index(np.argmax(speed), speed.shape)
    assert speed.max() > 1.5 * 0.05 and at[0] >= flow.resolution[0] - 8, (speed.max(), at)


def test_pressure_outlet_channel_5000_steps_and_drag(lgb):
    """The full 512x128x128 channel with lettuce's pressure outlet
    (EquilibriumOutletP, rho 1; obstacle.py:119-120) in place of the
    anti-bounce-back outlet runs the configuration's 5000 steps with the
    status word clear and the mass kept to 1e-4; with the sphere as the
    example project's halfway bounce-back its drag coefficient at step 5000
    lies in the range of a confined sphere at Re 300 (0.5 - 1.2; the
    unconfined value is about 0.66) and the lift is small."""
    import math
    from lettuce_gb300._reporter import reduce_flow

    class ObstacleP(lt.Obstacle):
        @property
        def post_boundaries(self):
            b = lt.Obstacle.post_boundaries.fget(self)
            return [b[0], lt.EquilibriumOutletP(self._unit_vector().tolist(), self,
                                                rho_outlet=1.0), b[2]]

    class EbbObstacleP(ObstacleP):
        psb = ()

        @property
        def post_streaming_boundaries(self):
            return list(self.psb)

    g = 256
    res = [2 * g, g // 2, g // 2]
    grid = np.meshgrid(*[np.arange(n) for n in res], indexing="ij", sparse=True)
    centre = [g / 2, (res[1] - 1) / 2, (res[2] - 1) / 2]
    solid = sum((x - c) ** 2 for x, c in zip(grid, centre)) < 12.0 ** 2
    ctx = lt.Context("cuda:0", torch.float32)
    flow = ObstacleP(ctx, res, 300, 0.05 * math.sqrt(3), res[0] / 24.0, stencil=lt.D3Q27)
    flow.mask = solid
    flow.initialize()
    sim = lt.Simulation(flow, lt.KBCCollision(), [],
                        streaming_strategy=lt.StreamingStrategy.PRE_STREAMING)
    m0 = reduce_flow(flow).cpu().numpy()
    sim(5000)
    m1 = reduce_flow(flow).cpu().numpy()
    assert sim.status == 0 and m1[3] == 0
    assert abs(m1[0] / m0[0] - 1) < 1e-4
    assert np.sqrt(m1[2]) < 0.1
    del sim, flow

    flow = EbbObstacleP(ctx, res, 300, 0.05 * math.sqrt(3), res[0] / 24.0, stencil=lt.D3Q27)
    flow.initialize()
    sbd = lt.SolidBoundaryData()
    sbd.solid_mask = solid
    b = lt.HalfwayBounceBackBoundary(ctx, flow, sbd, calc_force=True)
    flow.psb = [b]
    sim = lt.EbbSimulation(flow, lt.KBCCollision(), [])
    sim(5000)
    assert sim.status == 0
    area_pu = math.pi * 0.5 ** 2
    cd = float(lt.DragCoefficient(flow, b, solid, area_pu)())
    cl = float(lt.LiftCoefficient(flow, b, solid, area_pu)())
    assert 0.5 < cd < 1.2, cd
    assert abs(cl) < 0.1 * cd, cl
