"""The x-slab decomposition through the step kernel, on one GPU: the lattice
is split into parts held by one process (halo planes moved by copies), and
the reassembled parts must equal the whole-grid ``Simulation`` bit for bit,
for the pull, push and double streaming patterns, shifted 16-bit storage,
KBC, and masked boundaries (bounce-back, an equilibrium boundary with a
velocity field varying along x)."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden
from lgb_helpers import GivenFlow

pytestmark = pytest.mark.gpu

S = lt.StreamingStrategy


def tgv(dtype=torch.float32, storage=None, res=(24, 16, 10), stencil=lt.D3Q19):
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    return lt.TaylorGreenVortex(ctx, list(res), 1600, 0.05, stencil)


def compare(make_flow, make_collision, parts, strategy, steps=7, boundaries=None):
    flow_a = make_flow()
    sim = lt.Simulation(flow_a, make_collision(flow_a), [], streaming_strategy=strategy,
                        use_graph=False)
    flow_b = make_flow()
    sim_b = lt.Simulation(flow_b, make_collision(flow_b), [], streaming_strategy=strategy)
    slabs = lt.SlabSimulation(sim_b, parts)
    sim(steps)
    slabs(steps)
    torch.cuda.synchronize()
    flow_a._settle()
    whole = flow_a.f_raw
    split = slabs.gather()
    assert split.shape == whole.shape
    assert torch.equal(split, whole)
    assert slabs.status == 0


@pytest.mark.parametrize("strategy", [S.PRE_STREAMING, S.POST_STREAMING, S.DOUBLE_STREAMING])
@pytest.mark.parametrize("parts", [2, 3, 5])
def test_slabs_equal_whole_grid_f32(lgb, strategy, parts):
    compare(tgv, lambda f: lt.BGKCollision(f.units.relaxation_parameter_lu), parts, strategy)


@pytest.mark.parametrize("storage", ["fp16_shifted", "bf16_shifted"])
def test_slabs_equal_whole_grid_shifted(lgb, storage):
    compare(lambda: tgv(storage=storage),
            lambda f: lt.TRTCollision(f.units.relaxation_parameter_lu), 3, S.PRE_STREAMING)


def test_slabs_equal_whole_grid_kbc(lgb):
    compare(lambda: tgv(dtype=torch.float64, stencil=lt.D3Q27, res=(12, 8, 8)),
            lambda f: lt.KBCCollision(f.units.relaxation_parameter_lu), 2, S.POST_STREAMING)


@pytest.mark.parametrize("strategy", [S.PRE_STREAMING, S.POST_STREAMING])
def test_slabs_with_masked_boundaries(lgb, strategy):
    f0 = golden("random_d2q9_bgk")["f0"]
    f0 = np.tile(f0, (1, 3, 2))  # 21 x 10
    res = f0.shape[1:]
    rng = np.random.default_rng(5)
    bb = torch.as_tensor(rng.random(res) < 0.1)
    inlet = torch.zeros(res, dtype=torch.bool)
    inlet[:, 0] = True
    bb[:, 0] = False

    def make():
        ctx = lt.Context("cuda:0", torch.float64)
        flow = GivenFlow(ctx, lt.D2Q9(), f0)
        ux = torch.linspace(0.01, 0.05, res[0], dtype=torch.float64).view(1, -1, 1)
        vel = torch.cat([ux, torch.zeros_like(ux)], 0)
        flow._bnds = [lt.BounceBackBoundary(bb),
                      lt.EquilibriumBoundaryPU(ctx, flow, inlet, vel)]
        return flow

    compare(make, lambda f: lt.BGKCollision(0.8), 3, strategy, steps=5)


def test_slab_simulation_rejects_outlets(lgb):
    z = golden("obstacle2d_d2q9_bgk")
    from conftest import meta
    from lgb_helpers import obstacle_flow
    flow = obstacle_flow(lt.Context("cuda:0", torch.float64), z, meta(z))
    sim = lt.Simulation(flow, lt.BGKCollision(0.6), [])
    with pytest.raises(ValueError):
        lt.SlabSimulation(sim, 2)
