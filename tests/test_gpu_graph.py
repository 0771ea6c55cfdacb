"""CUDA-graph replay inside ``Simulation``: a captured pair of steps replayed
between reporter firings must give the same populations, bit for bit, as
launching every step from Python, for every streaming strategy, both memory
patterns, shifted storage and masked boundaries; reporters still see the
steps at which their interval fires."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden, meta
from lgb_helpers import obstacle_flow

pytestmark = pytest.mark.gpu

S = lt.StreamingStrategy


def tgv(dtype=torch.float32, storage=None, n=32):
    ctx = lt.Context("cuda:0", dtype, storage=storage)
    return lt.TaylorGreenVortex(ctx, [n, n, 16], 1600, 0.05, lt.D3Q19)


def run(make_flow, steps_list, use_graph, reporters=(), **kw):
    flow = make_flow()
    sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu),
                        list(reporters), use_graph=use_graph, **kw)
    for n in steps_list:
        sim(n)
    torch.cuda.synchronize()
    return flow.f.detach().clone(), flow.i


@pytest.mark.parametrize("strategy", [S.POST_STREAMING, S.PRE_STREAMING, S.DOUBLE_STREAMING])
def test_graph_replay_bit_identical_ab(lgb, strategy):
    a, ia = run(tgv, [1, 7, 10, 3], False, streaming_strategy=strategy)
    b, ib = run(tgv, [1, 7, 10, 3], True, streaming_strategy=strategy)
    assert ia == ib == 21
    assert torch.equal(a, b)


@pytest.mark.parametrize("storage", [None, "fp16_shifted"])
def test_graph_replay_bit_identical_aa(lgb, storage):
    mk = lambda: tgv(storage=storage)  # noqa: E731
    a, _ = run(mk, [5, 9, 2], False, memory_pattern="aa")
    b, _ = run(mk, [5, 9, 2], True, memory_pattern="aa")
    assert torch.equal(a, b)


def test_graph_replay_with_boundaries(lgb):
    z = golden("obstacle2d_d2q9_bgk")
    m = meta(z)
    mk = lambda: obstacle_flow(lt.Context("cuda:0", torch.float64), z, m)  # noqa: E731
    a, _ = run(mk, [13, 6], False)
    b, _ = run(mk, [13, 6], True)
    assert torch.equal(a, b)


def test_graph_reporters_fire_at_their_interval(lgb):
    def make():
        flow = tgv()
        rep = lt.ObservableReporter(lt.MaximumVelocity(flow), interval=5, out=None)
        return flow, rep

    flow_e, rep_e = make()
    sim_e = lt.Simulation(flow_e, lt.BGKCollision(flow_e.units.relaxation_parameter_lu),
                          [rep_e], use_graph=False)
    sim_e(23)
    flow_g, rep_g = make()
    sim_g = lt.Simulation(flow_g, lt.BGKCollision(flow_g.units.relaxation_parameter_lu),
                          [rep_g], use_graph=True)
    sim_g(23)
    assert [r[0] for r in rep_g.out] == [0, 5, 10, 15, 20]
    assert np.array_equal(np.array(rep_e.out), np.array(rep_g.out))
    assert torch.equal(flow_e.f, flow_g.f)


def test_graph_default_off_with_reporters(lgb):
    flow = tgv()
    rep = lt.ObservableReporter(lt.MaximumVelocity(flow), interval=1, out=None)
    sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [rep])
    assert not sim._graphs_enabled()
    sim(3)
    assert [r[0] for r in rep.out] == [0, 1, 2, 3]
    sim2 = lt.Simulation(tgv(), lt.BGKCollision(0.6), [])
    assert sim2._graphs_enabled()


def test_graph_with_post_as_pull_and_reporters(lgb):
    """POST_STREAMING as pull steps, replayed from graphs, with a reporter
    every 10 steps (each report applies the pending stream): the same
    populations and reports as the push kernels launched step by step"""
    outs, reps = [], []
    for use_graph, pap in ((False, False), (True, True)):
        flow = tgv()
        rep = lt.ObservableReporter(lt.IncompressibleKineticEnergy(flow), interval=10, out=None)
        sim = lt.Simulation(flow, lt.BGKCollision(flow.units.relaxation_parameter_lu), [rep],
                            streaming_strategy=S.POST_STREAMING, use_graph=use_graph,
                            post_as_pull=pap)
        assert sim._pull_post == pap
        sim(47)
        outs.append(flow.f.clone())
        reps.append(np.array(rep.out))
    assert torch.equal(outs[0], outs[1])
    assert np.array_equal(reps[0], reps[1]) and len(reps[0]) == 5
