"""native_invoke on the GPU: the ``invoke(simulation)`` lettuce would install
at lettuce/_simulation.py:229, driving lgb_step from a Simulation's own
attributes (flow.f / flow.f_next, collision, boundaries, lettuce's masks,
streaming strategy) and swapping the fields as lettuce/cuda_native/
_template.py:35-40 does. lettuce cannot be imported where the GPU runs, so the
simulations are this package's mirror objects, which carry the same
attributes (tests/test_lettuce_binding.py checks that lettuce's own objects
give the same descriptors); the results are held to lettuce's golden runs
and to the oracle."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden, meta
from lgb_helpers import obstacle_flow, obstacle_oracle_boundaries, rel_max, to_np

pytestmark = pytest.mark.gpu
STRATS = {"PRE_STREAMING": lt.StreamingStrategy.PRE_STREAMING,
          "POST_STREAMING": lt.StreamingStrategy.POST_STREAMING}


def _run_installed(sim, steps):
    """lettuce's Simulation.__call__ loop body (lettuce/_simulation.py:311-323)
    over the installed step"""
    invoke = lt.install(sim)
    for _ in range(steps):
        sim._collide_and_stream(sim)
        sim.flow.i += 1
    torch.cuda.synchronize()
    return invoke


@pytest.mark.parametrize("strategy", list(STRATS))
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_obstacle_through_binding(lgb, strategy, dtype):
    z = golden("obstacle3d_d3q27_kbc")
    m = meta(z)
    flow = obstacle_flow(lt.Context("cuda:0", dtype), z, m)
    sim = lt.Simulation(flow, lt.KBCCollision(), [], streaming_strategy=STRATS[strategy])
    invoke = _run_installed(sim, int(z["steps"]))
    err = rel_max(to_np(flow.f), z[f"f_{strategy}"])
    assert err < (1e-12 if dtype == torch.float64 else 2e-5), err
    assert int(invoke.status.item()) == 0


@pytest.mark.parametrize("strategy", list(STRATS))
def test_taylor_green_through_binding(lgb, strategy):
    z = golden("tgv3d_d3q19_bgk")
    m = meta(z)
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", torch.float64), m["res"], m["re"], m["ma"],
                                lt.D3Q19)
    flow.f = torch.as_tensor(z["f0"])
    sim = lt.Simulation(flow, lt.BGKCollision(float(z["tau"])), [],
                        streaming_strategy=STRATS[strategy])
    _run_installed(sim, int(z["steps"]))
    assert rel_max(to_np(flow.f), z[f"f_{strategy}"]) < 1e-12


@pytest.mark.parametrize("strategy", ["DOUBLE_STREAMING", "NO_STREAMING"])
def test_obstacle_2d_strategies_against_oracle(lgb, oracle, strategy):
    z = golden("obstacle2d_d2q9_bgk")
    m = meta(z)
    flow = obstacle_flow(lt.Context("cuda:0", torch.float64), z, m)
    f0 = to_np(flow.f)
    tau = flow.units.relaxation_parameter_lu
    sim = lt.Simulation(flow, lt.BGKCollision(tau), [],
                        streaming_strategy=getattr(lt.StreamingStrategy, strategy))
    _run_installed(sim, 7)
    ref = oracle.run("D2Q9", f0, 7, collision="bgk", tau=tau, strategy=strategy,
                     post=obstacle_oracle_boundaries(z, m))
    assert rel_max(to_np(flow.f), ref) < 1e-12


def test_invoke_refuses_a_replaced_field(lgb):
    flow = lt.TaylorGreenVortex(lt.Context("cuda:0", torch.float32), [16, 16], 100, 0.05, lt.D2Q9)
    sim = lt.Simulation(flow, lt.BGKCollision(0.6), [])
    invoke = lt.native_invoke(sim)
    invoke(sim)
    flow.f = torch.zeros(9, 16, 8, device="cuda:0")
    with pytest.raises(RuntimeError, match="rebuild the step"):
        invoke(sim)
