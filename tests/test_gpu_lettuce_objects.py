"""lettuce's own Simulation objects stepping on the kernels, on the GPU.

lettuce itself (its install in ``baseline/_ref``, or ``$LETTUCE_SRC``) builds
each simulation of ``tests/lettuce_cases.py`` twice on cuda:0: one steps on
lettuce's own torch path (``Simulation.__call__`` over its
``_collide_and_stream``, lettuce/_simulation.py:128-166 and 311-323), the
other through the same ``__call__`` after ``lettuce_gb300.install``, which
makes the assignment lettuce makes for its own native module
(lettuce/_simulation.py:229). From the same initial field, after the same
steps, the two fields agree to float64 / float32 rounding: every streaming
strategy, BGK (with Guo and Shan-Chen forces), TRT, KBC, regularized,
Smagorinsky, MRT, no collision, bounce-back, equilibrium inlet,
anti-bounce-back and pressure outlets, partially saturated cells, a
pre-collision boundary."""
import warnings

import pytest
import torch

import lettuce_gb300 as lt
from lettuce_cases import cases, import_lettuce
from lgb_helpers import rel_max, to_np

pytestmark = pytest.mark.gpu
STEPS = 6
TOL = {torch.float64: 1e-11, torch.float32: 5e-5}


@pytest.fixture
def lettuce(monkeypatch):
    L = import_lettuce()
    if L is None:
        pytest.skip("lettuce is not importable (install it in baseline/_ref or set LETTUCE_SRC)")
    # lettuce's Obstacle multiplies a CPU unit vector with its mask
    # (lettuce/ext/_flows/obstacle.py:94-99, 123-124); the mask starts on the
    # CPU (obstacle.py:63) but the setter puts it on the context's device, so
    # on a CUDA context the initialize() after setting a mask is refused by
    # torch. The unit vector is put where the mask is, the only change to
    # lettuce's objects.
    unit = L.Obstacle._unit_vector
    monkeypatch.setattr(L.Obstacle, "_unit_vector",
                        lambda self, i=0: unit(self, i).to(self._mask.device))
    return L


def _build(L, dtype):
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ctx = L.Context(device=torch.device("cuda:0"), dtype=dtype, use_native=False)
        return cases(L, ctx)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32], ids=["f64", "f32"])
def test_lettuce_simulations_step_on_the_kernels(lgb, lettuce, dtype):
    theirs, ours = _build(lettuce, dtype), _build(lettuce, dtype)
    errs = {}
    for name, a in theirs.items():
        b = ours[name]
        assert type(b).__module__.startswith("lettuce"), type(b)
        assert torch.equal(a.flow.f, b.flow.f), name
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            a(STEPS)
            invoke = lt.install(b)
            b(STEPS)
        torch.cuda.synchronize()
        assert b._collide_and_stream is invoke
        assert int(invoke.status.item()) == 0, name
        assert b.flow.i == STEPS
        errs[name] = rel_max(to_np(b.flow.f), to_np(a.flow.f))
    bad = {k: v for k, v in errs.items() if not v < TOL[dtype]}
    assert not bad, (bad, errs)
