"""The drop-in binding for lettuce's own Simulation objects
(lettuce_gb300.native_step / native_invoke / install), without a GPU.

``tests/golden/binding_descriptors.npz`` holds what ``native_step`` built
from lettuce's objects (lettuce imported from its sources by
``tests/golden/make_binding_golden.py``): the step descriptor with its
pointers zeroed, the launch patterns, the flag byte and no-streaming word
packed from lettuce's own masks, the inlet and MRT tables. The simulations
of ``tests/lettuce_cases.py`` built from this package's mirror classes must
give the same, and the mirror's own ``Simulation`` descriptor must agree with
the binding's. With lettuce importable (its source folder in
``$LETTUCE_SRC`` or its install in ``baseline/_ref``, the stand-ins of
``tests/golden/_stubs`` for its optional imports) the binding is also run on
lettuce's objects directly."""
import os

import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import GOLDEN
from lettuce_cases import cases, desc_signature, import_lettuce, step_record

DTYPES = {"f64": torch.float64, "f32": torch.float32}


def _fixture():
    z = np.load(os.path.join(GOLDEN, "binding_descriptors.npz"))
    out = {}
    for key in z.files:
        tag, name, field = key.split("/")
        out.setdefault((tag, name), {})[field] = z[key]
    return out


def _compare(rec, ref, what):
    assert sorted(rec) == sorted(ref), (what, sorted(rec), sorted(ref))
    for k in ref:
        if k.endswith("_rho") or k.endswith("_u"):
            np.testing.assert_allclose(rec[k], ref[k], rtol=1e-15, atol=0, err_msg=f"{what} {k}")
        elif k.endswith("_mrt"):
            # the mirror derives M^-1 by inversion; lettuce tabulates it
            np.testing.assert_allclose(rec[k], ref[k], rtol=0, atol=1e-15, err_msg=f"{what} {k}")
        else:
            assert np.array_equal(rec[k], ref[k]), (what, k)


@pytest.mark.parametrize("tag", list(DTYPES))
def test_mirror_builds_lettuces_descriptors(tag):
    fx = _fixture()
    sims = cases(lt, lt.Context("cpu", DTYPES[tag]))
    assert {n for t, n in fx if t == tag} == set(sims)
    for name, sim in sims.items():
        step = lt.native_step(sim)
        _compare(step_record(step), fx[(tag, name)], f"{tag}/{name}")
        # the mirror's own Simulation packs the same descriptor
        assert desc_signature(sim._desc) == desc_signature(step.desc), name
        if sim._flags is not None:
            assert torch.equal(sim._flags, step.flags)


def _import_lettuce():
    lettuce = import_lettuce()
    if lettuce is None:
        pytest.skip("lettuce is not importable (set LETTUCE_SRC to its source folder "
                    "or install it in baseline/_ref)")
    return lettuce


@pytest.mark.parametrize("tag", list(DTYPES))
def test_binding_on_lettuce_objects(tag):
    import warnings
    lettuce = _import_lettuce()
    fx = _fixture()
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        ctx = lettuce.Context(device="cpu", dtype=DTYPES[tag], use_native=False)
        sims = cases(lettuce, ctx)
    for name, sim in sims.items():
        _compare(step_record(lt.native_step(sim)), fx[(tag, name)], f"lettuce {tag}/{name}")


def test_binding_refusals():
    sim = cases(lt, lt.Context("cpu", torch.float64))["tgv2d_trt_post"]
    with pytest.raises(RuntimeError, match="no CPU path"):
        lt.native_invoke(sim)

    class CumulantCollision:  # a collision without a kernel
        pass
    sim.collision = CumulantCollision()
    with pytest.raises(NotImplementedError, match="CumulantCollision"):
        lt.native_step(sim)
    sim = cases(lt, lt.Context("cpu", torch.float64))["obstacle2d_bgk_pre"]

    class VelocityOutlet:
        pass
    sim.post_boundaries = list(sim.post_boundaries) + [VelocityOutlet()]
    with pytest.raises(NotImplementedError, match="VelocityOutlet"):
        lt.native_step(sim)
    flow = lt.TaylorGreenVortex(lt.Context("cpu", torch.float16), [8, 8], 100, 0.05, lt.D2Q9)
    sim = lt.Simulation(flow, lt.BGKCollision(0.6), [])
    sim.flow = type("F", (), {"f": torch.zeros(9, 8, 8, dtype=torch.float16),
                              "stencil": flow.stencil, "resolution": [8, 8],
                              "units": flow.units, "equilibrium": flow.equilibrium})()
    with pytest.raises(NotImplementedError, match="float32 or float64"):
        lt.native_step(sim)
