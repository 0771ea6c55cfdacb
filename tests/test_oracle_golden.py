"""Pins the CPU oracle to lettuce: every golden vector in tests/golden was
produced by lettuce's own float64 torch step (tests/golden/make_golden.py);
the oracle must reproduce each to float64 round-off."""
import numpy as np
import pytest

from conftest import golden, golden_names, meta

STRATS = ["PRE_STREAMING", "POST_STREAMING"]


def rel(a, b):
    return np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b)))


@pytest.mark.parametrize("name", golden_names("random_") + golden_names("tgv2d_d2q9")
                         + golden_names("tgv3d"))
@pytest.mark.parametrize("strategy", STRATS)
def test_periodic_cases(oracle, name, strategy):
    z = golden(name)
    m = meta(z)
    out = oracle.run(m["stencil"], z["f0"], int(z["steps"]), collision=m["collision"],
                     tau=float(z["tau"]), tau_minus=1.0, strategy=strategy)
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


def obstacle_boundaries(z, m):
    res = m["res"]
    d = len(res)
    x = np.arange(res[0]).reshape([-1] + [1] * (d - 1)) * np.ones(res)
    return [{"kind": "equilibrium_pu", "mask": np.abs(x) < 1e-6,
             "rho": z["inlet_rho_lu"].reshape([1] * d),
             "u": z["inlet_u_lu"].reshape([d] + [1] * d)},
            {"kind": "anti_bounce_back", "direction": [1] + [0] * (d - 1)},
            {"kind": "bounce_back", "mask": z["mask"]}]


@pytest.mark.parametrize("name", golden_names("obstacle"))
def test_obstacle_masks_bit_exact(oracle, name):
    z = golden(name)
    m = meta(z)
    ncm, nsm = oracle.assemble_masks(m["res"], z["f0"].shape[0], m["stencil"], [],
                                     obstacle_boundaries(z, m))
    assert np.array_equal(ncm, z["ncm"])
    assert np.array_equal(nsm, z["nsm"])


@pytest.mark.parametrize("name", golden_names("obstacle"))
@pytest.mark.parametrize("strategy", STRATS)
def test_obstacle_cases(oracle, name, strategy):
    z = golden(name)
    m = meta(z)
    out = oracle.run(m["stencil"], z["f0"], int(z["steps"]), collision=m["collision"],
                     tau=float(z["tau"]), strategy=strategy,
                     post=obstacle_boundaries(z, m))
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


@pytest.mark.parametrize("strategy", STRATS)
def test_equilibrium_boundary_field(oracle, strategy):
    z = golden("eqpu_field_d2q9")
    post = [{"kind": "equilibrium_pu", "mask": z["mask"], "rho": z["rho_lu"][0],
             "u": z["u_lu"]}]
    out = oracle.run("D2Q9", z["f0"], int(z["steps"]), collision="bgk",
                     tau=float(z["tau"]), strategy=strategy, post=post)
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


def test_native_known_answers(oracle):
    """lettuce tests/native/test_native_streaming.py (impulse per direction)
    and test_native_bounce_back.py"""
    z = golden("native_kats")
    out = oracle.run("D2Q9", z["stream_f0"], 1, collision="none")
    assert np.array_equal(out, z["stream_f1"])
    post = [{"kind": "bounce_back", "mask": z["bb_mask"]}]
    assert np.array_equal(oracle.run("D2Q9", z["bb_f0"], 1, collision="none", post=post),
                          z["bb_f1"])
    assert np.array_equal(oracle.run("D2Q9", z["bb_f0"], 2, collision="none", post=post),
                          z["bb_f2"])


def test_oracle_moments_match_golden(oracle):
    z = golden("observables")
    rho, u = oracle.moments("D2Q9", z["2d_f"])
    assert np.allclose(rho, z["2d_rho"][0], rtol=1e-14, atol=0)
    assert np.allclose(u, z["2d_u"], rtol=1e-12, atol=1e-16)


def test_oracle_energy_decay_series(oracle):
    """config 1: D2Q9 BGK TGV 256^2, Re 1000, f64, POST_STREAMING; the oracle
    must follow lettuce's kinetic energy series (first 100 steps here)"""
    z = golden("observables")  # noqa: F841  (units checked in test_host)
    e = golden("tgv2d_energy_256")
    import lettuce_gb300 as lt
    import torch
    ctx = lt.Context("cpu", torch.float64)
    flow = lt.TaylorGreenVortex(ctx, 256, 1000, 0.05, lt.D2Q9)
    f0 = flow.f.numpy()
    tau = flow.units.relaxation_parameter_lu
    f100 = oracle.run("D2Q9", f0, 100, collision="bgk", tau=tau, strategy="POST_STREAMING")
    dx = flow.units.convert_length_to_pu(1.0)
    k = flow.units.convert_incompressible_energy_to_pu(oracle.kinetic_energy("D2Q9", f100))
    assert abs(k * dx ** 2 / e["energy"][1] - 1) < 1e-12


def outletp_boundaries(z, m):
    res = m["res"]
    d = len(res)
    x = np.arange(res[0]).reshape([-1] + [1] * (d - 1)) * np.ones(res)
    return [{"kind": "equilibrium_pu", "mask": np.abs(x) < 1e-6,
             "rho": z["inlet_rho_lu"].reshape([1] * d),
             "u": z["inlet_u_lu"].reshape([d] + [1] * d)},
            {"kind": "equilibrium_outlet_p", "direction": [1] + [0] * (d - 1),
             "rho": m["rho_outlet"]},
            {"kind": "bounce_back", "mask": z["mask"]}]


@pytest.mark.parametrize("name", golden_names("outletp"))
@pytest.mark.parametrize("strategy", STRATS)
def test_pressure_outlet_cases(oracle, name, strategy):
    z = golden(name)
    m = meta(z)
    post = outletp_boundaries(z, m)
    ncm, nsm = oracle.assemble_masks(m["res"], z["f0"].shape[0], m["stencil"], [], post)
    assert np.array_equal(ncm, z["ncm"]) and np.array_equal(nsm, z["nsm"])
    out = oracle.run(m["stencil"], z["f0"], int(z["steps"]), collision="bgk",
                     tau=float(z["tau"]), strategy=strategy, post=post)
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


@pytest.mark.parametrize("name", golden_names("psm"))
@pytest.mark.parametrize("strategy", STRATS)
def test_partially_saturated_cases(oracle, name, strategy):
    z = golden(name)
    m = meta(z)
    post = [{"kind": "partially_saturated", "mask": z["mask"], "tau": float(z["tau"]),
             "B": float(z["B"])}]
    out = oracle.run(m["stencil"], z["f0"], int(z["steps"]), collision="bgk",
                     tau=float(z["tau"]), strategy=strategy, post=post)
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


EXT_FORCE = {"bgk_guo": ("bgk", "guo"), "bgk_shanchen": ("bgk", "shan_chen"),
             "smagorinsky_guo": ("smagorinsky", "guo"), "smagorinsky": ("smagorinsky", None),
             "regularized": ("regularized", None)}


@pytest.mark.parametrize("name", golden_names("ext_"))
@pytest.mark.parametrize("strategy", STRATS)
def test_forces_and_collisions(oracle, name, strategy):
    """regularized and Smagorinsky collisions, BGK / Smagorinsky with Guo and
    Shan-Chen forces (random fields, lettuce float64)"""
    z = golden(name)
    m = meta(z)
    coll, force = EXT_FORCE[m["kind"]]
    out = oracle.run(m["stencil"], z["f0"], int(z["steps"]), collision=coll,
                     tau=float(z["tau"]), strategy=strategy, force=force,
                     force_tau=float(z["force_tau"]), accel=z["accel"],
                     smagorinsky_constant=m["smagorinsky_constant"])
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


@pytest.mark.parametrize("name", golden_names("poiseuille"))
def test_poiseuille_force(oracle, name):
    """lettuce's forced Poiseuille channel (bounce-back walls, Guo or
    Shan-Chen), 300 POST_STREAMING steps"""
    z = golden(name)
    m = meta(z)
    mask = np.zeros([17, 17], dtype=bool)
    mask[:, [0, -1]] = True
    post = [{"kind": "bounce_back", "mask": mask}]
    ncm, _ = oracle.assemble_masks([17, 17], 9, "D2Q9", [], post)
    assert np.array_equal(ncm, z["ncm"])
    out = oracle.run("D2Q9", z["f0"], int(z["steps"]), collision="bgk", tau=float(z["tau"]),
                     strategy="POST_STREAMING", post=post, force=m["force"],
                     force_tau=float(z["tau"]), accel=z["accel"])
    assert rel(out, z["f_final"]) < 1e-12


@pytest.mark.parametrize("name", golden_names("mrt_"))
@pytest.mark.parametrize("strategy", STRATS)
def test_mrt_cases(oracle, name, strategy):
    """lettuce's MRT collision with its Lallemand, Dellar and Hermite moment
    transforms (random fields, per-moment relaxation times, float64)"""
    z = golden(name)
    m = meta(z)
    eq = {"D2Q9Lallemand": "lallemand", "D2Q9Dellar": "dellar",
          "D3Q27Hermite": "hermite"}[m["transform"]]
    out = oracle.run(m["stencil"], z["f0"], int(z["steps"]), collision="mrt",
                     strategy=strategy, mrt=(eq, z["matrix"], z["inverse"], z["relaxation"]))
    assert rel(out, z[f"f_{strategy}"]) < 1e-13


@pytest.mark.parametrize("name", golden_names("mrt_"))
def test_moment_bases_are_lettuces(name):
    """the package builds each basis from its polynomials in e and inverts it;
    the result equals lettuce's tabulated matrices"""
    import lettuce_gb300 as lt
    import torch
    z = golden(name)
    m = meta(z)
    T = getattr(lt, m["transform"])
    t = T(getattr(lt, m["stencil"])(), lt.Context("cpu", torch.float64))
    assert np.max(np.abs(t.matrix_np - z["matrix"])) < 1e-15
    assert np.max(np.abs(t.inverse_np - z["inverse"])) < 1e-14
