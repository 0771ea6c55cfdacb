"""Host-side logic on CPU: stencil tables, unit conversion, initial fields,
mask assembly and packing -- checked against lettuce's golden vectors and
against lettuce's own property tests (tests/stencil, tests/boundary)."""
import json

import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from lettuce_gb300 import _lib
from lettuce_gb300._simulation import pack_masks
from conftest import golden, meta

STENCILS = [lt.D1Q3, lt.D2Q9, lt.D3Q15, lt.D3Q19, lt.D3Q27]
CPU64 = lt.Context("cpu", torch.float64)


@pytest.mark.parametrize("S", STENCILS)
def test_stencil_invariants(S, oracle):
    s = S()
    # lettuce tests/stencil: weights sum to one, opposite, symmetry, first zero
    assert abs(sum(s.w) - 1) < 1e-15
    e = np.array(s.e)
    assert (e[s.opposite] == -e).all()
    assert (e.sum(axis=0) == 0).all()
    assert (e[0] == 0).all()
    # same tables (and q order) as the oracle's restatement of lettuce
    oe, ow, oo = oracle.stencil_tables(S.__name__)
    assert np.array_equal(e, oe) and np.allclose(s.w, ow, rtol=0, atol=0)
    assert list(oo) == list(s.opposite)


def test_units_match_lettuce():
    z = golden("observables")
    for tag, S, n in [("2d", lt.D2Q9, 16), ("3d", lt.D3Q19, 8)]:
        ref = json.loads(str(z[f"{tag}_units"]))
        flow = lt.TaylorGreenVortex(CPU64, n, 1000, 0.05, S)
        u = flow.units
        assert u.relaxation_parameter_lu == ref["relaxation_parameter_lu"]
        assert u.viscosity_lu == ref["viscosity_lu"]
        assert u.characteristic_velocity_lu == ref["characteristic_velocity_lu"]
        assert u.characteristic_length_lu == ref["characteristic_length_lu"]
        assert u.convert_time_to_pu(100) == ref["time_pu_100"]


@pytest.mark.parametrize("name,S,n", [("tgv2d_d2q9_bgk", lt.D2Q9, 16),
                                      ("tgv2d_d2q9_trt", lt.D2Q9, [16, 12]),
                                      ("tgv3d_d3q19_bgk", lt.D3Q19, 8),
                                      ("tgv3d_d3q27_kbc", lt.D3Q27, 8)])
def test_taylor_green_initial_field(name, S, n):
    z = golden(name)
    re = meta(z)["re"]
    flow = lt.TaylorGreenVortex(CPU64, n, re, 0.05, S)
    assert np.allclose(flow.f.numpy(), z["f0"], rtol=1e-13, atol=1e-16)


def _obstacle(name):
    z = golden(name)
    m = meta(z)
    S = getattr(lt, m["stencil"])
    flow = lt.Obstacle(CPU64, m["res"], m["re"], m["ma"], m["domain_length_x"], stencil=S)
    flow.mask = z["mask"]
    flow.initialize()
    return z, m, flow


@pytest.mark.parametrize("name", ["obstacle2d_d2q9_bgk", "obstacle3d_d3q27_kbc"])
def test_obstacle_setup_bit_exact(name):
    z, m, flow = _obstacle(name)
    assert np.array_equal(flow.f.numpy(), z["f0"])
    sim = lt.Simulation(flow, lt.KBCCollision() if m["collision"] == "kbc"
                        else lt.BGKCollision(flow.units.relaxation_parameter_lu), [])
    assert np.array_equal(sim.no_collision_mask.numpy(), z["ncm"])
    assert np.array_equal(sim.no_streaming_mask.numpy(), z["nsm"])
    # KBC relaxes with the flow's tau, like lettuce
    if m["collision"] == "kbc":
        assert sim.collision.tau == flow.units.relaxation_parameter_lu
    # equilibrium inlet in lattice units, as lettuce converts it
    inlet = sim._natives[1]
    assert inlet.kind == _lib.SUB_EQUILIBRIUM_PU
    assert np.allclose(inlet.u.numpy().ravel(), z["inlet_u_lu"].ravel(), rtol=1e-15)
    assert np.allclose(inlet.rho.numpy().ravel(), z["inlet_rho_lu"].ravel(), rtol=1e-15)


def test_pack_masks_bits():
    _, _, flow = _obstacle("obstacle3d_d3q27_kbc")
    sim = lt.Simulation(flow, lt.KBCCollision(), [])
    flags, bits = sim._flags.numpy(), sim._nsb.numpy()
    ncm, nsm = sim.no_collision_mask.numpy(), sim.no_streaming_mask.numpy()
    assert np.array_equal(flags & _lib.FLAG_INDEX_MASK, ncm)
    q = nsm.shape[0]
    keep = (nsm == 1)
    keep[0] = False
    for k in range(q):
        assert np.array_equal((bits >> k) & 1, keep[k].astype(np.int32))
    assert np.array_equal((flags & _lib.FLAG_NO_STREAM) != 0, keep.any(axis=0))
    # outlet plane: the populations entering from +x do not stream
    assert keep[:, -1].sum() == 9 * 8 * 8
    # push guard: x is marked where some x + e_q keeps population q
    e = np.asarray(flow.stencil.e)
    res = flow.resolution
    guard = np.zeros(res, dtype=bool)
    for x in np.ndindex(*res):
        for k in range(1, q):
            dst = tuple((np.asarray(x) + e[k]) % res)
            guard[x] |= keep[k][dst]
    assert np.array_equal((flags & _lib.FLAG_PUSH_GUARD) != 0, guard)
    assert sim._desc.options & _lib.OPT_PUSH_GUARD


def test_pack_masks_collision_index_quirk():
    """lettuce's torch stream keeps a population only where the
    no-streaming value is exactly 1; with pre-boundaries the mask starts at
    the collision index (lettuce/_simulation.py:106-107, 254-255)"""
    ncm = torch.full([4, 4], 1, dtype=torch.uint8)
    nsm = torch.full([9, 4, 4], 1, dtype=torch.uint8)  # collision_index == 1
    flags, bits = pack_masks(ncm, nsm)
    assert bits is not None and int(bits[0, 0]) == (1 << 9) - 2
    nsm2 = torch.full([9, 4, 4], 2, dtype=torch.uint8)  # collision_index == 2
    _, bits2 = pack_masks(torch.full([4, 4], 2, dtype=torch.uint8), nsm2)
    assert bits2 is None


def test_equilibrium_checked_tensor_shapes():
    flow = lt.TaylorGreenVortex(CPU64, [8, 6], 100, 0.05, lt.D2Q9)
    ct = lt.EquilibriumBoundaryPU.checked_tensor
    assert list(ct(0.5, CPU64, flow).shape) == [1, 1, 1]
    assert list(ct([0.1, 0.2], CPU64, flow).shape) == [2, 1, 1]
    assert list(ct(np.zeros([8, 6]), CPU64, flow).shape) == [1, 8, 6]
    assert list(ct(np.zeros([2, 8, 1]), CPU64, flow).shape) == [2, 8, 1]
    with pytest.raises(ValueError):
        ct(np.zeros([3, 8, 6]), CPU64, flow)
    with pytest.raises(ValueError):
        ct(np.zeros([2, 7, 6]), CPU64, flow)


def test_anti_bounce_back_masks():
    flow = lt.TaylorGreenVortex(CPU64, [6, 5, 4], 100, 0.05, lt.D3Q19)
    b = lt.AntiBounceBackOutlet([1, 0, 0], flow)
    assert list(b.velocities) == [1, 11, 13, 15, 17]
    nsm = b.make_no_streaming_mask([19, 6, 5, 4], CPU64)
    assert nsm.sum() == 5 * 5 * 4 and nsm[[2, 12, 14, 16, 18], -1].all()
    b2 = lt.AntiBounceBackOutlet([0, -1, 0], flow)
    ncm = b2.make_no_collision_mask([6, 5, 4], CPU64)
    assert ncm[:, 0].all() and ncm.sum() == 6 * 4
    with pytest.raises(AssertionError):
        lt.AntiBounceBackOutlet([1, 1, 0], flow)


def test_context_semantics():
    c = lt.Context("cpu")
    assert c.dtype == torch.float32 and not c.use_native and c.storage == _lib.F32
    c16 = lt.Context("cpu", torch.float16)
    assert c16.storage == _lib.F16_SHIFTED and c16.dtype == torch.float32
    cb = lt.Context("cpu", storage="bf16_shifted")
    assert cb.storage_dtype == torch.bfloat16
    with pytest.raises(AssertionError):
        lt.Context("cpu", use_native=True)
    with pytest.raises(ValueError):
        lt.Context("cpu", storage="fp8")
    with pytest.raises(AssertionError):
        lt.Context("mps")
    if not torch.cuda.is_available():
        with pytest.raises(AssertionError):
            lt.Context("cuda:0")
        with pytest.raises(AssertionError):
            lt.Context(None, use_native=True)
        # lettuce's placement without a device but with use_native=False
        assert lt.Context(None, use_native=False).device == torch.device("cuda:0")
        assert lt.Context().device == torch.device("cpu") and not lt.Context().use_native
    # masks keep an integer type, everything else takes the context dtype
    assert c.convert_to_tensor(np.array([True, False])).dtype == torch.uint8
    assert c.convert_to_tensor(torch.zeros(2, dtype=torch.bool)).dtype == torch.uint8
    assert c.convert_to_tensor([1, 2]).dtype == torch.float32
    assert c.convert_to_tensor(0.1).item() == np.float32(0.1)
    assert lt.Context("cpu", torch.float64).convert_to_tensor(np.arange(3)).dtype == torch.float64


def test_shifted_storage_round_trip_on_host():
    ctx = lt.Context("cpu", storage="fp16_shifted")
    flow = lt.TaylorGreenVortex(ctx, 16, 1000, 0.05, lt.D2Q9)
    ref = lt.TaylorGreenVortex(lt.Context("cpu", torch.float32), 16, 1000, 0.05, lt.D2Q9)
    assert flow.f_raw.dtype == torch.float16
    # the deviation from w is stored with fp16's 11-bit mantissa: at most
    # half an fp16 ulp of the largest deviation (plus float32 rounding)
    w = ref.torch_stencil.w.view(-1, 1, 1)
    hmax = (ref.f - w).abs().max().item()
    err = (flow.f - ref.f).abs().max().item()
    assert err <= hmax * 2.0 ** -10


def test_no_cpu_path():
    flow = lt.TaylorGreenVortex(lt.Context("cpu"), 8, 100, 0.05, lt.D2Q9)
    sim = lt.Simulation(flow, lt.BGKCollision(0.6), [])
    with pytest.raises(RuntimeError, match="no CPU path"):
        sim(1)


def test_force_without_kernel_is_refused():
    """a user force that offers no kernel is refused, not run in torch"""
    class TorchOnlyForce(lt.Guo):
        def native_available(self):
            return False

    flow = lt.TaylorGreenVortex(lt.Context("cpu"), 8, 100, 0.05, lt.D2Q9)
    with pytest.raises(NotImplementedError):
        lt.Simulation(flow, lt.BGKCollision(0.6, force=TorchOnlyForce(flow, 0.6, [1e-4, 0])), [])


def test_force_descriptors():
    flow = lt.PoiseuilleFlow2D(CPU64, 17, 1, 0.02)
    a = flow.units.convert_acceleration_to_lu(flow.acceleration)
    tau = flow.units.relaxation_parameter_lu
    for F, kind in [(lt.Guo, _lib.FORCE_GUO), (lt.ShanChen, _lib.FORCE_SHAN_CHEN)]:
        sim = lt.Simulation(flow, lt.BGKCollision(tau, force=F(flow, 0.9, a)), [])
        d = sim._desc
        assert (d.collision, d.force, d.force_tau) == (_lib.BGK, kind, 0.9)
        assert list(d.accel)[:2] == a.tolist()
    g = lt.Guo(flow, 0.9, a)
    assert g.ueq_scaling_factor == 0.5 and lt.ShanChen(flow, 0.9, a).ueq_scaling_factor == 0.9
    # Guo's source term restated on torch tensors: zero acceleration, zero term
    u = torch.zeros([2, 17, 17], dtype=torch.float64)
    assert torch.count_nonzero(lt.Guo(flow, 0.9, [0.0, 0.0]).source_term(u)) == 0
    sim = lt.Simulation(flow, lt.SmagorinskyCollision(0.7, smagorinsky_constant=0.2), [])
    assert (sim._desc.collision, sim._desc.smagorinsky_constant) == (_lib.SMAGORINSKY, 0.2)
    reg = lt.RegularizedCollision(0.6)
    sim = lt.Simulation(flow, reg, [])
    assert sim._desc.collision == _lib.REGULARIZED and sim._desc.tau == tau == reg.tau


def test_checkpoint_round_trip(tmp_path):
    flow = lt.TaylorGreenVortex(CPU64, 8, 100, 0.05, lt.D2Q9)
    f0 = flow.f.clone()
    flow.dump(tmp_path / "f.pkl")
    flow.f = torch.zeros_like(f0)
    flow.load(tmp_path / "f.pkl")
    assert torch.equal(flow.f, f0)


def test_checkpoint_compatible_with_lettuce(tmp_path):
    """a file written by lettuce's Flow.dump loads here, and this package's
    dump writes the same array lettuce's load expects (a pickled ndarray)"""
    import os
    import pickle
    from conftest import GOLDEN
    ref = np.load(os.path.join(GOLDEN, "lettuce_dump_d2q9_12.npz"))["f"]
    flow = lt.TaylorGreenVortex(CPU64, 12, 100, 0.05, lt.D2Q9)
    flow.f = torch.zeros_like(flow.f)
    flow.load(os.path.join(GOLDEN, "lettuce_dump_d2q9_12.pkl"))
    assert np.array_equal(flow.f.numpy(), ref)
    flow.dump(tmp_path / "ours.pkl")
    with open(tmp_path / "ours.pkl", "rb") as fh:
        back = pickle.load(fh)
    assert isinstance(back, np.ndarray) and np.array_equal(back, ref)


def test_lower_memory_equilibrium_is_the_quadratic_one():
    """lettuce's QuadraticEquilibriumLessMemory evaluates the same
    equilibrium; here it is accepted by the step (same kernels)"""
    import lettuce_gb300 as lt
    ctx = lt.Context("cpu", torch.float64)
    eq = lt.QuadraticEquilibriumLessMemory()
    flow = lt.TaylorGreenVortex(ctx, [8, 6], 100, 0.05, lt.D2Q9, equilibrium=eq)
    assert torch.equal(eq(flow), lt.QuadraticEquilibrium()(flow))
    assert eq.native_available()
    lt.Simulation(flow, lt.BGKCollision(0.7), [])   # set-up accepts it
