"""Halfway, linear interpolated and full-way bounce-back of lettuce's
example project (the post-streaming boundaries of
examples/advanced_projects/efficient_bounce_back_obstacle), on CPU: the oracle against the golden vectors the example itself produced
(populations after every step's collide, stream, bounce, and the
momentum-exchange force of each step), the product's neighbour search
against the example's link lists, and the masks, link bits and force links
``EbbSimulation`` builds on a CPU context (set-up only)."""
import numpy as np
import pytest
import torch

import lettuce_gb300 as lt
from conftest import golden, golden_names, meta
from lgb_helpers import fwbb_case, hwbb_case, ibb_case

CASES = golden_names("hwbb_")
IBB_CASES = golden_names("ibb_")
FWBB_CASES = golden_names("fwbb_")


def _post(z, m):
    if not m["inlet"]:
        return []
    res = list(m["res"])
    mask = np.zeros(res, dtype=bool)
    mask[0] = True
    return [dict(kind="equilibrium_pu", mask=mask, rho=z["inlet_rho_lu"], u=z["inlet_u_lu"])]


def test_cases_present():
    assert len(CASES) == 3


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_example(oracle, name):
    z = golden(name)
    m = meta(z)
    steps = int(z["steps"])
    forces = np.zeros((steps, 3))
    out = oracle.run(m["stencil"], z["f0"], steps, collision=m["collision"],
                     tau=float(z["tau"]), tau_minus=1.0, post=_post(z, m),
                     post_streaming=[dict(solid=z["solid"], f_index=z["f_index"])],
                     forces=forces)
    np.testing.assert_allclose(out, z["f"], rtol=0, atol=1e-14)
    d = len(m["res"])
    np.testing.assert_allclose(forces[:, :d], z["force"], rtol=0, atol=1e-13)
    assert np.all(forces[:, d:] == 0)
    ncm, nsm = oracle.ebb_masks(list(m["res"]), z["f0"].shape[0], m["stencil"], [],
                                _post(z, m), [dict(solid=z["solid"])])
    assert np.array_equal(ncm, z["ncm"]) and np.array_equal(nsm, z["nsm"])


@pytest.mark.parametrize("name", CASES)
def test_neighbour_search_matches_example(name):
    """same rows in the same order, negative coordinates kept as the
    example writes them (the non-periodic wrap of Python indexing)"""
    z = golden(name)
    m = meta(z)
    st = getattr(lt, m["stencil"])()
    per = m["periodicity"]
    g = None if "global_extra" not in z else (z["solid"] | z["global_extra"])
    rows = lt.hwbb_links(st.e, st.opposite, z["solid"], g,
                         None if per is None else tuple(per)[:st.d])
    assert rows.dtype == np.int64
    assert np.array_equal(rows, z["f_index"])


def test_given_link_lists_take_precedence():
    z = golden("hwbb_d2q9_bgk")
    m = meta(z)
    flow, hw = hwbb_case(lt.Context("cpu", torch.float64), z, m)
    sbd = lt.SolidBoundaryData()
    sbd.solid_mask = z["solid"]
    sbd.f_index_lt = z["f_index"][:10]
    sbd.f_index_gt = z["f_index"][10:12]
    b = lt.HalfwayBounceBackBoundary(flow.context, flow, sbd)
    assert np.array_equal(b.f_index.numpy(), z["f_index"][:12])


@pytest.mark.parametrize("name", CASES)
def test_ebb_masks_and_links_on_cpu(name):
    z = golden(name)
    m = meta(z)
    flow, hw = hwbb_case(lt.Context("cpu", torch.float64), z, m)
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.8), [])
    assert np.array_equal(sim.no_collision_mask.numpy(), z["ncm"])
    assert np.array_equal(sim.no_streaming_mask.numpy(), z["nsm"])
    # link bits: bit opp(q) at the fluid cell of every link (q, x)
    bits = sim._link_bits.numpy().view(np.uint32)
    st = flow.stencil
    res = np.array(m["res"])
    want = np.zeros(bits.shape, dtype=np.uint32)
    for row in z["f_index"]:
        c = tuple(np.where(row[1:] < 0, row[1:] + res, row[1:]))
        want[c] |= np.uint32(1 << st.opposite[row[0]])
    assert np.array_equal(bits, want)
    flags = sim._flags.numpy()
    assert np.array_equal((flags & lt._lib.FLAG_LINKS) != 0, want != 0)
    assert not np.any(z["solid"] & (want != 0))          # links sit on fluid cells
    assert int(sim._desc.link_bits) == sim._link_bits.data_ptr()
    trip = sim._force_links.numpy().view(np.uint32)
    assert trip.shape == (len(z["f_index"]), 3)
    flat = np.ravel_multi_index(tuple(np.where(z["f_index"][:, 1:] < 0,
                                               z["f_index"][:, 1:] + res,
                                               z["f_index"][:, 1:]).T), tuple(res))
    assert np.array_equal(trip[:, 0], z["f_index"][:, 0]) and np.array_equal(trip[:, 1], flat)
    assert np.all(trip[:, 2] == 0xFFFFFFFF)       # halfway links: no value table
    assert sim._pull_post and sim._desc.n_force_links == len(trip)
    assert not sim._desc.link_val


def test_ebb_rejections_on_cpu():
    z = golden("hwbb_d2q9_bgk")
    m = meta(z)
    flow, hw = hwbb_case(lt.Context("cpu", torch.float64), z, m)
    with pytest.raises(RuntimeError, match="EbbSimulation"):
        hw(flow)
    hw2 = lt.HalfwayBounceBackBoundary(flow.context, flow, type("S", (), {"solid_mask": z["solid"]})(),
                                       calc_force=True)
    flow.psb = [hw, hw2]
    with pytest.raises(NotImplementedError, match="force"):
        lt.EbbSimulation(flow, lt.BGKCollision(0.8), [])
    flow.psb = [lt.BounceBackBoundary(torch.as_tensor(z["solid"]))]
    with pytest.raises(NotImplementedError, match="BounceBackBoundary"):
        lt.EbbSimulation(flow, lt.BGKCollision(0.8), [])
    flow.psb = [hw]
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.8), [])
    with pytest.raises(ValueError, match="slabs"):
        lt.SlabSimulation(sim, 2)
    with pytest.raises(RuntimeError, match="CUDA"):
        sim(1)


def _ibb_rows(z):
    return (np.concatenate([z["f_index_lt"], z["f_index_gt"]]),
            np.concatenate([z["d_lt"], z["d_gt"]]))


def test_ibb_cases_present():
    assert len(IBB_CASES) == 2


@pytest.mark.parametrize("name", IBB_CASES)
def test_oracle_matches_example_interpolated(oracle, name):
    z = golden(name)
    m = meta(z)
    steps = int(z["steps"])
    forces = np.zeros((steps, 3))
    rows, dist = _ibb_rows(z)
    out = oracle.run(m["stencil"], z["f0"], steps, collision=m["collision"],
                     tau=float(z["tau"]), tau_minus=1.0,
                     post_streaming=[dict(solid=z["solid"], f_index=rows, d=dist)],
                     forces=forces)
    np.testing.assert_allclose(out, z["f"], rtol=0, atol=1e-14)
    d = len(m["res"])
    np.testing.assert_allclose(forces[:, :d], z["force"], rtol=0, atol=1e-13)


@pytest.mark.parametrize("name", IBB_CASES)
def test_ibb_value_table_on_cpu(name):
    """the sorted link table: a cell's k-th link bit (in population order)
    is entry base[cell] + k, whose pair names the link's population into
    the solid and the cell; the force triplets point at their links"""
    z = golden(name)
    m = meta(z)
    flow, b = ibb_case(lt.Context("cpu", torch.float64), z, m)
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.8), [])
    assert np.array_equal(sim.no_collision_mask.numpy(), z["ncm"])
    assert np.array_equal(sim.no_streaming_mask.numpy(), z["nsm"])
    st = flow.stencil
    bits = sim._link_bits.numpy().reshape(-1).view(np.uint32)
    base = sim._link_base.numpy().view(np.uint32)
    pairs = sim._link_pairs.numpy().view(np.uint32)
    dist = sim._link_d.numpy()
    rows, d0 = _ibb_rows(z)
    assert len(pairs) == len(rows) == sim._desc.n_links
    for j, (q, cell) in enumerate(pairs):
        pop = st.opposite[q]
        below = bin(int(bits[cell]) & ((1 << pop) - 1)).count("1")
        assert (bits[cell] >> pop) & 1 and base[cell] + below == j
    res = np.array(m["res"])
    flat = np.ravel_multi_index(tuple(rows[:, 1:].T), tuple(res))
    got = {(int(q), int(c)): float(w) for (q, c), w in zip(pairs, dist)}
    assert got == {(int(q), int(c)): float(w) for q, c, w in zip(rows[:, 0], flat, d0)}
    trip = sim._force_links.numpy().view(np.uint32)
    assert np.array_equal(pairs[trip[:, 2]], trip[:, :2])
    assert sim._link_val.dtype == flow.context.storage_dtype and len(sim._link_val) == len(rows)


def _fw_post(z):
    return [dict(solid=z["solid"], f_index=z["f_index"], d=np.zeros(len(z["f_index"])),
                 fullway=True)]


def test_fwbb_cases_present():
    assert len(FWBB_CASES) == 2


@pytest.mark.parametrize("name", FWBB_CASES)
def test_oracle_matches_example_fullway(oracle, name):
    z = golden(name)
    m = meta(z)
    steps = int(z["steps"])
    forces = np.zeros((steps, 3))
    out = oracle.run(m["stencil"], z["f0"], steps, collision=m["collision"],
                     tau=float(z["tau"]), tau_minus=1.0, post_streaming=_fw_post(z),
                     forces=forces)
    np.testing.assert_allclose(out, z["f"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(forces[:, :len(m["res"])], z["force"], rtol=0, atol=1e-13)
    ncm, nsm = oracle.ebb_masks(list(m["res"]), z["f0"].shape[0], m["stencil"], [], [],
                                _fw_post(z))
    assert np.array_equal(ncm, z["ncm"]) and np.array_equal(nsm, z["nsm"])


@pytest.mark.parametrize("name", FWBB_CASES)
def test_fullway_search_and_table_on_cpu(name):
    """the solid-cell links reproduce the example's list row for row; in
    the table they are distance-0 entries whose force triplets carry bit 31"""
    z = golden(name)
    m = meta(z)
    st = getattr(lt, m["stencil"])()
    per = m["periodicity"]
    g = None if "global_extra" not in z else (z["solid"] | z["global_extra"])
    rows = lt.fwbb_links(st.e, st.opposite, z["solid"], g,
                         None if per is None else tuple(per)[:st.d])
    assert np.array_equal(rows, z["f_index"])
    flow, b = fwbb_case(lt.Context("cpu", torch.float64), z, m)
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.8), [])
    assert np.array_equal(sim.no_collision_mask.numpy(), z["ncm"])
    assert np.array_equal(sim.no_streaming_mask.numpy(), z["nsm"])
    assert sim._nsb is None                     # the solid cells stream
    bits = sim._link_bits.numpy().reshape(-1).view(np.uint32)
    solid = np.asarray(z["solid"]).reshape(-1)
    assert np.all(solid[bits != 0])             # the links sit on solid cells
    assert np.all(sim._link_d.numpy() == 0)
    trip = sim._force_links.numpy().view(np.uint32)
    assert np.all(trip[:, 2] & 0x80000000)
    pairs = sim._link_pairs.numpy().view(np.uint32)
    assert np.array_equal(pairs[trip[:, 2] & 0x7FFFFFFF], trip[:, :2])


def _loop_search(e, opp, mask, other, periodicity, at_solid):
    """the example's neighbour search written as its loops
    (halfway_bounce_back_boundary.py:70-161, fullway_bounce_back_boundary.py:
    47-131): border shifts on periodic axes, Python indexing (negative
    indices wrap, past-the-end ones raise and drop the link)"""
    rows = []
    shape = mask.shape
    for p in zip(*np.nonzero(mask)):
        for i in range(len(e)):
            border = [0] * mask.ndim
            for k in range(mask.ndim):
                if p[k] == 0 and e[i][k] == -1 and periodicity[k]:
                    border[k] = -1
                elif p[k] == shape[k] - 1 and e[i][k] == 1 and periodicity[k]:
                    border[k] = 1
            c = tuple(int(p[k] + e[i][k] - border[k] * shape[k]) for k in range(mask.ndim))
            try:
                hit = (not mask[c]) and (not other[c])
            except IndexError:
                continue
            if hit:
                rows.append([opp[i]] + (list(map(int, p)) if at_solid else list(c)))
    return np.array(rows, dtype=np.int64).reshape(-1, mask.ndim + 1)


@pytest.mark.parametrize("stencil,shape", [("D2Q9", (9, 7)), ("D3Q19", (6, 5, 4)),
                                           ("D3Q27", (5, 5, 4))])
def test_link_searches_equal_the_loops(stencil, shape):
    import itertools
    st = getattr(lt, stencil)()
    rng = np.random.default_rng(sum(shape))
    for trial, per in enumerate(itertools.product([False, True], repeat=len(shape))):
        mask = rng.random(shape) < 0.25
        extra = (rng.random(shape) < 0.15) & ~mask
        glob = mask | extra
        want = _loop_search(st.e, st.opposite, mask, glob, per, at_solid=False)
        assert np.array_equal(lt.hwbb_links(st.e, st.opposite, mask, glob, per), want)
        want = _loop_search(st.e, st.opposite, mask, mask, per, at_solid=False)
        assert np.array_equal(lt.hwbb_links(st.e, st.opposite, mask, None, per), want)
        want = _loop_search(st.e, st.opposite, mask, extra, per, at_solid=True)
        assert np.array_equal(lt.fwbb_links(st.e, st.opposite, mask, glob, per), want)
        want = _loop_search(st.e, st.opposite, mask, np.zeros_like(mask), per, at_solid=True)
        assert np.array_equal(lt.fwbb_links(st.e, st.opposite, mask, None, per), want)


def test_ebb_masks_with_ordinary_boundaries_on_cpu(oracle):
    """an equilibrium inlet and an anti-bounce-back outlet (lettuce's
    post-collision boundaries) plus a halfway, an interpolated and a
    full-way solid: the masks EbbSimulation builds equal the oracle's
    restatement of ebb_simulation.py:28-57"""
    from lgb_helpers import HwbbFlow
    res = [18, 9]
    st = lt.D2Q9()
    rng = np.random.default_rng(4)
    f0 = np.asarray(st.w).reshape(-1, 1, 1) * (1 + 0.01 * rng.standard_normal([9] + res))
    ctx = lt.Context("cpu", torch.float64)
    flow = HwbbFlow(ctx, st, f0)
    inlet = np.zeros(res, dtype=bool)
    inlet[0] = True
    flow._bnds = [lt.EquilibriumBoundaryPU(ctx, flow, torch.as_tensor(inlet),
                                           torch.tensor([0.01, 0.0], dtype=torch.float64)),
                  lt.AntiBounceBackOutlet([1, 0], flow)]
    s1 = np.zeros(res, dtype=bool)
    s1[3:5, 2:5] = True
    s2 = np.zeros(res, dtype=bool)
    s2[8:10, 4:7] = True
    s3 = np.zeros(res, dtype=bool)
    s3[13:15, 1:3] = True
    glob = s1 | s2 | s3
    d1 = lt.SolidBoundaryData()
    d1.solid_mask = s1
    hw = lt.HalfwayBounceBackBoundary(ctx, flow, d1, global_solid_mask=glob)
    rows = lt.hwbb_links(st.e, st.opposite, s2, glob)
    d2 = lt.SolidBoundaryData()
    d2.solid_mask = s2
    d2.f_index_lt, d2.f_index_gt = rows[:5], rows[5:]
    d2.d_lt, d2.d_gt = np.full(5, 0.3), np.full(len(rows) - 5, 0.7)
    ib = lt.LinearInterpolatedBounceBackBoundary(ctx, flow, d2)
    fw = lt.FullwayBounceBackBoundary(ctx, flow, s3, global_solid_mask=glob, calc_force=True)
    flow.psb = [hw, ib, fw]
    sim = lt.EbbSimulation(flow, lt.BGKCollision(0.7), [])
    post = [{"kind": "equilibrium_pu", "mask": inlet, "rho": np.ones([1, 1]),
             "u": np.zeros([2, 1, 1])},
            {"kind": "anti_bounce_back", "direction": [1, 0]}]
    ps = [dict(solid=s1, f_index=hw.f_index.numpy()),
          dict(solid=s2, f_index=rows, d=np.r_[np.full(5, 0.3), np.full(len(rows) - 5, 0.7)]),
          dict(solid=s3, f_index=fw.f_index_fwbb.numpy(), fullway=True)]
    ncm, nsm = oracle.ebb_masks(res, 9, "D2Q9", [], post, ps)
    assert np.array_equal(sim.no_collision_mask.numpy(), ncm)
    assert np.array_equal(sim.no_streaming_mask.numpy(), nsm)
    assert set(np.unique(ncm)) == {0, 1, 2, 3, 4, 5}
    # every link in the table once; the force triplets are the full-way ones
    assert sim._desc.n_links == len(hw.f_index) + len(rows) + len(fw.f_index_fwbb)
    trip = sim._force_links.numpy().view(np.uint32)
    assert len(trip) == len(fw.f_index_fwbb) and np.all(trip[:, 2] & 0x80000000)


def test_bench_sphere_distances():
    """the bench's wall distances put x + d e_q on the sphere's surface"""
    import importlib.util
    import os
    spec = importlib.util.spec_from_file_location(
        "bench_mod", os.path.join(os.path.dirname(os.path.dirname(__file__)), "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    res = [40, 20, 20]
    centre, r = [12.0, 9.5, 9.5], 4.3
    g = np.meshgrid(*[np.arange(k) for k in res], indexing="ij", sparse=True)
    solid = sum((gi - ci) ** 2 for gi, ci in zip(g, centre)) < r * r
    st = lt.D3Q27()
    rows = lt.hwbb_links(st.e, st.opposite, solid)
    d = bench.sphere_link_distances(rows, centre, r)
    e = np.asarray(st.e)[rows[:, 0]]
    p = rows[:, 1:] + d[:, None] * e
    dist = np.sqrt(np.sum((p - np.asarray(centre)) ** 2, axis=1))
    assert np.all((d > 0) & (d <= 1))
    np.testing.assert_allclose(dist[d > 1e-3], r, rtol=1e-9)


def test_boundaries_without_links_on_cpu():
    """an empty solid and a solid enclosed by other solids give no links:
    the descriptors still describe a valid launch (no value table, a force
    over zero links)"""
    from lgb_helpers import HwbbFlow
    res = [8, 6]
    st = lt.D2Q9()
    f0 = np.asarray(st.w).reshape(-1, 1, 1) * np.ones([9] + res)
    ctx = lt.Context("cpu", torch.float64)
    empty = np.zeros(res, dtype=bool)
    inner = np.zeros(res, dtype=bool)
    inner[3, 2] = True
    ring = np.zeros(res, dtype=bool)
    ring[2:5, 1:4] = True
    ring[3, 2] = False
    for kind in ("halfway", "interpolated", "fullway"):
        for solid, glob in ((empty, None), (inner, inner | ring)):
            flow = HwbbFlow(ctx, st, f0)
            sbd = lt.SolidBoundaryData()
            sbd.solid_mask = solid
            if kind == "halfway":
                b = lt.HalfwayBounceBackBoundary(ctx, flow, sbd, global_solid_mask=glob,
                                                 calc_force=True)
            elif kind == "interpolated":
                sbd.f_index_lt = np.zeros((0, 3), dtype=np.int64)
                sbd.f_index_gt = np.zeros((0, 3), dtype=np.int64)
                sbd.d_lt, sbd.d_gt = np.zeros(0), np.zeros(0)
                b = lt.LinearInterpolatedBounceBackBoundary(ctx, flow, sbd, calc_force=True)
            else:
                b = lt.FullwayBounceBackBoundary(ctx, flow, solid, global_solid_mask=glob,
                                                 calc_force=True)
            assert len(b.link_rows()[0]) == 0
            flow.psb = [b]
            sim = lt.EbbSimulation(flow, lt.BGKCollision(0.7), [])
            d = sim._desc
            assert d.n_links == 0 and not d.link_val
            assert d.n_force_links == 0 and d.force_out and d.force_scratch
            assert int(sim._link_bits.abs().sum()) == 0


@pytest.mark.parametrize("kind", ["halfway", "interpolated"])
def test_oracle_momentum_balance(oracle, kind):
    """in the oracle, as in the kernels: on a periodic box the total
    momentum changes by minus the summed momentum-exchange forces"""
    st = lt.D2Q9()
    res = [40, 30]
    rng = np.random.default_rng(9)
    e = np.asarray(st.e, dtype=np.float64)
    w = np.asarray(st.w).reshape(-1, 1, 1)
    f0 = w * (1.0 + 0.05 * rng.standard_normal([9] + res))
    g = np.meshgrid(np.arange(res[0]), np.arange(res[1]), indexing="ij")
    solid = (g[0] - 17.2) ** 2 + (g[1] - 14.6) ** 2 < 5.1 ** 2
    rows = lt.hwbb_links(st.e, st.opposite, solid, None, (True, True))
    b = dict(solid=solid, f_index=rows)
    if kind == "interpolated":
        b["d"] = rng.uniform(0.05, 0.95, len(rows))
    steps = 25
    forces = np.zeros((steps, 3))
    f = oracle.run("D2Q9", f0, steps, collision="bgk", tau=0.66, post_streaming=[b],
                   forces=forces)
    dj = np.einsum("qd,qxy->d", e, f) - np.einsum("qd,qxy->d", e, f0)
    fsum = forces.sum(axis=0)[:2]
    assert np.abs(fsum).max() > 1e-3
    np.testing.assert_allclose(dj, -fsum, rtol=0, atol=1e-11)
