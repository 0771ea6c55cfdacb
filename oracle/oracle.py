"""CPU oracle for the lattice Boltzmann step -- TEST INFRASTRUCTURE ONLY.

Python face of ``oracle/lbm_oracle.c``: a restatement of lettuce's torch step
(stream by periodic roll, masked collide substeps, boundary operators) in
plain C. Only the test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use this module, always as the reference of a comparison
or the timed CPU baseline, never as part of the product path.

Boundaries are described by plain dicts so the oracle does not depend on the
product's classes:

* ``{"kind": "bounce_back", "mask": bool[*res]}``
  (lettuce/ext/_boundary/bounce_back_boundary.py:10-32)
* ``{"kind": "equilibrium_pu", "mask": bool[*res], "rho": arr, "u": arr}``
  with ``rho`` broadcastable to ``[*res]`` and ``u`` to ``[D, *res]``, both in
  lattice units (lettuce/ext/_boundary/equilibrium_boundary_pu.py:71-84)
* ``{"kind": "anti_bounce_back", "direction": [1, 0, 0]}``
  (lettuce/ext/_boundary/anti_bounce_back_outlet.py:22-103)
* ``{"kind": "equilibrium_outlet_p", "direction": [1, 0], "rho": 1.0}``
  (lettuce/ext/_boundary/equilibrium_outlet_p.py:12-91)
* ``{"kind": "partially_saturated", "mask": bool[*res], "tau": t, "B": b}``
  (lettuce/ext/_boundary/partially_saturated_boundary.py:6-51)
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liblbm_oracle.so")
_lock = threading.Lock()
_lib = None

STENCIL_IDS = {"D1Q3": 1, "D2Q9": 2, "D3Q15": 3, "D3Q19": 4, "D3Q27": 5}
COLLISION_IDS = {"none": 0, "bgk": 1, "trt": 2, "kbc": 3, "regularized": 4, "smagorinsky": 5,
                 "mrt": 6}
MRT_EQ_IDS = {"generic": 0, "dellar": 1, "lallemand": 2, "hermite": 3}
FORCE_IDS = {None: 0, "guo": 1, "shan_chen": 2}
SUB_KIND = {"collision": 0, "bounce_back": 1, "equilibrium_pu": 2,
            "anti_bounce_back": 3, "none": 4, "equilibrium_outlet_p": 5,
            "partially_saturated": 6}
# lettuce/cuda_native/_default_code_gen.py:13-17
STRATEGY_IDS = {"NO_STREAMING": 0, "POST_STREAMING": 1, "PRE_STREAMING": 2,
                "DOUBLE_STREAMING": 3}

# Velocity sets, lettuce/ext/_stencil/*.py (same q ordering).
_E = {
    "D1Q3": [[0], [1], [-1]],
    "D2Q9": [[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1], [1, 1], [-1, 1],
             [-1, -1], [1, -1]],
    "D3Q15": [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
              [0, 0, 1], [0, 0, -1], [1, 1, 1], [-1, -1, -1], [1, 1, -1],
              [-1, -1, 1], [1, -1, 1], [-1, 1, -1], [1, -1, -1], [-1, 1, 1]],
    "D3Q19": [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
              [0, 0, 1], [0, 0, -1], [0, 1, 1], [0, -1, -1], [0, 1, -1],
              [0, -1, 1], [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1],
              [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0]],
}
_E["D3Q27"] = _E["D3Q19"] + [[1, 1, 1], [-1, -1, -1], [1, 1, -1],
                             [-1, -1, 1], [1, -1, 1], [-1, 1, -1],
                             [1, -1, -1], [-1, 1, 1]]
_W = {
    "D1Q3": [2 / 3, 1 / 6, 1 / 6],
    "D2Q9": [4 / 9] + [1 / 9] * 4 + [1 / 36] * 4,
    "D3Q15": [2 / 9] + [1 / 9] * 6 + [1 / 72] * 8,
    "D3Q19": [1 / 3] + [1 / 18] * 6 + [1 / 36] * 12,
    "D3Q27": [8 / 27] + [2 / 27] * 6 + [1 / 54] * 12 + [1 / 216] * 8,
}


def stencil_tables(name):
    e = np.array(_E[name], dtype=np.int64)
    w = np.array(_W[name], dtype=np.float64)
    opp = np.array([int(np.where((e == -e[i]).all(axis=1))[0][0])
                    for i in range(len(e))], dtype=np.int64)
    return e, w, opp


class _Sub(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32),
                ("rho", ctypes.c_void_p),
                ("u", ctypes.c_void_p),
                ("rho_stride", ctypes.c_int64 * 3),
                ("u_stride", ctypes.c_int64 * 4),
                ("axis", ctypes.c_int32),
                ("sign", ctypes.c_int32),
                ("param", ctypes.c_double * 2)]


class _Problem(ctypes.Structure):
    _fields_ = [("stencil", ctypes.c_int32),
                ("res", ctypes.c_int32 * 3),
                ("collision", ctypes.c_int32),
                ("strategy", ctypes.c_int32),
                ("tau", ctypes.c_double),
                ("tau_minus", ctypes.c_double),
                ("ncm", ctypes.c_void_p),
                ("nsm", ctypes.c_void_p),
                ("n_sub", ctypes.c_int32),
                ("collision_index", ctypes.c_int32),
                ("sub", ctypes.POINTER(_Sub)),
                ("force", ctypes.c_int32),
                ("force_tau", ctypes.c_double),
                ("accel", ctypes.c_double * 3),
                ("smagorinsky_constant", ctypes.c_double),
                ("mrt_equilibrium", ctypes.c_int32),
                ("mrt_tables", ctypes.c_void_p),
                ("n_links", ctypes.c_int64),
                ("links", ctypes.c_void_p),
                ("force_out", ctypes.c_void_p),
                ("link_d", ctypes.c_void_p),
                ("link_force", ctypes.c_void_p)]


def build():
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(_LIB_PATH):
                build()
            L = ctypes.CDLL(_LIB_PATH)
            P = ctypes.c_void_p
            L.orc_run_f64.argtypes = [ctypes.POINTER(_Problem), P, P, ctypes.c_int, ctypes.c_int]
            L.orc_run_f32.argtypes = [ctypes.POINTER(_Problem), P, P, ctypes.c_int, ctypes.c_int]
            L.orc_moments_f64.argtypes = [ctypes.c_int, P, P, P, P, ctypes.c_int]
            L.orc_moments_f32.argtypes = [ctypes.c_int, P, P, P, P, ctypes.c_int]
            L.orc_equilibrium_f64.argtypes = [ctypes.c_int, P, P, P, P, ctypes.c_int]
            _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _bcast_strides(arr, shape):
    """element strides of ``arr`` broadcast to ``shape`` (0 on broadcast dims)"""
    assert arr.ndim == len(shape), (arr.shape, shape)
    out = []
    for i, n in enumerate(shape):
        if arr.shape[i] == 1:
            out.append(0)
        else:
            assert arr.shape[i] == n, (arr.shape, shape)
            out.append(arr.strides[i] // arr.itemsize)
    return out


def boundary_masks(b, resolution, q, name):
    """(no_collision_mask, no_streaming_mask) of one boundary dict, following
    the boundaries' make_no_collision_mask / make_no_streaming_mask."""
    res = list(resolution)
    kind = b["kind"]
    if kind in ("bounce_back", "equilibrium_pu", "partially_saturated"):
        return np.asarray(b["mask"], dtype=bool), None
    if kind == "equilibrium_outlet_p":
        # lettuce/ext/_boundary/equilibrium_outlet_p.py:73-85
        e, _, _ = stencil_tables(name)
        direction = list(b["direction"])
        vel = np.where(e @ np.array(direction) > 1 - 1e-6)[0]
        index = [slice(None) if i == 0 else (-1 if i == 1 else 0) for i in direction]
        nsm = np.zeros([q] + res, dtype=bool)
        nsm[tuple([np.setdiff1d(np.arange(q), vel)] + index)] = True
        ncm = np.zeros(res, dtype=bool)
        ncm[tuple(index)] = True
        return ncm, nsm
    if kind == "anti_bounce_back":
        # lettuce/ext/_boundary/anti_bounce_back_outlet.py:37-58, 93-103
        e, _, opp = stencil_tables(name)
        direction = list(b["direction"])
        vel = np.where(e @ np.array(direction) > 1 - 1e-6)[0]
        index = []
        for i in direction:
            if i == 0:
                index.append(slice(None))
            elif i == 1:
                index.append(-1)
            else:
                index.append(0)
        nsm = np.zeros([q] + res, dtype=bool)
        nsm[tuple([opp[vel]] + index)] = True
        ncm = np.zeros(res, dtype=bool)
        ncm[tuple(index)] = True
        return ncm, nsm
    if kind == "none":
        return None, None
    raise ValueError(kind)


def assemble_masks(resolution, q, name, pre, post):
    """no_collision_mask / no_streaming_mask as lettuce/_simulation.py:100-146
    builds them (integer index field, last writer wins; OR of the boolean
    no-streaming masks onto a field initialised to the collision index)."""
    ci = len(pre)
    if len(pre) + len(post) == 0:
        return None, None
    ncm = np.full(list(resolution), ci, dtype=np.uint8)
    nsm = np.full([q] + list(resolution), ci, dtype=np.uint8)
    for i, b in list(enumerate(pre)) + list(enumerate(post, start=ci + 1)):
        c, s = boundary_masks(b, resolution, q, name)
        if c is not None:
            ncm[c] = i
        if s is not None:
            nsm |= s.astype(np.uint8)
    return ncm, nsm


def ebb_masks(resolution, q, name, pre, post, post_streaming):
    """the masks of the example EbbSimulation
    (examples/advanced_projects/efficient_bounce_back_obstacle/simulation/
    ebb_simulation.py:28-57): lettuce's masks, created filled with the
    collision index if there were none, then each post-streaming
    boundary's solid cells take index collision_index + 1 + len(post) + j
    and, except for the full-way variant's, keep all populations in the
    stream"""
    ncm, nsm = assemble_masks(resolution, q, name, pre, post)
    if not post_streaming:
        return ncm, nsm
    ci = len(pre)
    if ncm is None:
        ncm = np.full(list(resolution), ci, dtype=np.uint8)
        nsm = np.full([q] + list(resolution), ci, dtype=np.uint8)
    for i, b in enumerate(post_streaming, start=ci + 1 + len(post)):
        solid = np.asarray(b["solid"], dtype=bool)
        ncm[solid] = i
        if not b.get("fullway"):
            # the full-way variant's solid cells stream
            # (fullway_bounce_back_boundary.py:182-184)
            nsm |= solid[None].astype(np.uint8)
    return ncm, nsm


def link_cells(f_index, resolution):
    """(q, flat cell index) rows of a halfway bounce-back link list given as
    (q, x, y[, z]) rows; negative coordinates count from the end, as the
    example's torch indexing reads them"""
    fi = np.asarray(f_index, dtype=np.int64).reshape(-1, len(resolution) + 1)
    res = np.array(resolution, dtype=np.int64)
    cells = np.where(fi[:, 1:] < 0, fi[:, 1:] + res, fi[:, 1:])
    flat = np.ravel_multi_index(tuple(cells.T), tuple(resolution))
    return np.ascontiguousarray(np.stack([fi[:, 0], flat], axis=1).astype(np.int64))


def run(name, f, nsteps, collision="bgk", tau=1.0, tau_minus=1.0,
        strategy="POST_STREAMING", pre=(), post=(), nthreads=None,
        masks=None, force=None, force_tau=1.0, accel=(0.0, 0.0, 0.0),
        smagorinsky_constant=0.17, mrt=None, post_streaming=(), forces=None):
    """Advance ``f`` ([Q, *res], float64 or float32) by ``nsteps`` steps and
    return the new array; ``f`` is not modified. ``force`` ("guo",
    "shan_chen" or None) with ``force_tau`` and ``accel`` (lattice units)
    applies to the BGK and Smagorinsky collisions. ``mrt`` = (equilibrium
    name, M, M^-1, relaxation times) for the "mrt" collision.
    ``post_streaming``: bounce-back boundaries of lettuce's example
    project, dicts with "solid" (mask), "f_index" (link rows q, x, y[, z])
    and, for the linear interpolated one, "d" (wall distance per row;
    without it the links are halfway), "force" (default True: its links
    count into ``forces``); the post-streaming full-way bounce-back is
    "fullway": True with its solid-cell links and d = 0 (the bounced value
    is then the streamed one); with any, every step runs collide,
    stream, bounce (the example EbbSimulation) whatever ``strategy`` says,
    and ``forces`` (float64 [nsteps, 3], optional) receives each step's
    momentum-exchange force over all links."""
    L = lib()
    f = np.ascontiguousarray(f)
    dt = f.dtype
    assert dt in (np.float64, np.float32)
    q = f.shape[0]
    res = list(f.shape[1:])
    pre, post = list(pre), list(post)
    post_streaming = list(post_streaming)
    if masks is None:
        ncm, nsm = ebb_masks(res, q, name, pre, post, post_streaming)
    else:
        ncm, nsm = masks
    keep = []
    subs = (_Sub * max(1, len(pre) + 1 + len(post)))()
    for i, b in enumerate(pre + [{"kind": "collision"}] + post):
        s = subs[i]
        s.kind = SUB_KIND[b["kind"]]
        if b["kind"] == "equilibrium_pu":
            rho = np.ascontiguousarray(np.asarray(b["rho"], dtype=dt))
            u = np.ascontiguousarray(np.asarray(b["u"], dtype=dt))
            rho = rho.reshape(rho.shape[-len(res):] if rho.ndim >= len(res) else [1] * len(res))
            if u.ndim == len(res):
                u = u[None]
            keep += [rho, u]
            rs = _bcast_strides(rho, res)
            us = _bcast_strides(u, [len(res)] + res)
            s.rho = rho.ctypes.data
            s.u = u.ctypes.data
            for k in range(3):
                s.rho_stride[k] = rs[k] if k < len(rs) else 0
            for k in range(4):
                s.u_stride[k] = us[k] if k < len(us) else 0
        if b["kind"] in ("anti_bounce_back", "equilibrium_outlet_p"):
            d = list(b["direction"])
            ax = [i for i, v in enumerate(d) if v != 0][0]
            s.axis = ax
            s.sign = int(d[ax])
        if b["kind"] == "equilibrium_outlet_p":
            s.param[0] = float(b.get("rho", 1.0))
        if b["kind"] == "partially_saturated":
            s.param[0] = float(b["tau"])
            s.param[1] = float(b["B"])
    p = _Problem()
    p.stencil = STENCIL_IDS[name]
    for k in range(3):
        p.res[k] = res[k] if k < len(res) else 1
    p.collision = COLLISION_IDS[collision]
    p.strategy = STRATEGY_IDS[strategy]
    p.tau = float(tau)
    p.tau_minus = float(tau_minus)
    p.force = FORCE_IDS[force]
    p.force_tau = float(force_tau)
    for k, a in enumerate(list(accel)[:3]):
        p.accel[k] = float(a)
    p.smagorinsky_constant = float(smagorinsky_constant)
    if mrt is not None:
        eq, M, Mi, srel = mrt
        tables = np.ascontiguousarray(np.concatenate(
            [np.asarray(M, np.float64).ravel(), np.asarray(Mi, np.float64).ravel(),
             np.asarray(srel, np.float64).ravel()]))
        keep.append(tables)
        p.mrt_equilibrium = MRT_EQ_IDS[eq]
        p.mrt_tables = tables.ctypes.data
    if ncm is not None:
        ncm = np.ascontiguousarray(ncm, dtype=np.uint8)
        nsm = np.ascontiguousarray(nsm, dtype=np.uint8)
        p.ncm = ncm.ctypes.data
        p.nsm = nsm.ctypes.data
    p.n_sub = len(pre) + 1 + len(post)
    p.collision_index = len(pre)
    p.sub = subs
    if post_streaming:
        links = np.concatenate([link_cells(b["f_index"], res) for b in post_streaming], axis=0)
        dist = np.ascontiguousarray(np.concatenate(
            [np.asarray(b["d"], dtype=np.float64).ravel() if "d" in b
             else np.full(len(np.asarray(b["f_index"]).reshape(-1, len(res) + 1)), -1.0)
             for b in post_streaming]))
        counted = np.ascontiguousarray(np.concatenate(
            [np.full(len(np.asarray(b["f_index"]).reshape(-1, len(res) + 1)),
                     0 if not b.get("force", True) else (2 if b.get("fullway") else 1),
                     dtype=np.uint8)
             for b in post_streaming]))
        keep += [links, dist, counted]
        p.n_links = len(links)
        p.links = links.ctypes.data
        p.link_d = dist.ctypes.data
        p.link_force = counted.ctypes.data
        if forces is not None:
            assert forces.dtype == np.float64 and forces.shape == (nsteps, 3)
            assert forces.flags["C_CONTIGUOUS"]
            p.force_out = forces.ctypes.data
    out = f.copy()
    work = np.empty_like(f)
    nthreads = nthreads or os.cpu_count() or 1
    fn = L.orc_run_f64 if dt == np.float64 else L.orc_run_f32
    rc = fn(ctypes.byref(p), _ptr(out), _ptr(work), int(nsteps), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle run failed ({rc})")
    return out


def moments(name, f, nthreads=None):
    """(rho [*res], u [D, *res]) of f, lettuce/_flow.py:157-193"""
    L = lib()
    f = np.ascontiguousarray(f)
    res = list(f.shape[1:])
    r3 = (ctypes.c_int32 * 3)(*(res + [1] * (3 - len(res))))
    rho = np.empty(res, dtype=f.dtype)
    u = np.empty([len(res)] + res, dtype=f.dtype)
    fn = L.orc_moments_f64 if f.dtype == np.float64 else L.orc_moments_f32
    rc = fn(STENCIL_IDS[name], ctypes.cast(r3, ctypes.c_void_p), _ptr(f), _ptr(rho), _ptr(u),
            int(nthreads or os.cpu_count() or 1))
    if rc != 0:
        raise RuntimeError("oracle moments failed")
    return rho, u


def equilibrium(name, rho, u, nthreads=None):
    """quadratic equilibrium [Q, *res] (float64)"""
    L = lib()
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    res = list(rho.shape)
    q = len(_E[name])
    r3 = (ctypes.c_int32 * 3)(*(res + [1] * (3 - len(res))))
    feq = np.empty([q] + res, dtype=np.float64)
    rc = L.orc_equilibrium_f64(STENCIL_IDS[name], ctypes.cast(r3, ctypes.c_void_p), _ptr(rho),
                               _ptr(u), _ptr(feq), int(nthreads or os.cpu_count() or 1))
    if rc != 0:
        raise RuntimeError("oracle equilibrium failed")
    return feq


def kinetic_energy(name, f):
    """sum over cells of 0.5 |u|^2 in lattice units, accumulated in float64
    (lettuce/_flow.py:200-204 summed as in
    lettuce/ext/_reporter/observable_reporter.py:34-42 before unit scaling)"""
    _, u = moments(name, np.asarray(f, dtype=np.float64))
    return float(0.5 * np.sum(u * u))
