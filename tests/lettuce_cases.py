"""Simulations built the same way from lettuce's classes or from this
package's mirror of them: ``cases(L, ctx)`` takes the module (``lettuce`` or
``lettuce_gb300``, whose public names are the same) and a context, and
returns ``{name: simulation}``. ``tests/golden/make_binding_golden.py`` runs
``lettuce_gb300.native_step`` on lettuce's objects and stores what it
builds; ``tests/test_lettuce_binding.py`` checks that the mirror's objects
give the same descriptors and masks.

Covered: every streaming strategy; BGK (with Guo and Shan-Chen forces), TRT,
KBC, regularized, Smagorinsky, MRT (Dellar), no collision; bounce-back,
equilibrium inlet, anti-bounce-back and pressure outlets, partially
saturated cells; a pre-collision boundary (lettuce's collision index 1, whose
no-streaming mask starts at 1 everywhere)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def import_lettuce():
    """lettuce itself, or None: from ``$LETTUCE_SRC`` (its source folder) or
    from its offline install in ``baseline/_ref`` (``pip install --target``),
    its optional file-output imports from the stand-ins in
    ``tests/golden/_stubs``"""
    root = os.path.dirname(HERE)
    for src in (os.environ.get("LETTUCE_SRC"), os.path.join(root, "baseline", "_ref")):
        if src and os.path.isfile(os.path.join(src, "lettuce", "__init__.py")):
            for p in (os.path.join(HERE, "golden", "_stubs"), src):
                if p not in sys.path:
                    sys.path.insert(0, p)
            break
    import warnings
    try:
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            import lettuce
    except ImportError:
        return None
    return lettuce if hasattr(lettuce, "Simulation") else None


def _sphere(res, centre, radius):
    grid = np.meshgrid(*[np.arange(n) for n in res], indexing="ij")
    return sum((g - c) ** 2 for g, c in zip(grid, centre)) < radius ** 2


def _transform(L, name):
    """lettuce keeps its moment transforms in lettuce.util.moments (not
    re-exported); this package exports them at the top level"""
    if hasattr(L, name):
        return getattr(L, name)
    import importlib
    return getattr(importlib.import_module(L.__name__ + ".util.moments"), name)


def cases(L, ctx):
    out = {}
    S = L.StreamingStrategy

    flow = L.TaylorGreenVortex(ctx, [12, 10, 8], 1600, 0.05, L.D3Q19())
    out["tgv3d_bgk_pre"] = L.Simulation(flow, L.BGKCollision(flow.units.relaxation_parameter_lu),
                                        [], streaming_strategy=S.PRE_STREAMING)

    flow = L.TaylorGreenVortex(ctx, [14, 12], 1000, 0.05, L.D2Q9())
    out["tgv2d_trt_post"] = L.Simulation(flow, L.TRTCollision(0.61, 0.83), [],
                                         streaming_strategy=S.POST_STREAMING)

    flow = L.TaylorGreenVortex(ctx, [10, 8, 6], 1000, 0.05, L.D3Q27())
    out["tgv3d_kbc_double"] = L.Simulation(flow, L.KBCCollision(), [],
                                           streaming_strategy=S.DOUBLE_STREAMING)

    flow = L.TaylorGreenVortex(ctx, [10, 8, 6], 1000, 0.05, L.D3Q19())
    out["tgv3d_smagorinsky_none"] = L.Simulation(flow, L.SmagorinskyCollision(0.57, 0.2), [],
                                                 streaming_strategy=S.NO_STREAMING)

    flow = L.TaylorGreenVortex(ctx, [12, 12], 1000, 0.05, L.D2Q9())
    out["tgv2d_regularized_pre"] = L.Simulation(flow, L.RegularizedCollision(), [],
                                                streaming_strategy=S.PRE_STREAMING)

    flow = L.TaylorGreenVortex(ctx, [12, 12], 1000, 0.05, L.D2Q9())
    srel = [1.0, 1.0, 1.0, 0.7, 0.7, 0.9, 0.9, 0.63, 0.63]
    out["tgv2d_mrt_dellar_pre"] = L.Simulation(
        flow, L.MRTCollision(_transform(L, "D2Q9Dellar")(L.D2Q9(), ctx), srel, ctx), [],
        streaming_strategy=S.PRE_STREAMING)

    flow = L.TaylorGreenVortex(ctx, [8, 8], 1000, 0.05, L.D2Q9())
    out["tgv2d_none_post"] = L.Simulation(flow, L.NoCollision(), [],
                                          streaming_strategy=S.POST_STREAMING)

    flow = L.PoiseuilleFlow2D(ctx, 17, 1, 0.02)
    a_lu = flow.units.convert_acceleration_to_lu(flow.acceleration)
    tau = flow.units.relaxation_parameter_lu
    out["poiseuille_guo_post"] = L.Simulation(
        flow, L.BGKCollision(tau, force=L.Guo(flow, tau, a_lu)), [])
    flow = L.PoiseuilleFlow2D(ctx, 17, 1, 0.02)
    out["poiseuille_shanchen_pre"] = L.Simulation(
        flow, L.BGKCollision(tau, force=L.ShanChen(flow, 0.8, a_lu)), [],
        streaming_strategy=S.PRE_STREAMING)

    for strat, tag in ((S.PRE_STREAMING, "pre"), (S.POST_STREAMING, "post")):
        res = [40, 20]
        flow = L.Obstacle(ctx, res, 100, 0.1, res[0] / 4.0, stencil=L.D2Q9())
        flow.mask = _sphere(res, [res[0] / 3.0, res[1] / 2.0 - 0.5], 4)
        flow.initialize()
        out[f"obstacle2d_bgk_{tag}"] = L.Simulation(
            flow, L.BGKCollision(flow.units.relaxation_parameter_lu), [],
            streaming_strategy=strat)

    res = [24, 10, 10]
    flow = L.Obstacle(ctx, res, 100, 0.1, res[0] / 4.0, stencil=L.D3Q27())
    flow.mask = _sphere(res, [8, 4.5, 4.5], 3)
    flow.initialize()
    out["obstacle3d_kbc_pre"] = L.Simulation(flow, L.KBCCollision(), [],
                                             streaming_strategy=S.PRE_STREAMING)

    class ObstacleP(L.Obstacle):
        @property
        def post_boundaries(self):
            b = L.Obstacle.post_boundaries.fget(self)
            return [b[0], L.EquilibriumOutletP(self._unit_vector().tolist(), self,
                                               rho_outlet=1.02), b[2]]
    res = [30, 14]
    flow = ObstacleP(ctx, res, 100, 0.1, res[0] / 4.0, stencil=L.D2Q9())
    flow.mask = _sphere(res, [10, 6.5], 3)
    flow.initialize()
    out["obstacle2d_outletp_post"] = L.Simulation(
        flow, L.BGKCollision(flow.units.relaxation_parameter_lu), [])

    solid = np.zeros([16, 12], dtype=bool)
    solid[4:9, 3:7] = True
    porous = np.zeros([16, 12], dtype=bool)
    porous[10:13, 2:5] = True

    class PreAndPost(L.TaylorGreenVortex):
        @property
        def pre_boundaries(self):
            return [L.BounceBackBoundary(self.context.convert_to_tensor(solid, dtype=bool))]

        @property
        def post_boundaries(self):
            return [L.PartiallySaturatedBC(self.context.convert_to_tensor(porous, dtype=bool),
                                           0.7, 0.3),
                    L.AntiBounceBackOutlet([0, -1], self)]
    flow = PreAndPost(ctx, [16, 12], 1000, 0.05, L.D2Q9())
    out["pre_and_post_bgk_post"] = L.Simulation(flow, L.BGKCollision(0.7), [],
                                                streaming_strategy=S.POST_STREAMING)
    return out


def desc_signature(desc) -> bytes:
    """the bytes of an lgb_step_desc with every pointer field zeroed (what
    remains: ids, sizes, relaxation times, substep kinds and parameters,
    strides, options)"""
    import ctypes
    copy = type(desc).from_buffer_copy(desc)

    def zero(struct):
        for name, typ in struct._fields_:
            if typ is ctypes.c_void_p:
                setattr(struct, name, None)
            elif isinstance(typ, type) and issubclass(typ, ctypes.Array) and \
                    issubclass(typ._type_, ctypes.Structure):
                for item in getattr(struct, name):
                    zero(item)
    zero(copy)
    return ctypes.string_at(ctypes.addressof(copy), ctypes.sizeof(copy))


def step_record(step) -> dict:
    """arrays describing a lettuce_gb300.NativeStep, for comparison"""
    rec = {"desc": np.frombuffer(desc_signature(step.desc), dtype=np.uint8).copy(),
           "patterns": np.asarray(step.patterns, dtype=np.int64)}
    if step.flags is not None:
        rec["flags"] = step.flags.cpu().numpy()
    if step.no_stream_bits is not None:
        rec["nsb"] = step.no_stream_bits.cpu().numpy()
    for k, nat in enumerate(step.natives):
        if getattr(nat, "rho", None) is not None:
            rec[f"sub{k}_rho"] = nat.rho.double().cpu().numpy()
            rec[f"sub{k}_u"] = nat.u.double().cpu().numpy()
        if getattr(nat, "mrt_tables", None) is not None:
            rec[f"sub{k}_mrt"] = np.asarray(nat.mrt_tables, dtype=np.float64)
    return rec
