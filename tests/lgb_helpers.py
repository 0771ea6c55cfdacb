"""Shared helpers of the GPU tests: a flow with given populations (like the
DummyFlow of lettuce's tests/conftest.py) and comparison utilities."""
import numpy as np
import torch

import lettuce_gb300 as lt


class GivenFlow(lt.ExtFlow):
    """populations set directly; optional post-boundaries"""

    def __init__(self, context, stencil, f0, boundaries=(), reynolds_number=100.0,
                 mach_number=0.05):
        self._f0 = np.asarray(f0)
        self._bnds = list(boundaries)
        super().__init__(context, list(self._f0.shape[1:]), reynolds_number, mach_number,
                         stencil=stencil)

    def make_resolution(self, resolution, stencil=None):
        return list(resolution)

    def make_units(self, reynolds_number, mach_number, resolution):
        return lt.UnitConversion(reynolds_number=reynolds_number, mach_number=mach_number)

    def initial_pu(self):
        raise NotImplementedError

    def initialize(self):
        self.f = torch.as_tensor(self._f0)

    @property
    def post_boundaries(self):
        return self._bnds


def collision_of(kind, tau, flow=None):
    if kind == "bgk":
        return lt.BGKCollision(tau)
    if kind == "trt":
        return lt.TRTCollision(tau, 1.0)
    if kind == "kbc":
        return lt.KBCCollision(tau)
    return lt.NoCollision()


def rel_max(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.max(np.abs(a - b)) / max(1e-300, np.max(np.abs(b))))


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(1e-300, np.linalg.norm(b)))


def to_np(t):
    return t.detach().to(torch.float64).cpu().numpy()


def obstacle_flow(context, z, m):
    S = getattr(lt, m["stencil"])
    flow = lt.Obstacle(context, m["res"], m["re"], m["ma"], m["domain_length_x"], stencil=S)
    flow.mask = z["mask"]
    flow.initialize()
    return flow


def obstacle_oracle_boundaries(z, m):
    res = m["res"]
    d = len(res)
    x = np.arange(res[0]).reshape([-1] + [1] * (d - 1)) * np.ones(res)
    return [{"kind": "equilibrium_pu", "mask": np.abs(x) < 1e-6,
             "rho": z["inlet_rho_lu"].reshape([1] * d),
             "u": z["inlet_u_lu"].reshape([d] + [1] * d)},
            {"kind": "anti_bounce_back", "direction": [1] + [0] * (d - 1)},
            {"kind": "bounce_back", "mask": z["mask"]}]


class HwbbFlow(GivenFlow):
    """a given-populations flow with post-streaming boundaries (the
    property the example EbbSimulation looks for on the flow's class)"""
    psb = ()

    @property
    def post_streaming_boundaries(self):
        return list(self.psb)


def hwbb_case(context, z, meta, f0=None):
    """(flow, boundary) of a halfway bounce-back golden case: the given
    populations, the optional equilibrium inlet on x = 0 and the boundary
    with its force computed"""
    stencil = getattr(lt, meta["stencil"])()
    f0 = z["f0"] if f0 is None else f0
    flow = HwbbFlow(context, stencil, f0)
    res = list(meta["res"])
    if meta["inlet"]:
        m = torch.zeros(res, dtype=torch.bool)
        m[0] = True
        vel = torch.tensor([0.02] + [0.0] * (len(res) - 1), dtype=context.dtype)
        flow._bnds = [lt.EquilibriumBoundaryPU(context, flow, m, vel)]
    sbd = lt.SolidBoundaryData()
    sbd.solid_mask = z["solid"]
    g = None if "global_extra" not in z else (z["solid"] | z["global_extra"])
    per = meta["periodicity"]
    hw = lt.HalfwayBounceBackBoundary(context, flow, sbd, global_solid_mask=g,
                                      periodicity=None if per is None else tuple(per),
                                      calc_force=True)
    flow.psb = [hw]
    return flow, hw


def ibb_case(context, z, meta, f0=None):
    """(flow, boundary) of an interpolated bounce-back golden case"""
    stencil = getattr(lt, meta["stencil"])()
    f0 = z["f0"] if f0 is None else f0
    flow = HwbbFlow(context, stencil, f0)
    sbd = lt.SolidBoundaryData()
    sbd.solid_mask = z["solid"]
    sbd.f_index_lt, sbd.f_index_gt = z["f_index_lt"], z["f_index_gt"]
    sbd.d_lt, sbd.d_gt = z["d_lt"], z["d_gt"]
    b = lt.LinearInterpolatedBounceBackBoundary(context, flow, sbd, calc_force=True)
    flow.psb = [b]
    return flow, b


def fwbb_case(context, z, meta, f0=None):
    """(flow, boundary) of a post-streaming full-way bounce-back golden case"""
    stencil = getattr(lt, meta["stencil"])()
    f0 = z["f0"] if f0 is None else f0
    flow = HwbbFlow(context, stencil, f0)
    g = None if "global_extra" not in z else (z["solid"] | z["global_extra"])
    per = meta["periodicity"]
    b = lt.FullwayBounceBackBoundary(context, flow, z["solid"], global_solid_mask=g,
                                     periodicity=None if per is None else tuple(per),
                                     calc_force=True)
    flow.psb = [b]
    return flow, b
