"""Observables and reporters (lettuce/ext/_reporter/observable_reporter.py,
error_reporter.py, failure_reporter.py).

The scalar observables are float64 reductions on the device
(``lgb_reduce``): the field is read once, nothing per cell is copied to the
host, and only the final scalars cross the bus when a reporter fires.
"""
from __future__ import annotations

import os
import sys
from abc import ABC, abstractmethod
from typing import List, Optional, Tuple

import numpy as np
import torch

from . import _device
from ._flow import torch_gradient
from ._simulation import Reporter

__all__ = ["Observable", "ObservableReporter", "MaximumVelocity",
           "IncompressibleKineticEnergy", "Enstrophy", "EnergySpectrum", "Mass",
           "DragCoefficient", "LiftCoefficient",
           "ErrorReporter", "FailureReporterBase", "NaNReporter", "HighMaReporter",
           "reduce_flow"]


def reduce_flow(flow, lo=None, hi=None, mask=None) -> torch.Tensor:
    """float64 device tensor [mass, 0.5*sum|u|^2, max|u|^2, non-finite cells,
    masked mass] of the flow's current populations (lattice units)"""
    m = None
    if mask is not None:
        m = torch.as_tensor(mask, device=flow.context.device).to(torch.uint8).contiguous()
    if flow._stream_pending is not None:
        flow._settle()
    return _device.reduce(flow.stencil.lgb_id, flow.context.storage, flow.resolution,
                          flow.f_raw, flow._aa_pending, lo, hi, m)


class Observable(ABC):
    def __init__(self, flow):
        self.context = flow.context
        self.flow = flow

    @abstractmethod
    def __call__(self, f: Optional[torch.Tensor] = None):
        ...


class MaximumVelocity(Observable):
    """max |u| in physical units (observable_reporter.py:27-31)"""

    def __call__(self, f: Optional[torch.Tensor] = None):
        r = reduce_flow(self.flow)
        return self.flow.units.convert_velocity_to_pu(torch.sqrt(r[2]))


class IncompressibleKineticEnergy(Observable):
    """dx^D * sum 0.5 |u|^2 in physical units (observable_reporter.py:34-42),
    accumulated in float64"""

    def __call__(self, f: Optional[torch.Tensor] = None):
        dx = self.flow.units.convert_length_to_pu(1.0)
        r = reduce_flow(self.flow)
        kin = self.flow.units.convert_incompressible_energy_to_pu(r[1])
        return kin * dx ** self.flow.stencil.d


class Enstrophy(Observable):
    """integral of the squared vorticity, periodic domains
    (observable_reporter.py:45-71)"""

    def __call__(self, f: Optional[torch.Tensor] = None):
        dx = self.flow.units.convert_length_to_pu(1.0)
        if self.flow.context.device.type == "cuda":
            # one fused float64 kernel over the velocity field: the sum of
            # |curl u|^2 in lattice units, then lettuce's unit scaling
            # (u_pu = c u_lu, d/dx_pu = d/dx_lu / dx)
            c = self.flow.units.convert_velocity_to_pu(1.0)
            ens = _device.enstrophy_lu(self.flow.u())
            return ens[0] * ((c / dx) ** 2 * dx ** self.flow.stencil.d)
        u = self.flow.units.convert_velocity_to_pu(self.flow.u())
        g0 = torch_gradient(u[0], dx=dx, order=6)
        g1 = torch_gradient(u[1], dx=dx, order=6)
        vort = torch.sum((g0[1] - g1[0]) * (g0[1] - g1[0]))
        if self.flow.stencil.d == 3:
            g2 = torch_gradient(u[2], dx=dx, order=6)
            vort = vort + torch.sum((g2[1] - g1[2]) * (g2[1] - g1[2])
                                    + (g0[2] - g2[0]) * (g0[2] - g2[0]))
        return vort * dx ** self.flow.stencil.d


class EnergySpectrum(Observable):
    """kinetic energy spectrum by shells of |k| (observable_reporter.py:74-137)"""

    def __init__(self, flow):
        super().__init__(flow)
        self.dx = flow.units.convert_length_to_pu(1.0)
        self.dimensions = flow.resolution
        freqs = [self.context.convert_to_tensor(np.fft.fftfreq(n, d=1 / n))
                 for n in self.dimensions]
        wavenumbers = torch.stack(torch.meshgrid(*freqs, indexing="ij"))
        wavenorms = torch.norm(wavenumbers, dim=0)
        if flow.stencil.d == 3:
            self.norm = self.dimensions[0] * np.sqrt(2 * np.pi) / self.dx ** 2
        else:
            self.norm = self.dimensions[0] / self.dx
        self.wavenumbers = torch.arange(int(torch.max(wavenorms)))
        k = self.wavenumbers.to(dtype=self.context.dtype, device=self.context.device)
        self.wavemask = ((wavenorms[..., None] > k - 0.5) & (wavenorms[..., None] <= k + 0.5))

    def __call__(self, f: Optional[torch.Tensor] = None):
        return self.spectrum_from_u(self.flow.u())

    def spectrum_from_u(self, u):
        u = self.flow.units.convert_velocity_to_pu(u)
        d = self.flow.stencil.d
        uh = torch.stack([torch.fft.fftn(u[i], dim=tuple(range(d))) for i in range(d)]) / self.norm
        ekin = torch.sum(0.5 * (uh.imag ** 2 + uh.real ** 2), dim=0)
        ek = ekin[..., None] * self.wavemask.to(dtype=self.context.dtype)
        return ek.sum(tuple(range(d)))


class Mass(Observable):
    """total mass in lattice units over f[..., 1:-1, 1:-1] minus the mass on
    ``no_mass_mask`` cells (observable_reporter.py:140-158), float64"""

    def __init__(self, flow, no_mass_mask=None):
        super().__init__(flow)
        self.mask = no_mass_mask

    def __call__(self, f: Optional[torch.Tensor] = None):
        res = self.flow.resolution
        d = len(res)
        lo = [0] * d
        hi = list(res)
        for i in range(max(0, d - 2), d):
            lo[i], hi[i] = 1, res[i] - 1
        mass = reduce_flow(self.flow, lo, hi)[0]
        if self.mask is not None:
            mass = mass - reduce_flow(self.flow, mask=self.mask)[4]
        return mass


class DragCoefficient(Observable):
    """Drag coefficient of an obstacle from its bounce-back boundary's
    momentum exchange (the efficient-bounce-back example's
    reporter/observables_force_coefficients.py:15-48):
    F_x / (0.5 rho_mean u_lu^2 A_lu), with rho_mean the mean density over
    the cells outside ``solid_mask`` (a float64 device reduction), u_lu the
    characteristic velocity and A_lu = area_pu (L_lu / L_pu)^(D-1). The
    boundary must compute its force (``calc_force=True``)."""
    _axis = 0

    def __init__(self, flow, obstacle_boundary, solid_mask, area_pu: float):
        super().__init__(flow)
        self.obstacle_boundary = obstacle_boundary
        self.solid_mask = torch.as_tensor(np.asarray(solid_mask, dtype=bool)
                                          if not isinstance(solid_mask, torch.Tensor)
                                          else solid_mask, device=flow.context.device).bool()
        self._fluid = (~self.solid_mask).to(torch.uint8).contiguous()
        self._n_fluid = int(self._fluid.sum().item())
        u = flow.units
        self.area_lu = area_pu * (u.characteristic_length_lu /
                                  u.characteristic_length_pu) ** (flow.stencil.d - 1)

    def __call__(self, f: Optional[torch.Tensor] = None):
        force = self.obstacle_boundary.force_sum[self._axis].double()
        rho_mean = reduce_flow(self.flow, mask=self._fluid)[4] / max(1, self._n_fluid)
        c = force / (0.5 * rho_mean * self.flow.units.characteristic_velocity_lu ** 2
                     * self.area_lu)
        return c.to(self.context.dtype)


class LiftCoefficient(DragCoefficient):
    """Lift coefficient: as ``DragCoefficient`` with the force along y
    (observables_force_coefficients.py:51-83)"""
    _axis = 1


class ObservableReporter(Reporter):
    """prints (or collects) an observable every ``interval`` steps"""

    def __init__(self, observable, interval=1, out=sys.stdout):
        super().__init__(interval)
        self.observable = observable
        self.out = [] if out is None else out
        self._parameter_name = observable.__class__.__name__
        if out is not None:
            print("steps    ", "time    ", self._parameter_name)

    def __call__(self, simulation):
        if simulation.flow.i % self.interval == 0:
            observed = self.observable.context.convert_to_ndarray(self.observable())
            assert len(observed.shape) < 2
            observed = [observed.item()] if len(observed.shape) == 0 else observed.tolist()
            entry = [simulation.flow.i,
                     simulation.units.convert_time_to_pu(simulation.flow.i)] + observed
            if isinstance(self.out, list):
                self.out.append(entry)
            else:
                print(*entry, file=self.out)


class ErrorReporter(Reporter):
    """L2 errors of u and p against an analytic solution (error_reporter.py:8-42)"""

    def __init__(self, analytical_solution, interval=1, out=sys.stdout):
        super().__init__(interval)
        self.analytical_solution = analytical_solution
        self.out = [] if out is None else out
        if not isinstance(self.out, list):
            print("#error_u         error_p", file=self.out)

    def __call__(self, simulation):
        i = simulation.flow.i
        if i % self.interval != 0:
            return
        t = simulation.units.convert_time_to_pu(i)
        pref, uref = self.analytical_solution(t=t)
        ctx = simulation.flow.context
        pref = ctx.convert_to_tensor(pref)
        uref = ctx.convert_to_tensor(uref)
        p = simulation.flow.p_pu
        u = simulation.flow.u_pu
        d = simulation.flow.stencil.d
        resolution = float(np.prod(p.shape)) ** (1.0 / d)
        err_u = torch.norm(u - uref) / resolution ** (d / 2)
        err_p = torch.norm(p - pref) / resolution ** (d / 2)
        if isinstance(self.out, list):
            self.out.append([err_u.item(), err_p.item()])
        else:
            print(err_u.item(), err_p.item(), file=self.out)


class FailureReporterBase(Reporter, ABC):
    """stops a BreakableSimulation when ``is_failed`` holds, by pushing flow.i
    far past the target step (failure_reporter.py:12-58); writes a log of the
    top-k offending locations when ``outdir`` is given. VTK frames are not
    written by this library."""

    def __init__(self, interval: int, k: int = 100, outdir: Optional[str] = None,
                 vtk_out: bool = False):
        super().__init__(interval)
        self.k = k
        self.outdir = outdir
        self.name = "FailureReporter"
        self.vtk_out = vtk_out
        self.failed_iteration = None

    def __call__(self, simulation):
        if simulation.flow.i % self.interval == 0 and self.is_failed(simulation):
            self.failed_iteration = simulation.flow.i
            if self.outdir is not None:
                self._write_log(simulation, self.get_results(simulation))
            print(f"(!) ABORT MESSAGE: {self.name}Reporter detected {self.name} "
                  f"(reporter-interval = {self.interval}) at iteration {simulation.flow.i}.")
            simulation.flow.i = int(simulation.flow.i + 1e10)

    def _top_failures(self, mask: torch.Tensor, values: torch.Tensor) -> List[Tuple]:
        failed = values[mask]
        coords = torch.nonzero(mask)
        n = min(self.k, failed.numel())
        if torch.isnan(failed).any():
            idx = torch.arange(n, device=values.device)
        else:
            _, idx = torch.topk(failed, k=n, largest=True, sorted=True)
        return [(list(c.astype(int)), float(v)) for c, v in
                zip(coords[idx].cpu().numpy(), failed[idx].cpu().numpy())]

    def _write_log(self, simulation, results):
        os.makedirs(self.outdir, exist_ok=True)
        path = os.path.join(str(self.outdir), f"{self.name}_reporter.log")
        with open(path, "w") as fh:
            fh.write(f"(!) {self.name} detected in step {simulation.flow.i} at following "
                     f"locations (top {self.k} listed):\n     ")
            for loc in self.locations_string(simulation):
                fh.write(f"{loc:6}   ")
            fh.write("\n")
            for pos, val in results:
                line = "".join(f"{int(p):6}   " for p in pos)
                fh.write(f"{line:<20} | {val:<15.6f}\n")
            fh.write("\n")

    @abstractmethod
    def locations_string(self, simulation) -> List[str]:
        ...

    @abstractmethod
    def is_failed(self, simulation) -> bool:
        ...

    @abstractmethod
    def get_results(self, simulation) -> List[Tuple]:
        ...


class NaNReporter(FailureReporterBase):
    """fails when a cell's density is not finite (a NaN or infinite
    population); the check is one float64 reduction on the device"""

    def __init__(self, interval: int, k: int = 100, outdir: Optional[str] = None,
                 vtk_out: bool = False):
        super().__init__(interval, k, outdir, vtk_out)
        self.name = "NaN"

    def is_failed(self, simulation) -> bool:
        return bool(reduce_flow(simulation.flow)[3].item() > 0)

    def get_results(self, simulation):
        f = simulation.flow.f
        return self._top_failures(torch.isnan(f), f)

    def locations_string(self, simulation):
        return ["q", "x", "y", "z"][: simulation.flow.stencil.d + 1]


class HighMaReporter(FailureReporterBase):
    """fails when max |u| / cs exceeds ``threshold``"""

    def __init__(self, interval: int, threshold: float = 0.3, k: int = 100,
                 outdir: Optional[str] = None, vtk_out: bool = False):
        super().__init__(interval, k, outdir, vtk_out)
        self.threshold = threshold
        self.name = "HighMa"

    def is_failed(self, simulation) -> bool:
        umax2 = reduce_flow(simulation.flow)[2].item()
        return bool(np.sqrt(umax2) / simulation.flow.stencil.cs > self.threshold)

    def get_results(self, simulation):
        u = simulation.flow.u()
        ma = torch.norm(u, dim=0) / simulation.flow.stencil.cs
        return self._top_failures(ma > self.threshold, ma)

    def locations_string(self, simulation):
        return ["x", "y", "z"][: simulation.flow.stencil.d] + ["Ma"]
