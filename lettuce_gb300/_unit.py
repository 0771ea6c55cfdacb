"""Conversion between lattice units (lu) and physical units (pu), with the
same characteristic scales and relations as lettuce's UnitConversion
(lettuce/_unit.py:13-145): u_lu = cs * Ma, nu = L U / Re,
tau = nu_lu / cs^2 + 1/2."""
from __future__ import annotations

import numpy as np

__all__ = ["UnitConversion"]


class UnitConversion:
    def __init__(self, reynolds_number, mach_number=0.05,
                 characteristic_length_pu=1, characteristic_velocity_pu=1,
                 characteristic_length_lu=1, characteristic_density_lu=1,
                 characteristic_density_pu=1, cs=1 / np.sqrt(3.0)):
        self.cs = cs
        self.reynolds_number = reynolds_number
        self.mach_number = mach_number
        self.characteristic_length_pu = characteristic_length_pu
        self.characteristic_velocity_pu = characteristic_velocity_pu
        self.characteristic_length_lu = characteristic_length_lu
        self.characteristic_density_lu = characteristic_density_lu
        self.characteristic_density_pu = characteristic_density_pu

    @property
    def characteristic_velocity_lu(self):
        return self.cs * self.mach_number

    @property
    def characteristic_pressure_pu(self):
        return self.characteristic_density_pu * self.characteristic_velocity_pu ** 2

    @property
    def characteristic_pressure_lu(self):
        return self.characteristic_density_lu * self.characteristic_velocity_lu ** 2

    @property
    def viscosity_lu(self):
        return (self.characteristic_length_lu * self.characteristic_velocity_lu
                / self.reynolds_number)

    @property
    def viscosity_pu(self):
        return (self.characteristic_length_pu * self.characteristic_velocity_pu
                / self.reynolds_number)

    @property
    def relaxation_parameter_lu(self):
        return self.viscosity_lu / self.cs ** 2 + 0.5

    # velocity / acceleration / time ------------------------------------
    def convert_velocity_to_pu(self, v):
        return v / self.characteristic_velocity_lu * self.characteristic_velocity_pu

    def convert_velocity_to_lu(self, v):
        return v / self.characteristic_velocity_pu * self.characteristic_velocity_lu

    def _acc_scales(self):
        return (self.characteristic_velocity_lu ** 2 / self.characteristic_length_lu,
                self.characteristic_velocity_pu ** 2 / self.characteristic_length_pu)

    def convert_acceleration_to_pu(self, a):
        lu, pu = self._acc_scales()
        return a / lu * pu

    def convert_acceleration_to_lu(self, a):
        lu, pu = self._acc_scales()
        return a / pu * lu

    def _time_scales(self):
        return (self.characteristic_length_lu / self.characteristic_velocity_lu,
                self.characteristic_length_pu / self.characteristic_velocity_pu)

    def convert_time_to_pu(self, t):
        lu, pu = self._time_scales()
        return t / lu * pu

    def convert_time_to_lu(self, t):
        lu, pu = self._time_scales()
        return t / pu * lu

    # density / pressure ---------------------------------------------------
    def convert_density_lu_to_pressure_pu(self, rho):
        return self.convert_pressure_to_pu(
            (rho - self.characteristic_density_lu) * self.cs ** 2)

    def convert_pressure_pu_to_density_lu(self, p):
        return (self.convert_pressure_to_lu(p) / self.cs ** 2
                + self.characteristic_density_lu)

    def convert_density_to_pu(self, rho):
        return rho / self.characteristic_density_lu * self.characteristic_density_pu

    def convert_density_to_lu(self, rho):
        return rho / self.characteristic_density_pu * self.characteristic_density_lu

    def convert_pressure_to_pu(self, p):
        return p / self.characteristic_pressure_lu * self.characteristic_pressure_pu

    def convert_pressure_to_lu(self, p):
        return p / self.characteristic_pressure_pu * self.characteristic_pressure_lu

    # length / energy ------------------------------------------------------
    def convert_length_to_pu(self, x):
        return x * self.characteristic_length_pu / self.characteristic_length_lu

    def convert_length_to_lu(self, x):
        return x * self.characteristic_length_lu / self.characteristic_length_pu

    def convert_energy_to_pu(self, e):
        return e * self.characteristic_pressure_pu / self.characteristic_pressure_lu

    def convert_energy_to_lu(self, e):
        return e * self.characteristic_pressure_lu / self.characteristic_pressure_pu

    def convert_incompressible_energy_to_pu(self, e):
        return (e * self.characteristic_velocity_pu ** 2
                / self.characteristic_velocity_lu ** 2)

    def convert_incompressible_energy_to_lu(self, e):
        return (e * self.characteristic_velocity_lu ** 2
                / self.characteristic_velocity_pu ** 2)
