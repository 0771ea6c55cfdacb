"""Moment transforms of the MRT collision (lettuce/util/moments.py:60-545).

Each basis is a list of polynomials in the lattice velocity e; its matrix is
M[i, q] = P_i(e_q) and the inverse is computed from it. The bases, in
lettuce's moment order:

* D1Q3Transform: 1, e_x, e_x^2 (rho, j, e);
* D2Q9Dellar: 1, e_x, e_y, 9/2 e_x^2 - 3/2, 9 e_x e_y, 9/2 e_y^2 - 3/2,
  (1 - 3 e_x^2)(1 - 3 e_y^2), 2 e_x (3 e_y^2 - 1), 2 e_y (3 e_x^2 - 1);
* D2Q9Lallemand (Lallemand & Luo 2000): 1, e_x, e_y, e_x^2 - e_y^2, e_x e_y,
  3|e|^2 - 4, (3|e|^2 - 5) e_x, (3|e|^2 - 5) e_y, 9/2|e|^4 - 21/2|e|^2 + 4;
* D3Q27Hermite: the tensor-product Hermite polynomials 1, e_a,
  H_a = e_a^2 - 1/3, e_a e_b, ... up to H_x H_y H_z, in lettuce's order.

The equilibrium moments are evaluated inside the step kernel
(``LGB_MRT_EQ_*``); ``transform``, ``inverse_transform`` and ``equilibrium``
restate them on torch tensors for callers outside the step (lettuce's
Transform interface).
"""
from __future__ import annotations

from typing import List

import numpy as np
import torch

from . import _lib

__all__ = ["Transform", "D1Q3Transform", "D2Q9Dellar", "D2Q9Lallemand", "D3Q27Hermite"]

_T = 1.0 / 3.0


def _e(stencil) -> np.ndarray:
    return np.asarray(stencil.e, dtype=np.float64)


class Transform:
    """base transform: identity moments, equilibrium M feq(rho, u)"""
    names: List[str] = []
    equilibrium_kind = _lib.MRT_EQ_GENERIC
    stencil_name = None

    def __init__(self, stencil, context, names=None):
        self.context = context
        self.stencil = stencil() if callable(stencil) else stencil
        if self.stencil_name is not None and type(self.stencil).__name__ != self.stencil_name:
            raise ValueError(f"{type(self).__name__} is a {self.stencil_name} basis")
        self.names = list(names) if names is not None else (
            list(self.names) if self.names else [f"m{i}" for i in range(self.stencil.q)])
        rows = self.rows(_e(self.stencil))
        self.matrix_np = np.asarray(rows, dtype=np.float64)
        self.inverse_np = np.linalg.inv(self.matrix_np)
        self.matrix = context.convert_to_tensor(self.matrix_np)
        self.inverse = context.convert_to_tensor(self.inverse_np)

    def rows(self, e: np.ndarray):
        return np.eye(len(e))

    def __getitem__(self, moment_names):
        if not isinstance(moment_names, tuple):
            moment_names = [moment_names]
        return [self.names.index(name) for name in moment_names]

    def _mv(self, m, v):
        return torch.einsum("ij,j...->i...", m.to(v.dtype), v)

    def transform(self, f):
        return self._mv(self.matrix, f)

    def inverse_transform(self, m):
        return self._mv(self.inverse, m)

    def equilibrium(self, m, flow):
        f = self.inverse_transform(m)
        rho = torch.sum(f, dim=0)[None]
        e = flow.torch_stencil.e.to(f.dtype)
        u = torch.einsum("qd,q...->d...", e, f) / rho
        return self.transform(flow.equilibrium(flow, rho, u))


class D1Q3Transform(Transform):
    names = ["rho", "j", "e"]
    stencil_name = "D1Q3"

    def __init__(self, stencil, context):
        super().__init__(stencil, context)

    def rows(self, e):
        x = e[:, 0]
        return [np.ones_like(x), x, x * x]


class D2Q9Dellar(Transform):
    names = ['rho', 'jx', 'jy', 'Pi_xx', 'Pi_xy', 'PI_yy', 'N', 'Jx', 'Jy']
    equilibrium_kind = _lib.MRT_EQ_DELLAR
    stencil_name = "D2Q9"

    def __init__(self, stencil, context):
        super().__init__(stencil, context)

    def rows(self, e):
        x, y = e[:, 0], e[:, 1]
        return [np.ones_like(x), x, y, 4.5 * x * x - 1.5, 9 * x * y, 4.5 * y * y - 1.5,
                (1 - 3 * x * x) * (1 - 3 * y * y), 2 * x * (3 * y * y - 1),
                2 * y * (3 * x * x - 1)]

    def equilibrium(self, m, flow=None):
        meq = torch.zeros_like(m)
        rho, jx, jy = m[0], m[1], m[2]
        meq[0], meq[1], meq[2] = rho, jx, jy
        meq[3] = jx * jx / rho * 9 / 2
        meq[4] = jx * jy / rho * 9
        meq[5] = jy * jy / rho * 9 / 2
        return meq


class D2Q9Lallemand(Transform):
    names = ['rho', 'jx', 'jy', 'pxx', 'pxy', 'e', 'qx', 'qy', 'eps']
    equilibrium_kind = _lib.MRT_EQ_LALLEMAND
    stencil_name = "D2Q9"

    def __init__(self, stencil, context):
        super().__init__(stencil, context)

    def rows(self, e):
        x, y = e[:, 0], e[:, 1]
        r2 = x * x + y * y
        return [np.ones_like(x), x, y, x * x - y * y, x * y, 3 * r2 - 4, (3 * r2 - 5) * x,
                (3 * r2 - 5) * y, 4.5 * r2 * r2 - 10.5 * r2 + 4]

    def equilibrium(self, m, flow=None):
        meq = torch.zeros_like(m)
        rho, jx, jy = m[0], m[1], m[2]
        jj = jx ** 2 + jy ** 2
        meq[0], meq[1], meq[2] = rho, jx, jy
        meq[3] = 1 / 2 * (2 / 3) * (jx ** 2 - jy ** 2)
        meq[4] = 1 / 2 * (2 / 3) * (jx * jy)
        meq[5] = 1 / 4 * -8 * rho + 1 / 6 * 18 * jj
        meq[6] = 1 / 2 * -2 * jx
        meq[7] = 1 / 2 * -2 * jy
        meq[8] = 1 / 4 * 4 * rho + 1 / 6 * -18 * jj
        return meq


class D3Q27Hermite(Transform):
    names = ['rho', 'jx', 'jy', 'jz',
             'Pi_xx', 'Pi_xy', 'PI_xz', 'PI_yy', 'PI_yz', 'PI_zz',
             'J_xxy', 'J_xxz', 'J_xyy', 'J_xyz', 'J_xzz', 'J_yyz', 'J_yzz',
             'J_xxyy', 'J_xxyz', 'J_xxzz', 'J_xyyz', 'J_xyzz', 'J_yyzz',
             'J_xxyyz', 'J_xxyzz', 'J_xyyzz', 'J_xyxzyz']
    equilibrium_kind = _lib.MRT_EQ_HERMITE
    stencil_name = "D3Q27"

    def __init__(self, stencil, context):
        super().__init__(stencil, context)

    def rows(self, e):
        x, y, z = e[:, 0], e[:, 1], e[:, 2]
        X, Y, Z = x * x - _T, y * y - _T, z * z - _T
        return [np.ones_like(x), x, y, z, X, x * y, x * z, Y, y * z, Z,
                X * y, X * z, x * Y, x * y * z, x * Z, Y * z, y * Z,
                X * Y, X * y * z, X * Z, x * Y * z, x * y * Z, Y * Z,
                X * Y * z, X * y * Z, x * Y * Z, X * Y * Z]

    def equilibrium(self, m, flow=None):
        meq = torch.zeros_like(m)
        rho, jx, jy, jz = m[0], m[1], m[2], m[3]
        meq[0], meq[1], meq[2], meq[3] = rho, jx, jy, jz
        meq[4] = jx * jx / rho
        meq[5] = jx * jy / rho
        meq[6] = jx * jz / rho
        meq[7] = jy * jy / rho
        meq[8] = jy * jz / rho
        meq[9] = jz * jz / rho
        meq[10] = jx * jx * jy / rho ** 2
        meq[11] = jx * jx * jz / rho ** 2
        meq[12] = jx * jy * jy / rho ** 2
        meq[13] = jx * jy * jz / rho ** 2
        meq[14] = jx * jz * jz / rho ** 2
        meq[15] = jy * jy * jz / rho ** 2
        meq[16] = jy * jz * jz / rho ** 2
        meq[17] = jx * jx * jy * jy / rho ** 3
        meq[18] = jx * jx * jy * jz / rho ** 3
        meq[19] = jx * jx * jz * jz / rho ** 3
        meq[20] = jx * jy * jy * jz / rho ** 3
        meq[21] = jx * jy * jz * jz / rho ** 3
        meq[22] = jy * jy * jz * jz / rho ** 3
        meq[23] = jx * jx * jy * jy * jz / rho ** 4
        meq[24] = jx * jx * jy * jz * jz / rho ** 4
        meq[25] = jx * jy * jy * jz * jz / rho ** 4
        meq[26] = jx * jy * jx * jz * jy * jz / rho ** 5
        return meq
