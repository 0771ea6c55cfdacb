"""Velocity sets with lettuce's q ordering (lettuce/_stencil.py:14-50,
lettuce/ext/_stencil/*.py). The ordering defines the population index of the
[Q, *resolution] field, so it is the same as lettuce's."""
from __future__ import annotations

from functools import cached_property
from typing import List

import numpy as np
import torch

from . import _lib

__all__ = ["Stencil", "TorchStencil", "D1Q3", "D2Q9", "D3Q15", "D3Q19", "D3Q27"]


class Stencil:
    e: List[List[int]]
    w: List[float]
    opposite: List[int]
    lgb_id: int
    cs: float = 1 / np.sqrt(3.0)

    @cached_property
    def d(self) -> int:
        assert len(self.e[0]) in [1, 2, 3]
        return len(self.e[0])

    @cached_property
    def q(self) -> int:
        return len(self.e)

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))


class TorchStencil:
    cs: float = 1 / np.sqrt(3.0)

    def __init__(self, stencil: Stencil, context):
        self.e = context.convert_to_tensor(stencil.e)
        self.w = context.convert_to_tensor(stencil.w)
        self.opposite = context.convert_to_tensor(stencil.opposite, dtype=torch.int64)

    @cached_property
    def d(self) -> int:
        return self.e.shape[1]

    @cached_property
    def q(self) -> int:
        return self.e.shape[0]


def _opposites(e):
    arr = np.array(e)
    return [int(np.where((arr == -arr[i]).all(axis=1))[0][0]) for i in range(len(e))]


class D1Q3(Stencil):
    lgb_id = _lib.D1Q3

    def __init__(self):
        self.e = [[0], [1], [-1]]
        self.w = [2.0 / 3.0, 1.0 / 6.0, 1.0 / 6.0]
        self.opposite = _opposites(self.e)


class D2Q9(Stencil):
    lgb_id = _lib.D2Q9

    def __init__(self):
        self.e = [[0, 0], [1, 0], [0, 1], [-1, 0], [0, -1],
                  [1, 1], [-1, 1], [-1, -1], [1, -1]]
        self.w = [4.0 / 9.0] + [1.0 / 9.0] * 4 + [1.0 / 36.0] * 4
        self.opposite = _opposites(self.e)


class D3Q15(Stencil):
    lgb_id = _lib.D3Q15

    def __init__(self):
        self.e = [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
                  [0, 0, 1], [0, 0, -1], [1, 1, 1], [-1, -1, -1], [1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [-1, 1, -1], [1, -1, -1], [-1, 1, 1]]
        self.w = [2.0 / 9.0] + [1.0 / 9.0] * 6 + [1.0 / 72.0] * 8
        self.opposite = _opposites(self.e)


_D3Q19_E = [[0, 0, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0],
            [0, 0, 1], [0, 0, -1], [0, 1, 1], [0, -1, -1], [0, 1, -1],
            [0, -1, 1], [1, 0, 1], [-1, 0, -1], [1, 0, -1], [-1, 0, 1],
            [1, 1, 0], [-1, -1, 0], [1, -1, 0], [-1, 1, 0]]


class D3Q19(Stencil):
    lgb_id = _lib.D3Q19

    def __init__(self):
        self.e = [list(v) for v in _D3Q19_E]
        self.w = [1.0 / 3.0] + [1.0 / 18.0] * 6 + [1.0 / 36.0] * 12
        self.opposite = _opposites(self.e)


class D3Q27(Stencil):
    lgb_id = _lib.D3Q27

    def __init__(self):
        self.e = [list(v) for v in _D3Q19_E] + [
            [1, 1, 1], [-1, -1, -1], [1, 1, -1], [-1, -1, 1],
            [1, -1, 1], [-1, 1, -1], [1, -1, -1], [-1, 1, 1]]
        self.w = ([8.0 / 27.0] + [2.0 / 27.0] * 6 + [1.0 / 54.0] * 12
                  + [1.0 / 216.0] * 8)
        self.opposite = _opposites(self.e)
