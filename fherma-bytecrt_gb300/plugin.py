"""Python mirror of the reference's plugin interface for this path.

Same names, argument meaning and error behaviour as the generated C++ ABI
(native-smoke/fherma.h:13-48 and the batched form native-batched/fherma.h:27-49):
``fherma_init(Point) -> state``, ``fherma_run(state, Inputs) -> Outputs``,
``fherma_free(state)``.  Tensors are numpy arrays shaped [N][L] (or [B][N][L]
when the point carries B) of uint32 little-endian limbs.  Errors raise
exceptions, as the reference's std::runtime_error does.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .native import Multiplier


@dataclass
class Point:
    N: int
    W: int
    L: int
    q: np.ndarray
    B: int = 0          # 0: the single-product ABI; >= 1: the batched ABI


@dataclass
class Inputs:
    a: np.ndarray
    b: np.ndarray


@dataclass
class Outputs:
    c: np.ndarray = field(default_factory=lambda: np.zeros(0, np.uint32))


class _State:
    def __init__(self, p: Point):
        if p.L != (p.W + 31) // 32:
            raise RuntimeError("point L mismatch")
        q = np.ascontiguousarray(p.q, dtype=np.uint32).reshape(-1)
        if q.shape[0] != p.L:
            raise RuntimeError("modulus limb count")
        if p.B > 128:
            raise RuntimeError("batch coverage B=1..128")
        self.point = p
        self.mult = Multiplier(p.N, p.W, q)
        self.batch = max(1, p.B)

    def shape(self):
        p = self.point
        return (p.B, p.N, p.L) if p.B else (p.N, p.L)


def fherma_init(p: Point) -> _State:
    return _State(p)


def fherma_run(state: _State, inp: Inputs) -> Outputs:
    shape = state.shape()
    total = int(np.prod(shape))
    a = np.ascontiguousarray(inp.a, dtype=np.uint32)
    b = np.ascontiguousarray(inp.b, dtype=np.uint32)
    if a.size != total or b.size != total:
        raise RuntimeError("input coefficient count")
    c = state.mult.multiply(a.reshape(shape), b.reshape(shape))
    return Outputs(c=c.reshape(shape))


def fherma_free(state: _State) -> None:
    state.mult.close()
