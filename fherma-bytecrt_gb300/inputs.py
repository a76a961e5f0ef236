"""Seeded synthetic operands and moduli in the wire format of the plugin ABI.

Every value is a coefficient of L little-endian uint32 limbs (``[N][L]`` row
major), matching ``fherma::Inputs`` (native-smoke/fherma.h:34-37).  The
stream is splitmix64 evaluated with numpy uint64 arithmetic, so the same seed
gives the same words on every machine and numpy version.

Workloads stand in for the FHERMA negacyclic challenge cases (not available
offline): moduli are seeded odd W-bit integers with the top bit set, operands
are uniform in [0, q), and the edge fixtures are all-zero, +-1, all q-1 and
the centre-lift bounds (q-1)/2 and (q+1)/2.
"""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, offset: int = 0) -> np.ndarray:
    """``count`` outputs of splitmix64 started at state ``seed`` (skipping ``offset``)."""
    with np.errstate(over="ignore"):
        idx = np.arange(offset + 1, offset + count + 1, dtype=np.uint64)
        z = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def random_words(seed: int, count: int, offset: int = 0) -> np.ndarray:
    return (splitmix64(seed, count, offset) >> np.uint64(16)).astype(np.uint32)


def limbs_for(W: int) -> int:
    return (W + 31) // 32


def modulus(W: int, seed: int) -> np.ndarray:
    """Odd W-bit modulus with the top bit set, as L words."""
    L = limbs_for(W)
    q = random_words(seed ^ 0x51A5E, L).astype(np.uint64)
    top = W - 32 * (L - 1)
    mask = (1 << top) - 1
    q[L - 1] &= np.uint64(mask)
    q[L - 1] |= np.uint64(1 << (top - 1))
    q[0] |= np.uint64(1)
    return q.astype(np.uint32)


def gap_modulus(W: int, gap: int) -> np.ndarray:
    """q = 2^W - gap (the FHERMA challenge form, native-smoke/rns-plan.hpp:186-197)."""
    L = limbs_for(W)
    v = (1 << W) - gap
    return np.array([(v >> (32 * i)) & 0xFFFFFFFF for i in range(L)], dtype=np.uint32)


def _less_than(x: np.ndarray, q: np.ndarray) -> np.ndarray:
    """Row-wise big-integer x < q for x of shape [n][L] (little-endian words)."""
    n, L = x.shape
    lt = np.zeros(n, dtype=bool)
    decided = np.zeros(n, dtype=bool)
    for limb in range(L - 1, -1, -1):
        xl = x[:, limb]
        ql = q[limb]
        newly_lt = (~decided) & (xl < ql)
        newly_gt = (~decided) & (xl > ql)
        lt |= newly_lt
        decided |= newly_lt | newly_gt
    return lt


def uniform(q: np.ndarray, N: int, seed: int) -> np.ndarray:
    """N coefficients uniform in [0, q) by rejection sampling."""
    q = np.asarray(q, dtype=np.uint32)
    L = q.shape[0]
    W = 32 * (L - 1) + int(q[L - 1]).bit_length()
    top_mask = np.uint32((1 << (W - 32 * (L - 1))) - 1) if W % 32 else np.uint32(0xFFFFFFFF)
    out = np.zeros((N, L), dtype=np.uint32)
    todo = np.arange(N)
    offset = 0
    while todo.size:
        cand = random_words(seed, todo.size * L, offset).reshape(todo.size, L)
        offset += todo.size * L
        cand[:, L - 1] &= top_mask
        ok = _less_than(cand, q)
        out[todo[ok]] = cand[ok]
        todo = todo[~ok]
    return out


def _int_words(v: int, L: int) -> np.ndarray:
    return np.array([(v >> (32 * i)) & 0xFFFFFFFF for i in range(L)], dtype=np.uint32)


def q_int(q: np.ndarray) -> int:
    v = 0
    for w in reversed([int(x) for x in q]):
        v = (v << 32) | w
    return v


def fixture(q: np.ndarray, N: int, kind: str) -> np.ndarray:
    """Edge operands: zero, one, minus_one (q-1), half_low ((q-1)/2), half_high ((q+1)/2)."""
    L = q.shape[0]
    qi = q_int(q)
    value = {"zero": 0, "one": 1, "minus_one": qi - 1,
             "half_low": (qi - 1) // 2, "half_high": (qi + 1) // 2}[kind]
    return np.tile(_int_words(value, L), (N, 1))
