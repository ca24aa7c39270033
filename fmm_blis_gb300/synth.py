"""Seeded synthetic operands, reproducible on any machine.

uniform(m, n, seed): column-major float64 in [-1, 1) from a splitmix64 stream
(element i of the column-major order uses the 64-bit state seed*2^32 + i).
hard(m, n, seed, phi): (u - 0.5) * exp(phi * g), u ~ U[0,1), g ~ N(0,1) by
Box-Muller, for the wide-exponent-range cases.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)


def _splitmix(state: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = state * _G + _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _unit(count: int, seed: int, stream: int = 0) -> np.ndarray:
    base = np.uint64((seed & 0xFFFFFFFF) << 32) + np.uint64(stream) * np.uint64(1 << 62)
    idx = np.arange(count, dtype=np.uint64) + base
    return (_splitmix(idx) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform(m: int, n: int, seed: int) -> np.ndarray:
    u = _unit(m * n, seed)
    return np.asfortranarray((2.0 * u - 1.0).reshape(n, m).T)


def hard(m: int, n: int, seed: int, phi: float) -> np.ndarray:
    u = _unit(m * n, seed, 1)
    a = np.maximum(_unit(m * n, seed, 2), 1e-300)
    b = _unit(m * n, seed, 3)
    g = np.sqrt(-2.0 * np.log(a)) * np.cos(2.0 * np.pi * b)
    return np.asfortranarray(((u - 0.5) * np.exp(phi * g)).reshape(n, m).T)
