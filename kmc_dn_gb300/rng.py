"""Replay streams: a pre-generated uniform stream shared by every hop loop.

Replay mode feeds one fixed sequence of uniforms u in (0, 1) to a hop loop,
two per hop in the reference's order: the first for the exponential clock,
the second for event selection (kmc_dopant_networks.py:100, :106).  The
stream is SplitMix64 (Steele, Lea and Flood, 2014) over a 64-bit seed, mapped
to ``((z >> 11) + 0.5) * 2**-53`` so that u is never 0 (the reference picks
the impossible transition (0, 0) when u == 0) and never 1.  It is
reproducible bit-for-bit from the seed on any machine with numpy.
"""
from __future__ import annotations

import numpy as np

__all__ = ["replay_uniforms"]

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def replay_uniforms(seed: int, n: int) -> np.ndarray:
    """n uniforms in (0, 1) (float64) from SplitMix64 seeded with ``seed``."""
    with np.errstate(over="ignore"):
        k = np.arange(1, n + 1, dtype=np.uint64)
        x = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) + k * _GOLDEN
        z = (x ^ (x >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return ((z >> np.uint64(11)).astype(np.float64) + 0.5) * (2.0 ** -53)
