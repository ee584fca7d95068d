"""Counter-based uniform random numbers shared bit-for-bit with the CUDA library.

The reference draws its rank-check vectors from MATLAB's unseeded global
``rand`` (Common/ID.m:68-86), which cannot be reproduced outside MATLAB.  Both
the oracle and the GPU library instead draw ``u(seed, stream, i)`` in [0, 1)
from a SplitMix64 finaliser over a 64-bit counter (Steele, Lea & Flood,
"Fast splittable pseudorandom number generators", OOPSLA 2014):

    z  = seed ^ (stream * 0xD1B54A32D192ED03)      (key)
    z += (i + 1) * 0x9E3779B97F4A7C15
    z  = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9
    z  = (z ^ (z >> 27)) * 0x94D049BB133111EB
    z ^= z >> 31
    u  = (z >> 11) * 2^-53

All arithmetic is modulo 2^64, so the stream is identical on every platform.
"""
from __future__ import annotations

import numpy as np

_M_KEY = np.uint64(0xD1B54A32D192ED03)
_M_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M_1 = np.uint64(0xBF58476D1CE4E5B9)
_M_2 = np.uint64(0x94D049BB133111EB)


def uniform(seed: int, stream: int, n: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        key = np.uint64(seed & 0xFFFFFFFFFFFFFFFF) ^ (np.uint64(stream & 0xFFFFFFFFFFFFFFFF) * _M_KEY)
        i = np.arange(1, n + 1, dtype=np.uint64)
        z = key + i * _M_GOLD
        z = (z ^ (z >> np.uint64(30))) * _M_1
        z = (z ^ (z >> np.uint64(27))) * _M_2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def id_stream(problem: int, draw: int) -> int:
    """Stream id of draw ``draw`` of the rank check of ID problem ``problem``."""
    return (problem << 8) | (draw & 0xFF)
