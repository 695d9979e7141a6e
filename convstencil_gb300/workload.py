"""Seeded synthetic workloads for the benchmarks: grids of doubles uniform in
[0, 1) from SplitMix64 (the top 53 bits of each output), and weights drawn
the same way and normalised to sum 1. The reference ships no datasets; its
benchmarks run on generated grids of the same shapes and sizes."""
from __future__ import annotations

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix_uniform(count: int, seed: int) -> np.ndarray:
    """`count` doubles in [0, 1): SplitMix64 outputs 1..count after `seed`,
    top 53 bits scaled by 2^-53."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + idx * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def seeded_weights(count: int, seed: int) -> np.ndarray:
    """`count` weights from splitmix_uniform, normalised to sum 1."""
    w = splitmix_uniform(count, seed)
    return w / w.sum()
