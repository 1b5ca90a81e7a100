"""Philox4x32-10 in numpy (TEST INFRASTRUCTURE ONLY: the oracle's copy of the
counter-based generator the CUDA library uses for Warren1995 noise).

Algorithm: Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as
1, 2, 3" (SC'11): ten rounds, each two 32x32->64-bit multiplies by
0xD2511F53 and 0xCD9E8D57, with the key bumped by 0x9E3779B9 / 0xBB67AE85.
Known-answer vectors of the published generator are checked in
tests/test_oracle.py.
"""
from __future__ import annotations

import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint64(0x9E3779B9)
_W1 = np.uint64(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)
_S32 = np.uint64(32)


def philox4x32_10(ctr, key):
    """ctr: 4 arrays (or ints) of 32-bit words; key: 2 words. Returns 4 uint64
    arrays holding the 32-bit output words."""
    c0, c1, c2, c3 = (np.asarray(x, dtype=np.uint64) & _MASK for x in ctr)
    k0, k1 = (np.asarray(x, dtype=np.uint64) & _MASK for x in key)
    for _ in range(10):
        p0 = _M0 * c0
        p1 = _M1 * c2
        hi0, lo0 = p0 >> _S32, p0 & _MASK
        hi1, lo1 = p1 >> _S32, p1 & _MASK
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        k0 = (k0 + _W0) & _MASK
        k1 = (k1 + _W1) & _MASK
    return c0, c1, c2, c3


def noise_uniform(seed: int, step: int, shape) -> np.ndarray:
    """U[0,1) per interior cell for time step `step`. Cells are grouped by
    four along the last axis: cell (row, col) of a 2-D grid (a 1-D grid is
    one row) takes output word col % 4 of Philox4x32-10 with counter
    (col // 4, row, step_lo, step_hi) and key (seed_lo, seed_hi); the word's
    top 24 bits times 2^-24 are the uniform number. Matches ppf::noise_group
    in the CUDA library."""
    shape = tuple(shape)
    rows, cols = (1, shape[0]) if len(shape) == 1 else (int(np.prod(shape[:-1])), shape[-1])
    nq = (cols + 3) // 4
    q = np.tile(np.arange(nq, dtype=np.uint64), rows)
    r = np.repeat(np.arange(rows, dtype=np.uint64), nq)
    step = int(step)
    seed = int(seed)
    words = philox4x32_10((q, r, step & 0xFFFFFFFF, step >> 32),
                          (seed & 0xFFFFFFFF, seed >> 32))
    w = np.stack(words, axis=-1).reshape(rows, nq * 4)[:, :cols]
    return ((w >> np.uint64(8)).astype(np.float64) * 2.0 ** -24).reshape(shape)
