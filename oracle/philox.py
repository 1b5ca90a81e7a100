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
    """U[0,1) per interior cell for time step `step`: first output word of
    Philox4x32-10 with counter (cell_lo, cell_hi, step_lo, step_hi) and key
    (seed_lo, seed_hi), top 24 bits times 2^-24 (cell = C-order linear index
    of the interior cell). Matches ppf::noise_bits in the CUDA library."""
    n = int(np.prod(shape))
    cell = np.arange(n, dtype=np.uint64)
    step = int(step)
    seed = int(seed)
    x, _, _, _ = philox4x32_10(
        (cell & _MASK, cell >> _S32, step & 0xFFFFFFFF, step >> 32),
        (seed & 0xFFFFFFFF, seed >> 32))
    return ((x >> np.uint64(8)).astype(np.float64) * 2.0 ** -24).reshape(shape)
