"""Counter-based random stream shared by the oracle and the CUDA engine.

TEST INFRASTRUCTURE: this package is the CPU oracle.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may use it.
The CUDA engine never imports it.

The reference (PETITE) draws every random number from two process-global
generators (numpy's ``RandomState`` and Python's ``random``), in the order the
Python loop happens to visit particles (``shower.py:30,540,561-562,583,671``,
``kinematics.py:33,93,128,233,261,325``, ``moliere.py:284,382``).  A parallel
engine cannot reproduce a global order, so both the engine and the oracle key
their uniforms by particle identity instead:

* generator: Philox4x32-10 (Salmon et al., "Parallel random numbers: as easy
  as 1, 2, 3", SC'11), key = 64-bit seed;
* counter  : (draw_block lo, draw_block hi, particle key lo, particle key hi);
* draw ``n`` of a particle uses block ``n >> 1`` and the 64-bit half ``n & 1``
  of the 128-bit output; the double is ``(u64 >> 11) * 2**-53`` in [0, 1).

Particle keys: primary ``i`` gets ``mix64(i + 1)``; the two daughters of a
hard interaction get ``mix64(parent + GOLDEN * (1 + bit))`` where ``bit`` is 0
for the first and 1 for the second returned four-vector (the same order the
reference uses for ``ID = 2*ID + bit`` at ``shower.py:486,494``).
"""
from __future__ import annotations

import numpy as np

M0 = np.uint64(0xD2511F53)
M1 = np.uint64(0xCD9E8D57)
W0 = 0x9E3779B9
W1 = 0xBB67AE85
MASK32 = np.uint64(0xFFFFFFFF)
GOLDEN = 0x9E3779B97F4A7C15
U64 = (1 << 64) - 1


def philox4x32_10(ctr, key):
    """Vectorised Philox4x32-10.

    ``ctr``: uint32 array of shape (..., 4); ``key``: uint32 array (..., 2).
    Returns uint32 array (..., 4).
    """
    c = np.asarray(ctr, dtype=np.uint64) & MASK32
    k = np.asarray(key, dtype=np.uint64) & MASK32
    c0, c1, c2, c3 = (c[..., i].copy() for i in range(4))
    k0 = np.broadcast_to(k[..., 0], c0.shape).copy()
    k1 = np.broadcast_to(k[..., 1], c0.shape).copy()
    for r in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        c0, c1, c2, c3 = hi1 ^ c1 ^ k0, lo1, hi0 ^ c3 ^ k1, lo0
        if r != 9:
            k0 = (k0 + np.uint64(W0)) & MASK32
            k1 = (k1 + np.uint64(W1)) & MASK32
    return np.stack([c0, c1, c2, c3], axis=-1).astype(np.uint32)


def mix64(z: int) -> int:
    """SplitMix64 finaliser (a bijection on 64-bit integers)."""
    z &= U64
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & U64
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & U64
    return z ^ (z >> 31)


def primary_key(index: int) -> int:
    return mix64(index + 1)


def daughter_key(parent_key: int, bit: int) -> int:
    return mix64(parent_key + GOLDEN * (1 + bit))


def uniforms(seed: int, pkey: int, start: int, count: int) -> np.ndarray:
    """Draws ``start .. start+count-1`` of particle ``pkey`` as float64 in [0, 1)."""
    if count <= 0:
        return np.zeros(0)
    n = np.arange(start, start + count, dtype=np.uint64)
    blk = n >> np.uint64(1)
    ctr = np.stack([blk & MASK32, blk >> np.uint64(32),
                    np.full_like(blk, pkey & 0xFFFFFFFF),
                    np.full_like(blk, (pkey >> 32) & 0xFFFFFFFF)], axis=-1)
    key = np.array([seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF], dtype=np.uint64)
    out = philox4x32_10(ctr, key).astype(np.uint64)
    half = (n & np.uint64(1)).astype(bool)
    lo = np.where(half, out[:, 2], out[:, 0])
    hi = np.where(half, out[:, 3], out[:, 1])
    u64 = lo | (hi << np.uint64(32))
    return (u64 >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


class Stream:
    """Sequential view of one particle's uniforms (buffered)."""

    __slots__ = ("seed", "key", "n", "_buf", "_pos")

    def __init__(self, seed: int, pkey: int):
        self.seed = seed
        self.key = pkey
        self.n = 0
        self._buf = np.zeros(0)
        self._pos = 0

    def next(self) -> float:
        if self._pos >= len(self._buf):
            self._buf = uniforms(self.seed, self.key, self.n, 64)
            self._pos = 0
        u = float(self._buf[self._pos])
        self._pos += 1
        self.n += 1
        return u

    def take(self, count: int) -> np.ndarray:
        return np.array([self.next() for _ in range(count)])
