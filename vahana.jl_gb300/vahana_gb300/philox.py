"""Philox4x32-10 (Salmon et al., SC'11) vectorised over numpy arrays.

Same stream as the kernels (csrc/vg_philox.cuh): key = (seed lo, seed hi),
counter = (nr lo, nr hi, step, tag).  Used by the model builders to draw
initial states on the host.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK32 = np.uint64(0xFFFFFFFF)

TAG_INIT, TAG_EDGE, TAG_INFECT, TAG_MOVE, TAG_SRC, TAG_DST, TAG_WEIGHT, TAG_PARAM = range(1, 9)


def philox4x32_10(c0, c1, c2, c3, seed):
    """Return the four u32 output words (uint64 arrays holding u32 values)."""
    c0, c1, c2, c3 = (np.asarray(c, dtype=np.uint64) & MASK32 for c in (c0, c1, c2, c3))
    shape = np.broadcast_shapes(c0.shape, c1.shape, c2.shape, c3.shape)
    c0, c1, c2, c3 = (np.broadcast_to(c, shape).copy() for c in (c0, c1, c2, c3))
    k0, k1 = int(seed) & 0xFFFFFFFF, (int(seed) >> 32) & 0xFFFFFFFF
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK32
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK32
        n0 = hi1 ^ c1 ^ np.uint64(k0)
        n2 = hi0 ^ c3 ^ np.uint64(k1)
        c0, c1, c2, c3 = n0, lo1, n2, lo0
        k0 = (k0 + W0) & 0xFFFFFFFF
        k1 = (k1 + W1) & 0xFFFFFFFF
    return c0, c1, c2, c3


def draw(seed, nr, step, tag):
    nr = np.asarray(nr, dtype=np.uint64)
    return philox4x32_10(nr & MASK32, nr >> np.uint64(32), np.uint64(step), np.uint64(tag), seed)


def to_u64(words):
    return (words[1] << np.uint64(32)) | words[0]


def unit(u64):
    """top 53 bits * 2^-53 in [0, 1)"""
    return (np.asarray(u64, dtype=np.uint64) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


def unit_open0(u64):
    return ((np.asarray(u64, dtype=np.uint64) >> np.uint64(11)) + np.uint64(1)).astype(np.float64) * (2.0 ** -53)


def bounded32(x, rng):
    return ((np.asarray(x, dtype=np.uint64) & MASK32) * np.uint64(rng)) >> np.uint64(32)
