"""Host-side PRNG keys in jax.random's layout (uint32[2]); PRNGKey(seed) and split under
jax_threefry_partitionable=True.  Device code draws the actual variates."""
from __future__ import annotations

import numpy as np

_ROT = ((13, 15, 26, 6), (17, 29, 16, 24))


def _rotl(v, r):
    return ((v << np.uint32(r)) | (v >> np.uint32(32 - r))).astype(np.uint32)


def threefry2x32(key, c0, c1):
    """Threefry-2x32-20 (Salmon et al. 2011) over uint32 arrays c0, c1 under a key."""
    with np.errstate(over="ignore"):
        k0 = np.uint32(key[0])
        k1 = np.uint32(key[1])
        ks = (k0, k1, np.uint32(k0 ^ k1 ^ np.uint32(0x1BD11BDA)))
        x0 = (np.asarray(c0, np.uint32) + ks[0]).astype(np.uint32)
        x1 = (np.asarray(c1, np.uint32) + ks[1]).astype(np.uint32)
        for blk in range(5):
            for r in _ROT[blk & 1]:
                x0 = (x0 + x1).astype(np.uint32)
                x1 = _rotl(x1, r)
                x1 = (x1 ^ x0).astype(np.uint32)
            x0 = (x0 + ks[(blk + 1) % 3]).astype(np.uint32)
            x1 = (x1 + ks[(blk + 2) % 3] + np.uint32(blk + 1)).astype(np.uint32)
    return x0, x1


def PRNGKey(seed: int) -> np.ndarray:
    """jax.random.PRNGKey with x64 enabled: [seed >> 32, seed & 0xFFFFFFFF]."""
    seed = int(seed)
    return np.array([(seed >> 32) & 0xFFFFFFFF, seed & 0xFFFFFFFF], np.uint32)


def split(key, num: int = 2) -> np.ndarray:
    i = np.arange(num, dtype=np.uint64)
    a, b = threefry2x32(key, (i >> np.uint64(32)).astype(np.uint32), (i & np.uint64(0xFFFFFFFF)).astype(np.uint32))
    return np.stack([a, b], axis=-1)
