"""Seeded input helpers shared by the CPU and GPU tests."""
import numpy as np


def split3(a):
    x = a.astype(np.uint64) & np.uint64(0x1FFFFF)
    x = (x | x << np.uint64(32)) & np.uint64(0x1F00000000FFFF)
    x = (x | x << np.uint64(16)) & np.uint64(0x1F0000FF0000FF)
    x = (x | x << np.uint64(8)) & np.uint64(0x100F00F00F00F00F)
    x = (x | x << np.uint64(4)) & np.uint64(0x10C30C30C30C30C3)
    x = (x | x << np.uint64(2)) & np.uint64(0x1249249249249249)
    return x


def morton(x, y, z):
    return (split3(x) << np.uint64(2)) | (split3(y) << np.uint64(1)) | split3(z)


def random_codes(depth, n, seed, cluster=False):
    """Uniform codes, or (cluster=True) points around 8 seeded centres, which
    share structure and give long runs of equal bricks."""
    rng = np.random.default_rng(seed)
    if cluster:
        g = 1 << depth
        c = rng.integers(0, g, (8, 3))
        p = c[rng.integers(0, 8, n)] + rng.integers(-6, 7, (n, 3))
        p = np.clip(p, 0, g - 1).astype(np.uint64)
        return morton(p[:, 0], p[:, 1], p[:, 2])
    return rng.integers(0, 1 << (3 * depth), n, dtype=np.uint64)


def chunks_of(codes, depth, levels_up):
    """Split into 8^levels_up Morton-ordered subvolumes with local codes."""
    sub = depth - levels_up
    chunk = (codes >> np.uint64(3 * sub)).astype(np.int64)
    local = codes & np.uint64((1 << (3 * sub)) - 1)
    return [local[chunk == i] for i in range(8 ** levels_up)], sub
