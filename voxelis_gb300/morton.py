"""Morton paths of voxel positions (utils/common.rs:6-111), vectorised with numpy.

encode_child_index_path puts x at bits 3n, y at 3n+1 and z at 3n+2 (10 bits per axis). The
bottom group of a voxel is path >> 3 and its slot inside the group is path & 7.
"""
import numpy as np

_M10, _M1, _M2, _M3, _M4 = 0x3FF, 0x30000FF, 0x300F00F, 0x30C30C3, 0x9249249


def _split(v):
    v = np.asarray(v, dtype=np.uint32) & _M10
    v = (v | (v << 16)) & _M1
    v = (v | (v << 8)) & _M2
    v = (v | (v << 4)) & _M3
    v = (v | (v << 2)) & _M4
    return v


def encode_child_index_path(x, y, z):
    """utils/common.rs:24-55 (scalar or array arguments)."""
    return _split(x) | (_split(y) << 1) | (_split(z) << 2)


def decode_path(path, depth):
    """Inverse of encode_child_index_path for a tree of `depth` levels; returns (x, y, z)."""
    p = np.asarray(path, dtype=np.uint32)
    x = np.zeros_like(p)
    y = np.zeros_like(p)
    z = np.zeros_like(p)
    for b in range(depth):
        x |= ((p >> (3 * b)) & 1) << b
        y |= ((p >> (3 * b + 1)) & 1) << b
        z |= ((p >> (3 * b + 2)) & 1) << b
    return x, y, z


def child_index(position, current, max_depth):
    """child_index_macro_2 (utils/common.rs:104-111)."""
    x, y, z = position
    shift = max_depth - current - 1
    return ((x >> shift) & 1) | (((y >> shift) & 1) << 1) | (((z >> shift) & 1) << 2)


def path_mask(max_depth, k):
    """PATH_MASKS[max_depth][k] (spatial/voxtree.rs:41-105) in closed form."""
    if max_depth <= 0 or k > max_depth - 1:
        return 0
    return ((1 << (3 * (k + 1))) - 1) << (3 * (max_depth - 1 - k))
