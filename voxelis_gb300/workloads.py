"""Seeded synthetic inputs of the named workload shapes (host-side, numpy, double precision).

perlin-dune terrain (dense chunks of a world tiled in XZ):
    h(wx, wz) = base + floor(amp * P(wx / scale, wz / scale)), P = 2D gradient noise with a
    256-entry permutation shuffled from the seed (Fisher-Yates driven by SplitMix64) and the quintic
    fade 6t^5 - 15t^4 + 10t^3. Voxels: y < h-4 -> 3 (stone), h-4 <= y < h-1 -> 2 (dirt),
    y == h-1 -> 1 (grass), above -> 0 (air).
caves (one large dense grid): voxel = 1 + floor(3|N|) where N(x/64, y/64, z/64) > 0.1, else 0,
    N = 3D gradient noise with the same permutation scheme.
random edits: uniform positions per chunk at a given density, 85% sets (material uniform in
    1..max_material) and 15% clears, applied last-write-wins as Batch::just_set does.
Heights and grids are generated once on the host and shipped as data, so the CPU and GPU paths see
identical inputs.
"""
import numpy as np

_MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.state = seed & _MASK64

    def next(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & _MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK64
        return z ^ (z >> 31)


def permutation(seed):
    """256-entry permutation shuffled by Fisher-Yates from SplitMix64(seed), doubled to 512."""
    rng = SplitMix64(seed)
    p = list(range(256))
    for i in range(255, 0, -1):
        j = rng.next() % (i + 1)
        p[i], p[j] = p[j], p[i]
    return np.array(p + p, dtype=np.int64)


def _fade(t):
    return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)


_G2 = np.array([[1, 1], [-1, 1], [1, -1], [-1, -1], [1, 0], [-1, 0], [0, 1], [0, -1]], dtype=np.float64)


def perlin2(x, z, perm):
    """2D gradient noise at arrays x, z (values roughly in [-1, 1])."""
    x = np.asarray(x, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    x0 = np.floor(x)
    z0 = np.floor(z)
    xi = x0.astype(np.int64) & 255
    zi = z0.astype(np.int64) & 255
    xf = x - x0
    zf = z - z0
    u = _fade(xf)
    v = _fade(zf)

    def g(hx, hz, dx, dz):
        h = perm[perm[hx] + hz] & 7
        return _G2[h, 0] * dx + _G2[h, 1] * dz

    n00 = g(xi, zi, xf, zf)
    n10 = g(xi + 1, zi, xf - 1, zf)
    n01 = g(xi, zi + 1, xf, zf - 1)
    n11 = g(xi + 1, zi + 1, xf - 1, zf - 1)
    nx0 = n00 + u * (n10 - n00)
    nx1 = n01 + u * (n11 - n01)
    return nx0 + v * (nx1 - nx0)


_G3 = np.array([[1, 1, 0], [-1, 1, 0], [1, -1, 0], [-1, -1, 0], [1, 0, 1], [-1, 0, 1], [1, 0, -1], [-1, 0, -1],
                [0, 1, 1], [0, -1, 1], [0, 1, -1], [0, -1, -1], [1, 1, 0], [0, -1, 1], [-1, 1, 0], [0, -1, -1]],
               dtype=np.float64)


def perlin3(x, y, z, perm):
    """3D gradient noise (improved-noise gradient set) at arrays x, y, z."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    z = np.asarray(z, dtype=np.float64)
    x0, y0, z0 = np.floor(x), np.floor(y), np.floor(z)
    xi = x0.astype(np.int64) & 255
    yi = y0.astype(np.int64) & 255
    zi = z0.astype(np.int64) & 255
    xf, yf, zf = x - x0, y - y0, z - z0
    u, v, w = _fade(xf), _fade(yf), _fade(zf)

    def g(ix, iy, iz, dx, dy, dz):
        h = perm[perm[perm[ix] + iy] + iz] & 15
        return _G3[h, 0] * dx + _G3[h, 1] * dy + _G3[h, 2] * dz

    n000 = g(xi, yi, zi, xf, yf, zf)
    n100 = g(xi + 1, yi, zi, xf - 1, yf, zf)
    n010 = g(xi, yi + 1, zi, xf, yf - 1, zf)
    n110 = g(xi + 1, yi + 1, zi, xf - 1, yf - 1, zf)
    n001 = g(xi, yi, zi + 1, xf, yf, zf - 1)
    n101 = g(xi + 1, yi, zi + 1, xf - 1, yf, zf - 1)
    n011 = g(xi, yi + 1, zi + 1, xf, yf - 1, zf - 1)
    n111 = g(xi + 1, yi + 1, zi + 1, xf - 1, yf - 1, zf - 1)
    x00 = n000 + u * (n100 - n000)
    x10 = n010 + u * (n110 - n010)
    x01 = n001 + u * (n101 - n001)
    x11 = n011 + u * (n111 - n011)
    y0_ = x00 + v * (x10 - x00)
    y1_ = x01 + v * (x11 - x01)
    return y0_ + w * (y1_ - y0_)


def dune_heights(nx, nz, side, seed=1234, base=12, amp=10, scale=48.0):
    """Integer heights h[wz][wx] of an (nx*side) x (nz*side) world."""
    perm = permutation(seed)
    wx = np.arange(nx * side, dtype=np.float64)
    wz = np.arange(nz * side, dtype=np.float64)
    X, Z = np.meshgrid(wx / scale, wz / scale, indexing="xy")
    return (base + np.floor(amp * perlin2(X, Z, perm))).astype(np.int64)


def terrain_column_values(h, side, y0=0, dtype=np.uint8):
    """Dense [y][z][x] block for heights h[z][x] and world y range [y0, y0 + side)."""
    y = np.arange(y0, y0 + side, dtype=np.int64)[:, None, None]
    hh = h[None, :, :]
    out = np.zeros((side, h.shape[0], h.shape[1]), dtype=dtype)
    out[y < hh - 4] = 3
    out[(y >= hh - 4) & (y < hh - 1)] = 2
    out[y == hh - 1] = 1
    return out


def dune_chunks(nx, nz, depth=5, seed=1234, base=12, amp=10, scale=48.0, dtype=np.uint8):
    """Dense grids of nx*nz chunks of side 2^depth tiled in XZ (chunk (i, k) covers
    wx in [side*i, side*i+side), wz in [side*k, side*k+side), y in [0, side)); chunk order is
    k-major (index = k*nx + i). Returns an array [n][side][side][side] ([y][z][x] per chunk)."""
    side = 1 << depth
    h = dune_heights(nx, nz, side, seed, base, amp, scale)
    grids = np.zeros((nz * nx, side, side, side), dtype=dtype)
    for k in range(nz):
        for i in range(nx):
            grids[k * nx + i] = terrain_column_values(h[k * side:(k + 1) * side, i * side:(i + 1) * side], side,
                                                      dtype=dtype)
    return grids


def dune_world_chunks(nx, nz, depth=5, seed=1234, base=12, amp=10, scale=48.0, dtype=np.uint8):
    """Same grids as dune_chunks, generated for the whole world at once (vectorised)."""
    side = 1 << depth
    h = dune_heights(nx, nz, side, seed, base, amp, scale)  # [wz][wx]
    world = terrain_column_values(h, side, dtype=dtype)    # [y][wz][wx]
    w = world.reshape(side, nz, side, nx, side)              # y, k, z, i, x
    return np.ascontiguousarray(w.transpose(1, 3, 0, 2, 4)).reshape(nz * nx, side, side, side)


def caves(depth, seed=99, dtype=np.uint8):
    """Dense [y][z][x] grid of side 2^depth: 1 + floor(3|N|) where N > 0.1, else 0."""
    side = 1 << depth
    perm = permutation(seed)
    out = np.zeros((side, side, side), dtype=dtype)
    zz, xx = np.meshgrid(np.arange(side) / 64.0, np.arange(side) / 64.0, indexing="ij")
    for y in range(side):
        n = perlin3(xx, np.full_like(xx, y / 64.0), zz, perm)
        out[y] = np.where(n > 0.1, 1 + np.floor(3 * np.abs(n)), 0).astype(dtype)
    return out


def caves_torch(depth, seed=99, device=None, y_block=64):
    """caves() computed with torch (float64, op for op the same arithmetic as perlin3), for grids too
    large to generate on the host in reasonable time; returns a [y][z][x] uint8 tensor on `device`."""
    import torch

    side = 1 << depth
    perm = torch.tensor(permutation(seed), dtype=torch.int64, device=device)
    g3 = torch.tensor(_G3, dtype=torch.float64, device=device)
    out = torch.empty((side, side, side), dtype=torch.uint8, device=device)
    zz, xx = torch.meshgrid(torch.arange(side, dtype=torch.float64, device=device) / 64.0,
                            torch.arange(side, dtype=torch.float64, device=device) / 64.0, indexing="ij")

    def fade(t):
        return t * t * t * (t * (t * 6.0 - 15.0) + 10.0)

    for y0 in range(0, side, y_block):
        yy = (torch.arange(y0, min(side, y0 + y_block), dtype=torch.float64, device=device) / 64.0)[:, None, None]
        x = xx[None].expand(yy.shape[0], side, side)
        z = zz[None].expand(yy.shape[0], side, side)
        y = yy.expand(yy.shape[0], side, side)
        x0, y0_, z0 = torch.floor(x), torch.floor(y), torch.floor(z)
        xi, yi, zi = x0.long() & 255, y0_.long() & 255, z0.long() & 255
        xf, yf, zf = x - x0, y - y0_, z - z0
        u, v, w = fade(xf), fade(yf), fade(zf)

        def g(ix, iy, iz, dx, dy, dz):
            h = perm[perm[perm[ix] + iy] + iz] & 15
            return g3[h, 0] * dx + g3[h, 1] * dy + g3[h, 2] * dz

        n000 = g(xi, yi, zi, xf, yf, zf)
        n100 = g(xi + 1, yi, zi, xf - 1, yf, zf)
        n010 = g(xi, yi + 1, zi, xf, yf - 1, zf)
        n110 = g(xi + 1, yi + 1, zi, xf - 1, yf - 1, zf)
        n001 = g(xi, yi, zi + 1, xf, yf, zf - 1)
        n101 = g(xi + 1, yi, zi + 1, xf - 1, yf, zf - 1)
        n011 = g(xi, yi + 1, zi + 1, xf, yf - 1, zf - 1)
        n111 = g(xi + 1, yi + 1, zi + 1, xf - 1, yf - 1, zf - 1)
        x00 = n000 + u * (n100 - n000)
        x10 = n010 + u * (n110 - n010)
        x01 = n001 + u * (n101 - n001)
        x11 = n011 + u * (n111 - n011)
        a = x00 + v * (x10 - x00)
        b = x01 + v * (x11 - x01)
        n = a + w * (b - a)
        out[y0:y0 + yy.shape[0]] = torch.where(n > 0.1, 1 + torch.floor(3 * torch.abs(n)),
                                               torch.zeros_like(n)).to(torch.uint8)
    return out


def random_edits(depth, density, seed, max_material=4095, clear_fraction=0.15, count=None):
    """(x, y, z, value) edits at uniform positions: count = density * voxels (or `count`); value 0 is
    a clear."""
    side = 1 << depth
    rng = np.random.default_rng(seed)
    n = count if count is not None else max(1, int(round(density * side ** 3)))
    xyz = rng.integers(0, side, size=(n, 3), dtype=np.int64)
    vals = rng.integers(1, max_material + 1, size=n, dtype=np.int64)
    vals[rng.random(n) < clear_fraction] = 0
    return xyz, vals


def edits_to_groups(depth, xyz, vals):
    """The Batch a sequence of just_set calls leaves behind (core/batch.rs:145-172), compacted:
    sorted touched bottom groups with their (set, clear) masks and 8 values. The last write to a
    voxel wins; a zero value records a clear (its value stays 0)."""
    from .morton import encode_child_index_path

    xyz = np.asarray(xyz, dtype=np.int64).reshape(-1, 3)
    vals = np.asarray(vals, dtype=np.int64).reshape(-1)
    path = encode_child_index_path(xyz[:, 0], xyz[:, 1], xyz[:, 2]).astype(np.int64)
    order = np.argsort(path, kind="stable")
    sp = path[order]
    last = np.ones(len(sp), dtype=bool)
    last[:-1] = sp[1:] != sp[:-1]
    sel = order[last]
    p = path[sel]
    v = vals[sel]
    g = p >> 3
    slot = p & 7
    groups, inv = np.unique(g, return_inverse=True)
    set_mask = np.zeros(len(groups), dtype=np.uint8)
    clear_mask = np.zeros(len(groups), dtype=np.uint8)
    np.bitwise_or.at(set_mask, inv, ((v != 0).astype(np.uint8) << slot.astype(np.uint8)))
    np.bitwise_or.at(clear_mask, inv, ((v == 0).astype(np.uint8) << slot.astype(np.uint8)))
    values = np.zeros((len(groups), 8), dtype=np.uint16)
    values[inv, slot] = v
    return groups.astype(np.uint32), set_mask, clear_mask, values


def terrain_params(depth):
    """Dune terrain scaled to chunks of side 2^depth (base 3s/8, amplitude 5s/16, scale 1.5s;
    s = 32 gives the 32^3 workload's 12, 10 and 48)."""
    s = 1 << depth
    return dict(base=3 * s // 8, amp=5 * s // 16, scale=1.5 * s)
