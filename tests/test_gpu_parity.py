"""GPU library vs oracle on identical inputs, through the C ABI.

Bit-exact criteria (integer work, no tolerance): the canonical DFS export of the DAG (node kinds,
types/mask bits, leaf and LOD values, refcounts, child links, roots), the interner's live node and
pattern counts, and get() of every voxel / of random positions.
"""
import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_PATCH_P1, VX_PATCH_P2, VX_PATCH_P3, VX_PATCH_P4
from voxelis_gb300.api import Batch, VoxInterner, VoxTree

pytestmark = pytest.mark.gpu


def pair(oracle_lib, gpu_lib, budget=64 << 20, bits=8, patches=0):
    return (VoxInterner(budget, bits, patches, lib=oracle_lib), VoxInterner(budget, bits, patches, lib=gpu_lib))


def assert_same(io, ig, to, tg):
    co, cg = io.export_canonical(to), ig.export_canonical(tg)
    for k in co:
        np.testing.assert_array_equal(co[k], cg[k], err_msg="canonical export differs in %s" % k)
    so, sg = io.stats(), ig.stats()
    for k in ("alive_nodes", "branch_patterns", "leaf_patterns"):
        assert so[k] == sg[k], (k, so[k], sg[k])
    ig.validate(tg)
    return co


def level_counts(c, roots):
    """collect_stats (utils/common.rs:302-333): nodes per depth with tree multiplicity."""
    out = {}
    stack = [(int(r), 0) for r in roots if r >= 0]
    memo = {}

    def counts(n):
        if n in memo:
            return memo[n]
        res = {0: 1}
        if c["kind"][n] == 0:
            for ch in c["children"][n]:
                if ch >= 0:
                    for d, k in counts(int(ch)).items():
                        res[d + 1] = res.get(d + 1, 0) + k
        memo[n] = res
        return res

    for r, _ in stack:
        for d, k in counts(r).items():
            out[d] = out.get(d, 0) + k
    return out


def grid(fn, depth=5):
    n = 1 << depth
    y, z, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return fn(x, y, z).astype(np.uint8)


PATTERNS = {
    "uniform": grid(lambda x, y, z: np.ones_like(x)),
    "checkerboard": grid(lambda x, y, z: np.where((x + y + z) % 2 == 0, 1, 0)),
    "sum": grid(lambda x, y, z: (x + y + z) % 256),
}


@pytest.mark.parametrize("path", ["dense", "batch"])
@pytest.mark.parametrize("name", list(PATTERNS))
def test_config1_fresh(oracle_lib, gpu_lib, name, path):
    io, ig = pair(oracle_lib, gpu_lib, 256 << 20)
    to, tg = VoxTree(5), VoxTree(5)
    b = to.create_batch(io)
    b.set_dense(PATTERNS[name])
    assert to.apply_batch(io, b)
    if path == "dense":
        assert ig.build_dense([tg], PATTERNS[name][None])[0] == 1
    else:
        bg = tg.create_batch(ig)
        bg.set_dense(PATTERNS[name])
        assert tg.apply_batch(ig, bg)
    assert_same(io, ig, [to], [tg])
    np.testing.assert_array_equal(to.to_vec(io), tg.to_vec(ig))


def test_config1_sequential(oracle_lib, gpu_lib):
    io, ig = pair(oracle_lib, gpu_lib, 256 << 20)
    to, tg = VoxTree(5), VoxTree(5)
    for name in ("uniform", "checkerboard", "sum"):
        bo, bg = to.create_batch(io), tg.create_batch(ig)
        bo.set_dense(PATTERNS[name])
        bg.set_dense(PATTERNS[name])
        assert to.apply_batch(io, bo) == tg.apply_batch(ig, bg)
        c = assert_same(io, ig, [to], [tg])
        assert level_counts(c, c["roots"]) == level_counts(ig.export_canonical([tg]), c["roots"])
        np.testing.assert_array_equal(to.to_vec(io), tg.to_vec(ig))


def build_terrain(lib, grids, depth, patches=0, budget=256 << 20, bits=8, dense=True):
    it = VoxInterner(budget, bits, patches, lib=lib)
    trees = [VoxTree(depth) for _ in range(len(grids))]
    if dense:
        it.build_dense(trees, grids)
    else:
        bs = []
        for t, g in zip(trees, grids):
            b = t.create_batch(it)
            b.set_dense(g)
            bs.append(b)
        it.apply_batches(trees, bs)
    return it, trees


@pytest.mark.parametrize("depth,patches", [(3, 0), (4, 0), (5, 0), (6, 0), (7, VX_PATCH_P2)])
def test_dense_terrain_matches_oracle(oracle_lib, gpu_lib, depth, patches):
    n = {3: 64, 4: 64, 5: 32, 6: 4, 7: 2}[depth]
    nx = int(np.sqrt(n))
    grids = W.dune_chunks(nx, n // nx, depth=depth, seed=7, base=(1 << depth) // 2 - 2,
                          amp=max(2, (1 << depth) // 3), scale=(1 << depth) * 1.5)
    io, to = build_terrain(oracle_lib, grids, depth, patches)
    ig, tg = build_terrain(gpu_lib, grids, depth, patches)
    c = assert_same(io, ig, to, tg)
    assert level_counts(c, c["roots"]) == level_counts(ig.export_canonical(tg), c["roots"])
    ig2, tg2 = build_terrain(gpu_lib, grids, depth, patches, dense=False)
    assert_same(io, ig2, to, tg2)


@pytest.mark.parametrize("depth,n,bits,patches", [(5, 32, 8, 0), (5, 16, 16, 0), (6, 4, 8, 0), (7, 1, 8, VX_PATCH_P2)])
def test_dense_noise_runs_the_quad_memo_out(oracle_lib, gpu_lib, depth, n, bits, patches):
    """Random voxels: nearly every quad (4^3) is distinct, so the build's quad memo runs out of
    records (a quarter of the quads as slots, half of those as records) and fills its slots: quads
    computed in the streaming kernel after the records are gone, records published without a free
    slot within 4 steps, records shared across the pieces of a host-memory build (n >= 8) and
    uniform quads between them (value 0 on a third of the voxels) all take part."""
    rng = np.random.default_rng(100 + depth)
    side = 1 << depth
    vals = rng.integers(1, 4 if bits == 8 else 4000, (n, side, side, side))
    g = np.where(rng.random((n, side, side, side)) < 0.33, 0, vals).astype(np.uint8 if bits == 8 else np.uint16)
    g[:, : side // 2] = 0  # uniform quads and octants too
    io, ig = pair(oracle_lib, gpu_lib, budget=256 << 20, bits=bits, patches=patches)
    to, tg = [VoxTree(depth) for _ in range(n)], [VoxTree(depth) for _ in range(n)]
    io.build_dense(to, g)
    ig.build_dense(tg, g)
    assert_same(io, ig, to, tg)


def test_per_chunk_equals_batched(gpu_lib):
    grids = W.dune_chunks(4, 4, depth=5, seed=3)
    ia, ta = build_terrain(gpu_lib, grids, 5)
    ib = VoxInterner(256 << 20, lib=gpu_lib)
    tb = [VoxTree(5) for _ in grids]
    for t, g in zip(tb, grids):
        ib.build_dense([t], g[None])
    ca, cb = ia.export_canonical(ta), ib.export_canonical(tb)
    for k in ca:
        np.testing.assert_array_equal(ca[k], cb[k])


def test_gets_match_oracle(oracle_lib, gpu_lib):
    grids = W.dune_chunks(4, 4, depth=5, seed=11)
    io, to = build_terrain(oracle_lib, grids, 5)
    ig, tg = build_terrain(gpu_lib, grids, 5)
    rng = np.random.default_rng(5)
    q = 20000
    tidx = rng.integers(0, len(grids), q)
    xyz = rng.integers(0, 32, (q, 3)).astype(np.int32)
    fo, vo = io.get_many(np.array([to[i].tree for i in tidx]), xyz)
    fg, vg = ig.get_many(np.array([tg[i].tree for i in tidx]), xyz)
    np.testing.assert_array_equal(fo, fg)
    np.testing.assert_array_equal(vo, vg)
    # every voxel of a few chunks against the input grid
    for i in (0, 5, 15):
        np.testing.assert_array_equal(tg[i].to_vec(ig), grids[i])


def edit_batches(trees, interner, depth, density, seed, max_material):
    bs = []
    for j, t in enumerate(trees):
        xyz, vals = W.random_edits(depth, density, seed + j, max_material=max_material)
        b = t.create_batch(interner)
        for (x, y, z), v in zip(xyz, vals):
            b.just_set((x, y, z), int(v))
        bs.append(b)
    return bs


@pytest.mark.parametrize("launch", [1, 0], ids=["single_launch", "per_phase"])
@pytest.mark.parametrize("bits,depths,patches", [
    (8, [5, 5, 5, 5], VX_PATCH_P1),
    (16, [5, 6, 5, 6], VX_PATCH_P1),
    (16, [7, 6, 5], VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P3),
    (8, [5, 5, 6], VX_PATCH_P1 | VX_PATCH_P4),
    (16, [7, 5], VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P3 | VX_PATCH_P4),
])
def test_batched_edits_match_sequential_oracle(oracle_lib, gpu_lib, bits, depths, patches, launch):
    """Batched apply_batch of several trees (both launch forms of the device apply) equals the
    oracle's apply_batch one tree after the other."""
    io, ig = pair(oracle_lib, gpu_lib, 256 << 20, bits, patches)
    gpu_lib.call("tune_set_launch", ig.handle, launch, handle=ig.handle)
    to = [VoxTree(d) for d in depths]
    tg = [VoxTree(d) for d in depths]
    for k, d in enumerate(depths):
        g = W.dune_chunks(1, 1, depth=d, seed=20 + k, base=(1 << d) // 2, amp=(1 << d) // 3,
                          scale=(1 << d) * 1.5, dtype=np.uint8 if bits == 8 else np.uint16)[0]
        io.build_dense([to[k]], g[None])
        ig.build_dense([tg[k]], g[None])
    assert_same(io, ig, to, tg)
    maxm = 255 if bits == 8 else 4095
    for rnd, density in enumerate((0.001, 0.01, 0.1)):
        bo, bg = [], []
        for k, (a, b) in enumerate(zip(to, tg)):
            xyz, vals = W.random_edits(depths[k], density, 100 * rnd + k, max_material=maxm)
            x1, x2 = a.create_batch(io), b.create_batch(ig)
            for (x, y, z), v in zip(xyz, vals):
                x1.just_set((x, y, z), int(v))
                x2.just_set((x, y, z), int(v))
            bo.append(x1)
            bg.append(x2)
        cho = [a.apply_batch(io, b) for a, b in zip(to, bo)]
        chg = ig.apply_batches(tg, bg)
        assert list(cho) == list(chg)
        assert_same(io, ig, to, tg)


def test_clear_everything_p4(oracle_lib, gpu_lib):
    """Clearing every voxel of a chunk under P4 empties the tree on both sides."""
    io, ig = pair(oracle_lib, gpu_lib, 64 << 20, 8, VX_PATCH_P1 | VX_PATCH_P4)
    to, tg = VoxTree(4), VoxTree(4)
    g = W.dune_chunks(1, 1, depth=4, seed=2, base=6, amp=4, scale=24.0)[0]
    io.build_dense([to], g[None])
    ig.build_dense([tg], g[None])
    for it, t in ((io, to), (ig, tg)):
        b = t.create_batch(it)
        b.set_dense(np.zeros_like(g))
        assert t.apply_batch(it, b)
        assert t.is_empty()
    assert_same(io, ig, [to], [tg])
    assert io.stats()["alive_nodes"] == 1


def test_fill_then_patches(oracle_lib, gpu_lib):
    io, ig = pair(oracle_lib, gpu_lib, 64 << 20, 8, VX_PATCH_P1)
    to, tg = VoxTree(5), VoxTree(5)
    for lib_it, t in ((io, to), (ig, tg)):
        b = t.create_batch(lib_it)
        b.just_fill(4)
        for i in range(0, 32, 3):
            b.just_set((i, 31 - i, (i * 7) % 32), 9)
        assert t.apply_batch(lib_it, b)
    assert_same(io, ig, [to], [tg])


def test_release_matches(oracle_lib, gpu_lib):
    grids = W.dune_chunks(3, 3, depth=5, seed=4)
    io, to = build_terrain(oracle_lib, grids, 5)
    ig, tg = build_terrain(gpu_lib, grids, 5)
    for k in (0, 4, 8):
        to[k].clear(io)
        tg[k].clear(ig)
    assert_same(io, ig, to, tg)
    for k in range(9):
        to[k].clear(io)
        tg[k].clear(ig)
    so, sg = io.stats(), ig.stats()
    assert so["alive_nodes"] == sg["alive_nodes"] == 1


def test_rebuild_after_release_reuses_slots(gpu_lib):
    grids = W.dune_chunks(2, 2, depth=5, seed=8)
    ig, tg = build_terrain(gpu_lib, grids, 5)
    s1 = ig.stats()
    for t in tg:
        t.clear(ig)
    tg2 = [VoxTree(5) for _ in grids]
    ig.build_dense(tg2, grids)
    s2 = ig.stats()
    assert s2["alive_nodes"] == s1["alive_nodes"]
    assert s2["next_index"] == s1["next_index"]


@pytest.mark.parametrize("launch", [1, 0], ids=["single_launch", "per_phase"])
@pytest.mark.parametrize("patches", [VX_PATCH_P1 | VX_PATCH_P2, VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P3 | VX_PATCH_P4])
def test_device_group_records_match_oracle(oracle_lib, gpu_lib, patches, launch):
    """vx_apply_groups_async (compacted groups already in HBM) equals sequential apply_batch."""
    import ctypes as C

    import torch

    depths = [7, 6, 6, 5, 5, 5]  # deepest first, as the entry point requires
    io, ig = pair(oracle_lib, gpu_lib, 256 << 20, 16, patches)
    gpu_lib.call("tune_set_launch", ig.handle, launch, handle=ig.handle)
    to = [VoxTree(d) for d in depths]
    tg = [VoxTree(d) for d in depths]
    for k, d in enumerate(depths):
        g = W.dune_chunks(1, 1, depth=d, seed=40 + k, dtype=np.uint16, **W.terrain_params(d))[0]
        io.build_dense([to[k]], g[None])
        ig.build_dense([tg[k]], g[None])
    recs = []
    for k, d in enumerate(depths):
        xyz, vals = W.random_edits(d, (0.001, 0.01, 0.1)[k % 3], 900 + k, max_material=4095)
        b = to[k].create_batch(io)
        b.set_many(xyz, vals)
        to[k].apply_batch(io, b)
        groups, sm, cm, vv = W.edits_to_groups(d, xyz, vals)
        recs.append((np.full(len(groups), k, np.uint32), groups, sm, cm, vv))
    item, group, sm, cm, vv = (np.concatenate([r[j] for r in recs]) for j in range(5))
    dev = torch.device("cuda", 0)

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a).view(np.int32 if a.dtype.itemsize == 4 else
                                                             (np.int16 if a.dtype.itemsize == 2 else np.uint8))).to(dev)

    handles = np.array([x._bind(ig) for x in tg], dtype=np.uint32)
    args = [t(handles), t(np.full(len(tg), 2, np.uint8)), t(np.zeros(len(tg), np.uint32)), len(item),
            t(item), t(group), t(sm), t(cm), t(vv.reshape(-1)), torch.zeros(len(tg), dtype=torch.uint8, device=dev)]
    ptrs = [C.c_void_p(a.data_ptr()) if isinstance(a, torch.Tensor) else a for a in args]
    torch.cuda.synchronize()
    gpu_lib.call("apply_groups_async", ig.handle, len(tg), *ptrs, max(depths), handle=ig.handle)
    ig.sync()
    for x in tg:
        x._dirty = True
    assert_same(io, ig, to, tg)


def test_dense_small_depths_in_any_order(oracle_lib, gpu_lib):
    """Dense builds of chunks of depth 2 and 3 (one CTA per chunk, a shared-memory size per depth),
    with a smaller build between two larger ones, equal the oracle's: a kernel's shared-memory
    opt-in must not shrink when it is launched with less."""
    for depth, bits in ((3, 8), (2, 8), (3, 8), (3, 16), (2, 16), (3, 16)):
        side = 1 << depth
        grids = W.dune_chunks(2, 4, depth=depth, seed=60 + depth, base=side // 2, amp=side // 3, scale=side * 1.5,
                              dtype=np.uint8 if bits == 8 else np.uint16)
        io, to = build_terrain(oracle_lib, grids, depth, bits=bits)
        ig, tg = build_terrain(gpu_lib, grids, depth, bits=bits)
        assert_same(io, ig, to, tg)


@pytest.mark.parametrize("bits,depths,patches", [
    (8, [5, 5, 6], VX_PATCH_P1),
    (16, [4, 6, 5], VX_PATCH_P1),
    (8, [3, 4, 2], 0),
    (8, [7, 5], VX_PATCH_P1 | VX_PATCH_P2),
])
def test_batched_set_matches_one_by_one_set(oracle_lib, gpu_lib, bits, depths, patches):
    """vx_trees_set_many equals VoxTree::set called one voxel at a time in order (the reference's
    single-voxel path: collapse at every level, removal by value 0): same canonical DAG, refcounts,
    live nodes and per-call results, on terrain trees whose uniform regions are collapsed leaves,
    with repeated voxels, unchanged values and removals mixed in."""
    io, ig = pair(oracle_lib, gpu_lib, 256 << 20, bits, patches)
    to = [VoxTree(d) for d in depths]
    tg = [VoxTree(d) for d in depths]
    dt = np.uint8 if bits == 8 else np.uint16
    for k, d in enumerate(depths):
        side = 1 << d
        g = W.dune_chunks(1, 1, depth=d, seed=70 + k, base=side // 2, amp=max(1, side // 3), scale=side * 1.5,
                          dtype=dt)[0]
        io.build_dense([to[k]], g[None])
        ig.build_dense([tg[k]], g[None])
    assert_same(io, ig, to, tg)
    rng = np.random.default_rng(sum(depths) + bits)
    maxm = 255 if bits == 8 else 4095
    for rnd in range(3):
        n = 400
        t_idx = rng.integers(0, len(depths), n)
        xyz = np.stack([rng.integers(0, 1 << depths[t], 3) for t in t_idx]).astype(np.int32)
        xyz[n // 2:n // 2 + 40] = xyz[:40]  # the same voxels again, later in the sequence
        t_idx[n // 2:n // 2 + 40] = t_idx[:40]
        vals = rng.integers(1, 4 if rnd == 0 else maxm, n).astype(np.uint32)  # few values first: collapses
        vals[rng.random(n) < 0.3] = 0
        cho = [to[t].set(io, tuple(int(c) for c in p), int(v)) for t, p, v in zip(t_idx, xyz, vals)]
        chg = ig.set_many([tg[t] for t in t_idx], xyz, vals)
        assert list(cho) == list(chg)
        assert_same(io, ig, to, tg)
