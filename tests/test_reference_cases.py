"""The reference's own unit tests for this path, restated over the C ABI.

Sources: voxelis/src/spatial/voxtree.rs:1128-2202 (32 tests), core/block_id.rs:475-609 and
core/max_depth.rs:157-230. Each test keeps the reference's inputs and assertions (every-voxel get,
root refcount 1, changed flags, dedup of equal content). The random-noise tests use a fixed seed
(the reference uses an unseeded rand::rng()).

The `lib` fixture runs every case on the CPU oracle and, in gpu-marked runs, on the GPU library.
"""
import numpy as np
import pytest

from voxelis_gb300 import block_id as B
from voxelis_gb300._abi import VX_PATCH_P2, ReferencePanic
from voxelis_gb300.api import VoxInterner, VoxTree


def every_voxel(interner, tree):
    """get() of every voxel, as a dense [y][z][x] array of Optional values (0 = None)."""
    n = tree.voxels_per_axis()
    ys, zs, xs = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    xyz = np.stack([xs.ravel(), ys.ravel(), zs.ravel()], axis=1)
    found, vals = interner.get_many(np.full(len(xyz), tree._bind(interner)), xyz)
    out = np.where(found, vals, 0).reshape(n, n, n)
    return out, found.reshape(n, n, n)


def expect_grid(interner, tree, fn):
    n = tree.voxels_per_axis()
    y, z, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    want = fn(x, y, z).astype(np.int64)
    got, found = every_voxel(interner, tree)
    assert np.array_equal(found, want != 0)
    assert np.array_equal(got.astype(np.int64), want)


def mk(lib, budget, bits=8, patches=0):
    return VoxInterner.with_memory_budget(budget, voxel_bits=bits, patches=patches, lib=lib)


# ---- voxtree.rs tests ---------------------------------------------------------------------------
def test_create(lib):
    tree = VoxTree(3)
    assert tree.is_empty()
    assert tree.max_depth(0) == 3
    assert tree.voxels_per_axis(0) == 8


def test_child_index():
    from voxelis_gb300.morton import child_index

    for max_depth in range(7):
        n = 1 << max_depth
        for depth in range(max_depth):
            for y in range(n):
                for z in range(n):
                    for x in range(n):
                        assert child_index((x, y, z), depth, max_depth) < 8


def test_set_and_get(lib):
    interner = mk(lib, 1024 * 2)
    tree = VoxTree(3)
    p = (0, 0, 0)
    assert tree.set(interner, p, 42)
    assert tree.get(interner, p) == 42
    assert tree.set(interner, p, 24)
    assert tree.get(interner, p) == 24
    assert tree.get(interner, (1, 1, 1)) is None
    assert tree.set(interner, (7, 7, 7), 99)
    assert tree.get(interner, (7, 7, 7)) == 99
    tree.clear(interner)
    positions = [(0, 0, 0), (0, 0, 1), (0, 1, 0), (0, 1, 1), (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)]
    for i, pos in enumerate(positions):
        tree.set(interner, pos, i + 1)
    for i, pos in enumerate(positions):
        assert tree.get(interner, pos) == i + 1


def test_is_empty(lib):
    interner = mk(lib, 1024)
    tree = VoxTree(3)
    assert tree.is_empty()
    assert tree.set(interner, (0, 0, 0), 1)
    assert not tree.is_empty()
    tree.clear(interner)
    assert tree.is_empty()


def test_clear(lib):
    interner = mk(lib, 1024 * 2)
    tree = VoxTree(3)
    positions = [(0, 0, 0), (0, 0, 1), (0, 1, 0), (0, 1, 1), (1, 0, 0), (1, 0, 1), (1, 1, 0), (1, 1, 1)]
    for i, pos in enumerate(positions):
        tree.set(interner, pos, i + 1)
    tree.clear(interner)
    assert tree.is_empty()
    for pos in positions:
        assert tree.get(interner, pos) is None


def test_no_default_leaf_nodes(lib):
    interner = mk(lib, 1024)
    tree = VoxTree(3)
    p = (0, 0, 0)
    assert tree.set(interner, p, 42)
    assert tree.get(interner, p) == 42
    assert not tree.is_empty()
    assert tree.set(interner, p, 0)
    assert tree.get(interner, p) is None
    assert tree.is_empty()


def test_dirty_flag(lib):
    interner = mk(lib, 1024)
    tree = VoxTree(3)
    assert not tree.is_dirty()
    assert tree.set(interner, (0, 0, 0), 1)
    assert tree.is_dirty()
    tree.clear_dirty()
    assert not tree.is_dirty()
    tree.clear(interner)
    assert tree.is_dirty()


def test_shared_interner_uniqueness(lib):
    interner = mk(lib, 1024)
    t1, t2 = VoxTree(3), VoxTree(3)
    assert t1.is_empty() and t2.is_empty()
    assert t1.set(interner, (0, 0, 0), 42)
    assert t1.get(interner, (0, 0, 0)) == 42
    assert t2.get(interner, (0, 0, 0)) is None
    assert t2.set(interner, (0, 0, 0), 24)
    assert t2.get(interner, (0, 0, 0)) == 24
    assert t1.get_root_id() != t2.get_root_id()


def test_shared_interner_deduplication(lib):
    interner = mk(lib, 1024)
    t1, t2 = VoxTree(3), VoxTree(3)
    assert t1.set(interner, (0, 0, 0), 42)
    assert t2.set(interner, (0, 0, 0), 42)
    assert t1.get_root_id() == t2.get_root_id()


def test_set_behaviour(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    p = (0, 0, 0)
    assert tree.set(interner, p, 3)
    assert tree.get(interner, p) == 3
    assert tree.set(interner, p, 4)
    assert tree.get(interner, p) == 4
    assert not tree.set(interner, p, 4)
    assert tree.get(interner, p) == 4


def test_batch_double_apply(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    batch.set(interner, (0, 0, 0), 3)
    assert tree.apply_batch(interner, batch)
    assert not tree.apply_batch(interner, batch)


def test_patterns_set_expand_shared_leaf(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    for value in range(1, 6):
        tree.fill(interner, value * 10)
        tree.set(interner, (0, 0, 0), value)
        expect_grid(interner, tree, lambda x, y, z, v=value: np.where((x == 0) & (y == 0) & (z == 0), v, v * 10))
    assert not tree.is_empty()
    assert not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_expand_shared_leaf(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    batch.fill(interner, 1)
    batch.set(interner, (0, 0, 0), 2)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: np.where((x == 0) & (y == 0) & (z == 0), 2, 1))
    assert not tree.is_empty()
    assert not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_set_checkerboard(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    n = 32
    for y in range(n):
        for z in range(n):
            for x in range(n):
                if (x + y + z) % 2 == 0:
                    assert tree.set(interner, (x, y, z), 2)
    expect_grid(interner, tree, lambda x, y, z: np.where((x + y + z) % 2 == 0, 2, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_checkerboard(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    n = 32
    for y in range(n):
        for z in range(n):
            for x in range(n):
                assert batch.set(interner, (x, y, z), 2 if (x + y + z) % 2 == 0 else 1)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: np.where((x + y + z) % 2 == 0, 2, 1))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_set_solid_fill_one_by_one(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    n = 32
    for y in range(n):
        for z in range(n):
            for x in range(n):
                assert tree.set(interner, (x, y, z), 3)
    expect_grid(interner, tree, lambda x, y, z: np.full(x.shape, 3))
    assert not tree.is_empty() and tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_solid_fill_one_by_one(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    n = 32
    for y in range(n):
        for z in range(n):
            for x in range(n):
                assert batch.set(interner, (x, y, z), 3)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: np.full(x.shape, 3))
    assert not tree.is_empty() and tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_set_solid_fill_half_one_by_one(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    n, half = 32, 16
    for value in range(1, 6):
        for y in range(half):
            for z in range(n):
                for x in range(n):
                    assert tree.set(interner, (x, y, z), value)
        expect_grid(interner, tree, lambda x, y, z, v=value: np.where(y < half, v, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_solid_fill_half_one_by_one(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    n, half = 32, 16
    for value in range(1, 6):
        batch = tree.create_batch(interner)
        for y in range(half):
            for z in range(n):
                for x in range(n):
                    assert batch.set(interner, (x, y, z), value)
        assert tree.apply_batch(interner, batch)
        expect_grid(interner, tree, lambda x, y, z, v=value: np.where(y < half, v, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_set_solid_fill_fill_op(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    tree.fill(interner, 3)
    expect_grid(interner, tree, lambda x, y, z: np.full(x.shape, 3))
    assert not tree.is_empty() and tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_solid_fill_fill_op(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    batch.fill(interner, 3)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: np.full(x.shape, 3))
    assert not tree.is_empty() and tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def _sparse(x, y, z):
    return np.where((x % 4 == 0) & (y % 4 == 0) & (z % 4 == 0), 3, 0)


def test_patterns_set_sparse_fill(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    for y in range(0, 32, 4):
        for z in range(0, 32, 4):
            for x in range(0, 32, 4):
                assert tree.set(interner, (x, y, z), 3)
                assert tree.get(interner, (x, y, z)) == 3
    expect_grid(interner, tree, _sparse)
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_sparse_fill(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    for y in range(0, 32, 4):
        for z in range(0, 32, 4):
            for x in range(0, 32, 4):
                assert batch.set(interner, (x, y, z), 3)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, _sparse)
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_set_gradient_fill(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    for x in range(32):
        value = x % 256
        for y in range(32):
            for z in range(32):
                assert tree.set(interner, (x, y, z), value) == (value > 0)
    expect_grid(interner, tree, lambda x, y, z: x % 256)
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_gradient_fill(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    for x in range(32):
        for y in range(32):
            for z in range(32):
                assert batch.set(interner, (x, y, z), x % 256)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: x % 256)
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def _edge(x, y, z, n=32):
    return (x == 0) | (x == n - 1) | (y == 0) | (y == n - 1) | (z == 0) | (z == n - 1)


def test_patterns_set_hollow_cube(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    for y in range(32):
        for z in range(32):
            for x in range(32):
                if _edge(x, y, z):
                    assert tree.set(interner, (x, y, z), 3)
    expect_grid(interner, tree, lambda x, y, z: np.where(_edge(x, y, z), 3, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_hollow_cube(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    for y in range(32):
        for z in range(32):
            for x in range(32):
                if _edge(x, y, z):
                    assert batch.set(interner, (x, y, z), 3)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: np.where(_edge(x, y, z), 3, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_set_diagonal(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    for i in range(32):
        assert tree.set(interner, (i, i, i), 3)
        assert tree.get(interner, (i, i, i)) == 3
    expect_grid(interner, tree, lambda x, y, z: np.where((x == y) & (x == z), 3, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_diagonal(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    for i in range(32):
        assert batch.set(interner, (i, i, i), 3)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, lambda x, y, z: np.where((x == y) & (x == z), 3, 0))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def _random_noise_edits(seed=1234, count=1000):
    rng = np.random.default_rng(seed)
    edits = []
    for _ in range(count):
        x, y, z = (int(v) for v in rng.integers(0, 32, 3))
        edits.append((x, y, z, int(rng.integers(1, 256))))
    return edits


def _noise_grid(edits):
    data = np.zeros((32, 32, 32), dtype=np.int64)  # [y][z][x]
    for x, y, z, v in edits:
        data[y, z, x] = v
    return lambda x, y, z: data[y, z, x]


def test_patterns_set_random_noise(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    edits = _random_noise_edits()
    for x, y, z, v in edits:
        assert tree.set(interner, (x, y, z), v)
        assert tree.get(interner, (x, y, z)) == v
    expect_grid(interner, tree, _noise_grid(edits))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_patterns_batch_random_noise(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(5)
    batch = tree.create_batch(interner)
    edits = _random_noise_edits()
    for x, y, z, v in edits:
        assert batch.set(interner, (x, y, z), v)
    assert tree.apply_batch(interner, batch)
    expect_grid(interner, tree, _noise_grid(edits))
    assert not tree.is_empty() and not tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


def test_max_depth_zero(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(0)
    assert tree.set(interner, (0, 0, 0), 1)
    assert tree.get(interner, (0, 0, 0)) == 1
    assert not tree.is_empty()
    assert tree.is_leaf()
    assert interner.get_ref(tree.get_root_id()) == 1


# ---- max_depth.rs / traversal_depth.rs caps -------------------------------------------------------
def test_max_depth_cap(lib):
    interner = mk(lib, 1 << 20)
    with pytest.raises(ReferencePanic):
        VoxTree(7)._bind(interner)
    VoxTree(6)._bind(interner)


def test_max_depth_cap_patched(lib):
    interner = mk(lib, 1 << 20, patches=VX_PATCH_P2)
    VoxTree(10)._bind(interner)
    with pytest.raises(ReferencePanic):
        VoxTree(11)._bind(interner)


def test_get_out_of_bounds(lib):
    interner = mk(lib, 1 << 20)
    tree = VoxTree(3)
    with pytest.raises(ReferencePanic):
        tree.get(interner, (8, 0, 0))
    with pytest.raises(ReferencePanic):
        tree.set(interner, (0, -1, 0), 1)


# ---- block_id.rs tests (bit layout of the id shared by the ABI) ----------------------------------
def test_block_id_layout():
    assert B.is_invalid(B.INVALID) and not B.is_valid(B.INVALID)
    e = B.EMPTY
    assert B.index(e) == 0 and B.generation(e) == 0 and B.types(e) == 0 and B.mask(e) == 0
    assert B.is_branch(e) and B.is_empty(e) and B.is_valid(e)
    leaf = B.new_leaf(123, 456)
    assert B.index(leaf) == 123 and B.generation(leaf) == 456 and B.is_leaf(leaf)
    assert leaf == 0x800001C80000007B  # block_id.rs:409 doc-test value
    br = B.new_branch(123, 456, 0xAB, 0xCD)
    assert (B.index(br), B.generation(br), B.types(br), B.mask(br)) == (123, 456, 0xAB, 0xCD)
    assert B.is_branch(br)
    mx = B.new_extended(B.MAX_INDEX, B.MAX_GENERATION, 0xFF, 0xFF, True)
    assert B.is_valid(mx) and mx != B.INVALID
    with pytest.raises(B.BlockIdPanic):
        B.new_leaf(0, B.MAX_GENERATION + 1)
    with pytest.raises(B.BlockIdPanic):
        B.types(B.new_leaf(0, 0))
    with pytest.raises(B.BlockIdPanic):
        B.mask(B.new_leaf(0, 0))
    with pytest.raises(B.BlockIdPanic):
        B.has_child(B.new_leaf(0, 0), 0)
    with pytest.raises(B.BlockIdPanic):
        B.has_child(B.new_branch(0, 0, 0xFF, 0xFF), 8)
    b = B.new_branch(0, 0, 0, 0b1010_1010)
    assert B.has_child(b, 1) and not B.has_child(b, 0) and B.has_child(b, 3) and not B.has_child(b, 2)
    assert B.describe(B.INVALID) == "Id(INVALID)" and B.describe(B.EMPTY) == "Id(EMPTY)"
    assert B.describe(B.new_leaf(1, 2)) == "Id(L, i: 00000001, g: 0002)"


def test_root_ids_follow_the_layout(lib):
    """Root ids returned through the ABI decode with the reference's BlockId layout."""
    interner = mk(lib, 1 << 20)
    tree = VoxTree(3)
    tree.fill(interner, 5)
    r = tree.get_root_id()
    assert B.is_leaf(r) and interner.get_value(r) == 5
    tree.set(interner, (1, 2, 3), 9)
    r = tree.get_root_id()
    assert B.is_branch(r) and B.mask(r) == 0xFF and B.types(r) != 0xFF
