"""Known answers derived by reading the reference path (voxtree.rs:724-1118, interner/mod.rs).

These pin behaviours the reference's own tests do not: the exact DAG and refcounts of the plain
single-chunk workload (uniform / checkerboard / (x+y+z) mod 256 at MaxDepth 5), the refcount leak
when a batch re-sets voxels of an ancestor leaf to the leaf's own value (Q5), the assert_ne! panic
when a batch rebuilds the same root (Q4) and the BlockId::types() panic on a partial edit of a
collapsed bottom group (Q3) together with its patched behaviour (P1).
Each case runs on the oracle and, in gpu-marked runs, on the GPU library.
"""
import numpy as np
import pytest

from voxelis_gb300 import block_id as B
from voxelis_gb300._abi import VX_PATCH_P1, VX_PATCH_P4, VX_PATCH_P5, ReferencePanic
from voxelis_gb300.api import VoxInterner, VoxTree

D = 5
N = 1 << D


def grid(fn):
    y, z, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    return fn(x, y, z).astype(np.uint8)


UNIFORM = grid(lambda x, y, z: np.ones_like(x))
CHECKER = grid(lambda x, y, z: np.where((x + y + z) % 2 == 0, 1, 0))
SUM = grid(lambda x, y, z: (x + y + z) % 256)


def build(lib, g, tree=None, interner=None, patches=0):
    interner = interner or VoxInterner.with_memory_budget(256 << 20, patches=patches, lib=lib)
    tree = tree or VoxTree(D)
    b = tree.create_batch(interner)
    b.set_dense(g)
    changed = tree.apply_batch(interner, b)
    return interner, tree, changed


def test_uniform_is_one_leaf(lib):
    interner, tree, changed = build(lib, UNIFORM)
    assert changed
    r = tree.get_root_id()
    assert B.is_leaf(r) and interner.get_value(r) == 1 and interner.get_ref(r) == 1
    c = interner.export_canonical([tree])
    assert len(c["kind"]) == 1 and c["kind"][0] == 1


def test_checkerboard_is_one_leaf_and_five_branches(lib):
    interner, tree, changed = build(lib, CHECKER)
    assert changed
    c = interner.export_canonical([tree])
    # pre-order: root, depth-1, depth-2, depth-3, bottom group branch, leaf(1)
    assert list(c["kind"]) == [0, 0, 0, 0, 0, 1]
    assert list(c["refcount"]) == [1, 8, 8, 8, 8, 4]
    assert list(c["mask"][:4]) == [0xFF] * 4 and list(c["types"][:4]) == [0] * 4
    assert c["mask"][4] == 0x69 and c["types"][4] == 0x69  # even-parity slots 0, 3, 5, 6
    assert c["value"][5] == 1
    assert list(c["children"][4]) == [5, -1, -1, 5, -1, 5, 5, -1]


def test_sum_pattern_gets(lib):
    interner, tree, changed = build(lib, SUM)
    assert changed
    assert np.array_equal(tree.to_vec(interner), SUM)
    assert interner.get_ref(tree.get_root_id()) == 1


def test_checkerboard_on_uniform_is_a_noop_that_leaks(lib):
    """Every set slot already holds leaf(1): each of the 4096 groups returns early after
    inc_ref_by(leaf, 8 - 4) (voxtree.rs:835-839, 865-868)."""
    interner, tree, _ = build(lib, UNIFORM)
    leaf = tree.get_root_id()
    _, _, changed = build(lib, CHECKER, tree=tree, interner=interner)
    assert not changed
    assert tree.get_root_id() == leaf
    assert interner.get_ref(leaf) == 1 + 4 * 4096


def test_sequential_config1(lib):
    interner, tree, _ = build(lib, UNIFORM)
    build(lib, CHECKER, tree=tree, interner=interner)
    _, _, changed = build(lib, SUM, tree=tree, interner=interner)
    assert changed
    # sets never clear: (x+y+z) mod 256 == 0 only at the origin, which keeps the uniform value 1
    want = SUM.copy()
    want[0, 0, 0] = 1
    assert np.array_equal(tree.to_vec(interner), want)


def test_reapplying_a_uniform_batch_panics(lib):
    """Q4: the rebuilt root equals the old root and apply_batch's assert_ne! fires (voxtree.rs:311)."""
    interner, tree, _ = build(lib, UNIFORM)
    with pytest.raises(ReferencePanic):
        build(lib, UNIFORM, tree=tree, interner=interner)


def test_reapplying_a_uniform_batch_p5(lib):
    """P5 skips the assert_ne!: the root is released and re-installed, so the DAG and every
    refcount are what they were before the second batch."""
    interner, tree, _ = build(lib, UNIFORM, patches=VX_PATCH_P5)
    root, rc, alive = tree.get_root_id(), interner.get_ref(tree.get_root_id()), interner.stats()["alive_nodes"]
    _, _, changed = build(lib, UNIFORM, tree=tree, interner=interner)
    assert changed
    assert tree.get_root_id() == root and interner.get_ref(root) == rc
    assert interner.stats()["alive_nodes"] == alive
    assert np.array_equal(tree.to_vec(interner), UNIFORM)
    interner.validate([tree])


def _collapsed_group_then_partial(lib, patches):
    interner = VoxInterner.with_memory_budget(1 << 20, patches=patches, lib=lib)
    tree = VoxTree(D)
    b = tree.create_batch(interner)
    for x in range(2):
        for y in range(2):
            for z in range(2):
                b.set(interner, (x, y, z), 1)
    assert tree.apply_batch(interner, b)
    b2 = tree.create_batch(interner)
    b2.set(interner, (0, 0, 0), 2)
    return interner, tree, b2


def test_partial_edit_of_collapsed_bottom_group_panics(lib):
    """Q3: the descent stops on a leaf at depth max-1 and BlockId::types() asserts."""
    interner, tree, b2 = _collapsed_group_then_partial(lib, 0)
    with pytest.raises(ReferencePanic):
        tree.apply_batch(interner, b2)


def test_partial_edit_of_collapsed_bottom_group_p1(lib):
    interner, tree, b2 = _collapsed_group_then_partial(lib, VX_PATCH_P1)
    assert tree.apply_batch(interner, b2)
    assert tree.get(interner, (0, 0, 0)) == 2
    assert tree.get(interner, (1, 0, 0)) == 1 and tree.get(interner, (1, 1, 1)) == 1
    assert tree.get(interner, (2, 0, 0)) is None
    interner.validate([tree])


def test_clears_are_ignored_without_p4(lib):
    interner, tree, _ = build(lib, UNIFORM)
    b = tree.create_batch(interner)
    b.set(interner, (3, 3, 3), 0)
    assert b.size() == 1 and b.has_patches()
    assert not tree.apply_batch(interner, b)
    assert tree.get(interner, (3, 3, 3)) == 1


def test_clears_with_p4(lib):
    interner = VoxInterner.with_memory_budget(256 << 20, patches=VX_PATCH_P4 | VX_PATCH_P1, lib=lib)
    tree = VoxTree(D)
    build(lib, UNIFORM, tree=tree, interner=interner)
    b = tree.create_batch(interner)
    b.set(interner, (3, 3, 3), 0)
    b.set(interner, (4, 3, 3), 7)
    assert tree.apply_batch(interner, b)
    assert tree.get(interner, (3, 3, 3)) is None
    assert tree.get(interner, (4, 3, 3)) == 7
    assert tree.get(interner, (5, 3, 3)) == 1
    interner.validate([tree])
    assert interner.get_ref(tree.get_root_id()) == 1
