"""to_vec (utils/common.rs:158-246) on the GPU: vx_trees_to_dense / vx_trees_to_dense_async against the
oracle's to_vec, tree by tree, bit-exact (integer work). Covers every depth 1..8, u8 and u16, EMPTY
trees, trees whose root is a leaf (fill), collapsed leaves at every level (P1 + uniform sub-cubes),
host and device output, and a size-independent round trip (dense build -> to_vec == input) on a
MaxDepth 9 tree. A tree of the wrong depth is refused. (MaxDepth 1 trees are made with fill and
single-voxel set: the reference's batch path needs MaxDepth >= 2.)"""
import ctypes as C

import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_E_INVALID_ARG, VX_OK, VX_PATCH_P1, VX_PATCH_P2
from voxelis_gb300.api import VoxInterner, VoxTree

pytestmark = pytest.mark.gpu


def _trees(lib, depth, bits, seed, n=5):
    """n trees of one depth in one interner: EMPTY, filled, blocky (uniform sub-cubes that collapse),
    and random edits."""
    patches = VX_PATCH_P1 | (VX_PATCH_P2 if depth > 6 else 0)
    it = VoxInterner(256 << 20, bits, patches, lib=lib)
    trees = [VoxTree(depth) for _ in range(n)]
    rng = np.random.default_rng(seed)
    side = 1 << depth
    hi = 255 if bits == 8 else 4095
    trees[1].fill(it, 7)
    if depth < 2:  # batches need MaxDepth >= 2 (the reference's batch path underflows below)
        trees[2].fill(it, 3)
        trees[3].set(it, (1, 0, 1), 9)
        trees[4].set(it, (0, 1, 0), 5)
        trees[4].set(it, (1, 1, 1), 6)
        return it, trees
    # blocky: 4^3-voxel (or whole-tree) blocks of one value, so leaves sit at several depths
    blk = max(1, side // 4)
    coarse = rng.integers(0, 4, (side // blk,) * 3)
    g = np.kron(coarse, np.ones((blk, blk, blk), dtype=np.int64)).astype(np.uint8 if bits == 8 else np.uint16)
    b = trees[2].create_batch(it)
    b.set_dense(g)
    trees[2].apply_batch(it, b)
    for t in trees[3:]:
        cnt = max(1, side ** 3 // 5)
        xyz = rng.integers(0, side, (cnt, 3)).astype(np.int32)
        vals = rng.integers(1, hi, cnt).astype(np.uint32)
        b = t.create_batch(it)
        b.set_many(xyz, vals)
        t.apply_batch(it, b)
    return it, trees


@pytest.mark.parametrize("bits", [8, 16])
@pytest.mark.parametrize("depth", [1, 2, 3, 4, 5, 6, 7, 8])
def test_to_vec_matches_oracle(oracle_lib, gpu_lib, depth, bits):
    if depth > 6 and bits == 16:
        pytest.skip("u16 covered at depths 1-6")
    io, to = _trees(oracle_lib, depth, bits, 100 + depth)
    ig, tg = _trees(gpu_lib, depth, bits, 100 + depth)
    many = ig.to_vec_many(tg)
    for k in range(len(to)):
        want = to[k].to_vec(io)
        np.testing.assert_array_equal(many[k], want, err_msg="tree %d" % k)
        np.testing.assert_array_equal(tg[k].to_vec(ig), want, err_msg="tree %d (single)" % k)


def test_to_vec_device_output_and_depth_check(gpu_lib):
    import torch

    ig, tg = _trees(gpu_lib, 6, 8, 7)
    want = ig.to_vec_many(tg)
    handles = np.array([t._bind(ig) for t in tg], dtype=np.uint32)
    dev = torch.device("cuda", 0)
    t_d = torch.from_numpy(handles.view(np.int32)).to(dev)
    out = torch.full((len(tg), 64, 64, 64), 0xAB, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    st = gpu_lib.status("trees_to_dense_async", ig.handle, len(tg), C.c_void_p(t_d.data_ptr()), 6,
                        C.c_void_p(out.data_ptr()))
    assert st == VX_OK
    ig.sync()
    np.testing.assert_array_equal(out.cpu().numpy(), want)
    # a tree of another depth is refused on the host path ...
    other = VoxTree(5)
    h = np.array([tg[0]._bind(ig), other._bind(ig)], dtype=np.uint32)
    buf = np.zeros((2, 64, 64, 64), np.uint8)
    st = gpu_lib.status("trees_to_dense", ig.handle, 2, C.c_void_p(h.ctypes.data), C.c_void_p(buf.ctypes.data), 0)
    assert st == VX_E_INVALID_ARG


def test_dense_build_round_trip_depth9(gpu_lib):
    """Size-independent property at a full MaxDepth 9 tree (512^3): to_vec(build_dense(g)) == g."""
    grid = W.caves_torch(9, seed=5, device="cpu", y_block=64).numpy()
    ig = VoxInterner(1 << 30, 8, VX_PATCH_P2, lib=gpu_lib)
    t = VoxTree(9)
    ig.build_dense([t], grid[None])
    np.testing.assert_array_equal(t.to_vec(ig), grid)
