"""A deep single tree (MaxDepth 8 here; the benchmark runs 10) under P1+P2+P3+P4: dense cave build,
then successive batches of random set/clear edits, compared with the oracle after every step."""
import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_PATCH_P1, VX_PATCH_P2, VX_PATCH_P3, VX_PATCH_P4
from voxelis_gb300.api import VoxInterner, VoxTree

pytestmark = pytest.mark.gpu

PATCHES = VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P3 | VX_PATCH_P4


def same(io, ig, to, tg):
    co, cg = io.export_canonical(to), ig.export_canonical(tg)
    for k in co:
        np.testing.assert_array_equal(co[k], cg[k], err_msg=k)
    assert io.stats()["alive_nodes"] == ig.stats()["alive_nodes"]
    ig.validate(tg)


def test_deep_caves_build_and_edits(oracle_lib, gpu_lib):
    depth = 8
    grid = W.caves_torch(depth, seed=99, device="cpu", y_block=32).numpy()
    io = VoxInterner(1 << 30, 8, PATCHES, lib=oracle_lib)
    ig = VoxInterner(1 << 30, 8, PATCHES, lib=gpu_lib)
    to, tg = VoxTree(depth), VoxTree(depth)
    io.build_dense([to], grid[None])
    ig.build_dense([tg], grid[None])
    same(io, ig, [to], [tg])
    for b in range(3):
        xyz, vals = W.random_edits(depth, 0, 500 + b, max_material=4, clear_fraction=0.2, count=40000)
        for it, t in ((io, to), (ig, tg)):
            bt = t.create_batch(it)
            bt.set_many(xyz, vals)
            assert t.apply_batch(it, bt)
        same(io, ig, [to], [tg])
    rng = np.random.default_rng(3)
    q = rng.integers(0, 1 << depth, (20000, 3)).astype(np.int32)
    fo, vo = io.get_many(np.full(len(q), to.tree), q)
    fg, vg = ig.get_many(np.full(len(q), tg.tree), q)
    np.testing.assert_array_equal(fo, fg)
    np.testing.assert_array_equal(vo, vg)
