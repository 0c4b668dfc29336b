"""Model serialisation (VoxModel::serialize + serialize_chunk, world/voxmodel.rs:177-282,
world/voxchunk.rs:382-405) — row f3 of the scope table.

The byte stream renumbers nodes in slot-index order, so it is byte-identical between two
implementations exactly when their allocation orders agree: the single-voxel path (VoxTree::set /
fill, one device thread with the reference's own order) must give the oracle's bytes, bit for bit.
Batched builds allocate in another order; there the streams are decoded and compared as DAGs (the
canonical form of every chunk's root, node counts, values and masks), and the decoder itself is
checked against the oracle's own trees."""
import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_PATCH_P1
from voxelis_gb300.api import VoxInterner, VoxTree


from voxelis_gb300.vtm import canonical, decode  # noqa: E402


def single_voxel_world(lib, bits):
    it = VoxInterner(64 << 20, bits, VX_PATCH_P1, lib=lib)
    trees = [VoxTree(4) for _ in range(3)]
    rng = np.random.default_rng(9)
    hi = 200 if bits == 8 else 3000
    for t in trees:
        for _ in range(300):
            x, y, z = (int(v) for v in rng.integers(0, 16, 3))
            t.set(it, (x, y, z), int(rng.integers(0, hi)))
    trees[2].fill(it, 5)
    trees[2].set(it, (1, 2, 3), 9)
    return it, trees


@pytest.mark.parametrize("bits", [8, 16])
def test_single_voxel_world_bytes(lib, oracle_lib, bits):
    pos = [(0, 0, 0), (1, 0, -2), (7, 3, 1)]
    io, to = single_voxel_world(oracle_lib, bits)
    want = io.serialize_model(to, pos)
    il, tl = single_voxel_world(lib, bits)
    got = il.serialize_model(tl, pos)
    assert got == want
    # the decoder reads back the oracle's own trees
    leaves, branches, chunks = decode(want, bits // 8)
    assert [c[0] for c in chunks] == pos
    assert len(leaves) == io.stats()["leaf_patterns"] and len(branches) == io.stats()["branch_patterns"] - 1


@pytest.mark.parametrize("bits", [8, 16])
def test_batched_world_decodes_to_the_same_dag(lib, oracle_lib, bits):
    dt = np.uint8 if bits == 8 else np.uint16
    grids = W.dune_world_chunks(3, 2, depth=5, seed=12, dtype=dt)
    pos = [(i, 0, k) for k in range(2) for i in range(3)]
    forms = []
    for l in (oracle_lib, lib):
        it = VoxInterner(64 << 20, bits, 0, lib=l)
        trees = [VoxTree(5) for _ in range(6)]
        it.build_dense(trees, grids)
        forms.append(canonical(*decode(it.serialize_model(trees, pos), bits // 8)))
    assert forms[0] == forms[1]
