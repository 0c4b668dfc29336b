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
from voxelis_gb300._abi import VX_PATCH_P1, ReferencePanic
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


# ---- deserialisation (VoxModel::deserialize, world/voxmodel.rs:284-408) ---------------------------

def _varint(v):
    out = bytearray()
    while v >= 0x80:
        out.append((v & 0x7F) | 0x80)
        v >>= 7
    out.append(v)
    return bytes(out)


def _stream(leaves, branches, chunks, vb=1):
    """A payload from records: leaves [(id, value)], branches [(id, mask, [child ids], lod)],
    chunks [((x, y, z), root id)]."""
    b = bytearray(len(leaves).to_bytes(4, "big"))
    for i, v in leaves:
        b += _varint(i) + int(v).to_bytes(vb, "big")
    b += len(branches).to_bytes(4, "big")
    for i, m, ch, lod in branches:
        b += _varint(i) + bytes([m]) + b"".join(_varint(c) for c in ch) + int(lod).to_bytes(vb, "big")
    b += len(chunks).to_bytes(4, "big")
    for p, r in chunks:
        b += b"VoxTreeChunk" + b"".join(int(a).to_bytes(4, "big", signed=True) for a in p) + _varint(r)
    return bytes(b)


def _leaf(i):
    return (1 << 63) | i


def _branch(i, types, mask):
    return (types << 55) | (mask << 47) | i


# a hand-made payload: leaves 1 (5) and 2 (7); branch 3 = [1, 2] under mask 0b11; branch 4 = [3, 1]
# under mask 0b10000001; chunks rooted at 4, 3 and EMPTY
KNOWN = _stream([(1, 5), (2, 7)], [(3, 0b11, [1, 2], 5), (4, 0b10000001, [3, 1], 5)],
                [((0, 0, 0), 4), ((1, 2, -3), 3), ((-1, 0, 0), 0)])


def test_deserialize_known_answer(lib):
    """deserialize_leaf / deserialize_branch / set_root_id on a payload worked out by hand: slots =
    ids, types = which children are leaves, refcounts = child slots naming the node + chunk roots
    (the EMPTY slot counts the EMPTY root), values and LOD as written."""
    it = VoxInterner(1 << 20, 8, 0, lib=lib)
    trees, pos = it.deserialize_model(KNOWN, 1)
    assert pos.tolist() == [[0, 0, 0], [1, 2, -3], [-1, 0, 0]]
    assert [t.get_root_id() for t in trees] == [_branch(4, 0b10000000, 0b10000001), _branch(3, 0b11, 0b11), 0]
    assert [t.max_depth() for t in trees] == [1, 1, 1]
    refs = {_leaf(1): 2, _leaf(2): 1, _branch(3, 0b11, 0b11): 2, _branch(4, 0b10000000, 0b10000001): 1, 0: 1}
    for bid, want in refs.items():
        assert it.get_ref(bid) == want, hex(bid)
    assert it.stats()["alive_nodes"] == VoxInterner(1 << 20, 8, 0, lib=lib).stats()["alive_nodes"] + 4
    # the tree rooted at branch 3 at MaxDepth 1: octant 0 = leaf 5, octant 1 = leaf 7, the rest empty
    assert trees[1].get(it, (0, 0, 0)) == 5 and trees[1].get(it, (1, 0, 0)) == 7
    assert trees[1].get(it, (0, 1, 0)) is None
    # re-serialising gives the same bytes (slots are the ids, so the renumbering is the identity)
    assert it.serialize_model(trees, pos) == KNOWN


def _world(lib, bits, n=6):
    dt = np.uint8 if bits == 8 else np.uint16
    grids = W.dune_world_chunks(3, 2, depth=5, seed=31, dtype=dt)[:n]
    it = VoxInterner(64 << 20, bits, VX_PATCH_P1, lib=lib)
    trees = [VoxTree(5) for _ in range(n)]
    it.build_dense(trees, grids)
    trees[1].set(it, (1, 2, 3), 9)
    trees[2].fill(it, 4)
    trees.append(VoxTree(5))  # an EMPTY chunk
    pos = [(i % 3, i // 3, -i) for i in range(len(trees))]
    return it, trees, pos


@pytest.mark.parametrize("bits", [8, 16])
def test_deserialize_round_trip(lib, bits):
    """serialize -> deserialize into a fresh interner -> serialize gives the same bytes; the trees
    hold the same voxels and the interner dedups against the loaded patterns afterwards."""
    it, trees, pos = _world(lib, bits)
    data = it.serialize_model(trees, pos)
    it2 = VoxInterner(64 << 20, bits, VX_PATCH_P1, lib=lib)
    t2, p2 = it2.deserialize_model(data, 5)
    assert p2.tolist() == [list(p) for p in pos]
    assert it2.serialize_model(t2, p2) == data
    for a, b in zip(trees, t2):
        np.testing.assert_array_equal(a.to_vec(it), b.to_vec(it2))
    # building the same chunk again finds every node: nothing is created, the root is shared
    created = it2.stats()["nodes_created"]
    again = VoxTree(5)
    it2.build_dense([again], np.stack([trees[0].to_vec(it)]))
    assert again.get_root_id() == t2[0].get_root_id()
    assert it2.stats()["nodes_created"] == created


def _canon_equal(io, to, ig, tg):
    co, cg = io.export_canonical(to), ig.export_canonical(tg)
    for k in co:
        np.testing.assert_array_equal(co[k], cg[k], err_msg=k)
    so, sg = io.stats(), ig.stats()
    for k in ("alive_nodes", "branch_patterns", "leaf_patterns", "next_index", "nodes_created"):
        assert so[k] == sg[k], (k, so[k], sg[k])


@pytest.mark.gpu
@pytest.mark.parametrize("bits", [8, 16])
def test_deserialize_gpu_equals_oracle(oracle_lib, gpu_lib, bits):
    """The same payload deserialised by the GPU and by the oracle: same trees, positions, canonical
    DAG with refcounts, slot-level BlockIds, counts; then the same edits on both stay equal."""
    io, to, pos = _world(oracle_lib, bits)
    data = io.serialize_model(to, pos)
    ro = VoxInterner(64 << 20, bits, VX_PATCH_P1, lib=oracle_lib)
    rg = VoxInterner(64 << 20, bits, VX_PATCH_P1, lib=gpu_lib)
    ao, po = ro.deserialize_model(data, 5)
    ag, pg = rg.deserialize_model(data, 5)
    np.testing.assert_array_equal(po, pg)
    assert [t.get_root_id() for t in ao] == [t.get_root_id() for t in ag]
    _canon_equal(ro, ao, rg, ag)
    assert ro.get_ref(0) == rg.get_ref(0) == 1
    rng = np.random.default_rng(5)
    for t_o, t_g in zip(ao, ag):
        b_o, b_g = t_o.create_batch(ro), t_g.create_batch(rg)
        for _ in range(50):
            p = tuple(int(v) for v in rng.integers(0, 32, 3))
            v = int(rng.integers(0, 6))
            b_o.set(ro, p, v)
            b_g.set(rg, p, v)
        assert t_o.apply_batch(ro, b_o) == t_g.apply_batch(rg, b_g)
    _canon_equal(ro, ao, rg, ag)


def _bad_streams():
    ok_leaves, ok_branches = [(1, 5), (2, 7)], [(3, 0b11, [1, 2], 5)]
    yield "leaf id out of sequence", _stream([(2, 5), (1, 7)], ok_branches, [])
    yield "leaf value zero", _stream([(1, 0), (2, 7)], ok_branches, [])
    yield "branch id out of sequence", _stream(ok_leaves, [(4, 0b11, [1, 2], 5)], [])
    yield "branch mask empty", _stream(ok_leaves, [(3, 0, [], 5)], [])
    yield "child names no node", _stream(ok_leaves, [(3, 0b11, [1, 9], 5)], [])
    yield "root names no node", _stream(ok_leaves, ok_branches, [((0, 0, 0), 4)])
    bad_magic = bytearray(_stream(ok_leaves, ok_branches, [((0, 0, 0), 3)]))
    bad_magic[-14] ^= 1
    yield "chunk magic", bytes(bad_magic)
    five = bytearray(_stream(ok_leaves, ok_branches, []))
    yield "six-byte varint", bytes(five[:4]) + b"\x81\x80\x80\x80\x80\x00" + bytes(five[5:])
    full = _stream(ok_leaves, ok_branches, [((0, 0, 0), 3), ((1, 0, 0), 0)])
    for cut in range(len(full)):
        yield "truncated at %d" % cut, full[:cut]


def test_deserialize_rejects_what_the_reference_panics_on(lib):
    """Every malformed payload is VX_E_REF_PANIC (the reference's unwrap / assert panics), on an
    interner that stays usable; a payload whose records are fine loads on an interner that already
    holds nodes only if it holds none."""
    for name, data in _bad_streams():
        it = VoxInterner(1 << 20, 8, 0, lib=lib)
        with pytest.raises(ReferencePanic):
            it.deserialize_model(data, 2)
        if lib.prefix != "vxo_":  # the device validates every record before it writes a node
            assert it.stats()["nodes_created"] == 0, name
    it = VoxInterner(1 << 20, 8, 0, lib=lib)
    t = VoxTree(2)
    t.set(it, (0, 0, 0), 3)
    with pytest.raises(ReferencePanic):
        it.deserialize_model(KNOWN, 1)
    # an EMPTY child under a set mask bit is what the reference's branch map gives for id 0: loaded
    data = _stream([(1, 5)], [(2, 0b11, [1, 0], 5)], [((0, 0, 0), 2)])
    it = VoxInterner(1 << 20, 8, 0, lib=lib)
    trees, _ = it.deserialize_model(data, 1)
    assert trees[0].get_root_id() == _branch(2, 0b01, 0b11)
    assert trees[0].get(it, (0, 0, 0)) == 5 and trees[0].get(it, (1, 0, 0)) is None


def test_deserialize_empty_model(lib):
    it = VoxInterner(1 << 20, 8, 0, lib=lib)
    trees, pos = it.deserialize_model(_stream([], [], []), 3)
    assert trees == [] and pos.shape == (0, 3)
    trees, pos = it.deserialize_model(_stream([], [], [((4, 5, 6), 0)] * 3), 3)
    assert len(trees) == 3 and all(t.is_empty() for t in trees) and it.get_ref(0) == 3


@pytest.mark.gpu
def test_deserialize_large_stream_gpu_equals_oracle(oracle_lib, gpu_lib):
    """A multi-megabyte payload (noise chunks: about 20 k nodes each; 3.2 MB in 256-byte segments,
    about 12 k of them, 400 level-1 and 13 level-2 tables), so that a section spans thousands of
    parse segments and all three table levels: GPU = oracle, and a round trip."""
    rng = np.random.default_rng(77)
    grids = rng.integers(1, 4, (160, 32, 32, 32), dtype=np.uint8)
    grids[rng.random(grids.shape) < 0.3] = 0
    ig = VoxInterner(256 << 20, 8, 0, lib=gpu_lib)
    trees = [VoxTree(5) for _ in range(len(grids))]
    ig.build_dense(trees, grids)
    pos = [(k, -k, 2 * k) for k in range(len(grids))]
    data = ig.serialize_model(trees, pos)
    assert len(data) > 2 << 20
    ro = VoxInterner(256 << 20, 8, 0, lib=oracle_lib)
    rg = VoxInterner(256 << 20, 8, 0, lib=gpu_lib)
    ao, po = ro.deserialize_model(data, 5)
    ag, pg = rg.deserialize_model(data, 5)
    np.testing.assert_array_equal(po, pg)
    _canon_equal(ro, ao, rg, ag)
    assert rg.serialize_model(ag, pg) == data


def test_deserialize_after_edits_and_releases(lib):
    """A model whose interner has recycled slots (edits replaced subtrees; free list and generations
    in use) serialises with renumbered ids and loads into a fresh interner with the same voxels, and
    re-serialising the loaded model gives the same bytes."""
    dt = np.uint8
    grids = W.dune_world_chunks(2, 2, depth=5, seed=41, dtype=dt)
    it = VoxInterner(64 << 20, 8, VX_PATCH_P1, lib=lib)
    trees = [VoxTree(5) for _ in range(len(grids))]
    it.build_dense(trees, grids)
    rng = np.random.default_rng(3)
    for t in trees:
        b = t.create_batch(it)
        for _ in range(400):
            b.set(it, tuple(int(v) for v in rng.integers(0, 32, 3)), int(rng.integers(1, 7)))
        t.apply_batch(it, b)
    assert it.stats()["free_count"] > 0  # the edits released replaced nodes
    pos = [(k, 0, 0) for k in range(len(trees))]
    data = it.serialize_model(trees, pos)
    it2 = VoxInterner(64 << 20, 8, VX_PATCH_P1, lib=lib)
    t2, p2 = it2.deserialize_model(data, 5)
    for a, b in zip(trees, t2):
        np.testing.assert_array_equal(a.to_vec(it), b.to_vec(it2))
    assert it2.serialize_model(t2, p2) == data
