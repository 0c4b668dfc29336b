"""Occupancy masks for greedy meshing (generate_occupancy_masks + fill_masks_for_region,
utils/mesh.rs:418-597) — row f4 of the scope table. The oracle restates the reference's traversal and
region fills; here it is pinned against an independent numpy derivation from the dense grid (each
non-default voxel (x, y, z) of material m sets bit x of YZ[y][z], bit y of XZ[z][x] and bit z of
XY[y][x], globally and in m's planes), and the GPU library must match the oracle bit for bit: several
chunks per builder at offsets, MaxDepth 2..6, u8 and u16, a uniform 64^3 chunk (the reference's
whole-builder fill), overlapping chunks and EMPTY trees."""
import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_PATCH_P1
from voxelis_gb300.api import VoxInterner, VoxTree


def numpy_masks(grids, offsets):
    glob = np.zeros((3, 64, 64), np.uint64)
    mats = {}
    for g, (ox, oy, oz) in zip(grids, offsets):
        ys, zs, xs = np.nonzero(g)
        vals = g[ys, zs, xs].astype(np.int64)
        X, Y, Z = xs + ox, ys + oy, zs + oz
        for m in np.unique(vals):
            sel = vals == m
            cnt, pm = mats.get(int(m), (0, np.zeros((3, 64, 64), np.uint64)))
            np.bitwise_or.at(pm[0], (Y[sel], Z[sel]), np.left_shift(np.uint64(1), X[sel].astype(np.uint64)))
            np.bitwise_or.at(pm[1], (Z[sel], X[sel]), np.left_shift(np.uint64(1), Y[sel].astype(np.uint64)))
            np.bitwise_or.at(pm[2], (Y[sel], X[sel]), np.left_shift(np.uint64(1), Z[sel].astype(np.uint64)))
            mats[int(m)] = (cnt + int(sel.sum()), pm)
        np.bitwise_or.at(glob[0], (Y, Z), np.left_shift(np.uint64(1), X.astype(np.uint64)))
        np.bitwise_or.at(glob[1], (Z, X), np.left_shift(np.uint64(1), Y.astype(np.uint64)))
        np.bitwise_or.at(glob[2], (Y, X), np.left_shift(np.uint64(1), Z.astype(np.uint64)))
    xs_ = np.bitwise_or.reduce(glob[0].ravel())
    ys_ = np.bitwise_or.reduce(glob[1].ravel())
    zs_ = np.bitwise_or.reduce(glob[2].ravel())
    active = np.array([ys_, zs_, zs_, xs_, ys_, xs_], np.uint64)
    return {"global": glob, "active": active, "materials": mats}


def same(a, b):
    np.testing.assert_array_equal(a["global"], b["global"])
    np.testing.assert_array_equal(a["active"], b["active"])
    assert sorted(a["materials"]) == sorted(b["materials"])
    for m in a["materials"]:
        assert a["materials"][m][0] == b["materials"][m][0], m
        np.testing.assert_array_equal(a["materials"][m][1], b["materials"][m][1], err_msg=str(m))


def cases(bits):
    dt = np.uint8 if bits == 8 else np.uint16
    out = []
    # 2 x 2 x 2 dune chunks of 32^3 (the reference's 8-chunks-per-builder packing)
    g = W.dune_world_chunks(2, 2, depth=5, seed=21, dtype=dt)
    grids = [g[0], g[1], g[2], g[3], g[0], g[3], np.zeros_like(g[0]), g[2]]
    offs = [(32 * (k & 1), 32 * ((k >> 1) & 1), 32 * (k >> 2)) for k in range(8)]
    out.append(("dunes_2x2x2_d5", 5, grids, offs))
    # one 64^3 chunk of terrain, one uniform 64^3 chunk
    out.append(("terrain_d6", 6, [W.dune_world_chunks(1, 1, depth=6, seed=5, dtype=dt, **W.terrain_params(6))[0]],
                [(0, 0, 0)]))
    out.append(("uniform_d6", 6, [np.full((64, 64, 64), 7, dt)], [(0, 0, 0)]))
    # 4^3 random chunks of 4^3 voxels at every other offset, overlapping pairs
    rng = np.random.default_rng(3)
    small = [rng.integers(0, 4, (4, 4, 4)).astype(dt) for _ in range(6)]
    out.append(("random_d2_overlap", 2, small, [(0, 0, 0), (0, 0, 0), (60, 8, 4), (12, 60, 0), (5, 9, 13), (5, 9, 13)]))
    return out


@pytest.mark.parametrize("bits", [8, 16])
def test_occupancy_masks(lib, bits):
    for name, d, grids, offs in cases(bits):
        it = VoxInterner(64 << 20, bits, VX_PATCH_P1, lib=lib)
        trees = [VoxTree(d) for _ in grids]
        for t, g in zip(trees, grids):
            b = t.create_batch(it)
            b.set_dense(g)
            t.apply_batch(it, b)
        got = it.occupancy_masks(trees, offs)
        # the numpy derivation works from what the trees hold (to_vec), the way the reference reads them
        want = numpy_masks([t.to_vec(it) for t in trees], offs)
        same(got, want)


@pytest.mark.gpu
def test_gpu_occupancy_matches_oracle(oracle_lib, gpu_lib):
    for name, d, grids, offs in cases(8):
        res = []
        for lib in (oracle_lib, gpu_lib):
            it = VoxInterner(64 << 20, 8, VX_PATCH_P1, lib=lib)
            trees = [VoxTree(d) for _ in grids]
            it.build_dense(trees, np.stack(grids)) if d >= 2 else None
            res.append(it.occupancy_masks(trees, offs))
        same(res[0], res[1])


@pytest.mark.gpu
def test_batched_builders_equal_one_call_per_builder(gpu_lib):
    import ctypes as C

    import torch

    it = VoxInterner(64 << 20, 8, VX_PATCH_P1, lib=gpu_lib)
    grids = W.dune_world_chunks(4, 4, depth=5, seed=8)
    trees = [VoxTree(5) for _ in range(16)]
    it.build_dense(trees, grids)
    # builder b takes chunks 4b .. 4b+3 at the four x/z quadrants; builder 4 stays empty
    n_b, mm = 5, 8
    builder_of = np.repeat(np.arange(4, dtype=np.uint32), 4)
    offs = np.array([(32 * (k & 1), 0, 32 * (k >> 1)) for k in range(4)] * 4, np.uint32)
    handles = np.array([t._bind(it) for t in trees], np.uint32)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.from_numpy(a.view(np.int32) if a.dtype == np.uint32 else a).to(dev)  # noqa: E731
    t_d, b_d, o_d = T(handles), T(builder_of), T(offs.ravel().copy())
    glob = torch.zeros(n_b * 3 * 4096, dtype=torch.int64, device=dev)
    act = torch.zeros(n_b * 6, dtype=torch.int64, device=dev)
    nm = torch.zeros(n_b, dtype=torch.int32, device=dev)
    ids = torch.zeros(n_b * mm, dtype=torch.int32, device=dev)
    cnt = torch.zeros(n_b * mm, dtype=torch.int64, device=dev)
    masks = torch.zeros(n_b * mm * 3 * 4096, dtype=torch.int64, device=dev)
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    torch.cuda.synchronize()
    it._call("occupancy_masks_async", n_b, 16, P(t_d), P(b_d), P(o_d), 5, mm, P(glob), P(act), P(nm), P(ids), P(cnt),
             P(masks))
    it.sync()
    glob = glob.cpu().numpy().view(np.uint64).reshape(n_b, 3, 64, 64)
    act = act.cpu().numpy().view(np.uint64).reshape(n_b, 6)
    nm, ids = nm.cpu().numpy(), ids.cpu().numpy().reshape(n_b, mm)
    cnt = cnt.cpu().numpy().reshape(n_b, mm)
    masks = masks.cpu().numpy().view(np.uint64).reshape(n_b, mm, 3, 64, 64)
    for b in range(n_b):
        sel = [k for k in range(16) if builder_of[k] == b]
        if not sel:
            assert nm[b] == 0 and not glob[b].any() and not act[b].any()
            continue
        one = it.occupancy_masks([trees[k] for k in sel], offs[sel], max_materials=mm)
        np.testing.assert_array_equal(glob[b], one["global"])
        np.testing.assert_array_equal(act[b], one["active"])
        assert nm[b] == len(one["materials"])
        for k, m in enumerate(sorted(one["materials"])):
            assert ids[b, k] == m and cnt[b, k] == one["materials"][m][0]
            np.testing.assert_array_equal(masks[b, k], one["materials"][m][1])
