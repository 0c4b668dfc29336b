"""The device-resident entry points can be recorded into a CUDA graph and replayed: a replayed dense
build gives the same DAG (canonical export, bit-exact) as direct calls, and so do replayed batched
gets. The interner's workspace is grown by one direct call before capture (allocation is not
allowed while a stream is capturing)."""
import ctypes as C

import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300.api import export_canonical as export

pytestmark = pytest.mark.gpu


def test_dense_build_and_gets_replay_from_a_cuda_graph(gpu_lib):
    import torch

    dev = torch.device("cuda", 0)
    n = 64
    grids_np = W.dune_world_chunks(8, 8, depth=5, seed=3)
    h = C.c_void_p()
    gpu_lib.call("interner_create", C.c_uint64(64 << 20), 8, 0, 0, C.byref(h))
    call = lambda name, *a: gpu_lib.call(name, h, *a, handle=h)  # noqa: E731
    stream = torch.cuda.Stream(device=dev)
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    trees = np.zeros(n, np.uint32)
    depths = np.full(n, 5, np.uint8)
    call("trees_create", n, depths.ctypes.data, trees.ctypes.data)
    with torch.cuda.stream(stream):
        t_d = torch.from_numpy(trees.view(np.int32)).to(dev)
        g_d = torch.from_numpy(grids_np).to(dev)
        rng = np.random.default_rng(5)
        q_t = torch.from_numpy(trees[rng.integers(0, n, 4096)].view(np.int32)).to(dev)
        q_xyz = torch.from_numpy(rng.integers(0, 32, (4096, 3)).astype(np.int32)).to(dev)
        found = torch.zeros(4096, dtype=torch.uint8, device=dev)
        vals = torch.zeros(4096, dtype=torch.uint8, device=dev)
    stream.synchronize()
    build = (n, C.c_void_p(t_d.data_ptr()), C.c_void_p(g_d.data_ptr()), None, 5)
    gets = (C.c_uint64(4096), C.c_void_p(q_t.data_ptr()), C.c_void_p(q_xyz.data_ptr()),
            C.c_void_p(found.data_ptr()), C.c_void_p(vals.data_ptr()))

    call("build_dense_async", *build)  # direct: grows the workspace
    call("get_many_async", *gets)
    call("interner_sync")
    want = export(gpu_lib, h, trees)
    want_found, want_vals = found.cpu().numpy().copy(), vals.cpu().numpy().copy()

    call("interner_reset")
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        call("build_dense_async", *build)
        call("get_many_async", *gets)
    for _ in range(2):  # the capture itself ran nothing; replay twice from an empty interner
        call("interner_reset")
        found.zero_()
        vals.zero_()
        stream.synchronize()
        with torch.cuda.stream(stream):
            graph.replay()
        call("interner_sync")
        got = export(gpu_lib, h, trees)
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
        np.testing.assert_array_equal(found.cpu().numpy(), want_found)
        np.testing.assert_array_equal(vals.cpu().numpy(), want_vals)
    gpu_lib.call("interner_destroy", h, handle=h)


def test_batched_apply_replays_from_a_cuda_graph(gpu_lib, oracle_lib):
    """A batched apply whose level passes take the one-pass scan over many tiles, captured once and
    replayed three times from an empty interner, gives the oracle's DAG every time: the scan's
    look-back state lives on the device and is clean at the start of every scan, whether the scan
    was launched directly or replayed."""
    import torch

    from voxelis_gb300._abi import VX_PATCH_P1
    from voxelis_gb300.api import Batch, VoxInterner, VoxTree

    depth, n = 5, 48
    grids = W.dune_world_chunks(8, 6, depth=depth, seed=11)
    edits = [W.random_edits(depth, 0.05, 900 + i, max_material=200) for i in range(n)]
    recs = [W.edits_to_groups(depth, xyz, v) for xyz, v in edits]
    R = sum(len(r[0]) for r in recs)
    assert 2 * 2048 < R < 64 * 2048  # several tiles, within the one-pass scan's range

    # the oracle: dense build, then one Batch per chunk (just_set in order) applied
    oi = VoxInterner(256 << 20, 8, VX_PATCH_P1, lib=oracle_lib)
    ot = [VoxTree(depth) for _ in range(n)]
    oi.build_dense(ot, grids)
    batches = []
    for xyz, v in edits:
        b = Batch(depth, 8, VX_PATCH_P1, lib=oracle_lib)
        b.set_many(xyz, v)
        batches.append(b)
    oi.apply_batches(ot, batches)
    want = oi.export_canonical(ot)

    dev = torch.device("cuda", 0)
    h = C.c_void_p()
    gpu_lib.call("interner_create", C.c_uint64(256 << 20), 8, VX_PATCH_P1, 0, C.byref(h))
    call = lambda name, *a: gpu_lib.call(name, h, *a, handle=h)  # noqa: E731
    stream = torch.cuda.Stream(device=dev)
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    trees = np.zeros(n, np.uint32)
    call("trees_create", n, np.full(n, depth, np.uint8).ctypes.data, trees.ctypes.data)
    item = np.concatenate([np.full(len(r[0]), i, np.uint32) for i, r in enumerate(recs)])
    group, sm, cm, vv = (np.concatenate([r[j] for r in recs]) for j in range(4))

    def dev_arr(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a).view(dt)).to(dev)

    with torch.cuda.stream(stream):
        t_d = dev_arr(trees, np.int32)
        g_d = torch.from_numpy(grids).to(dev)
        it_d, gr_d = dev_arr(item, np.int32), dev_arr(group, np.int32)
        s_d, c_d, v_d = dev_arr(sm, np.uint8), dev_arr(cm, np.uint8), dev_arr(vv.reshape(-1), np.int16)
        flags = torch.full((n,), 2, dtype=torch.uint8, device=dev)
        fill = torch.zeros(n, dtype=torch.int32, device=dev)
    stream.synchronize()
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731

    def work():
        call("build_dense_async", n, P(t_d), P(g_d), None, depth)
        call("apply_groups_async", n, P(t_d), P(flags), P(fill), R, P(it_d), P(gr_d), P(s_d), P(c_d), P(v_d),
             None, depth)

    work()  # direct: grows the workspace
    call("interner_sync")
    got = export(gpu_lib, h, trees)
    for k in want:
        np.testing.assert_array_equal(got[k], want[k], err_msg="direct " + k)

    call("interner_reset")
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        work()
    for rep in range(3):
        call("interner_reset")
        stream.synchronize()
        with torch.cuda.stream(stream):
            graph.replay()
        call("interner_sync")
        got = export(gpu_lib, h, trees)
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg="replay %d %s" % (rep, k))
    gpu_lib.call("interner_destroy", h, handle=h)
