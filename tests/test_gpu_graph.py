"""The device-resident entry points can be recorded into a CUDA graph and replayed: a replayed dense
build gives the same DAG (canonical export, bit-exact) as direct calls, and so do replayed batched
gets. The interner's workspace is grown by one direct call before capture (allocation is not
allowed while a stream is capturing)."""
import ctypes as C

import numpy as np
import pytest

from voxelis_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def test_dense_build_and_gets_replay_from_a_cuda_graph(gpu_lib):
    import torch

    from bench import export

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
