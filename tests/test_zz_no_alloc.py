"""vx_build_dense_noalloc: the dense build for callers that cannot allocate device memory.

Some callers cannot let a library call cudaMalloc while they run: code recorded into a CUDA graph
(allocation is not allowed during stream capture), frame loops and servers that reserve their device
memory up front, and hosts whose allocator belongs to another runtime. This entry point stages the
levels above the 32^3 blocks (chunks of depth 6 and more) in a fixed device array compiled into the
library instead of a workspace grown on demand; shallower chunks (a CTA per 32^3 block, a warp per
16^3 octant at depth 4, a CTA per chunk at depths 2-3) stage nothing. Its output must be identical
to the regular dense-build entry point's (integer work: no tolerance), on two calls in a row that
share the array, and requests larger than the array must be refused before any work is queued.

This file is collected last so that, should it fail, a run stopping at the first failure has
already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_E_BUFFER, VX_OK, VX_PATCH_P2
from voxelis_gb300.api import VoxInterner, VoxTree

pytestmark = pytest.mark.gpu

SCRATCH_BYTES = 3 << 20  # VX_NOALLOC_SCRATCH_BYTES in include/voxelis_gb300.h


def scratch_bytes(n, depth):
    """Bytes a call stages: node rows (12 B) of the levels above the unit one CTA reduces (32^3 blocks
    at depths 5-10, 16^3 octants at depth 4), rounded up to 256, then their arrival counts (4 B)."""
    unit = 5 if depth >= 5 else 4
    rows = sum(n << (3 * k) for k in range(1, depth - unit + 1))
    counts = sum(n << (3 * k) for k in range(0, depth - unit))
    return (12 * rows + 255) // 256 * 256 + 4 * counts + 256


def _noalloc(lib):
    f = lib.lib.vx_build_dense_noalloc
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
    f.restype = C.c_int
    return f


def _grids(depth, n, seed):
    side = 1 << depth
    nx = 2 if n > 1 else 1
    return W.dune_chunks(nx, n // nx, depth=depth, seed=seed, base=side // 2, amp=side // 3, scale=side * 1.5)


@pytest.mark.parametrize("depth,n,patches", [(6, 4, 0), (7, 2, VX_PATCH_P2), (5, 8, 0), (4, 8, 0), (3, 8, 0)])
def test_noalloc_matches_regular_build_on_two_calls(gpu_lib, depth, n, patches):
    import torch

    f = _noalloc(gpu_lib)
    first, second = _grids(depth, n, 31), _grids(depth, n, 32)

    # the regular entry point (host buffers, workspace grown on demand)
    ref = VoxInterner(256 << 20, 8, patches, lib=gpu_lib)
    ref_a, ref_b = [VoxTree(depth) for _ in range(n)], [VoxTree(depth) for _ in range(n)]
    ch_ref_a = ref.build_dense(ref_a, first)
    ch_ref_b = ref.build_dense(ref_b, second)

    # the no-allocation entry point, called twice in a row on the same interner
    it = VoxInterner(256 << 20, 8, patches, lib=gpu_lib)
    out_a, out_b = [VoxTree(depth) for _ in range(n)], [VoxTree(depth) for _ in range(n)]
    dev = torch.device("cuda", 0)
    for trees, grids, ch_ref in ((out_a, first, ch_ref_a), (out_b, second, ch_ref_b)):
        handles = np.array([t._bind(it) for t in trees], dtype=np.uint32)
        t_d = torch.from_numpy(handles.view(np.int32)).to(dev)
        g_d = torch.from_numpy(np.ascontiguousarray(grids)).to(dev)
        c_d = torch.zeros(n, dtype=torch.uint8, device=dev)
        torch.cuda.synchronize()
        st = f(it.handle, n, C.c_void_p(t_d.data_ptr()), C.c_void_p(g_d.data_ptr()), C.c_void_p(c_d.data_ptr()), depth)
        assert st == VX_OK, gpu_lib.last_error(it.handle)
        it.sync()
        np.testing.assert_array_equal(c_d.cpu().numpy(), ch_ref)
        for t in trees:
            t._dirty = True

    for mine, theirs in ((out_a, ref_a), (out_a + out_b, ref_a + ref_b)):
        c_mine, c_ref = it.export_canonical(mine), ref.export_canonical(theirs)
        for k in c_ref:
            np.testing.assert_array_equal(c_mine[k], c_ref[k], err_msg=k)
    assert it.stats()["alive_nodes"] == ref.stats()["alive_nodes"]
    it.validate(out_a + out_b)
    for k in (0, n - 1):
        np.testing.assert_array_equal(out_b[k].to_vec(it), second[k])


def test_noalloc_refuses_requests_beyond_its_array(gpu_lib):
    import torch

    f = _noalloc(gpu_lib)
    it = VoxInterner(1 << 20, 8, 0, lib=gpu_lib)
    tree = VoxTree(6)
    tree._bind(it)
    small = torch.zeros(64, dtype=torch.uint8, device="cuda")
    per_chunk = scratch_bytes(2, 6) - scratch_bytes(1, 6)
    too_many = SCRATCH_BYTES // per_chunk + 1
    assert scratch_bytes(too_many, 6) > SCRATCH_BYTES
    st = f(it.handle, too_many, C.c_void_p(small.data_ptr()), C.c_void_p(small.data_ptr()), None, 6)
    assert st == VX_E_BUFFER
    assert it.stats()["alive_nodes"] == 1
    assert tree.is_empty()


def test_noalloc_replays_from_a_cuda_graph(gpu_lib):
    """The reason the entry point exists: after one direct call on the device (which resolves the
    array's address), the call is recorded into a CUDA graph and replayed into fresh trees, twice,
    with the regular build's result each time."""
    import torch

    f = _noalloc(gpu_lib)
    depth, n = 6, 4
    grids = _grids(depth, n, 41)
    ref = VoxInterner(64 << 20, 8, 0, lib=gpu_lib)
    ref_trees = [VoxTree(depth) for _ in range(n)]
    ch_ref = ref.build_dense(ref_trees, grids)
    want = ref.export_canonical(ref_trees)

    it = VoxInterner(64 << 20, 8, 0, lib=gpu_lib)
    trees = [VoxTree(depth) for _ in range(n)]
    handles = np.array([t._bind(it) for t in trees], dtype=np.uint32)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    it.set_stream(stream.cuda_stream)
    with torch.cuda.stream(stream):
        t_d = torch.from_numpy(handles.view(np.int32)).to(dev)
        g_d = torch.from_numpy(np.ascontiguousarray(grids)).to(dev)
        c_d = torch.zeros(n, dtype=torch.uint8, device=dev)
    stream.synchronize()
    args = (it.handle, n, C.c_void_p(t_d.data_ptr()), C.c_void_p(g_d.data_ptr()), C.c_void_p(c_d.data_ptr()), depth)
    assert f(*args) == VX_OK, gpu_lib.last_error(it.handle)  # direct call before any capture
    it.sync()
    gpu_lib.call("interner_reset", it.handle, handle=it.handle)
    stream.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        assert f(*args) == VX_OK
    for rep in range(2):
        gpu_lib.call("interner_reset", it.handle, handle=it.handle)
        c_d.zero_()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            graph.replay()
        it.sync()
        np.testing.assert_array_equal(c_d.cpu().numpy(), ch_ref)
        for t in trees:
            t._dirty = True
        got = it.export_canonical(trees)
        for k in want:
            np.testing.assert_array_equal(got[k], want[k], err_msg="replay %d %s" % (rep, k))
