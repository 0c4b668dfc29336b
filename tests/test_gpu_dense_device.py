"""Dense builds from device memory run as one piece: for 8-bit interners the lanes that create nodes
count their children's references and the top-level kernel's last CTA closes the allocation epoch
(16-bit interners count in one pass over the epoch's allocations), and the record kernel computes
only the listed claims (placed ones, and those left without a memo slot). Each case builds its
grids in two calls into one interner, so the second call's epoch starts from the first one's close,
and compares with the oracle's host build of the same grids: canonical export (kinds, masks,
values, refcounts, child links, roots) and the live node and pattern counts, bit-exact."""
import ctypes as C

import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_MEM_DEVICE, VX_PATCH_P2
from voxelis_gb300.api import VoxInterner, VoxTree

pytestmark = pytest.mark.gpu


def _grids(kind, depth, n, bits, seed):
    if kind == "dunes":
        nx = max(1, int(np.sqrt(n)))
        return W.dune_chunks(nx, n // nx, depth=depth, seed=seed, base=(1 << depth) // 2 - 2,
                             amp=max(2, (1 << depth) // 3), scale=(1 << depth) * 1.5)
    rng = np.random.default_rng(seed)  # nearly every quad distinct: the memo runs out of records
    side = 1 << depth
    vals = rng.integers(1, 4 if bits == 8 else 4000, (n, side, side, side))
    g = np.where(rng.random((n, side, side, side)) < 0.33, 0, vals)
    g[:, : side // 2] = 0
    return g.astype(np.uint8 if bits == 8 else np.uint16)


def _build_from_device(it, trees, grids):
    import torch

    dev = torch.device("cuda", 0)
    handles = np.ascontiguousarray([t._bind(it) for t in trees], dtype=np.uint32)
    g = np.ascontiguousarray(grids)
    t_d = torch.from_numpy(handles.view(np.int32)).to(dev)
    g_d = torch.from_numpy(g.view(np.int8 if g.dtype == np.uint8 else np.int16)).to(dev)
    ch_d = torch.zeros(len(trees), dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    it._call("build_dense", len(trees), C.c_void_p(t_d.data_ptr()), C.c_void_p(g_d.data_ptr()),
             C.c_void_p(ch_d.data_ptr()), VX_MEM_DEVICE)
    it.sync()
    for t in trees:
        t._dirty = True
    return ch_d.cpu().numpy()


@pytest.mark.parametrize("kind,depth,n,bits", [
    ("dunes", 5, 64, 8),
    ("dunes", 6, 16, 8),
    ("dunes", 7, 4, 8),
    ("noise", 5, 32, 8),
    ("noise", 6, 4, 8),
    ("noise", 5, 16, 16),
])
def test_device_dense_build_equals_oracle(oracle_lib, gpu_lib, kind, depth, n, bits):
    pytest.importorskip("torch")
    grids = _grids(kind, depth, n, bits, seed=11 + depth)
    patches = VX_PATCH_P2 if depth >= 7 else 0
    io = VoxInterner(256 << 20, bits, patches, lib=oracle_lib)
    ig = VoxInterner(256 << 20, bits, patches, lib=gpu_lib)
    to, tg = [VoxTree(depth) for _ in range(n)], [VoxTree(depth) for _ in range(n)]
    half = n // 2
    for part in (slice(0, half), slice(half, n)):
        want = io.build_dense(to[part], grids[part])
        got = _build_from_device(ig, tg[part], grids[part])
        np.testing.assert_array_equal(got, want)
    co, cg = io.export_canonical(to), ig.export_canonical(tg)
    for k in co:
        np.testing.assert_array_equal(cg[k], co[k], err_msg="canonical export differs in %s" % k)
    so, sg = io.stats(), ig.stats()
    for k in ("alive_nodes", "branch_patterns", "leaf_patterns"):
        assert so[k] == sg[k], (k, so[k], sg[k])
    assert sg["error_flags"] == 0
    ig.validate(tg)
