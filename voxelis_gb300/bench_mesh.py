"""Occupancy masks for greedy meshing (bench.py --workload mesh).

The 4096 perlin-dune chunks of 32^3 u8 of the default workload, built once into a device-resident
interner, then packed 8 to a 64^3 builder (2 x 2 x 2 chunks at offsets 0/32, the reference's
8-chunks-of-32^3 packing, utils/mesh.rs:1195-1225): 512 vx_occupancy_masks calls through the C ABI
(host outputs: the builder's global planes, active masks, per-material counts and planes). Every
builder is checked against the CPU oracle's restatement of generate_occupancy_masks on the same
trees for a sample; the oracle is timed on the same sample (one thread).
"""
import ctypes as C
import json
import statistics
import time

import numpy as np

from . import workloads as W
from ._abi import gpu_lib

N_SIDE = 64
MAX_MAT = 16


def run(args):
    import torch

    from .build import build as build_lib

    build_lib()
    lib = gpu_lib()
    dev = torch.device("cuda", 0)
    grids = W.dune_world_chunks(N_SIDE, N_SIDE, depth=5, seed=1234)
    n = grids.shape[0]
    h = C.c_void_p()
    lib.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(h))
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731
    trees = np.zeros(n, np.uint32)
    call("trees_create", n, np.full(n, 5, np.uint8).ctypes.data, trees.ctypes.data)
    t_d = torch.from_numpy(trees.view(np.int32)).to(dev)
    g_d = torch.from_numpy(grids).to(dev)
    call("build_dense_async", n, C.c_void_p(t_d.data_ptr()), C.c_void_p(g_d.data_ptr()), None, 5)
    call("interner_sync")
    # builders: chunk (i, k) of the 64 x 64 tiling goes to builder (i // 2, k // 2) at (32 (i & 1), 0, 32 (k & 1))
    groups = []
    for bk in range(N_SIDE // 2):
        for bi in range(N_SIDE // 2):
            ids, offs = [], []
            for dk in range(2):
                for di in range(2):
                    c = (2 * bk + dk) * N_SIDE + (2 * bi + di)
                    ids.append(trees[c])
                    offs.append((32 * di, 0, 32 * dk))
            groups.append((np.array(ids, np.uint32), np.array(offs, np.uint32)))
    glob = np.zeros(3 * 4096, np.uint64)
    active = np.zeros(6, np.uint64)
    nm = C.c_uint32()
    mids = np.zeros(MAX_MAT, np.uint32)
    mcnt = np.zeros(MAX_MAT, np.uint64)
    mmask = np.zeros(MAX_MAT * 3 * 4096, np.uint64)

    def one(ids, offs):
        call("occupancy_masks", len(ids), C.c_void_p(ids.ctypes.data), C.c_void_p(offs.ctypes.data),
             C.c_void_p(glob.ctypes.data), C.c_void_p(active.ctypes.data), MAX_MAT, C.byref(nm),
             C.c_void_p(mids.ctypes.data), C.c_void_p(mcnt.ctypes.data), C.c_void_p(mmask.ctypes.data))

    for g in groups[:8]:
        one(*g)
    reps = max(1, args.steps // 200)
    t0 = time.perf_counter()
    for _ in range(reps):
        for g in groups:
            one(*g)
    gpu_s = (time.perf_counter() - t0) / reps
    # oracle on a sample of builders, same trees rebuilt there
    import bench as B

    ol = B.oracle_lib()
    oh = C.c_void_p()
    ol.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(oh))
    sample = groups[:: max(1, len(groups) // 32)][:32]
    ok = True
    cpu_s = 0.0
    o_glob = np.zeros_like(glob)
    o_active = np.zeros_like(active)
    o_nm = C.c_uint32()
    o_ids = np.zeros_like(mids)
    o_cnt = np.zeros_like(mcnt)
    o_mask = np.zeros_like(mmask)
    for ids, offs in sample:
        o_trees = np.zeros(len(ids), np.uint32)
        for k, t in enumerate(ids):
            out = C.c_uint32()
            ol.call("tree_create", oh, 5, C.byref(out))
            o_trees[k] = out.value
            g = np.ascontiguousarray(grids[int(np.nonzero(trees == t)[0][0])])
            ol.call("build_dense", oh, 1, C.c_void_p(o_trees[k:k + 1].ctypes.data), C.c_void_p(g.ctypes.data), None, 0)
        t1 = time.perf_counter()
        ol.call("occupancy_masks", oh, len(ids), C.c_void_p(o_trees.ctypes.data), C.c_void_p(offs.ctypes.data),
                C.c_void_p(o_glob.ctypes.data), C.c_void_p(o_active.ctypes.data), MAX_MAT, C.byref(o_nm),
                C.c_void_p(o_ids.ctypes.data), C.c_void_p(o_cnt.ctypes.data), C.c_void_p(o_mask.ctypes.data))
        cpu_s += time.perf_counter() - t1
        one(ids, offs)
        k = o_nm.value
        ok = ok and nm.value == k and np.array_equal(glob, o_glob) and np.array_equal(active, o_active) and \
            np.array_equal(mids[:k], o_ids[:k]) and np.array_equal(mcnt[:k], o_cnt[:k]) and \
            np.array_equal(mmask[:k * 3 * 4096], o_mask[:k * 3 * 4096])
    ol.status("interner_destroy", oh)
    call("interner_destroy")
    line = {"metric": "chunks/s (occupancy masks, 8 chunks of 32^3 per 64^3 builder)",
            "value": n / gpu_s, "unit": "chunks/s", "higher_is_better": True,
            "config": {"workload": "occupancy masks of the 4096 dune chunks, 512 builders, through the C ABI with host outputs"},
            "builders": len(groups), "ms_per_builder": gpu_s / len(groups) * 1e3, "checked_against_oracle": ok,
            "cpu_baseline": {"value": 8 * len(sample) / cpu_s, "unit": "chunks/s", "cores": 1, "kind": "port",
                             "sample": "%d builders (generate_occupancy_masks per chunk, one thread)" % len(sample)}}
    print(json.dumps(line))
