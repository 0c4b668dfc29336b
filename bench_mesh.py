"""Occupancy masks for greedy meshing (bench.py --workload mesh).

The 4096 perlin-dune chunks of 32^3 u8 of the default workload, built once into a device-resident
interner, packed 4 to a 64^3 builder (2 x 2 chunks in x and z at offsets 0/32: the tiling is one
chunk high; the reference packs up to 8 chunks of 32^3, utils/mesh.rs:1195-1225), 1024 builders:

  value        vx_occupancy_masks_async over all 1024 builders, outputs resident in HBM (CUDA events)
  e2e          the same call plus the device-to-host copy of every output into pinned memory
  per_builder  one vx_occupancy_masks call per builder through the C ABI (host outputs)
  cpu_baseline the oracle's restatement of generate_occupancy_masks, one thread, on a sample

Every builder of the batched result is compared with the per-builder call, and a sample of builders
with the oracle. Also timed on the same world: vx_serialize_model of all 4096 chunks (the
VoxModel::serialize payload, host output) against the oracle's restatement of it.
"""
import ctypes as C
import json
import statistics
import time

import numpy as np

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import gpu_lib

N_SIDE = 64
MAX_MAT = 8


def run(args):
    import torch

    from voxelis_gb300.build import build as build_lib

    build_lib()
    lib = gpu_lib()
    dev = torch.device("cuda", 0)
    grids = W.dune_world_chunks(N_SIDE, N_SIDE, depth=5, seed=1234)
    n = grids.shape[0]
    h = C.c_void_p()
    lib.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(h))
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731
    stream = torch.cuda.Stream(device=dev)
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    trees = np.zeros(n, np.uint32)
    depths = np.full(n, 5, np.uint8)  # named: ctypes.data of a temporary would dangle
    call("trees_create", n, depths.ctypes.data, trees.ctypes.data)
    # builder (bi, bk) takes chunks (2bi + di, 2bk + dk) at (32 di, 0, 32 dk)
    nb = (N_SIDE // 2) ** 2
    order, builder_of, offs = [], [], []
    for bk in range(N_SIDE // 2):
        for bi in range(N_SIDE // 2):
            for dk in range(2):
                for di in range(2):
                    order.append((2 * bk + dk) * N_SIDE + (2 * bi + di))
                    builder_of.append(bk * (N_SIDE // 2) + bi)
                    offs.append((32 * di, 0, 32 * dk))
    order = np.array(order)
    tr = np.ascontiguousarray(trees[order])
    builder_of = np.array(builder_of, np.uint32)
    offs = np.array(offs, np.uint32)
    with torch.cuda.stream(stream):
        t_all = torch.from_numpy(trees.view(np.int32)).to(dev)
        g_d = torch.from_numpy(grids).to(dev)
        t_d = torch.from_numpy(tr.view(np.int32)).to(dev)
        b_d = torch.from_numpy(builder_of.view(np.int32)).to(dev)
        o_d = torch.from_numpy(offs.ravel().view(np.int32)).to(dev)
        plane = 3 * 4096
        glob = torch.zeros(nb * plane, dtype=torch.int64, device=dev)
        act = torch.zeros(nb * 6, dtype=torch.int64, device=dev)
        nm = torch.zeros(nb, dtype=torch.int32, device=dev)
        ids = torch.zeros(nb * MAX_MAT, dtype=torch.int32, device=dev)
        cnt = torch.zeros(nb * MAX_MAT, dtype=torch.int64, device=dev)
        masks = torch.zeros(nb * MAX_MAT * plane, dtype=torch.int64, device=dev)
    stream.synchronize()
    call("build_dense_async", n, C.c_void_p(t_all.data_ptr()), C.c_void_p(g_d.data_ptr()), None, 5)
    call("interner_sync")
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731
    args_async = (nb, len(tr), P(t_d), P(b_d), P(o_d), 5, MAX_MAT, P(glob), P(act), P(nm), P(ids), P(cnt), P(masks))
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    for _ in range(3):
        call("occupancy_masks_async", *args_async)
    call("interner_sync")
    steps = max(5, args.steps // 50)
    ms = []
    launches = 0
    for k in range(steps):
        with torch.cuda.stream(stream):
            flush.fill_(k)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        l0 = lib.kernel_launches()
        call("occupancy_masks_async", *args_async)
        launches += lib.kernel_launches() - l0
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    call("interner_sync")
    dev_ms = statistics.median(ms)
    out_bytes = (glob.numel() + act.numel() + cnt.numel() + masks.numel()) * 8 + (nm.numel() + ids.numel()) * 4
    # e2e: the same call + D2H of every output into pinned memory
    hosts = [torch.empty(x.shape, dtype=x.dtype, pin_memory=True) for x in (glob, act, nm, ids, cnt, masks)]
    e2e = []
    for _ in range(steps):
        stream.synchronize()
        t0 = time.perf_counter()
        call("occupancy_masks_async", *args_async)
        with torch.cuda.stream(stream):
            for hbuf, dbuf in zip(hosts, (glob, act, nm, ids, cnt, masks)):
                hbuf.copy_(dbuf, non_blocking=True)
        stream.synchronize()
        e2e.append(time.perf_counter() - t0)
    e2e_ms = statistics.median(e2e) * 1e3
    g_h = hosts[0].numpy().view(np.uint64).reshape(nb, plane)
    a_h = hosts[1].numpy().view(np.uint64).reshape(nb, 6)
    n_h = hosts[2].numpy()
    i_h = hosts[3].numpy().reshape(nb, MAX_MAT)
    c_h = hosts[4].numpy().reshape(nb, MAX_MAT)
    m_h = hosts[5].numpy().view(np.uint64).reshape(nb, MAX_MAT, plane)
    # per-builder path, and its agreement with the batched result
    glob1 = np.zeros(plane, np.uint64)
    act1 = np.zeros(6, np.uint64)
    nm1 = C.c_uint32()
    ids1 = np.zeros(MAX_MAT, np.uint32)
    cnt1 = np.zeros(MAX_MAT, np.uint64)
    masks1 = np.zeros(MAX_MAT * plane, np.uint64)

    def one(b):
        sel = slice(4 * b, 4 * b + 4)
        tb, ob = np.ascontiguousarray(tr[sel]), np.ascontiguousarray(offs[sel])
        call("occupancy_masks", 4, C.c_void_p(tb.ctypes.data), C.c_void_p(ob.ctypes.data), C.c_void_p(glob1.ctypes.data),
             C.c_void_p(act1.ctypes.data), MAX_MAT, C.byref(nm1), C.c_void_p(ids1.ctypes.data),
             C.c_void_p(cnt1.ctypes.data), C.c_void_p(masks1.ctypes.data))
        return tb, ob

    same = True
    t0 = time.perf_counter()
    for b in range(nb):
        one(b)
        k = nm1.value
        same = same and n_h[b] == k and np.array_equal(g_h[b], glob1) and np.array_equal(a_h[b], act1) and \
            np.array_equal(i_h[b, :k], ids1[:k]) and np.array_equal(c_h[b, :k], cnt1[:k]) and \
            np.array_equal(m_h[b, :k].ravel(), masks1[:k * plane])
    per_builder_s = time.perf_counter() - t0
    # oracle on a sample of builders
    import bench as B

    ol = B.oracle_lib()
    oh = C.c_void_p()
    ol.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(oh))
    sample = list(range(0, nb, max(1, nb // 32)))[:32]
    cpu_s = 0.0
    ok = True
    o_glob = np.zeros_like(glob1)
    o_act = np.zeros_like(act1)
    o_nm = C.c_uint32()
    o_ids = np.zeros_like(ids1)
    o_cnt = np.zeros_like(cnt1)
    o_mask = np.zeros_like(masks1)
    for b in sample:
        o_trees = np.zeros(4, np.uint32)
        for k in range(4):
            out = C.c_uint32()
            ol.call("tree_create", oh, 5, C.byref(out))
            o_trees[k] = out.value
            g = np.ascontiguousarray(grids[order[4 * b + k]])
            ol.call("build_dense", oh, 1, C.c_void_p(o_trees[k:k + 1].ctypes.data), C.c_void_p(g.ctypes.data), None, 0)
        ob = np.ascontiguousarray(offs[4 * b:4 * b + 4])
        t1 = time.perf_counter()
        ol.call("occupancy_masks", oh, 4, C.c_void_p(o_trees.ctypes.data), C.c_void_p(ob.ctypes.data),
                C.c_void_p(o_glob.ctypes.data), C.c_void_p(o_act.ctypes.data), MAX_MAT, C.byref(o_nm),
                C.c_void_p(o_ids.ctypes.data), C.c_void_p(o_cnt.ctypes.data), C.c_void_p(o_mask.ctypes.data))
        cpu_s += time.perf_counter() - t1
        k = o_nm.value
        ok = ok and n_h[b] == k and np.array_equal(g_h[b], o_glob) and np.array_equal(a_h[b], o_act) and \
            np.array_equal(i_h[b, :k], o_ids[:k]) and np.array_equal(c_h[b, :k], o_cnt[:k]) and \
            np.array_equal(m_h[b, :k].ravel(), o_mask[:k * plane])
    ol.status("interner_destroy", oh)

    # model serialisation of the whole world (VoxModel::serialize payload), GPU vs oracle
    pos = np.array([(c % N_SIDE, 0, c // N_SIDE) for c in range(n)], np.int32)
    size = C.c_uint64()
    call("serialize_model", n, C.c_void_p(trees.ctypes.data), C.c_void_p(pos.ctypes.data), None, C.c_uint64(0),
         C.byref(size))
    blob = np.zeros(size.value, np.uint8)
    ser = []
    for _ in range(5):
        t0 = time.perf_counter()
        call("serialize_model", n, C.c_void_p(trees.ctypes.data), C.c_void_p(pos.ctypes.data),
             C.c_void_p(blob.ctypes.data), C.c_uint64(size.value), C.byref(size))
        ser.append(time.perf_counter() - t0)
    ser_ms = statistics.median(ser) * 1e3
    oh = C.c_void_p()
    ol.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(oh))
    o_trees = np.zeros(n, np.uint32)
    for c in range(n):
        out = C.c_uint32()
        ol.call("tree_create", oh, 5, C.byref(out))
        o_trees[c] = out.value
    ol.call("build_dense", oh, n, C.c_void_p(o_trees.ctypes.data), C.c_void_p(grids.ctypes.data), None, 0)
    o_size = C.c_uint64()
    ol.call("serialize_model", oh, n, C.c_void_p(o_trees.ctypes.data), C.c_void_p(pos.ctypes.data), None, C.c_uint64(0),
            C.byref(o_size))
    o_blob = np.zeros(o_size.value, np.uint8)
    t0 = time.perf_counter()
    ol.call("serialize_model", oh, n, C.c_void_p(o_trees.ctypes.data), C.c_void_p(pos.ctypes.data),
            C.c_void_p(o_blob.ctypes.data), C.c_uint64(o_size.value), C.byref(o_size))
    o_ms = (time.perf_counter() - t0) * 1e3
    ol.status("interner_destroy", oh)
    call("interner_destroy")
    from voxelis_gb300.api import export_canonical
    from voxelis_gb300.vtm import canonical, decode

    # model deserialisation of the same payload into a fresh interner (VoxModel::deserialize), GPU vs
    # oracle: per call the host bytes go to the device, are parsed there and the nodes placed
    h2 = C.c_void_p()
    lib.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(h2))
    d_trees = np.zeros(n, np.uint32)
    d_pos = np.zeros((n, 3), np.int32)
    d_n = C.c_uint32()
    des = []
    for _ in range(5):
        lib.call("interner_reset", h2, handle=h2)
        t0 = time.perf_counter()
        lib.call("deserialize_model", h2, C.c_void_p(blob.ctypes.data), C.c_uint64(size.value), 5, n,
                 C.c_void_p(d_trees.ctypes.data), C.c_void_p(d_pos.ctypes.data), C.byref(d_n), handle=h2)
        des.append(time.perf_counter() - t0)
        if _ < 4:
            for t in d_trees:
                lib.call("tree_destroy", h2, int(t), handle=h2)
    des_ms = statistics.median(des) * 1e3
    oh = C.c_void_p()
    ol.call("interner_create", C.c_uint64(256 << 20), 8, 0, 0, C.byref(oh))
    o_dt = np.zeros(n, np.uint32)
    o_dp = np.zeros((n, 3), np.int32)
    t0 = time.perf_counter()
    ol.call("deserialize_model", oh, C.c_void_p(blob.ctypes.data), C.c_uint64(size.value), 5, n,
            C.c_void_p(o_dt.ctypes.data), C.c_void_p(o_dp.ctypes.data), C.byref(d_n), handle=oh)
    o_des_ms = (time.perf_counter() - t0) * 1e3
    cg, co = export_canonical(lib, h2, d_trees), export_canonical(ol, oh, o_dt)
    des_equal = bool(np.array_equal(d_pos, o_dp) and all(np.array_equal(cg[k], co[k]) for k in co))
    re = np.zeros(size.value, np.uint8)
    lib.call("serialize_model", h2, n, C.c_void_p(d_trees.ctypes.data), C.c_void_p(d_pos.ctypes.data),
             C.c_void_p(re.ctypes.data), C.c_uint64(size.value), C.byref(size), handle=h2)
    ol.status("interner_destroy", oh)
    lib.status("interner_destroy", h2)
    deserialize = {"bytes": int(size.value), "ms": des_ms, "MB_per_s": size.value / (des_ms * 1e-3) / 1e6,
                   "oracle_equal": des_equal, "round_trip_bytes_equal": bool(np.array_equal(re, blob)),
                   "cpu_baseline": {"ms": o_des_ms, "cores": 1, "kind": "port", "sample": "the same payload"}}

    same_model = canonical(*decode(blob.tobytes(), 1)) == canonical(*decode(o_blob.tobytes(), 1))
    serialize = {"bytes": int(size.value), "ms": ser_ms, "MB_per_s": size.value / (ser_ms * 1e-3) / 1e6,
                 "same_model_as_oracle": bool(same_model),
                 "cpu_baseline": {"ms": o_ms, "cores": 1, "kind": "port", "sample": "the same 4096-chunk world"}}
    line = {"metric": "chunks/s (occupancy masks, 4 chunks of 32^3 per 64^3 builder)",
            "value": n / (dev_ms * 1e-3), "unit": "chunks/s", "higher_is_better": True, "dtype": "u8",
            "config": {"workload": "occupancy masks of the 4096 dune chunks, 1024 builders, one batched call",
                       "l2": "flushed between steps (256 MiB write)"},
            "ms_per_step": dev_ms, "output_bytes": int(out_bytes), "gpu_launches": launches / steps,
            "e2e": {"value": n / (e2e_ms * 1e-3), "unit": "chunks/s", "ms": e2e_ms, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(out_bytes)},
            "per_builder_gpu": {"value": n / per_builder_s, "unit": "chunks/s", "same_as_batched": bool(same)},
            "checked_against_oracle": bool(ok), "serialize_model": serialize, "deserialize_model": deserialize,
            "cpu_baseline": {"value": 4 * len(sample) / cpu_s, "unit": "chunks/s", "cores": 1, "kind": "port",
                             "sample": "%d builders (generate_occupancy_masks per chunk, one thread)" % len(sample)}}
    print(json.dumps(line))
