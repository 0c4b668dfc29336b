"""Uneven batched edits on GB300 (bench.py --workload edits; also part of the default bench.py line).

1536 chunks in one VoxInterner<u16> (patches P1 + P2): 512 each of MaxDepth 7, 6 and 5 (128^3, 64^3,
32^3), built from the dune terrain rule scaled to each chunk side. Each chunk then gets one batch of
uniform-random edits at density 0.001, 0.01 or 0.1 of its voxels (chunk i takes density i mod 3); an
edit is a set (material uniform in 1..4095) with probability 0.85, else a clear (ignored without P4,
voxtree.rs:779). All 1536 batches go to the device as compacted touched groups and are applied by one
launch sequence (vx_apply_groups_async); the launch shape is picked by the autotuner first.

Reported beside it: the plain per-chunk GPU path (one call per chunk, same DAG checked), e2e through
vx_apply_batches with host Batch objects, and the CPU oracle over the whole workload: its terrain
build and its 1536 Batches (just_set, then apply_batch in order) give the reference DAG that the GPU
result is compared with (canonical export, live nodes, per-depth counts), and its apply time is the
CPU baseline.
"""
import ctypes as C
import statistics
import time

import numpy as np

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_PATCH_P1, VX_PATCH_P2, VX_PROF_N, VX_PROF_NAMES, gpu_lib, vx_interner_stats
from voxelis_gb300.api import Batch, export_canonical, same_dag
from voxelis_gb300.tune import autotune_apply

DEPTHS = (7, 6, 5)
PER_DEPTH = 512
DENSITIES = (0.001, 0.01, 0.1)
BUDGET = 8 << 30
PATCHES = VX_PATCH_P1 | VX_PATCH_P2
WORKLOAD = ("uneven batched edits: 1536 chunks u16 (512 each MaxDepth 7/6/5, dune terrain), one batch per chunk "
            "at density 0.001/0.01/0.1, 85% set / 15% clear, P1+P2")


def make_world(per_depth=PER_DEPTH):
    """Dense u16 grids per depth ([per_depth][s][s][s]) and the items' edit records (deepest first)."""
    nz = max(1, per_depth // 32)
    grids = {d: W.dune_world_chunks(per_depth // nz, nz, depth=d, seed=1234 + d, dtype=np.uint16,
                                    **W.terrain_params(d)) for d in DEPTHS}
    recs, edits = [], []
    i = 0
    for d in DEPTHS:
        for _ in range(per_depth):
            xyz, vals = W.random_edits(d, DENSITIES[i % 3], 7000 + i, max_material=4095)
            g, sm, cm, vv = W.edits_to_groups(d, xyz, vals)
            recs.append((np.full(len(g), i, np.uint32), g, sm, cm, vv))
            edits.append((xyz, vals))
            i += 1
    return grids, recs, edits


def oracle_leg(grids_np, edits, per_depth, budget):
    """The oracle over the whole workload: terrain built per chunk (Batch from the dense grid, then
    apply_batch), then every chunk's edit Batch filled by just_set and applied in chunk order.
    Returns (canonical export, live nodes, fill seconds, apply seconds)."""
    import bench as B

    ol = B.oracle_lib()
    oh = C.c_void_p()
    ol.call("interner_create", C.c_uint64(budget), 16, PATCHES, 0, C.byref(oh))
    n = len(edits)
    trees = np.zeros(n, np.uint32)
    for i in range(n):
        out = C.c_uint32()
        ol.call("tree_create", oh, DEPTHS[i // per_depth], C.byref(out), handle=oh)
        trees[i] = out.value
    for k, d in enumerate(DEPTHS):
        tr = np.ascontiguousarray(trees[k * per_depth:(k + 1) * per_depth])
        ol.call("build_dense", oh, per_depth, C.c_void_p(tr.ctypes.data), C.c_void_p(grids_np[d].ctypes.data), None, 0,
                handle=oh)
    t0 = time.perf_counter()
    batches = []
    for i, (xyz, vals) in enumerate(edits):
        b = Batch(DEPTHS[i // per_depth], 16, PATCHES, lib=ol)
        b.set_many(xyz, vals)
        batches.append(b)
    t1 = time.perf_counter()
    ptrs = (C.c_void_p * n)(*[b.handle.value for b in batches])
    changed = np.zeros(n, np.uint8)
    ol.call("apply_batches", oh, n, C.c_void_p(trees.ctypes.data), C.cast(ptrs, C.c_void_p),
            C.c_void_p(changed.ctypes.data), handle=oh)
    t2 = time.perf_counter()
    for b in batches:
        b.close()
    canon = export_canonical(ol, oh, trees)
    st = vx_interner_stats()
    ol.call("interner_stats_get", oh, C.byref(st), handle=oh)
    ol.status("interner_destroy", oh)
    return canon, int(st.alive_nodes), t1 - t0, t2 - t1


def measure(args, full_line=False):
    import torch

    import bench as B
    from voxelis_gb300.build import build as build_lib

    build_lib()
    lib = gpu_lib()
    dev = torch.device("cuda", 0)
    t0 = time.time()
    per_depth = getattr(args, "edits_chunks", PER_DEPTH)
    grids_np, recs, edits = make_world(per_depth)
    gen_s = time.time() - t0
    n = len(recs)
    n_edits = int(sum(len(v) for _, v in edits))
    item, group, sm, cm, vv = (np.concatenate([r[j] for r in recs]) for j in range(5))
    R = len(item)

    h = C.c_void_p()
    budget = max(512 << 20, BUDGET * per_depth // PER_DEPTH)
    lib.call("interner_create", C.c_uint64(budget), 16, PATCHES, 0, C.byref(h))
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731
    stream = torch.cuda.Stream(device=dev)
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    depths = np.concatenate([np.full(per_depth, d, np.uint8) for d in DEPTHS])
    trees = np.zeros(n, np.uint32)
    call("trees_create", n, depths.ctypes.data, trees.ctypes.data)

    def to_dev(a):
        a = np.ascontiguousarray(a)
        view = {1: np.uint8, 2: np.int16, 4: np.int32}[a.dtype.itemsize]
        return torch.from_numpy(a.view(view)).to(dev)

    with torch.cuda.stream(stream):
        g_d = {d: to_dev(grids_np[d]) for d in DEPTHS}
        t_d = to_dev(trees)
        rec = dict(item=to_dev(item), group=to_dev(group), set=to_dev(sm), clear=to_dev(cm), vals=to_dev(vv.reshape(-1)),
                   flags=to_dev(np.full(n, 2, np.uint8)), fill=to_dev(np.zeros(n, np.uint32)),
                   changed=torch.zeros(n, dtype=torch.uint8, device=dev))
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream.synchronize()
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731

    def rebuild():
        call("interner_reset")
        off = 0
        for d in DEPTHS:
            call("build_dense_async", per_depth, C.c_void_p(t_d.data_ptr() + 4 * off), P(g_d[d]), None, d)
            off += per_depth
        with torch.cuda.stream(stream):
            flush.fill_(3)  # L2 holds none of the interner when the apply starts
        call("interner_sync")

    def apply_all():
        call("apply_groups_async", n, P(t_d), P(rec["flags"]), P(rec["fill"]), R, P(rec["item"]), P(rec["group"]),
             P(rec["set"]), P(rec["clear"]), P(rec["vals"]), P(rec["changed"]), max(DEPTHS))

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    launch = getattr(args, "launch", None)
    if launch is not None:  # a fixed launch form instead of the autotuner's choice
        call("tune_set_launch", int(launch))
        tune = {"fixed_single_launch": int(launch)}
    elif args.quick:
        tune = {"skipped": True}
    else:
        tune = autotune_apply(lib, h, rebuild, lambda: timed(apply_all), signature="edits%d" % per_depth)
    prof_ms = (C.c_double * VX_PROF_N)()
    prof_n = (C.c_uint64 * VX_PROF_N)()
    for _ in range(args.warmup):
        rebuild()
        apply_all()
        call("interner_sync")
    steps = max(3, args.steps)
    ms, launches, phases = [], 0, {}
    st = vx_interner_stats()
    clocks = B.Clocks(0)
    for _ in range(steps):
        rebuild()
        call("interner_stats_get", C.byref(st))
        created_before = int(st.nodes_created)
        l0 = lib.kernel_launches()
        ms.append(timed(apply_all))
        launches += lib.kernel_launches() - l0
        call("interner_sync")
    clk = clocks.stop()
    # the phase split from the same applies run again with the library's per-phase events (kept out
    # of the timed steps above: an event between two kernels holds the second one back)
    n_prof = max(1, min(steps, 5))
    for _ in range(n_prof):
        rebuild()
        call("interner_stats_get", C.byref(st))
        created_before = int(st.nodes_created)
        call("profile_enable", 1)
        call("profile_collect", prof_ms, prof_n)
        apply_all()
        call("interner_sync")
        call("profile_collect", prof_ms, prof_n)
        call("profile_enable", 0)
        for k in range(VX_PROF_N):
            if prof_n[k]:
                phases[VX_PROF_NAMES[k]] = phases.get(VX_PROF_NAMES[k], 0.0) + prof_ms[k] * steps / n_prof
    launches = launches / steps
    apply_ms = statistics.median(ms)
    call("interner_stats_get", C.byref(st))
    nodes_after = int(st.alive_nodes)
    created = int(st.nodes_created) - created_before  # nodes the apply created (interner misses)
    phases_ms = {k: v / steps for k, v in phases.items()}
    if args.quick:
        call("interner_destroy")
        return {"quick": True, "ms_per_step": apply_ms, "steps_ms": ms, "phases_ms_per_step": phases_ms,
                "edits": n_edits, "records": R, "gpu_launches": launches}

    canon = export_canonical(lib, h, trees)

    # plain per-chunk GPU path on the same inputs
    rebuild()
    starts = np.searchsorted(item, np.arange(n + 1))
    zero_items = to_dev(np.zeros(max(1, int(np.max(np.diff(starts)))), np.uint32))

    def per_chunk():
        for i in range(n):
            a, b = int(starts[i]), int(starts[i + 1])
            call("apply_groups_async", 1, C.c_void_p(t_d.data_ptr() + 4 * i), P(rec["flags"]), P(rec["fill"]), b - a,
                 P(zero_items), C.c_void_p(rec["group"].data_ptr() + 4 * a), C.c_void_p(rec["set"].data_ptr() + a),
                 C.c_void_p(rec["clear"].data_ptr() + a), C.c_void_p(rec["vals"].data_ptr() + 16 * a), None,
                 int(depths[i]))

    pc_ms = timed(per_chunk)
    call("interner_sync")
    pc_same = same_dag(canon, export_canonical(lib, h, trees))

    # e2e: host Batch objects through vx_apply_batches (host staging, H2D, apply, D2H of flags)
    batches = []
    for i, (xyz, vals) in enumerate(edits):
        b = Batch(int(depths[i]), 16, PATCHES, lib=lib)
        b.set_many(xyz, vals)
        batches.append(b)
    ptrs = (C.c_void_p * n)(*[b.handle.value for b in batches])
    changed_h = np.zeros(n, np.uint8)
    e2e = []
    for _ in range(max(3, args.steps // 4)):
        rebuild()
        t1 = time.perf_counter()
        call("apply_batches", n, C.c_void_p(trees.ctypes.data), C.cast(ptrs, C.c_void_p), C.c_void_p(changed_h.ctypes.data))
        e2e.append(time.perf_counter() - t1)
    e2e_same = same_dag(canon, export_canonical(lib, h, trees))
    for b in batches:
        b.close()
    e2e_ms = statistics.median(e2e) * 1e3
    call("interner_destroy")
    del g_d, rec, flush
    torch.cuda.empty_cache()

    # the oracle over the whole workload: reference DAG and CPU baseline
    ocanon, oalive, fill_s, apply_s = oracle_leg(grids_np, edits, per_depth, budget)
    parity = B.parity_report(canon, nodes_after, ocanon, oalive)
    del ocanon

    # algorithmic bytes: the compacted records (set + clear masks, 8 u16 values, item index), the nodes
    # the apply created (node_size 80 B for u16) and one root id per chunk
    algo = R * (2 + 8 * 2 + 4) + created * 80 + n * 8
    peak, peak_kind = B.peaks()
    achieved = algo / (apply_ms * 1e-3) / 1e9
    out = {
        "metric": "edits/s", "value": n_edits / (apply_ms * 1e-3), "unit": "edits/s", "ms_per_step": apply_ms,
        "steps": steps, "warmup": args.warmup, "higher_is_better": True, "dtype": "u16", "data": "synthetic",
        "config": {"workload": WORKLOAD, "edits": n_edits, "touched_groups": R, "chunks": n, "budget_bytes": budget,
                   "l2": "flushed before every timed apply (256 MiB write); records %.0f MB" % (R * 26 / 1e6)},
        "chunks_per_s": n / (apply_ms * 1e-3),
        "autotune": tune,
        "per_chunk_gpu": {"value": n_edits / (pc_ms * 1e-3), "unit": "edits/s", "ms": pc_ms, "same_dag": pc_same},
        "batched_over_per_chunk": pc_ms / apply_ms,
        "phases_ms_per_step": phases_ms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": B.profiled_traffic("apply_edits_uneven192.md"),
                     "kernel": "whole apply sequence (bottom groups, level passes, refcount epoch, release)",
                     "algorithmic_bytes": int(algo), "peak_kind": peak_kind},
        "e2e": {"value": n_edits / (e2e_ms * 1e-3), "unit": "edits/s", "ms": e2e_ms,
                "h2d_bytes_per_step": int(R * 26 + n * 16), "d2h_bytes_per_step": int(n), "same_dag": e2e_same},
        "cpu_baseline": {"value": n_edits / apply_s, "unit": "edits/s", "cores": 1, "kind": "port",
                         "sample": "the whole workload once, one thread: %.2f s of apply_batch over the 1536 Batches "
                                   "(their just_set fill took %.2f s more)" % (apply_s, fill_s)},
        "parity": parity,
        "nodes_after": nodes_after, "nodes_created": created, "gpu_launches": launches, "generation_s": gen_s,
        "clocks": clk,
    }
    if full_line:
        out.update({"n_gpus": 1, "scaling": "weak", "vs_baseline": None})
    return out
