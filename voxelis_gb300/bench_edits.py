"""Uneven batched edits on GB300 (bench.py --workload edits).

1536 chunks in one VoxInterner<u16> (patches P1 + P2): 512 each of MaxDepth 7, 6 and 5 (128^3, 64^3,
32^3), built from the dune terrain rule scaled to each chunk side. Each chunk then gets one batch of
uniform-random edits at density 0.001, 0.01 or 0.1 of its voxels (chunk i takes density i mod 3); an
edit is a set (material uniform in 1..4095) with probability 0.85, else a clear (ignored without P4,
voxtree.rs:779). All 1536 batches go to the device as compacted touched groups and are applied by one
launch sequence (vx_apply_groups_async); the launch shape is picked by the autotuner first.

Reported beside it: the plain per-chunk GPU path (one call per chunk, same DAG checked), e2e through
vx_apply_batches with host Batch objects, and the CPU oracle on a sample of chunks.
"""
import ctypes as C
import json
import os
import statistics
import time

import numpy as np

from . import workloads as W
from ._abi import VX_PATCH_P1, VX_PATCH_P2, VX_PROF_N, VX_PROF_NAMES, gpu_lib
from .tune import autotune_apply

DEPTHS = (7, 6, 5)
PER_DEPTH = 512
DENSITIES = (0.001, 0.01, 0.1)
BUDGET = 8 << 30
PATCHES = VX_PATCH_P1 | VX_PATCH_P2


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


def run(args):
    import torch

    from .build import build as build_lib

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
    stream.synchronize()
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731

    def rebuild():
        call("interner_reset")
        off = 0
        for d in DEPTHS:
            call("build_dense_async", per_depth, C.c_void_p(t_d.data_ptr() + 4 * off), P(g_d[d]), None, d)
            off += per_depth
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

    if args.quick:
        tune = {"skipped": True}
    else:
        tune = autotune_apply(lib, h, rebuild, lambda: timed(apply_all))
    prof_ms = (C.c_double * VX_PROF_N)()
    prof_n = (C.c_uint64 * VX_PROF_N)()
    for _ in range(args.warmup):
        rebuild()
        apply_all()
        call("interner_sync")
    call("profile_enable", 1)
    call("profile_collect", prof_ms, prof_n)
    ms = []
    launches = 0
    phases = {}
    for _ in range(args.steps):
        call("profile_enable", 0)
        rebuild()
        call("profile_enable", 1)
        l0 = lib.kernel_launches()
        ms.append(timed(apply_all))
        launches += lib.kernel_launches() - l0
        call("interner_sync")
        call("profile_collect", prof_ms, prof_n)
        for k in range(VX_PROF_N):
            if prof_n[k]:
                phases[VX_PROF_NAMES[k]] = phases.get(VX_PROF_NAMES[k], 0.0) + prof_ms[k]
    launches = launches / args.steps
    call("profile_enable", 0)
    apply_ms = statistics.median(ms)
    from ._abi import vx_interner_stats

    st = vx_interner_stats()
    call("interner_stats_get", C.byref(st))
    import bench as B

    if args.quick:
        print(json.dumps({"quick": True, "ms_per_step": statistics.median(ms), "steps_ms": ms,
                          "phases_ms_per_step": {k: v / max(1, args.steps) for k, v in phases.items()},
                          "edits": n_edits, "records": R}))
        call("interner_destroy")
        return
    # canonical DAG of the batched result
    canon = B.export(lib, h, trees)
    nodes_after = st.alive_nodes

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
    canon_pc = B.export(lib, h, trees)
    same_dag = all(np.array_equal(canon[k], canon_pc[k]) for k in canon)

    # e2e: host Batch objects through vx_apply_batches (host staging, H2D, apply, D2H of flags)
    from .api import Batch

    batches = []
    for i, (xyz, vals) in enumerate(edits):
        b = Batch(int(depths[i]), 16, PATCHES, lib=lib)
        b.set_many(xyz, vals)
        batches.append(b)
    ptrs = (C.c_void_p * n)(*[b.handle.value for b in batches])
    changed_h = np.zeros(n, np.uint8)
    e2e = []
    for k in range(max(2, args.steps // 2)):
        rebuild()
        t1 = time.perf_counter()
        call("apply_batches", n, C.c_void_p(trees.ctypes.data), C.cast(ptrs, C.c_void_p), C.c_void_p(changed_h.ctypes.data))
        e2e.append(time.perf_counter() - t1)
    canon_e2e = B.export(lib, h, trees)
    same_dag = same_dag and all(np.array_equal(canon[k], canon_e2e[k]) for k in canon)
    e2e_ms = statistics.median(e2e) * 1e3
    call("interner_destroy")

    # CPU oracle on a sample: 2 chunks per depth, full Batch + apply_batch
    ol = B.oracle_lib()
    oh = C.c_void_p()
    ol.call("interner_create", C.c_uint64(1 << 30), 16, PATCHES, 0, C.byref(oh))
    sample = [k * per_depth + j for k in range(len(DEPTHS)) for j in (0, 2)]
    cpu_s, cpu_edits = 0.0, 0
    for i in sample:
        out = C.c_uint32()
        ol.call("tree_create", oh, int(depths[i]), C.byref(out))
        d = int(depths[i])
        g = np.ascontiguousarray(grids_np[d][i % per_depth])
        tr = np.array([out.value], np.uint32)
        ol.call("build_dense", oh, 1, C.c_void_p(tr.ctypes.data), C.c_void_p(g.ctypes.data), None, 0)
        b = Batch(d, 16, PATCHES, lib=ol)
        xyz, vals = edits[i]
        t1 = time.perf_counter()
        b.set_many(xyz, vals)
        ch = C.c_int()
        ol.call("apply_batch", oh, out.value, b.handle, C.byref(ch))
        cpu_s += time.perf_counter() - t1
        cpu_edits += len(vals)
    ol.status("interner_destroy", oh)

    algo = R * 22 + max(0, nodes_after - 1) * 80
    bottom_ms = phases.get("apply_bottom", 0.0) / max(1, args.steps)
    peak, peak_kind = B.peaks()
    line = {
        "metric": "edits/s", "value": n_edits / (apply_ms * 1e-3), "unit": "edits/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": apply_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u16", "data": "synthetic",
        "config": {"workload": "uneven batched edits: 1536 chunks u16 (512 each MaxDepth 7/6/5), one batch per chunk "
                               "at density 0.001/0.01/0.1, 85% set / 15% clear, P1+P2",
                   "edits": n_edits, "touched_groups": R, "chunks": n, "budget_bytes": budget,
                   "l2": "inputs and records larger than L2 (records %.0f MB)" % (R * 26 / 1e6)},
        "chunks_per_s": n / (apply_ms * 1e-3),
        "autotune": tune,
        "per_chunk_gpu": {"value": n_edits / (pc_ms * 1e-3), "unit": "edits/s", "ms": pc_ms, "same_dag": same_dag},
        "batched_over_per_chunk": pc_ms / apply_ms,
        "phases_ms_per_step": {k: v / max(1, args.steps) for k, v in phases.items()},
        "roofline": {"bound": "hbm", "achieved": algo / (apply_ms * 1e-3) / 1e9, "peak": peak, "unit": "GB/s",
                     "frac": algo / (apply_ms * 1e-3) / 1e9 / peak, "traffic": None,
                     "kernel": "whole apply sequence", "algorithmic_bytes": int(algo), "peak_kind": peak_kind,
                     "bottom_kernel_ms": bottom_ms},
        "e2e": {"value": n_edits / (e2e_ms * 1e-3), "unit": "edits/s", "ms": e2e_ms,
                "h2d_bytes_per_step": int(R * 26 + n * 16), "d2h_bytes_per_step": int(n)},
        "cpu_baseline": {"value": cpu_edits / cpu_s, "unit": "edits/s", "cores": 1, "kind": "port",
                         "sample": "%d chunks (2 per depth): Batch filled by just_set, then apply_batch" % len(sample)},
        "nodes_after": int(nodes_after), "gpu_launches": int(launches), "generation_s": gen_s,
    }
    print(json.dumps(line))
