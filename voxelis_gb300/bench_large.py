"""Large single tree on GB300 (bench.py --workload large).

One VoxTree of MaxDepth 10 (1024^3 u8, patches P1 + P2 + P3 + P4) built from a dense 1 GiB grid of
caves (voxel = 1 + floor(3|N|) where N(x/64, y/64, z/64) > 0.1, else 0; N = 3D gradient noise with a
seed-shuffled permutation), then 16M uniform-random get() queries, then 8 successive batches of 1M
random edits (materials 1..4, 80% set / 20% clear; clears honoured, P4). After each batch the interner's
node counts and the UB fence (every reachable child live, refcount > 0) are checked; with --check the
canonical DAG (nodes, refcounts, links) is compared with the CPU oracle after the build and after each
batch (slow: minutes of CPU).
"""
import ctypes as C
import json
import statistics
import time

import numpy as np

from . import workloads as W
from ._abi import VX_PATCH_P1, VX_PATCH_P2, VX_PATCH_P3, VX_PATCH_P4, VX_PROF_N, VX_PROF_NAMES, gpu_lib

DEPTH = 10
PATCHES = VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P3 | VX_PATCH_P4
BUDGET = 16 << 30
N_GETS = 1 << 24
N_BATCHES = 8
EDITS_PER_BATCH = 1 << 20


def run(args, check=False):
    import torch

    from .build import build as build_lib

    build_lib()
    lib = gpu_lib()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.Stream(device=dev)
    t0 = time.time()
    with torch.cuda.stream(stream):
        grid = W.caves_torch(DEPTH, seed=99, device=dev)
    stream.synchronize()
    gen_s = time.time() - t0
    h = C.c_void_p()
    lib.call("interner_create", C.c_uint64(BUDGET), 8, PATCHES, 0, C.byref(h))
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    tree = np.zeros(1, np.uint32)
    d = np.array([DEPTH], np.uint8)
    call("trees_create", 1, d.ctypes.data, tree.ctypes.data)
    with torch.cuda.stream(stream):
        t_d = torch.from_numpy(tree.view(np.int32)).to(dev)
    P = lambda x: C.c_void_p(x.data_ptr())  # noqa: E731

    def timed(fn):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    prof_ms = (C.c_double * VX_PROF_N)()
    prof_n = (C.c_uint64 * VX_PROF_N)()
    build_ms = []
    for k in range(1 + max(1, args.warmup)):
        call("interner_reset")
        call("profile_enable", 1)
        call("profile_collect", prof_ms, prof_n)
        build_ms.append(timed(lambda: call("build_dense_async", 1, P(t_d), P(grid), None, DEPTH)))
        call("interner_sync")
        call("profile_collect", prof_ms, prof_n)
        call("profile_enable", 0)
    build_phases = {VX_PROF_NAMES[k]: prof_ms[k] for k in range(VX_PROF_N) if prof_n[k]}
    from ._abi import vx_interner_stats

    st = vx_interner_stats()
    call("interner_stats_get", C.byref(st))
    nodes_built = int(st.alive_nodes)

    report = {"metric": "voxels/s (dense build, MaxDepth 10)", "unit": "voxels/s", "higher_is_better": True,
              "config": {"workload": "large tree: MaxDepth 10 (1024^3 u8) caves grid, 16M gets, 8 x 1M edits "
                                     "(80/20 set/clear, P1+P2+P3+P4)"},
              "grid_generation_s": gen_s, "build_ms": build_ms[-1], "value": (1 << 30) / (build_ms[-1] * 1e-3),
              "build_phases_ms": build_phases, "nodes_after_build": nodes_built}

    oracle = None
    if check:
        import bench as B

        ol = B.oracle_lib()
        oh = C.c_void_p()
        ol.call("interner_create", C.c_uint64(BUDGET), 8, PATCHES, 0, C.byref(oh))
        ot = C.c_uint32()
        ol.call("tree_create", oh, DEPTH, C.byref(ot))
        g_host = grid.cpu().numpy()
        otr = np.array([ot.value], np.uint32)
        t1 = time.time()
        ol.call("build_dense", oh, 1, C.c_void_p(otr.ctypes.data), C.c_void_p(g_host.ctypes.data), None, 0)
        report["oracle_build_s"] = time.time() - t1
        oracle = (ol, oh, ot.value)
        report["check_build"] = compare(lib, h, tree, oracle)

    # 16M uniform-random gets
    rng = np.random.default_rng(17)
    xyz = rng.integers(0, 1 << DEPTH, (N_GETS, 3)).astype(np.int32)
    with torch.cuda.stream(stream):
        q_d = torch.from_numpy(xyz).to(dev)
        qt_d = torch.zeros(N_GETS, dtype=torch.int32, device=dev) + int(tree[0])
        f_d = torch.empty(N_GETS, dtype=torch.uint8, device=dev)
        v_d = torch.empty(N_GETS, dtype=torch.uint8, device=dev)
    get_ms = []
    for _ in range(5):
        get_ms.append(timed(lambda: call("get_many_async", C.c_uint64(N_GETS), P(qt_d), P(q_d), P(f_d), P(v_d))))
    call("interner_sync")
    g_host = grid.cpu().numpy() if oracle is None else g_host
    sample = slice(0, 1 << 16)
    want = g_host[xyz[sample, 1], xyz[sample, 2], xyz[sample, 0]]
    report["gets"] = {"value": N_GETS / (statistics.median(get_ms) * 1e-3), "unit": "gets/s",
                      "ms": statistics.median(get_ms),
                      "checked": bool(np.array_equal(v_d[sample].cpu().numpy(), want))}

    # 8 batches of 1M random set/clear edits (P4)
    batches = []
    for b in range(N_BATCHES):
        exyz, vals = W.random_edits(DEPTH, 0, 1000 + b, max_material=4, clear_fraction=0.2, count=EDITS_PER_BATCH)
        g, sm, cm, vv = W.edits_to_groups(DEPTH, exyz, vals)
        batches.append((exyz, vals, g, sm, cm, vv))
    one = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    flags, fill, item0 = one(np.array([2], np.uint8)), one(np.zeros(1, np.int32)), None
    edit_ms, checks = [], []
    for b, (exyz, vals, g, sm, cm, vv) in enumerate(batches):
        R = len(g)
        with torch.cuda.stream(stream):
            ri = torch.zeros(R, dtype=torch.int32, device=dev)
            rg, rs, rc = one(g.view(np.int32)), one(sm), one(cm)
            rv = one(vv.reshape(-1).view(np.int16))
        stream.synchronize()
        edit_ms.append(timed(lambda: call("apply_groups_async", 1, P(t_d), P(flags), P(fill), R, P(ri), P(rg), P(rs),
                                          P(rc), P(rv), None, DEPTH)))
        call("interner_maintain")
        call("validate", 1, C.c_void_p(tree.ctypes.data))
        if oracle is not None:
            ol, oh, ot = oracle
            from .api import Batch

            bb = Batch(DEPTH, 8, PATCHES, lib=ol)
            bb.set_many(exyz, vals)
            ch = C.c_int()
            ol.call("apply_batch", oh, ot, bb.handle, C.byref(ch))
            bb.close()
            checks.append(compare(lib, h, tree, oracle))
    call("interner_stats_get", C.byref(st))
    report["edits"] = {"value": EDITS_PER_BATCH / (statistics.median(edit_ms) * 1e-3), "unit": "edits/s",
                       "ms_per_batch": edit_ms, "touched_groups_per_batch": [len(b[2]) for b in batches]}
    report["nodes_after_edits"] = int(st.alive_nodes)
    if checks:
        report["check_edits"] = checks
    call("interner_destroy")
    print(json.dumps(report))


def compare(lib, h, tree, oracle):
    """Canonical DAG of the GPU tree vs the oracle's: identical arrays, plus per-depth counts."""
    import bench as B

    ol, oh, ot = oracle
    cg = B.export(lib, h, tree)
    co = B.export(ol, oh, np.array([ot], np.uint32))
    same = all(np.array_equal(cg[k], co[k]) for k in cg)
    return {"same_dag": bool(same), "canonical_nodes": int(len(cg["kind"]))}
