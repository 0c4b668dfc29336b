"""Large single tree on GB300 (bench.py --workload large; also part of the default bench.py line).

One VoxTree of MaxDepth 10 (1024^3 u8, patches P1 + P2 + P3 + P4) built from a dense 1 GiB grid of
caves (voxel = 1 + floor(3|N|) where N(x/64, y/64, z/64) > 0.1, else 0; N = 3D gradient noise with a
seed-shuffled permutation), then 16M uniform-random get() queries (every result checked against the
grid), then 8 successive batches of 1M random edits (materials 1..4, 80% set / 20% clear; clears
honoured, P4). After every batch the UB fence runs (every reachable child live, refcount > 0). The CPU
oracle builds the same tree and applies the same 8 Batches; its canonical DAG (nodes, refcounts,
links), live node count and per-depth counts are compared with the GPU's after the build and after
every batch (--no-check skips the oracle).
"""
import ctypes as C
import statistics
import time

import numpy as np

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import (VX_PATCH_P1, VX_PATCH_P2, VX_PATCH_P3, VX_PATCH_P4, VX_PROF_N, VX_PROF_NAMES, gpu_lib,
                                vx_interner_stats)
from voxelis_gb300.api import Batch, export_canonical

DEPTH = 10
PATCHES = VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P3 | VX_PATCH_P4
BUDGET = 16 << 30
N_GETS = 1 << 24
N_BATCHES = 8
EDITS_PER_BATCH = 1 << 20
WORKLOAD = ("large tree: MaxDepth 10 (1024^3 u8) caves grid, 16M gets, 8 x 1M edits (80/20 set/clear), "
            "P1+P2+P3+P4")


def _stats(lib, h):
    st = vx_interner_stats()
    lib.call("interner_stats_get", h, C.byref(st), handle=h)
    return st


def compare(lib, h, tree, oracle):
    """GPU tree vs the oracle's: canonical DAG (every array), live nodes, per-depth counts."""
    import bench as B

    ol, oh, ot = oracle
    cg = export_canonical(lib, h, tree)
    co = export_canonical(ol, oh, np.array([ot], np.uint32))
    rep = B.parity_report(cg, int(_stats(lib, h).alive_nodes), co, int(_stats(ol, oh).alive_nodes))
    rep.pop("fields_equal") if rep["oracle_equal"] else None
    return rep


class Prepared:
    """The caves grid generated on the GPU and, when checking, the oracle's build of the same tree
    running in a background thread (it takes about a minute of one core; the oracle's C calls release
    the interpreter, so other work proceeds meanwhile)."""

    def __init__(self, check):
        import threading

        import torch

        import bench as B

        self.dev = torch.device("cuda", 0)
        self.stream = torch.cuda.Stream(device=self.dev)
        t0 = time.time()
        with torch.cuda.stream(self.stream):
            self.grid = W.caves_torch(DEPTH, seed=99, device=self.dev)
        self.stream.synchronize()
        self.gen_s = time.time() - t0
        self.check = check
        self.oracle = self.error = None
        self.oracle_build_s = None
        self.done = threading.Event()
        if not check:
            self.done.set()
            return
        host = self.grid.cpu().numpy()

        def work():
            try:
                ol = B.oracle_lib()
                oh = C.c_void_p()
                ol.call("interner_create", C.c_uint64(BUDGET), 8, PATCHES, 0, C.byref(oh))
                ot = C.c_uint32()
                ol.call("tree_create", oh, DEPTH, C.byref(ot), handle=oh)
                otr = np.array([ot.value], np.uint32)
                t1 = time.time()
                ol.call("build_dense", oh, 1, C.c_void_p(otr.ctypes.data), C.c_void_p(host.ctypes.data), None, 0,
                        handle=oh)
                self.oracle_build_s = time.time() - t1
                self.oracle = (ol, oh, ot.value)
            except Exception as e:  # reported by measure()
                self.error = e
            self.done.set()

        threading.Thread(target=work, daemon=True).start()


def measure(args, full_line=False, check=None, prepared=None):
    import torch

    import bench as B
    from voxelis_gb300.build import build as build_lib

    if check is None:
        check = not getattr(args, "no_check", False)
    build_lib()
    lib = gpu_lib()
    pre = prepared if prepared is not None else Prepared(check)
    check = pre.check
    dev, stream, grid, gen_s = pre.dev, pre.stream, pre.grid, pre.gen_s
    h = C.c_void_p()
    lib.call("interner_create", C.c_uint64(BUDGET), 8, PATCHES, 0, C.byref(h))
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    tree = np.zeros(1, np.uint32)
    call("trees_create", 1, np.array([DEPTH], np.uint8).ctypes.data, tree.ctypes.data)
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
    clocks = B.Clocks(0)
    for _ in range(1 + max(1, min(args.warmup, 3))):
        call("interner_reset")
        build_ms.append(timed(lambda: call("build_dense_async", 1, P(t_d), P(grid), None, DEPTH)))
        call("interner_sync")
    clk = clocks.stop()
    # the phase split from one more build with the library's per-phase events (kept out of the timed
    # builds: an event between two kernels holds the second one back)
    call("interner_reset")
    call("profile_enable", 1)
    call("profile_collect", prof_ms, prof_n)
    call("build_dense_async", 1, P(t_d), P(grid), None, DEPTH)
    call("interner_sync")
    call("profile_collect", prof_ms, prof_n)
    call("profile_enable", 0)
    build_phases = {VX_PROF_NAMES[k]: prof_ms[k] for k in range(VX_PROF_N) if prof_n[k]}
    st = _stats(lib, h)
    nodes_built = int(st.alive_nodes)
    peak, peak_kind = B.peaks()
    algo = grid.numel() + int(st.nodes_created) * int(st.node_size) + 8
    report = {"metric": "voxels/s (dense build, MaxDepth 10)", "unit": "voxels/s", "higher_is_better": True,
              "config": {"workload": WORKLOAD, "budget_bytes": BUDGET},
              "grid_generation_s": gen_s, "build_ms": build_ms[-1], "value": (1 << 30) / (build_ms[-1] * 1e-3),
              "build_phases_ms": build_phases, "nodes_after_build": nodes_built,
              "roofline": {"bound": "hbm", "kernel": "whole dense build", "algorithmic_bytes": algo,
                           "achieved": algo / (build_ms[-1] * 1e-3) / 1e9, "peak": peak,
                           "frac": algo / (build_ms[-1] * 1e-3) / 1e9 / peak, "unit": "GB/s", "peak_kind": peak_kind},
              "clocks": clk}

    oracle, checks = None, []
    if check:
        pre.done.wait()
        if pre.error is not None:
            raise pre.error
        oracle = pre.oracle
        report["oracle_build_s"] = pre.oracle_build_s
        checks.append(dict(after="build", **compare(lib, h, tree, oracle)))

    # 16M uniform-random gets, every result checked against the grid
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
    with torch.cuda.stream(stream):
        want = grid[q_d[:, 1].long(), q_d[:, 2].long(), q_d[:, 0].long()]
        gets_ok = bool(torch.equal(v_d, want) and torch.equal(f_d.bool(), want != 0))
    gms = statistics.median(get_ms)
    report["gets"] = {"value": N_GETS / (gms * 1e-3), "unit": "gets/s", "ms": gms, "checked_all": gets_ok,
                      "roofline_frac": N_GETS * 14 / (gms * 1e-3) / 1e9 / peak}
    del q_d, qt_d, f_d, v_d, want
    del grid
    torch.cuda.empty_cache()

    # 8 batches of 1M random set/clear edits (P4)
    flags, fill = (torch.from_numpy(a).to(dev) for a in (np.array([2], np.uint8), np.zeros(1, np.int32)))
    edit_ms, created = [], []
    for b in range(N_BATCHES):
        exyz, vals = W.random_edits(DEPTH, 0, 1000 + b, max_material=4, clear_fraction=0.2, count=EDITS_PER_BATCH)
        g, sm, cm, vv = W.edits_to_groups(DEPTH, exyz, vals)
        R = len(g)
        with torch.cuda.stream(stream):
            ri = torch.zeros(R, dtype=torch.int32, device=dev)
            rg, rs, rc = (torch.from_numpy(np.ascontiguousarray(a)).to(dev) for a in (g.view(np.int32), sm, cm))
            rv = torch.from_numpy(np.ascontiguousarray(vv.reshape(-1).view(np.int16))).to(dev)
        stream.synchronize()
        c0 = int(_stats(lib, h).nodes_created)
        edit_ms.append(timed(lambda: call("apply_groups_async", 1, P(t_d), P(flags), P(fill), R, P(ri), P(rg), P(rs),
                                          P(rc), P(rv), None, DEPTH)))
        call("interner_maintain")
        call("validate", 1, C.c_void_p(tree.ctypes.data))
        created.append((R, int(_stats(lib, h).nodes_created) - c0))
        if oracle is not None:
            ol, oh, ot = oracle
            bb = Batch(DEPTH, 8, PATCHES, lib=ol)
            bb.set_many(exyz, vals)
            ch = C.c_int()
            ol.call("apply_batch", oh, ot, bb.handle, C.byref(ch), handle=oh)
            bb.close()
            checks.append(dict(after="batch %d" % b, **compare(lib, h, tree, oracle)))
    st = _stats(lib, h)
    em = statistics.median(edit_ms)
    # algorithmic bytes of a batch: compacted records (2 + 8 + 4 B), created nodes x 79 B, the root
    eb = statistics.median([r * 14 + c * int(st.node_size) + 8 for r, c in created])
    report["edits"] = {"value": EDITS_PER_BATCH / (em * 1e-3), "unit": "edits/s", "ms_per_batch": edit_ms,
                       "touched_groups_per_batch": [r for r, _ in created],
                       "nodes_created_per_batch": [c for _, c in created],
                       "roofline_frac": eb / (em * 1e-3) / 1e9 / peak}
    report["nodes_after_edits"] = int(st.alive_nodes)
    if oracle is not None:
        ol.status("interner_destroy", oh)
        report["parity"] = {"oracle_equal": all(c["oracle_equal"] for c in checks), "checks": checks}
    call("interner_destroy")
    if full_line:
        report.update({"n_gpus": 1, "steps": len(build_ms) - 1, "warmup": 1, "dtype": "u8", "data": "synthetic",
                       "scaling": "weak", "vs_baseline": None, "ms_per_step": build_ms[-1]})
    return report
