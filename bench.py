#!/usr/bin/env python3
"""Benchmark of the batched dense-chunk build (the spec workload) on GB300.

Workload (one step): intern 4096 perlin-dune chunks of 32^3 u8 voxels, tiled 64 x 64 in XZ, into one
device-resident interner with a single batched call (vx_build_dense_async: one persistent fused
kernel plus the refcount epoch). Inputs are resident in HBM when the timed region starts. Between
steps (untimed) the interner is reset to an empty store and L2 is flushed by writing 256 MiB.

Also measured in the same run:
  gets        4,194,304 uniform-random get() queries on the built world (vx_get_many_async)
  per_chunk   the plain per-chunk GPU path: one build call per chunk, same DAG (checked)
  e2e         the same build through the public C ABI with HOST buffers (vx_build_dense,
              VX_MEM_HOST): H2D of the grids from pinned memory, build, D2H of the changed flags
  roofline    the dense phase (dense_quads16_kernel streaming the grids, then dense_memo_compute_kernel
              for the distinct quads): algorithmic bytes of the build (input grids + new nodes x
              node_size + roots x 8) / the phase's CUDA-event duration (the level passes are the
              "levels" phase), against the measured HBM copy bandwidth
  cpu_baseline the CPU restatement of the reference (oracle), one thread, whole 4096-chunk workload

--impl reference times the reference's CPU algorithm (the oracle port; the Rust reference cannot be
built here) with all host threads: Batches filled in parallel, applied serially to one interner, as
voxelis-voxelize does.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CHUNKS_X = 64
CHUNKS_Z = 64
DEPTH = 5
SEED = 1234
BUDGET = 256 << 20
N_GETS = 1 << 22
WORKLOAD = "batched dense build: 4096 perlin-dune chunks 32^3 u8 (64x64 XZ tiling), one interner"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=1000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--workload", default="dunes", choices=["dunes", "edits", "serve", "large", "mesh"],
                   help="dunes: batched dense build of 4096 32^3 chunks (default); edits: uneven batched edits")
    p.add_argument("--check", action="store_true", help="large: compare with the CPU oracle after every step")
    p.add_argument("--edits-chunks", type=int, default=512,
                   help="edits: chunks per depth (512 is the benchmark; fewer for profiling)")
    p.add_argument("--quick", action="store_true",
                   help="timed build steps and gets only (no per-chunk, e2e or CPU legs); for profiling")
    return p.parse_args()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")),
            int(os.environ.get("WORLD_SIZE", "1")))


def max_over_ranks(ms, world, device=None):
    """The step time of the whole job: the slowest replica's (all-reduce MAX; NCCL on GPUs, gloo on CPU)."""
    if world <= 1:
        return ms
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, world, ms):
    """Whole-job units/s of `world` replicas that each processed units_per_rank in `ms` (max over ranks)."""
    return world * units_per_rank / (ms * 1e-3)


def config(extra=None):
    c = {"workload": WORKLOAD, "chunks": CHUNKS_X * CHUNKS_Z, "max_depth": DEPTH, "voxel": "u8",
         "seed": SEED, "budget_bytes": BUDGET, "gets": N_GETS,
         "l2": "flushed between steps (256 MiB write); inputs 128 MiB"}
    if extra:
        c.update(extra)
    return c


# ---- clocks sampler ----------------------------------------------------------------------------
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        self.file.seek(0)
        rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, n in enumerate(names):
                    if r[5 + k].strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(summary):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) recorded from one ncu
    capture in profiles/<summary>: the line 'traffic_bytes_per_launch: N', or None."""
    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            for ln in f:
                if ln.strip().startswith("traffic_bytes_per_launch:"):
                    return int(float(ln.split(":", 1)[1].split()[0]))
    except (OSError, ValueError):
        pass
    return None


# ---- the CPU legs ----------------------------------------------------------------------------------
def oracle_lib():
    from oracle import build as oracle_build
    from voxelis_gb300._abi import NativeLib

    return NativeLib(oracle_build.build(), "vxo_")


def cpu_baseline(grids):
    """The oracle (a line-faithful CPU restatement of the reference) on one thread: every chunk's
    Batch filled by just_set, then apply_batch, serially into one interner."""
    import ctypes as C

    ol = oracle_lib()
    h = C.c_void_p()
    ol.call("interner_create", C.c_uint64(BUDGET), 8, 0, 0, C.byref(h))
    n = grids.shape[0]
    trees = np.zeros(n, dtype=np.uint32)
    for i in range(n):
        out = C.c_uint32()
        ol.call("tree_create", h, DEPTH, C.byref(out))
        trees[i] = out.value
    secs = C.c_double()
    f = ol.lib.vxo_time_build_dense
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    f.restype = C.c_int
    st = f(h, n, trees.ctypes.data, grids.ctypes.data, C.byref(secs))
    ol.status("interner_destroy", h)
    if st != 0:
        raise RuntimeError("oracle build failed: %d" % st)
    return n / secs.value, secs.value


def run_reference(args):
    rank, _, world = dist_env()
    if rank != 0:
        return
    import ctypes as C

    grids = np_grids()
    ol = oracle_lib()
    threads = os.cpu_count() or 1
    sample = 512  # chunks per step: a bounded sample of the 4096-chunk workload
    f = ol.lib.vxo_build_dense_mt
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_double),
                  C.POINTER(C.c_double)]
    f.restype = C.c_int
    times = []
    for step in range(args.warmup + args.steps):
        lo = (step * sample) % grids.shape[0]
        g = np.ascontiguousarray(grids[lo:lo + sample])
        h = C.c_void_p()
        ol.call("interner_create", C.c_uint64(64 << 20), 8, 0, 0, C.byref(h))
        trees = np.zeros(sample, dtype=np.uint32)
        for i in range(sample):
            out = C.c_uint32()
            ol.call("tree_create", h, DEPTH, C.byref(out))
            trees[i] = out.value
        fs, ap = C.c_double(), C.c_double()
        t0 = time.perf_counter()
        st = f(h, sample, trees.ctypes.data, g.ctypes.data, threads, C.byref(fs), C.byref(ap))
        t1 = time.perf_counter()
        ol.status("interner_destroy", h)
        if st != 0:
            raise RuntimeError("oracle build failed: %d" % st)
        if step >= args.warmup:
            times.append(t1 - t0)
    per_step = statistics.mean(times)
    value = sample / per_step
    line = {
        "metric": "chunks/s", "value": value, "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
        "config": config({"reference_sample_chunks_per_step": sample}),
        "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": "port",
                         "sample": "%d consecutive chunks of the 4096-chunk workload per step, fresh interner; "
                                   "Batches filled on %d threads, applied serially" % (sample, threads)},
        "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def np_grids():
    from voxelis_gb300 import workloads as W

    return W.dune_world_chunks(CHUNKS_X, CHUNKS_Z, depth=DEPTH, seed=SEED)


# ---- our arm --------------------------------------------------------------------------------------
def run_ours(args):
    import ctypes as C

    import torch

    rank, local_rank, world = dist_env()
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    from voxelis_gb300 import build as lib_build
    from voxelis_gb300._abi import VX_PROF_N, VX_PROF_NAMES, gpu_lib

    lib_build.build()
    lib = gpu_lib()
    grids_np = np_grids()
    n = grids_np.shape[0]
    stream = torch.cuda.Stream(device=dev)
    h = C.c_void_p()
    lib.call("interner_create", C.c_uint64(BUDGET), 8, 0, 0, C.byref(h))
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731
    call("interner_set_stream", C.c_void_p(stream.cuda_stream))
    depths = np.full(n, DEPTH, dtype=np.uint8)
    trees = np.zeros(n, dtype=np.uint32)
    call("trees_create", n, depths.ctypes.data, trees.ctypes.data)

    with torch.cuda.stream(stream):
        grids = torch.from_numpy(grids_np).to(dev)
        trees_d = torch.from_numpy(trees.view(np.int32)).to(dev)
        changed = torch.zeros(n, dtype=torch.uint8, device=dev)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream.synchronize()

    def build_async():
        call("build_dense_async", n, C.c_void_p(trees_d.data_ptr()), C.c_void_p(grids.data_ptr()),
             C.c_void_p(changed.data_ptr()), DEPTH)

    def step_prepare():
        with torch.cuda.stream(stream):
            flush.fill_(1)
        call("interner_reset")

    for _ in range(args.warmup):
        step_prepare()
        build_async()
        call("interner_sync")

    prof_ms = (C.c_double * VX_PROF_N)()
    prof_n = (C.c_uint64 * VX_PROF_N)()
    call("profile_enable", 1)
    call("profile_collect", prof_ms, prof_n)
    clocks = Clocks(local_rank)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = lib.kernel_launches()
    step_ms = []
    dense_ms = 0.0
    for _ in range(args.steps):
        step_prepare()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        build_async()
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    launches = lib.kernel_launches() - launches0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    call("interner_sync")
    call("profile_collect", prof_ms, prof_n)
    call("profile_enable", 0)
    phases = {VX_PROF_NAMES[k]: {"ms_total": prof_ms[k], "count": int(prof_n[k])} for k in range(VX_PROF_N)
              if prof_n[k]}
    dense_ms = prof_ms[0] / max(1, prof_n[0])
    ms = max_over_ranks(statistics.mean(step_ms), world, dev)

    # DAG size after the last timed step
    from voxelis_gb300._abi import vx_interner_stats

    st = vx_interner_stats()
    call("interner_stats_get", C.byref(st))
    new_nodes = st.alive_nodes - 1
    n_changed = int(changed.sum().item())
    node_size = st.node_size
    algo_bytes = grids_np.nbytes + new_nodes * node_size + n_changed * 8

    # gets on the built world
    rng = np.random.default_rng(SEED + 1)
    qt = trees[rng.integers(0, n, N_GETS)]
    qxyz = rng.integers(0, 1 << DEPTH, (N_GETS, 3)).astype(np.int32)
    with torch.cuda.stream(stream):
        qt_d = torch.from_numpy(qt.view(np.int32)).to(dev)
        qxyz_d = torch.from_numpy(qxyz).to(dev)
        found_d = torch.empty(N_GETS, dtype=torch.uint8, device=dev)
        val_d = torch.empty(N_GETS, dtype=torch.uint8, device=dev)
    stream.synchronize()
    get_args = (C.c_uint64(N_GETS), C.c_void_p(qt_d.data_ptr()), C.c_void_p(qxyz_d.data_ptr()),
                C.c_void_p(found_d.data_ptr()), C.c_void_p(val_d.data_ptr()))
    for _ in range(3):
        call("get_many_async", *get_args)
    get_ms = []
    for _ in range(max(5, args.steps // 5)):
        with torch.cuda.stream(stream):
            flush.fill_(2)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        call("get_many_async", *get_args)
        e1.record(stream)
        e1.synchronize()
        get_ms.append(e0.elapsed_time(e1))
    call("interner_sync")
    gms = statistics.mean(get_ms)
    # spot-check gets against the dense input
    f_h = found_d[:65536].cpu().numpy()
    v_h = val_d[:65536].cpu().numpy()
    ti = {int(t): i for i, t in enumerate(trees)}
    ref_v = np.array([grids_np[ti[int(qt[k])], qxyz[k, 1], qxyz[k, 2], qxyz[k, 0]] for k in range(65536)])
    gets_ok = bool(np.array_equal(v_h, ref_v) and np.array_equal(f_h.astype(bool), ref_v != 0))

    if args.quick:
        print(json.dumps({"quick": True, "ms_per_step": ms, "chunks_per_s": n / (ms * 1e-3), "gets_ms": gms,
                          "dense_kernel_ms": dense_ms, "algorithmic_bytes": int(algo_bytes), "gets_ok": gets_ok,
                          "gpu_launches": int(launches)}))
        call("interner_destroy")
        return

    # canonical DAG of the batched build, then the per-chunk path on the same grids
    canon = export(lib, h, trees)
    call("interner_reset")
    stream.synchronize()
    pc_ms = []
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for i in range(n):
        call("build_dense_async", 1, C.c_void_p(trees_d.data_ptr() + 4 * i),
             C.c_void_p(grids.data_ptr() + grids_np[0].nbytes * i), C.c_void_p(changed.data_ptr() + i), DEPTH)
    e1.record(stream)
    e1.synchronize()
    call("interner_sync")
    pc_ms = e0.elapsed_time(e1)
    canon_pc = export(lib, h, trees)
    same_dag = all(np.array_equal(canon[k], canon_pc[k]) for k in canon)

    # e2e through the public API with host buffers (pinned)
    pinned = torch.from_numpy(grids_np).pin_memory()
    trees_h = trees.copy()
    changed_h = np.zeros(n, dtype=np.uint8)
    e2e_s = []
    for k in range(args.warmup + max(5, args.steps // 5)):
        step_prepare()
        stream.synchronize()
        t0 = time.perf_counter()
        call("build_dense", n, C.c_void_p(trees_h.ctypes.data), C.c_void_p(pinned.data_ptr()),
             C.c_void_p(changed_h.ctypes.data), 0)
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_s.append(t1 - t0)
    e2e_ms = statistics.mean(e2e_s) * 1e3
    canon_e2e = export(lib, h, trees)
    same_dag = same_dag and all(np.array_equal(canon[k], canon_e2e[k]) for k in canon)

    peak, peak_kind = peaks()
    achieved = algo_bytes / (dense_ms * 1e-3) / 1e9
    line = {
        "metric": "chunks/s",
        "value": replica_throughput(n, world, ms),
        "unit": "chunks/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u8",
        "data": "synthetic",
        "config": config({"parallelism": "replicas" if world > 1 else "single"}),
        "voxel_edits_per_s": world * grids_np.size / (ms * 1e-3),
        "gets": {"value": N_GETS / (gms * 1e-3), "unit": "gets/s", "ms": gms, "checked": gets_ok},
        "per_chunk_gpu": {"value": n / (pc_ms * 1e-3), "unit": "chunks/s", "ms": pc_ms, "same_dag": same_dag},
        "batched_over_per_chunk": pc_ms / ms,
        "dag": {"nodes": int(new_nodes), "canonical_nodes": int(len(canon["kind"])), "node_size": int(node_size)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": profiled_traffic("dense_phase_dunes4096.md"),
                     "kernel": "dense phase: dense_quads16_kernel + dense_memo_compute_kernel",
                     "kernel_ms": dense_ms, "algorithmic_bytes": int(algo_bytes), "peak_kind": peak_kind},
        "phases": phases,
        "e2e": {"value": world * n / (e2e_ms * 1e-3), "unit": "chunks/s", "ms": e2e_ms,
                "h2d_bytes_per_step": int(grids_np.nbytes + 4 * n), "d2h_bytes_per_step": int(n)},
        "clocks": clk,
        "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_cpu:
        v, secs = cpu_baseline(grids_np)
        line["cpu_baseline"] = {"value": v, "unit": "chunks/s", "cores": 1, "kind": "port",
                                "sample": "the whole 4096-chunk workload once (%.2f s), one thread: Batch filled "
                                          "by just_set then apply_batch per chunk" % secs}
    call("interner_destroy")
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def export(lib, h, trees):
    import ctypes as C

    from voxelis_gb300._abi import vx_canonical

    n_nodes = C.c_uint64()
    lib.call("export_canonical", h, len(trees), C.c_void_p(trees.ctypes.data), None, C.byref(n_nodes), handle=h)
    m = n_nodes.value
    out = {"kind": np.zeros(m, np.uint8), "types": np.zeros(m, np.uint8), "mask": np.zeros(m, np.uint8),
           "value": np.zeros(m, np.uint32), "refcount": np.zeros(m, np.uint32),
           "children": np.zeros(m * 8, np.int32), "roots": np.zeros(len(trees), np.int32)}
    c = vx_canonical()
    for k in ("kind", "types", "mask"):
        setattr(c, k, out[k].ctypes.data_as(C.POINTER(C.c_uint8)))
    for k in ("value", "refcount"):
        setattr(c, k, out[k].ctypes.data_as(C.POINTER(C.c_uint32)))
    for k in ("children", "roots"):
        setattr(c, k, out[k].ctypes.data_as(C.POINTER(C.c_int32)))
    c.capacity = m
    lib.call("export_canonical", h, len(trees), C.c_void_p(trees.ctypes.data), C.byref(c), C.byref(n_nodes), handle=h)
    return out


def main():
    args = parse()
    if args.workload == "edits":
        from voxelis_gb300 import bench_edits

        bench_edits.run(args)
    elif args.workload == "large":
        from voxelis_gb300 import bench_large

        bench_large.run(args, check=args.check)
    elif args.workload == "mesh":
        from voxelis_gb300 import bench_mesh

        bench_mesh.run(args)
    elif args.workload == "serve":
        from voxelis_gb300 import bench_serve

        bench_serve.run(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
