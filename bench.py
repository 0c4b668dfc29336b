#!/usr/bin/env python3
"""Benchmark of the batched dense-chunk build (4096 perlin-dune chunks of 32^3 u8) on GB300.

Workload (one step): intern 4096 perlin-dune chunks of 32^3 u8 voxels, tiled 64 x 64 in XZ, into one
device-resident interner with a single batched call (vx_build_dense_async). Inputs are resident in
HBM when the timed region starts. Between steps (untimed) the interner is reset to an empty store and
L2 is flushed by writing 256 MiB. Clocks are sampled through NVML during the timed steps.

Also measured in the same run:
  gets         4,194,304 uniform-random get() queries on the built world, every result checked
  per_chunk    the plain per-chunk GPU path: one build call per chunk, same DAG (checked)
  e2e          the same build through the public C ABI with HOST buffers (vx_build_dense,
               VX_MEM_HOST): H2D of the grids from pinned memory, build, D2H of the changed flags
  roofline     the dense phase (dense_quads16_kernel, then dense_memo_compute_kernel): algorithmic
               bytes of the build (input grids + new nodes x node_size + roots x 8) / the phase's
               CUDA-event duration, against the measured HBM copy bandwidth
  cpu_baseline the CPU restatement of the reference (oracle), one thread, the whole 4096-chunk workload
  parity       the oracle's DAG of that workload against the GPU's: canonical export (kinds, types,
               masks, values, refcounts, children, roots), live nodes, per-depth counts; the run exits
               non-zero when they differ
  configs      the other workloads at full size, each with its own oracle parity, roofline and clocks
               (bench_edits.py, bench_serve.py, bench_large.py); --no-extras skips them

--impl reference times the reference's CPU algorithm (the oracle port; the Rust reference cannot be
built here) with all host threads on the same workload: all 4096 chunks per step into one interner,
Batches filled in parallel and applied serially, as voxelis-voxelize does. --gpus N outside torchrun
re-launches the script as N ranks (replicas).
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
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline and oracle parity legs")
    p.add_argument("--no-extras", action="store_true",
                   help="dunes: skip the other configurations (uneven edits, served world, large tree)")
    p.add_argument("--workload", default="dunes", choices=["dunes", "edits", "serve", "large", "mesh"],
                   help="dunes: batched dense build of 4096 32^3 chunks (default); edits: uneven batched edits")
    p.add_argument("--check", action="store_true", help="large: compare with the CPU oracle after every step")
    p.add_argument("--edits-chunks", type=int, default=512,
                   help="edits: chunks per depth (512 is the benchmark; fewer for profiling)")
    p.add_argument("--launch", type=int, choices=[0, 1], default=None,
                   help="edits: apply as one cooperative launch (1) or one launch per phase (0) instead of autotuning")
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
    """SM clock and clock-event reasons sampled during the timed region: a background thread reads
    NVML through ctypes every `period` seconds (read-only queries), so that even a region of a few
    milliseconds holds samples; without NVML it falls back to `nvidia-smi -lms`."""

    REASON_BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
                   0x80: "hw_power_brake_slowdown"}

    def __init__(self, device_index, period=0.001):
        import threading

        self.samples = []
        self.max_mhz = None
        self.proc = None
        self._stop = threading.Event()
        self._thread = None
        self._nvml = self._open_nvml(device_index)
        if self._nvml is not None:
            self._thread = threading.Thread(target=self._loop, args=(period,), daemon=True)
            self._thread.start()
            deadline = time.time() + 2.0
            while not self.samples and time.time() < deadline:  # the region starts with a sample
                time.sleep(0.001)
        else:
            self._start_smi(device_index)

    def _open_nvml(self, device_index):
        import ctypes as C

        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            handle = C.c_void_p()
            ok = False
            try:  # the NVML device with the CUDA device's PCI bus id (NVML and CUDA may order devices differently)
                import torch

                p = torch.cuda.get_device_properties(device_index)
                bus = ("%08x:%02x:%02x.0" % (p.pci_domain_id, p.pci_bus_id, p.pci_device_id)).encode()
                ok = lib.nvmlDeviceGetHandleByPciBusId_v2(C.c_char_p(bus), C.byref(handle)) == 0
            except Exception:
                ok = False
            if not ok and lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(device_index), C.byref(handle)) != 0:
                return None
            reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = C.c_uint()
            if lib.nvmlDeviceGetMaxClockInfo(handle, 1, C.byref(mx)) == 0:  # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            return lib, handle, reasons
        except (OSError, AttributeError):
            return None

    def _loop(self, period):
        import ctypes as C

        lib, handle, reasons = self._nvml
        mhz, bits = C.c_uint(), C.c_ulonglong()
        while True:
            if lib.nvmlDeviceGetClockInfo(handle, 1, C.byref(mhz)) == 0 and reasons(handle, C.byref(bits)) == 0:
                self.samples.append((float(mhz.value), int(bits.value)))
            if self._stop.wait(period):
                break

    def _start_smi(self, device_index):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        fields = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                  "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device_index), "--query-gpu=" + fields,
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self._thread is not None:
            self._stop.set()
            self._thread.join(timeout=5)
            sm = [s for s, _ in self.samples]
            reasons = sorted({name for _, b in self.samples for bit, name in self.REASON_BITS.items() if b & bit})
            src = "nvml"
        elif self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.file.flush()
            self.file.seek(0)
            rows = [r.split(",") for r in self.file.read().strip().splitlines() if r.strip()]
            os.unlink(self.file.name)
            sm, reasons = [], set()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for r in rows:
                try:
                    sm.append(float(r[0]))
                    self.max_mhz = max(self.max_mhz or 0.0, float(r[1]))
                    reasons.update(n for k, n in enumerate(names) if r[2 + k].strip().lower() == "active")
                except (ValueError, IndexError):
                    continue
            reasons = sorted(reasons)
            src = "nvidia-smi"
        else:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0, "source": None}
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": reasons, "samples": 0, "source": src}
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(sm), "source": src}


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


def oracle_dunes(grids):
    """The oracle (a line-faithful CPU restatement of the reference) on one thread over the whole
    workload: every chunk's Batch filled by just_set, then apply_batch, serially into one interner of
    the workload's budget. Returns (chunks/s, seconds, canonical export, live nodes): the time is the
    CPU baseline and the export the parity reference of the GPU build."""
    import ctypes as C

    from voxelis_gb300._abi import vx_interner_stats
    from voxelis_gb300.api import export_canonical

    ol = oracle_lib()
    h = C.c_void_p()
    ol.call("interner_create", C.c_uint64(BUDGET), 8, 0, 0, C.byref(h))
    n = grids.shape[0]
    trees = np.zeros(n, dtype=np.uint32)
    for i in range(n):
        out = C.c_uint32()
        ol.call("tree_create", h, DEPTH, C.byref(out), handle=h)
        trees[i] = out.value
    secs = C.c_double()
    f = ol.lib.vxo_time_build_dense
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.POINTER(C.c_double)]
    f.restype = C.c_int
    st = f(h, n, trees.ctypes.data, grids.ctypes.data, C.byref(secs))
    if st != 0:
        ol.status("interner_destroy", h)
        raise RuntimeError("oracle build failed: %d" % st)
    canon = export_canonical(ol, h, trees)
    stats = vx_interner_stats()
    ol.call("interner_stats_get", h, C.byref(stats), handle=h)
    ol.status("interner_destroy", h)
    return n / secs.value, secs.value, canon, int(stats.alive_nodes)


def parity_report(gpu_canon, gpu_alive, oracle_canon, oracle_alive):
    """Bit-exact comparison of two canonical exports (every array), live node counts and per-depth
    node counts with tree multiplicity."""
    from voxelis_gb300.api import level_counts

    fields = {k: bool(np.array_equal(gpu_canon[k], oracle_canon[k])) for k in oracle_canon}
    lg, lo = level_counts(gpu_canon), level_counts(oracle_canon)
    ok = all(fields.values()) and gpu_alive == oracle_alive and lg == lo
    return {"oracle_equal": ok, "canonical_nodes": int(len(oracle_canon["kind"])), "alive_nodes_gpu": gpu_alive,
            "alive_nodes_oracle": oracle_alive, "level_counts_equal": lg == lo, "level_counts": lo,
            "fields_equal": fields}


def run_reference(args):
    """The reference's CPU algorithm (the oracle port: the Rust reference cannot be built here) on
    the host cores, on the same workload and config as our arm: each step builds all 4096 chunks into
    one fresh interner of the workload's budget, Batches filled from the grids on every host thread
    and applied serially (the pattern of voxelis-voxelize/src/lib.rs:284-361)."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    import ctypes as C

    grids = np_grids()
    n = grids.shape[0]
    ol = oracle_lib()
    threads = os.cpu_count() or 1
    f = ol.lib.vxo_build_dense_mt
    f.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_double),
                  C.POINTER(C.c_double)]
    f.restype = C.c_int
    times = []
    for step in range(args.warmup + args.steps):
        h = C.c_void_p()
        ol.call("interner_create", C.c_uint64(BUDGET), 8, 0, 0, C.byref(h))
        trees = np.zeros(n, dtype=np.uint32)
        for i in range(n):
            out = C.c_uint32()
            ol.call("tree_create", h, DEPTH, C.byref(out), handle=h)
            trees[i] = out.value
        fs, ap = C.c_double(), C.c_double()
        t0 = time.perf_counter()
        st = f(h, n, trees.ctypes.data, grids.ctypes.data, threads, C.byref(fs), C.byref(ap))
        t1 = time.perf_counter()
        ol.status("interner_destroy", h)
        if st != 0:
            raise RuntimeError("oracle build failed: %d" % st)
        if step >= args.warmup:
            times.append(t1 - t0)
    per_step = statistics.mean(times)
    value = n / per_step
    line = {
        "metric": "chunks/s", "value": value, "unit": "chunks/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u8", "data": "synthetic", "impl": "reference",
        "config": config({"parallelism": "replicas" if world > 1 else "single"}),
        "cpu_baseline": {"value": value, "unit": "chunks/s", "cores": threads, "kind": "port",
                         "sample": "the whole 4096-chunk workload per step into one fresh %d MiB interner; Batches "
                                   "filled on %d threads, applied serially" % (BUDGET >> 20, threads)},
        "e2e": {"value": value, "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
    from voxelis_gb300.api import export_canonical, same_dag

    lib_build.build()
    lib = gpu_lib()
    grids_np = np_grids()
    n = grids_np.shape[0]
    stream = torch.cuda.Stream(device=dev)
    depths = np.full(n, DEPTH, dtype=np.uint8)

    def make(table_log2):
        """A fresh interner of the workload's budget (table_log2 0: the default branch table) with the
        workload's trees, on the bench's stream."""
        hh = C.c_void_p()
        lib.call("interner_create", C.c_uint64(BUDGET), 8, 0, int(table_log2), C.byref(hh))
        lib.call("interner_set_stream", hh, C.c_void_p(stream.cuda_stream), handle=hh)
        tr = np.zeros(n, dtype=np.uint32)
        lib.call("trees_create", hh, n, depths.ctypes.data, tr.ctypes.data, handle=hh)
        return hh, tr

    h, trees = make(0)
    lib.status("interner_destroy", h)
    call = lambda name, *a: lib.call(name, h, *a, handle=h)  # noqa: E731

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

    # the autotuner picks the branch table's size and the quad memo's geometry on this workload; the
    # timed interner is then created with them (same trees, same DAG)
    tune = None
    if not args.quick:
        from voxelis_gb300.tune import autotune_dense

        def trial(hh):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            lib.call("interner_reset", hh, handle=hh)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            lib.call("build_dense_async", hh, n, C.c_void_p(trees_d.data_ptr()), C.c_void_p(grids.data_ptr()),
                     C.c_void_p(changed.data_ptr()), DEPTH, handle=hh)
            e1.record(stream)
            e1.synchronize()
            lib.call("interner_sync", hh, handle=hh)
            return e0.elapsed_time(e1)

        tune = autotune_dense(lib, lambda t: make(t)[0], trial, signature="dunes%d" % n)
    h, trees2 = make(tune["table_log2"] if tune else 0)
    assert np.array_equal(trees, trees2)
    if tune:
        call("tune_set_dense", tune["memo_shift"])

    for _ in range(args.warmup):
        step_prepare()
        build_async()
        call("interner_sync")

    prof_ms = (C.c_double * VX_PROF_N)()
    prof_n = (C.c_uint64 * VX_PROF_N)()
    clocks = Clocks(local_rank)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = lib.kernel_launches()
    step_ms = []
    for _ in range(args.steps):
        step_prepare()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        build_async()
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
    launches = lib.kernel_launches() - launches0  # this library's kernels in the timed region
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    call("interner_sync")
    # the phase split (and the dense phase's duration for the roofline) from the same steps run again
    # with the library's per-phase CUDA events: events between kernels hold back the early launch of
    # the next kernel, so the headline above is taken without them
    call("profile_enable", 1)
    call("profile_collect", prof_ms, prof_n)
    for _ in range(min(args.steps, 200)):
        step_prepare()
        build_async()
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
    gpu_alive = int(st.alive_nodes)
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
    # every get against the dense input
    f_h = found_d.cpu().numpy()
    v_h = val_d.cpu().numpy()
    slot = np.zeros(int(trees.max()) + 1, dtype=np.int64)
    slot[trees] = np.arange(n)
    ref_v = grids_np[slot[qt], qxyz[:, 1], qxyz[:, 2], qxyz[:, 0]]
    gets_ok = bool(np.array_equal(v_h, ref_v) and np.array_equal(f_h.astype(bool), ref_v != 0))

    if args.quick:
        print(json.dumps({"quick": True, "ms_per_step": ms, "chunks_per_s": n / (ms * 1e-3), "gets_ms": gms,
                          "dense_kernel_ms": dense_ms, "algorithmic_bytes": int(algo_bytes), "gets_ok": gets_ok,
                          "gpu_launches": launches}))
        call("interner_destroy")
        return 0

    # canonical DAG of the batched build, then the per-chunk path on the same grids
    canon = export_canonical(lib, h, trees)
    call("interner_reset")
    stream.synchronize()
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
    pc_same = same_dag(canon, export_canonical(lib, h, trees))

    # e2e through the public API with host buffers (pinned)
    pinned = torch.from_numpy(grids_np).pin_memory()
    trees_h = trees.copy()
    changed_h = np.zeros(n, dtype=np.uint8)
    e2e_s = []
    for k in range(args.warmup + max(30, args.steps // 5)):  # at least 30: a slow host step moves a short mean
        step_prepare()
        stream.synchronize()
        t0 = time.perf_counter()
        call("build_dense", n, C.c_void_p(trees_h.ctypes.data), C.c_void_p(pinned.data_ptr()),
             C.c_void_p(changed_h.ctypes.data), 0)
        t1 = time.perf_counter()
        if k >= args.warmup:
            e2e_s.append(t1 - t0)
    e2e_ms = statistics.mean(e2e_s) * 1e3
    e2e_same = same_dag(canon, export_canonical(lib, h, trees))
    call("interner_destroy")

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
        "autotune": tune,
        "voxel_edits_per_s": world * grids_np.size / (ms * 1e-3),
        "gets": {"value": N_GETS / (gms * 1e-3), "unit": "gets/s", "ms": gms, "checked_all": gets_ok},
        "per_chunk_gpu": {"value": n / (pc_ms * 1e-3), "unit": "chunks/s", "ms": pc_ms, "same_dag": pc_same},
        "batched_over_per_chunk": pc_ms / ms,
        "dag": {"nodes": int(new_nodes), "canonical_nodes": int(len(canon["kind"])), "node_size": int(node_size)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": profiled_traffic("dense_phase_dunes4096.md"),
                     "kernel": "dense phase: dense_quads16_kernel + dense_memo_compute_kernel",
                     "kernel_ms": dense_ms, "algorithmic_bytes": int(algo_bytes), "peak_kind": peak_kind,
                     "step_frac": algo_bytes / (ms * 1e-3) / 1e9 / peak},
        "phases": phases,
        "e2e": {"value": world * n / (e2e_ms * 1e-3), "unit": "chunks/s", "ms": e2e_ms,
                "h2d_bytes_per_step": int(grids_np.nbytes + 4 * n), "d2h_bytes_per_step": int(n),
                "same_dag": e2e_same},
        "clocks": clk,
        "gpu_launches": int(launches),
        "gpu_launches_per_step": launches / max(1, args.steps),
    }
    ok = pc_same and e2e_same and gets_ok
    if rank == 0 and not args.no_cpu:
        v, secs, ocanon, oalive = oracle_dunes(grids_np)
        line["cpu_baseline"] = {"value": v, "unit": "chunks/s", "cores": 1, "kind": "port",
                                "sample": "the whole 4096-chunk workload once (%.2f s), one thread: Batch filled "
                                          "by just_set then apply_batch per chunk, one interner" % secs}
        line["parity"] = parity_report(canon, gpu_alive, ocanon, oalive)
        ok = ok and line["parity"]["oracle_equal"]
    if world == 1 and not args.no_extras:
        line["configs"] = run_extras(args)
        for c in line["configs"].values():
            ok = ok and c.get("parity", {}).get("oracle_equal", True) is not False and "error" not in c
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0 if ok else 3


def run_extras(args):
    """The other benchmark configurations, measured in the same run at their full sizes (each with
    its own oracle comparison, roofline and clocks): uneven batched edits, the served world and the
    MaxDepth-10 tree. A failure of one is recorded in its entry."""
    import traceback

    import torch

    out = {}
    prepared = None
    try:  # the large tree's grid, and the oracle's minute-long build of it started in the background
        import bench_large

        prepared = bench_large.Prepared(check=True)
    except Exception as e:
        out["large_tree"] = {"error": "%s: %s" % (type(e).__name__, e), "trace": traceback.format_exc()[-600:]}
    for key, mod in (("uneven_edits", "bench_edits"), ("served_world", "bench_serve"), ("large_tree", "bench_large")):
        if key in out:
            continue
        t0 = time.time()
        try:
            m = __import__(mod)
            out[key] = m.measure(args, prepared=prepared) if key == "large_tree" else m.measure(args)
        except Exception as e:  # keep the headline line; the entry says what failed
            out[key] = {"error": "%s: %s" % (type(e).__name__, e), "trace": traceback.format_exc()[-600:]}
        out[key]["wall_s"] = time.time() - t0
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


def spawn_ranks(args):
    """`--gpus N` outside torchrun: re-run this script under torch.distributed.run with N ranks (one
    per GPU, rendezvous on 127.0.0.1) and return its exit code."""
    import socket

    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    if args.impl == "ours":  # build once before N ranks start
        from voxelis_gb300 import build as lib_build

        lib_build.build()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", str(args.gpus),
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + sys.argv[1:]
    return subprocess.call(cmd)


def main():
    args = parse()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        sys.exit(spawn_ranks(args))
    if args.workload == "edits":
        import bench_edits

        print(json.dumps(bench_edits.measure(args, full_line=True)), flush=True)
    elif args.workload == "large":
        import bench_large

        print(json.dumps(bench_large.measure(args, full_line=True)), flush=True)
    elif args.workload == "mesh":
        import bench_mesh

        bench_mesh.run(args)
    elif args.workload == "serve":
        import bench_serve

        print(json.dumps(bench_serve.measure(args, full_line=True)), flush=True)
    elif args.impl == "reference":
        run_reference(args)
    else:
        sys.exit(run_ours(args))


if __name__ == "__main__":
    main()
