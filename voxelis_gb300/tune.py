"""Autotuner of the batched-apply launch.

Tries the launch form (the whole apply as one cooperative launch, or one kernel per phase) with
threads-per-block x blocks-per-SM combinations of the branch-creating kernels on the caller's own
workload (each trial: `reset()` to the same starting state, then `trial()` returning milliseconds),
keeps the fastest, applies it with vx_tune_set / vx_tune_set_launch and caches the choice per GPU and
workload signature in voxelis_gb300/_build/tune_cache.json.
"""
import json
import os

# (single launch, threads per block, blocks per SM); a single launch caps blocks per SM at what can
# be resident at once
SHAPES = [(1, 256, 4), (1, 512, 2), (1, 256, 8), (0, 128, 8), (0, 256, 4), (0, 256, 8), (0, 256, 16), (0, 512, 4)]
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "tune_cache.json")


def _gpu_name():
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def _apply(lib, handle, single, threads, bps):
    lib.call("tune_set_launch", handle, single, handle=handle)
    lib.call("tune_set", handle, threads, bps, handle=handle)


def autotune_apply(lib, handle, reset, trial, signature="default", repeats=2):
    key = "%s|%s" % (_gpu_name(), signature)
    cache = {}
    if os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except ValueError:
            cache = {}
    results = {}
    for single, threads, bps in SHAPES:
        _apply(lib, handle, single, threads, bps)
        best = None
        for _ in range(repeats):
            reset()
            ms = trial()
            best = ms if best is None else min(best, ms)
        results["%s:%dx%d" % ("single" if single else "phases", threads, bps)] = best
    choice = min(results, key=results.get)
    form, shape = choice.split(":")
    threads, bps = (int(v) for v in shape.split("x"))
    single = 1 if form == "single" else 0
    _apply(lib, handle, single, threads, bps)
    cache[key] = {"single_launch": single, "threads": threads, "blocks_per_sm": bps, "trials_ms": results}
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    json.dump(cache, open(CACHE, "w"), indent=1)
    return {"single_launch": single, "threads": threads, "blocks_per_sm": bps, "trials_ms": results}


# dense builds: the branch table's size relative to the default (2 x capacity, rounded up to a power
# of two: load factor at most 1/2) and the quad memo's slots (the call's quads >> shift)
TABLE_STEPS = (-1, 0, 1)
MEMO_SHIFTS = (1, 2, 3)
DEFAULT_MEMO_SHIFT = 2  # the interner's default (vx_interner_create)


def autotune_dense(lib, make, build, signature="dense", repeats=5, margin=0.02):
    """Tries branch-table sizes (load factor) and quad-memo geometries on the caller's own dense
    build. make(table_log2) returns a fresh interner handle (table_log2 0: the default size) with the
    caller's trees; build(handle) resets it, runs one build and returns milliseconds. Each candidate
    is the median of `repeats` builds; the fastest replaces the default geometry only when it is
    faster by more than `margin` (differences below that are run-to-run spread). Returns
    {table_log2, memo_shift, trials_ms} and caches it; the caller recreates its interner with that
    table size and applies the shift with vx_tune_set_dense."""
    import statistics
    import ctypes as C

    from ._abi import vx_interner_stats

    key = "%s|%s" % (_gpu_name(), signature)
    results = {}
    h0 = make(0)
    st = vx_interner_stats()
    lib.call("interner_stats_get", h0, C.byref(st), handle=h0)
    lib.status("interner_destroy", h0)
    default_log2 = int(st.table_slots).bit_length() - 1
    for step in TABLE_STEPS:
        t_log2 = default_log2 + step
        h = make(t_log2)
        for shift in MEMO_SHIFTS:
            lib.call("tune_set_dense", h, shift, handle=h)
            results["t%d:m%d" % (t_log2, shift)] = statistics.median(build(h) for _ in range(repeats))
        lib.status("interner_destroy", h)
    choice = min(results, key=results.get)
    default = "t%d:m%d" % (default_log2, DEFAULT_MEMO_SHIFT)
    if default in results and results[choice] > (1.0 - margin) * results[default]:
        choice = default
    t_log2, shift = (int(v[1:]) for v in choice.split(":"))
    out = {"table_log2": t_log2, "default_table_log2": default_log2, "memo_shift": shift, "trials_ms": results}
    cache = {}
    if os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except ValueError:
            cache = {}
    cache[key] = out
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    json.dump(cache, open(CACHE, "w"), indent=1)
    return out
