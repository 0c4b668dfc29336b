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
