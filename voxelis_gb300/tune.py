"""Autotuner of the batched-apply launch shape.

Tries threads-per-block x blocks-per-SM combinations of the bottom-group and level kernels on the
caller's own workload (each trial: `reset()` to the same starting state, then `trial()` returning
milliseconds), keeps the fastest, applies it with vx_tune_set and caches the choice per GPU and
workload signature in voxelis_gb300/_build/tune_cache.json.
"""
import ctypes as C
import json
import os

SHAPES = [(128, 8), (256, 4), (256, 8), (256, 16), (512, 4), (512, 8)]
CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "tune_cache.json")


def _gpu_name():
    try:
        import torch

        return torch.cuda.get_device_name(0)
    except Exception:
        return "unknown"


def autotune_apply(lib, handle, reset, trial, signature="default", repeats=2):
    key = "%s|%s" % (_gpu_name(), signature)
    cache = {}
    if os.path.exists(CACHE):
        try:
            cache = json.load(open(CACHE))
        except ValueError:
            cache = {}
    results = {}
    for threads, bps in SHAPES:
        lib.call("tune_set", handle, threads, bps, handle=handle)
        best = None
        for _ in range(repeats):
            reset()
            ms = trial()
            best = ms if best is None else min(best, ms)
        results["%dx%d" % (threads, bps)] = best
    choice = min(results, key=results.get)
    threads, bps = (int(v) for v in choice.split("x"))
    lib.call("tune_set", handle, threads, bps, handle=handle)
    cache[key] = {"threads": threads, "blocks_per_sm": bps, "trials_ms": results}
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    json.dump(cache, open(CACHE, "w"), indent=1)
    return {"threads": threads, "blocks_per_sm": bps, "trials_ms": results}
