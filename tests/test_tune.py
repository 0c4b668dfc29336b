"""Host logic of the autotuners (voxelis_gb300/tune.py) against a fake library: the fastest launch
shape is kept and applied, a dense-build geometry replaces the default only when it is faster by
more than the margin, and each choice is cached per GPU and workload signature."""
import json

import pytest

from voxelis_gb300 import tune


class FakeLib:
    """Records the calls the tuners make; interner handles are integers."""

    def __init__(self, table_slots=1 << 20):
        self.calls = []
        self.table_slots = table_slots
        self.live = set()

    def call(self, name, *args, handle=None):
        self.calls.append((name, args))
        if name == "interner_stats_get":
            args[1]._obj.table_slots = self.table_slots
        return 0

    def status(self, name, *args):
        self.calls.append((name, args))
        if name == "interner_destroy":
            self.live.discard(args[0])
        return 0


@pytest.fixture(autouse=True)
def cache_in_tmp(tmp_path, monkeypatch):
    monkeypatch.setattr(tune, "CACHE", str(tmp_path / "tune_cache.json"))
    monkeypatch.setattr(tune, "_gpu_name", lambda: "fake-gpu")


def test_apply_tuner_keeps_and_applies_the_fastest_shape():
    lib = FakeLib()
    state = {}
    times = {(0, 256, 8): 1.0}  # every other shape 2.0 ms

    def trial():
        return times.get((state["single"], state["threads"], state["bps"]), 2.0)

    def record(name, *args, handle=None):
        if name == "tune_set_launch":
            state["single"] = args[1]
        if name == "tune_set":
            state["threads"], state["bps"] = args[1], args[2]
        return 0

    lib.call = record
    out = tune.autotune_apply(lib, 7, reset=lambda: None, trial=trial, signature="w")
    assert (out["single_launch"], out["threads"], out["blocks_per_sm"]) == (0, 256, 8)
    assert (state["single"], state["threads"], state["bps"]) == (0, 256, 8)  # applied last
    assert len(out["trials_ms"]) == len(tune.SHAPES)
    cached = json.load(open(tune.CACHE))
    assert cached["fake-gpu|w"]["threads"] == 256


def _dense(lib, times):
    handles = iter(range(1, 100))
    current = {}

    def make(table_log2):
        h = next(handles)
        lib.live.add(h)
        current[h] = {"t": table_log2, "m": tune.DEFAULT_MEMO_SHIFT}
        return h

    orig = lib.call

    def call(name, *args, handle=None):
        if name == "tune_set_dense":
            current[args[0]]["m"] = args[1]
        return orig(name, *args, handle=handle)

    lib.call = call

    def build(h):
        return times.get((current[h]["t"], current[h]["m"]), 1.0)

    return make, build


def test_dense_tuner_keeps_the_default_within_the_margin():
    lib = FakeLib(table_slots=1 << 20)
    make, build = _dense(lib, {(21, 3): 0.99})  # 1% faster than the default (20, 2): within 2%
    out = tune.autotune_dense(lib, make, build, signature="d", repeats=3)
    assert out["default_table_log2"] == 20
    assert (out["table_log2"], out["memo_shift"]) == (20, tune.DEFAULT_MEMO_SHIFT)
    assert len(out["trials_ms"]) == len(tune.TABLE_STEPS) * len(tune.MEMO_SHIFTS)
    assert not lib.live  # every trial interner destroyed


def test_dense_tuner_takes_a_clearly_faster_geometry_and_caches_it():
    lib = FakeLib(table_slots=1 << 22)
    make, build = _dense(lib, {(21, 3): 0.90, (23, 1): 0.95})
    out = tune.autotune_dense(lib, make, build, signature="d2", repeats=3)
    assert (out["table_log2"], out["memo_shift"]) == (21, 3)
    assert json.load(open(tune.CACHE))["fake-gpu|d2"]["memo_shift"] == 3
