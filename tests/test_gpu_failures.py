"""Failure paths, made to happen on purpose without faulting anything: each device limit runs out,
the device records a sticky error bit, the host turns it into the matching status at the next
synchronising call, and the interner stays usable: after vx_interner_reset the next call on the same
interner succeeds and matches the oracle.

  out of nodes      a budget too small for the build (interner/macros.rs:38 panics "Out of memory")
  table full        a 16-slot branch table, so inserts run out of probes
  timeout           a round limit of 0 for the warp-cooperative insert loop and a table a fifth
                    full, so lanes whose first probe meets another key's slot give up

Every wait in device code is bounded, and a failed insert yields the EMPTY id, which no consumer
dereferences, so these runs stay within their buffers (the results of the failed call are wrong until
the reset, as the status says).
"""
import ctypes as C

import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300._abi import VX_E_OOM, VX_E_TABLE_FULL, VX_E_TIMEOUT, VoxelisError, vx_interner_stats
from voxelis_gb300.api import VoxInterner, VoxTree

pytestmark = pytest.mark.gpu


def _build(it, grids, depth):
    trees = [VoxTree(depth) for _ in range(len(grids))]
    it.build_dense(trees, grids)
    return trees


def _stats(lib, it):
    """The interner's counters, read without raising on the sticky status."""
    s = vx_interner_stats()
    lib.status("interner_stats_get", it.handle, C.byref(s))
    return s


def _reset(lib, it):
    lib.call("interner_reset", it.handle, handle=it.handle)


def _recovers(lib, oracle_lib, it, grids):
    """After a reset, a build on the same interner equals the oracle's."""
    _reset(lib, it)
    trees = _build(it, grids, 5)
    io = VoxInterner(64 << 20, 8, 0, lib=oracle_lib)
    to = _build(io, grids, 5)
    co, cg = io.export_canonical(to), it.export_canonical(trees)
    for k in co:
        np.testing.assert_array_equal(cg[k], co[k], err_msg=k)
    assert it.stats()["error_flags"] == 0


def test_out_of_nodes_is_reported_then_recovered(gpu_lib, oracle_lib):
    grids = W.dune_chunks(8, 8, depth=5, seed=3)  # about 3,500 nodes
    it = VoxInterner(300 * 79, 8, 0, lib=gpu_lib)  # capacity = budget / node_size = 300 nodes
    assert it.stats()["capacity"] == 300
    with pytest.raises(VoxelisError) as e:
        _build(it, grids, 5)
    assert e.value.status == VX_E_OOM
    s = _stats(gpu_lib, it)
    assert s.next_index <= 300 and s.error_flags  # nothing was allocated past the pool
    _recovers(gpu_lib, oracle_lib, it, grids[:1])


def test_table_full_is_reported_then_recovered(gpu_lib, oracle_lib):
    grids = W.dune_chunks(4, 4, depth=5, seed=5)  # about 1,200 distinct branches
    it = VoxInterner(64 << 20, 8, 0, table_log2=4, lib=gpu_lib)  # 16 branch slots, 16 probes
    assert it.stats()["table_slots"] == 16
    with pytest.raises(VoxelisError) as e:
        _build(it, grids, 5)
    assert e.value.status == VX_E_TABLE_FULL
    one = np.zeros((1, 32, 32, 32), np.uint8)
    one[0, 3, 4, 5] = 7  # a single voxel: one branch per level, five in all
    _recovers(gpu_lib, oracle_lib, it, one)


def test_insert_round_limit_times_out_then_recovers(gpu_lib, oracle_lib):
    grids = W.dune_chunks(8, 8, depth=5, seed=7)  # about 3,300 branches into 16,384 slots
    it = VoxInterner(64 << 20, 8, 0, table_log2=14, lib=gpu_lib)
    probes, rounds, spins = C.c_uint32(), C.c_uint32(), C.c_uint32()
    gpu_lib.call("interner_get_limits", it.handle, C.byref(probes), C.byref(rounds), C.byref(spins), handle=it.handle)
    assert rounds.value == 1 << 20 and spins.value == 1 << 22
    gpu_lib.call("interner_set_limits", it.handle, probes.value, 0, spins.value, handle=it.handle)
    with pytest.raises(VoxelisError) as e:
        _build(it, grids, 5)
    assert e.value.status == VX_E_TIMEOUT
    gpu_lib.call("interner_set_limits", it.handle, probes.value, rounds.value, spins.value, handle=it.handle)
    _recovers(gpu_lib, oracle_lib, it, grids[:4])
