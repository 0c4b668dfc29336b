"""Generates the golden fixtures in this folder from the CPU oracle (oracle/, a line-by-line
restatement of voxtree.rs / interner/mod.rs; its own pins are tests/test_reference_cases.py, which
re-runs the reference's unit tests, and tests/test_known_answers.py).

Each fixture is a compressed .npz holding the workload's inputs and its results: the canonical DFS
export of the DAG (kind, types, mask, value, refcount, children, roots), the interner's node
counts, and get() answers at seeded positions. tests/test_golden.py checks that the oracle keeps
reproducing them and that the GPU library reproduces them bit for bit, so any change of either
side's semantics shows up as a fixture diff.

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from voxelis_gb300 import workloads as W  # noqa: E402
from voxelis_gb300._abi import VX_PATCH_P1, VX_PATCH_P2, VX_PATCH_P4  # noqa: E402
from voxelis_gb300.api import VoxInterner, VoxTree  # noqa: E402


def _config1_grids():
    n = 32
    y, z, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    return {
        "uniform": np.ones((n, n, n), np.uint8),
        "checker": np.where((x + y + z) % 2 == 0, 1, 0).astype(np.uint8),
        "sum": ((x + y + z) % 256).astype(np.uint8),
    }


def _queries(trees, depth, n, seed):
    rng = np.random.default_rng(seed)
    t = rng.integers(0, len(trees), n)
    xyz = rng.integers(0, 1 << depth, (n, 3)).astype(np.int32)
    return t.astype(np.int32), xyz


def run_case(name, lib):
    """Runs fixture `name` on `lib` (oracle or GPU library); returns the dict that is stored."""
    out = {}
    if name == "config1_sequential":
        g = _config1_grids()
        it = VoxInterner(256 << 20, 8, 0, lib=lib)
        t = VoxTree(5)
        changed = []
        for k in ("uniform", "checker", "sum"):
            b = t.create_batch(it)
            b.set_dense(g[k])
            changed.append(t.apply_batch(it, b))
        trees, depth = [t], 5
        out["changed"] = np.array(changed, np.uint8)
    elif name.startswith("config1_"):
        g = _config1_grids()[name.split("_")[1]]
        it = VoxInterner(256 << 20, 8, 0, lib=lib)
        t = VoxTree(5)
        b = t.create_batch(it)
        b.set_dense(g)
        out["changed"] = np.array([t.apply_batch(it, b)], np.uint8)
        trees, depth = [t], 5
    elif name == "dunes16_d5":
        grids = W.dune_world_chunks(4, 4, depth=5, seed=1234)
        it = VoxInterner(256 << 20, 8, 0, lib=lib)
        trees, depth = [VoxTree(5) for _ in range(16)], 5
        out["changed"] = it.build_dense(trees, grids).astype(np.uint8)
    elif name == "terrain4_d6_p1":
        grids = W.dune_world_chunks(2, 2, depth=6, seed=77, **W.terrain_params(6))
        it = VoxInterner(256 << 20, 8, VX_PATCH_P1, lib=lib)
        trees, depth = [VoxTree(6) for _ in range(4)], 6
        out["changed"] = it.build_dense(trees, grids).astype(np.uint8)
        # then one batch of random edits per chunk
        bs = []
        for k, t in enumerate(trees):
            xyz, vals = W.random_edits(6, 0.01, 900 + k, max_material=255, clear_fraction=0.0)
            b = t.create_batch(it)
            b.set_many(xyz, vals)
            bs.append(b)
        out["changed_edits"] = it.apply_batches(trees, bs).astype(np.uint8)
    elif name == "edits_u16_p1p2p4":
        patches = VX_PATCH_P1 | VX_PATCH_P2 | VX_PATCH_P4
        it = VoxInterner(256 << 20, 16, patches, lib=lib)
        trees = []
        depth = None
        for d in (7, 6, 5):
            for k in range(1 if d == 7 else 2):
                t = VoxTree(d)
                grid = W.dune_world_chunks(1, 1, depth=d, seed=40 + k, dtype=np.uint16, **W.terrain_params(d))[0]
                b = t.create_batch(it)
                b.set_dense(grid)
                t.apply_batch(it, b)
                trees.append(t)
        bs = []
        for k, t in enumerate(trees):
            d = t.max_depth_value
            xyz, vals = W.random_edits(d, 0.002 if d == 7 else 0.01, 500 + k)
            b = t.create_batch(it)
            b.set_many(xyz, vals)
            bs.append(b)
        out["changed_edits"] = it.apply_batches(trees, bs).astype(np.uint8)
    else:
        raise KeyError(name)
    c = it.export_canonical(trees)
    for k, v in c.items():
        out["canon_" + k] = v
    st = it.stats()
    out["alive_nodes"] = np.array([st["alive_nodes"]], np.int64)
    # gets at seeded positions (per tree depth)
    qt, qxyz = [], []
    for i, t in enumerate(trees):
        d = depth or t.max_depth_value
        _, xyz = _queries([t], d, 512, 31 + i)
        qt.append(np.full(len(xyz), t._bind(it), np.uint32))
        qxyz.append(xyz)
    qt, qxyz = np.concatenate(qt), np.concatenate(qxyz)
    found, vals = it.get_many(qt, qxyz)
    out["get_xyz"] = qxyz
    out["get_found"] = found.astype(np.uint8)
    out["get_value"] = vals
    return out


CASES = ["config1_uniform", "config1_checker", "config1_sum", "config1_sequential", "dunes16_d5",
         "terrain4_d6_p1", "edits_u16_p1p2p4"]


def main():
    from oracle import build as oracle_build
    from voxelis_gb300._abi import NativeLib

    lib = NativeLib(oracle_build.build(), "vxo_")
    for name in CASES:
        res = run_case(name, lib)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print(name, "nodes", len(res["canon_kind"]), "alive", int(res["alive_nodes"][0]))


if __name__ == "__main__":
    main()
