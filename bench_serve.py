"""Served world on GB300 (bench.py --workload serve; also part of the default bench.py line).

A device-resident world of 64 x 4 x 64 chunks (x, y, z) of MaxDepth 6 (64^3 u8) in one interner with
a 16 GiB budget (patches P1 + P4, so carves are honoured); the dune terrain rule scaled to 64-voxel
chunks fills the bottom chunk layer. Requests arrive as a Poisson stream (70% edits: a sphere of radius
uniform in 2..12 at a uniform world position that carves (value 0) or fills (material 1..8), possibly
spanning chunks; 30% gets of 65,536 uniform world points) and are served by voxelis_gb300.serve
(continuous batching in waves, admission by interner memory). Per arrival rate: p50/p99 latency of
edits and gets, the sustained request, voxel-edit and get rates, and the HBM-roofline fraction of the
served work (algorithmic bytes of the requests served over wall time).
"""
import time

import numpy as np

from voxelis_gb300 import workloads as W
from voxelis_gb300.serve import EDIT, Server, World, make_trace

RATES = (1000, 2000, 5000, 10000, 20000, 40000)
WORKLOAD = "served world 64x4x64 chunks of 64^3 u8, 16 GiB budget, Poisson 70/30 edits/gets, P1+P4+P5"


def measure(args, full_line=False):
    import bench as B
    from voxelis_gb300.build import build as build_lib

    build_lib()
    t0 = time.time()
    world = World(64, 4, 64, 6, budget=16 << 30)
    grids = W.dune_world_chunks(64, 64, depth=6, seed=4321, **W.terrain_params(6))
    world.build_terrain(grids, np.arange(64 * 64))
    del grids
    build_s = time.time() - t0
    duration = max(0.5, min(3.0, args.steps * 0.1))
    peak, peak_kind = B.peaks()
    out = {"metric": "p99 edit latency (ms) at sustained rate", "unit": "ms", "higher_is_better": False,
           "config": {"workload": WORKLOAD, "duration_s_per_rate": duration, "points_per_get": 65536},
           "world_build_s": build_s, "rates": [], "peak_kind": peak_kind}
    node_size = int(world.stats().node_size)
    clocks = B.Clocks(0)
    for rate in RATES:
        reqs, pool = make_trace(world, rate=float(rate), duration=duration, seed=rate)
        server = Server(world, pool)
        if rate == RATES[0]:  # warm-up on a short trace
            wr, _ = make_trace(world, rate=float(rate), duration=0.2, seed=1)
            server.run(wr, realtime=True)
            server.records = server.items = server.points = 0
            server.waves = 0
        created0 = int(world.stats().nodes_created)
        t1 = time.perf_counter()
        lat, _ = server.run(reqs, realtime=True)
        wall = time.perf_counter() - t1
        created = int(world.stats().nodes_created) - created0
        kinds = np.array([r["kind"] for r in reqs])
        le, lg = lat[kinds == EDIT] * 1e3, lat[kinds != EDIT] * 1e3
        vox = sum(int(4.19 * r["radius"] ** 3) for r in reqs if r["kind"] == EDIT)
        # algorithmic bytes served: group records (set + clear masks, 8 u8 values, item index),
        # created nodes, one root per chunk apply, and 12 + 1 + 1 bytes per point read
        algo = server.records * 14 + created * node_size + server.items * 8 + server.points * 14
        out["rates"].append({
            "offered_req_per_s": rate, "requests": len(reqs), "served_req_per_s": len(reqs) / wall,
            "edit_p50_ms": float(np.percentile(le, 50)), "edit_p99_ms": float(np.percentile(le, 99)),
            "get_p50_ms": float(np.percentile(lg, 50)), "get_p99_ms": float(np.percentile(lg, 99)),
            "voxel_edits_per_s": vox / wall, "gets_per_s": int((kinds != EDIT).sum()) * 65536 / wall,
            "waves": server.waves, "requests_per_wave": len(reqs) / max(1, server.waves),
            "algorithmic_bytes": int(algo), "roofline_frac": algo / wall / 1e9 / peak,
        })
    out["clocks"] = clocks.stop()
    st = world.stats()
    out["nodes_alive"] = int(st.alive_nodes)
    # the headline: p99 at the highest offered rate that is sustained (served >= 95% of offered) with
    # p99 <= 2 ms; beside it the highest sustained rate whatever its p99, and the most served
    held = [r for r in out["rates"] if r["served_req_per_s"] >= 0.95 * r["offered_req_per_s"]]
    within = [r for r in held if r["edit_p99_ms"] <= 2.0]
    best = max(within or held or out["rates"][:1], key=lambda r: r["offered_req_per_s"])
    out["value"] = best["edit_p99_ms"]
    out["at_rate"] = best["offered_req_per_s"]
    out["roofline_frac_at_rate"] = best["roofline_frac"]
    if held:
        top = max(held, key=lambda r: r["offered_req_per_s"])
        out["highest_sustained"] = {"offered_req_per_s": top["offered_req_per_s"], "edit_p99_ms": top["edit_p99_ms"]}
    out["max_served_req_per_s"] = max(r["served_req_per_s"] for r in out["rates"])
    world.close()
    if full_line:
        out.update({"n_gpus": 1, "steps": len(RATES), "warmup": 1, "dtype": "u8", "data": "synthetic",
                    "scaling": "weak", "vs_baseline": None, "ms_per_step": duration * 1e3})
    return out
