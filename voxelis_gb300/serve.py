"""A serving loop over a device-resident voxel world (continuous batching of edit and get requests).

World: nx x ny x nz chunks of MaxDepth d in one interner (patches P1 + P4 + P5: carves are honoured,
and a fill that leaves a chunk as it was is a no-op instead of the reference's assert_ne! panic).
Requests arrive over time; each is either
  edit  a sphere brush (center, radius, value; value 0 carves) applied as Batch::just_set calls
        into one Batch per touched chunk, then apply_batch on each of those chunks, or
  get   a set of world points read with VoxTree::get.
Semantics are those of executing the requests one by one in arrival order. The loop executes them in
waves: a wave is the longest arrival-order prefix of pending requests made of edits touching pairwise
disjoint chunks followed by gets; its edits run as one batched apply (vx_apply_groups_async) and its
gets as batched world gets after them, so every result equals the one-by-one result. Requests that
arrive while a wave is on the GPU are admitted into the next one, which is staged on the host
(vx_stage_spheres, pinned buffers, async copies) while the device works. Edits are admitted only
while the interner's free node headroom covers a conservative estimate of the nodes they can create;
replaced roots are released (nodes recycled with a new generation) by every apply, and the branch
table is rebuilt from live nodes when deletions pile up (vx_interner_maintain).
"""
import ctypes as C
import math
import time

import numpy as np

from . import workloads as W
from ._abi import VX_PATCH_P1, VX_PATCH_P4, VX_PATCH_P5, vx_interner_stats, vx_world, gpu_lib

EDIT, GET = 0, 1


class World:
    """nx*ny*nz chunks of depth d; chunk id = (cy * nz + cz) * nx + cx."""

    def __init__(self, nx, ny, nz, depth, budget, bits=8, patches=VX_PATCH_P1 | VX_PATCH_P4 | VX_PATCH_P5, lib=None):
        import torch

        self.torch = torch
        self.lib = lib or gpu_lib()
        self.nx, self.ny, self.nz, self.depth = nx, ny, nz, depth
        self.side = 1 << depth
        self.bits = bits
        self.dev = torch.device("cuda", torch.cuda.current_device())
        h = C.c_void_p()
        self.lib.call("interner_create", C.c_uint64(budget), bits, patches, 0, C.byref(h))
        self.h = h
        self.stream = torch.cuda.Stream(device=self.dev)
        self.call("interner_set_stream", C.c_void_p(self.stream.cuda_stream))
        n = nx * ny * nz
        self.n_chunks = n
        depths = np.full(n, depth, np.uint8)
        self.trees = np.zeros(n, np.uint32)
        self.call("trees_create", n, depths.ctypes.data, self.trees.ctypes.data)
        self.trees_d = torch.from_numpy(self.trees.view(np.int32)).to(self.dev)
        self.wdesc = vx_world(nx, ny, nz, depth, C.c_void_p(self.trees_d.data_ptr()))

    def call(self, name, *args):
        return self.lib.call(name, self.h, *args, handle=self.h)

    def build_terrain(self, grids, chunk_ids):
        """Dense construction of the given chunks (grids [k][s][s][s] in chunk_ids order)."""
        torch = self.torch
        with torch.cuda.stream(self.stream):
            g = torch.from_numpy(np.ascontiguousarray(grids)).to(self.dev)
            t = torch.from_numpy(self.trees[np.asarray(chunk_ids)].view(np.int32)).to(self.dev)
        self.call("build_dense_async", len(chunk_ids), C.c_void_p(t.data_ptr()), C.c_void_p(g.data_ptr()), None,
                  self.depth)
        self.call("interner_sync")

    def stats(self):
        st = vx_interner_stats()
        self.call("interner_stats_get", C.byref(st))
        return st

    def close(self):
        if self.h:
            self.call("interner_destroy")
            self.h = None


def sphere_chunks(world, c, r):
    """Chunk ids a sphere's bounding box (clipped to the world) can touch."""
    s = world.side
    lo = [max(0, c[k] - r) for k in range(3)]
    hi = [min((world.nx, world.ny, world.nz)[k] * s - 1, c[k] + r) for k in range(3)]
    if any(lo[k] > hi[k] for k in range(3)):
        return frozenset()
    out = []
    for cy in range(lo[1] // s, hi[1] // s + 1):
        for cz in range(lo[2] // s, hi[2] // s + 1):
            for cx in range(lo[0] // s, hi[0] // s + 1):
                out.append((cy * world.nz + cz) * world.nx + cx)
    return frozenset(out)


def make_trace(world, rate, duration, seed, edit_fraction=0.7, points_pool=16, points_per_get=65536,
               r_min=2, r_max=12, material_max=8):
    """Poisson arrivals at `rate` req/s for `duration` s. Returns (requests, point pool)."""
    rng = np.random.default_rng(seed)
    t, reqs = 0.0, []
    W_ = (world.nx * world.side, world.ny * world.side, world.nz * world.side)
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        if rng.random() < edit_fraction:
            c = tuple(int(rng.integers(0, W_[k])) for k in range(3))
            r = int(rng.integers(r_min, r_max + 1))
            v = 0 if rng.random() < 0.5 else int(rng.integers(1, material_max + 1))
            reqs.append({"kind": EDIT, "t": t, "center": c, "radius": r, "value": v,
                         "chunks": sphere_chunks(world, c, r)})
        else:
            reqs.append({"kind": GET, "t": t, "pool": int(rng.integers(0, points_pool))})
    pool = [np.stack([rng.integers(0, W_[0], points_per_get), rng.integers(0, W_[1], points_per_get),
                      rng.integers(0, W_[2], points_per_get)], 1).astype(np.int32) for _ in range(points_pool)]
    return reqs, pool


class Server:
    def __init__(self, world, pool, max_wave_edits=512, max_wave_gets=64, headroom_nodes=None):
        torch = world.torch
        self.w = world
        self.torch = torch
        self.max_e, self.max_g = max_wave_edits, max_wave_gets
        self.lib = world.lib
        dev = world.dev
        self.pool_h = [torch.from_numpy(p).pin_memory() for p in pool]
        self.ppg = pool[0].shape[0]
        cap_items, cap_recs = 1 << 16, 1 << 22
        self.cap_items, self.cap_recs = cap_items, cap_recs
        pin = lambda n, dt: torch.empty(n, dtype=dt).pin_memory()  # noqa: E731
        # two sets of pinned staging buffers: wave k+1 is staged while wave k's copies may be queued
        self.hset = [dict(items=pin(cap_items, torch.int32), item_trees=pin(cap_items, torch.int32),
                          ri=pin(cap_recs, torch.int32), rg=pin(cap_recs, torch.int32), rs=pin(cap_recs, torch.uint8),
                          rc=pin(cap_recs, torch.uint8), rv=pin(cap_recs * 8, torch.int16)) for _ in range(2)]
        for k, hs in enumerate(self.hset):  # numpy views of the pinned buffers (no torch call per wave)
            hs["k"] = k
            hs["np"] = {"items": hs["items"].numpy(), "item_trees": hs["item_trees"].numpy()}
        self.parity = 0
        self.d_item_trees = torch.empty(cap_items, dtype=torch.int32, device=dev)
        self.d_flags = torch.full((cap_items,), 2, dtype=torch.uint8, device=dev)
        self.d_fill = torch.zeros(cap_items, dtype=torch.int32, device=dev)
        self.d_ri = torch.empty(cap_recs, dtype=torch.int32, device=dev)
        self.d_rg = torch.empty(cap_recs, dtype=torch.int32, device=dev)
        self.d_rs = torch.empty(cap_recs, dtype=torch.uint8, device=dev)
        self.d_rc = torch.empty(cap_recs, dtype=torch.uint8, device=dev)
        self.d_rv = torch.empty(cap_recs * 8, dtype=torch.int16, device=dev)
        # per pinned set: the 6 staged arrays' device and host addresses for one vx_copy_to_device_async
        dsts = [self.d_item_trees, self.d_ri, self.d_rg, self.d_rs, self.d_rc, self.d_rv]
        self.copies = [{"dst": np.array([t.data_ptr() for t in dsts], np.uint64),
                        "src": np.array([hs[k].data_ptr() for k in ("item_trees", "ri", "rg", "rs", "rc", "rv")],
                                        np.uint64),
                        "bytes": np.zeros(6, np.uint64)} for hs in self.hset]
        self.d_pts = torch.empty((max_wave_gets, self.ppg, 3), dtype=torch.int32, device=dev)
        self.pool_ptr = [p.data_ptr() for p in self.pool_h]
        self.get_dst = np.array([self.d_pts[k].data_ptr() for k in range(max_wave_gets)], np.uint64)
        self.get_src = np.zeros(max_wave_gets, np.uint64)
        self.get_bytes = np.full(max_wave_gets, self.ppg * 3 * 4, np.uint64)
        self.d_found = torch.empty((max_wave_gets, self.ppg), dtype=torch.uint8, device=dev)
        vt = torch.uint8 if world.bits == 8 else torch.int16
        self.d_vals = torch.empty((max_wave_gets, self.ppg), dtype=vt, device=dev)
        self.h_found = pin(max_wave_gets * self.ppg, torch.uint8).view(max_wave_gets, self.ppg)
        self.h_vals = pin(max_wave_gets * self.ppg, vt).view(max_wave_gets, self.ppg)
        st = world.stats()
        self.capacity = st.capacity
        self.alive_est = st.alive_nodes
        self.headroom = headroom_nodes if headroom_nodes is not None else st.capacity // 16
        self.stage = self.lib.lib.vx_stage_spheres
        self.stage.restype = C.c_int
        self.waves = 0
        # work done, for the algorithmic-bytes count: staged group records, items (chunk applies), points read
        self.records = self.items = self.points = 0

    # -- wave formation ------------------------------------------------------------------------------
    def form_wave(self, pending, start):
        """Longest prefix pending[start:] of chunk-disjoint edits then gets (bounded sizes)."""
        edits, gets, touched = [], [], set()
        i = start
        while i < len(pending):
            r = pending[i]
            if r["kind"] == EDIT:
                if gets or len(edits) >= self.max_e or (r["chunks"] & touched):
                    break
                est = 2 * math.ceil((4.19 * r["radius"] ** 3) / 8 + 1) * self.w.depth
                if self.alive_est + est > self.capacity - self.headroom:
                    break  # memory admission: wait for releases
                self.alive_est += est
                edits.append(r)
                touched |= r["chunks"]
            else:
                if len(gets) >= self.max_g:
                    break
                gets.append(r)
            i += 1
        return edits, gets, i

    # -- staging and launch ----------------------------------------------------------------------------
    def launch(self, edits, gets):
        w, torch = self.w, self.torch
        P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        hs = self.hset[self.parity]
        self.parity ^= 1
        if edits:
            n = len(edits)
            cen = np.array([e["center"] for e in edits], np.int32)
            rad = np.array([e["radius"] for e in edits], np.int32)
            val = np.array([e["value"] for e in edits], np.uint32)
            ni, nr = C.c_uint64(), C.c_uint64()
            st = self.stage(w.depth, w.nx, w.ny, w.nz, n, C.c_void_p(cen.ctypes.data), C.c_void_p(rad.ctypes.data),
                            C.c_void_p(val.ctypes.data), C.c_uint64(self.cap_items), P(hs["items"]),
                            C.c_uint64(self.cap_recs), P(hs["ri"]), P(hs["rg"]), P(hs["rs"]), P(hs["rc"]),
                            P(hs["rv"]), C.byref(ni), C.byref(nr))
            if st != 0:
                raise RuntimeError("vx_stage_spheres failed: %d" % st)
            ni, nr = ni.value, nr.value
            self.records += nr
            self.items += ni
            if ni:
                hn = hs["np"]
                np.take(w.trees.view(np.int32), hn["items"][:ni], out=hn["item_trees"][:ni])
                cp = self.copies[hs["k"]]
                cp["bytes"][:] = (4 * ni, 4 * nr, 4 * nr, nr, nr, 16 * nr)  # item trees, ri, rg, rs, rc, rv
                w.call("copy_to_device_async", 6, cp["dst"].ctypes.data, cp["src"].ctypes.data, cp["bytes"].ctypes.data)
                w.call("apply_groups_async", ni, P(self.d_item_trees), P(self.d_flags), P(self.d_fill), nr,
                       P(self.d_ri), P(self.d_rg), P(self.d_rs), P(self.d_rc), P(self.d_rv), None, w.depth)
        if gets:  # the gets' point sets in one call, then one batched world get each
            ng = len(gets)
            self.points += ng * self.ppg
            self.get_src[:ng] = [self.pool_ptr[g["pool"]] for g in gets]
            w.call("copy_to_device_async", ng, self.get_dst.ctypes.data, self.get_src.ctypes.data,
                   self.get_bytes.ctypes.data)
        for k, g in enumerate(gets):
            w.call("world_get_async", C.byref(w.wdesc), C.c_uint64(self.ppg), P(self.d_pts[k]), P(self.d_found[k]),
                   P(self.d_vals[k]))
        if gets:
            with torch.cuda.stream(w.stream):
                self.h_found[:len(gets)].copy_(self.d_found[:len(gets)], non_blocking=True)
                self.h_vals[:len(gets)].copy_(self.d_vals[:len(gets)], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record(w.stream)
        return ev

    def run(self, reqs, realtime=True, keep_results=False, one_by_one=False):
        """Serves `reqs` (sorted by arrival). Returns per-request latencies (s) and, optionally, the
        get results."""
        t0 = time.perf_counter()
        pending, pend_reqs, results = [], [], {}  # arrived requests: indices and the requests themselves
        lat = np.full(len(reqs), np.nan)
        nxt, start = 0, 0
        inflight = None
        while start < len(reqs) or inflight is not None:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and (not realtime or reqs[nxt]["t"] <= now):
                pending.append(nxt)
                pend_reqs.append(reqs[nxt])
                nxt += 1
            wave = None
            if start < len(pending):
                if one_by_one:
                    r = pend_reqs[start]
                    e, g, end = ([r], [], start + 1) if r["kind"] == EDIT else ([], [r], start + 1)
                else:
                    e, g, end = self.form_wave(pend_reqs, start)
                if end > start:
                    wave = (pending[start:end], e, g)
                    ev = self.launch(e, g)
                    start = end
            if inflight is not None:
                ids, e_, g_, ev_ = inflight
                ev_.synchronize()
                done = time.perf_counter() - t0
                for j in ids:
                    lat[j] = done - reqs[j]["t"] if realtime else 0.0
                self.waves += 1
                if self.waves % 64 == 0:
                    self.w.call("interner_maintain")
                    self.alive_est = self.w.stats().alive_nodes
                inflight = None
            if wave is not None:
                ids, e, g = wave
                if keep_results and g:
                    ev.synchronize()
                    for k, r in enumerate(g):
                        results[ids[len(e) + k]] = (self.h_found[k].clone().numpy(), self.h_vals[k].clone().numpy())
                inflight = (ids, e, g, ev)
            elif inflight is None and nxt < len(reqs) and realtime:
                time.sleep(max(0.0, min(0.0005, reqs[nxt]["t"] - (time.perf_counter() - t0))))
        self.w.call("interner_maintain")
        return lat, results
