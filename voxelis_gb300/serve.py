"""A serving loop over a device-resident voxel world (continuous batching of edit and get requests).

World: nx x ny x nz chunks of MaxDepth d in one interner (patches P1 + P4 + P5: carves are honoured,
and a fill that leaves a chunk as it was is a no-op instead of the reference's assert_ne! panic).
Requests arrive over time; each is either
  edit  a sphere brush (center, radius, value; value 0 carves) applied as Batch::just_set calls
        into one Batch per touched chunk, then apply_batch on each of those chunks, or
  get   a set of world points read with VoxTree::get.
Semantics are those of executing the requests one by one in arrival order. The loop executes them in
waves, scanning the pending requests in arrival order: an edit joins the wave unless one of its
chunks is already edited in the wave or belongs to an edit held back before it (then it is held back
too, so the edits of a chunk keep their order); a get joins the wave with its cut, the number of the
wave's edits that arrived before it, unless an edit before it was held back (the wave ends there).
The wave's edits run as one batched apply (vx_apply_groups_async). When a get must not see some of
them, the current roots of the edited chunks are held first (vx_world_hold_async: one more
reference each) and the get reads every chunk edited at or after its cut at the held root
(vx_world_get_at_async); the holds are released after the wave's gets (vx_world_release_async). So
every get sees exactly the edits that arrived before it, every result equals the one-by-one result,
and a backlog forms large waves. Requests that arrive while a wave is on the GPU are admitted into
the next one, which is staged on the host (vx_stage_spheres, pinned buffers, async copies) while the
device works. Edits are admitted only while the interner's free node headroom covers a conservative
estimate of the nodes they can create; replaced roots are released (nodes recycled with a new
generation) by every apply, and the branch table is rebuilt from live nodes when deletions pile up
(vx_interner_maintain).
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
        # per chunk: the root held for reads before a wave's edit, and that edit's rank in the wave
        self.old_roots = torch.zeros(n, dtype=torch.int64, device=self.dev)
        self.edit_rank = torch.full((n,), -1, dtype=torch.int32, device=self.dev)

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
                          rc=pin(cap_recs, torch.uint8), rv=pin(cap_recs * 8, torch.int16),
                          ranks=pin(cap_items, torch.int32)) for _ in range(2)]
        for k, hs in enumerate(self.hset):  # numpy views of the pinned buffers (no torch call per wave)
            hs["k"] = k
            hs["np"] = {"items": hs["items"].numpy(), "item_trees": hs["item_trees"].numpy(),
                        "ranks": hs["ranks"].numpy()}
        self.parity = 0
        self.d_item_chunks = torch.empty(cap_items, dtype=torch.int32, device=dev)
        self.d_ranks = torch.empty(cap_items, dtype=torch.int32, device=dev)
        self.d_held = torch.empty(cap_items, dtype=torch.int64, device=dev)
        self.d_item_trees = torch.empty(cap_items, dtype=torch.int32, device=dev)
        self.d_flags = torch.full((cap_items,), 2, dtype=torch.uint8, device=dev)
        self.d_fill = torch.zeros(cap_items, dtype=torch.int32, device=dev)
        self.d_ri = torch.empty(cap_recs, dtype=torch.int32, device=dev)
        self.d_rg = torch.empty(cap_recs, dtype=torch.int32, device=dev)
        self.d_rs = torch.empty(cap_recs, dtype=torch.uint8, device=dev)
        self.d_rc = torch.empty(cap_recs, dtype=torch.uint8, device=dev)
        self.d_rv = torch.empty(cap_recs * 8, dtype=torch.int16, device=dev)
        # per pinned set: the staged arrays' device and host addresses for one vx_copy_to_device_async
        # (the item chunks and their edit ranks only go over when the wave holds roots)
        dsts = [self.d_item_trees, self.d_ri, self.d_rg, self.d_rs, self.d_rc, self.d_rv, self.d_item_chunks,
                self.d_ranks]
        names = ("item_trees", "ri", "rg", "rs", "rc", "rv", "items", "ranks")
        self.copies = [{"dst": np.array([t.data_ptr() for t in dsts], np.uint64),
                        "src": np.array([hs[k].data_ptr() for k in names], np.uint64),
                        "bytes": np.zeros(len(names), np.uint64)} for hs in self.hset]
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
    def form_wave(self, pending, scan_limit=None):
        """The next wave from `pending` (unserved requests in arrival order): (edits, gets, taken), the
        edits touching pairwise disjoint chunks, each get as (request, cut) where cut is the number of
        the wave's edits that arrived before it, and `taken` the positions in `pending` of the
        requests the wave serves. An edit whose chunks meet an edit of the wave, or an edit held back
        before it, is held back; a get after a held-back edit ends the wave, as do the size limits
        and memory admission."""
        edits, gets, taken = [], [], []
        touched, blocked = set(), set()
        held_back = False
        limit = scan_limit if scan_limit is not None else 4 * (self.max_e + self.max_g)
        for i, r in enumerate(pending):
            if i >= limit:
                break
            if r["kind"] == EDIT:
                if len(edits) >= self.max_e:
                    break
                if r["chunks"] & touched or r["chunks"] & blocked:
                    blocked |= r["chunks"]
                    held_back = True
                    continue
                est = 2 * math.ceil((4.19 * r["radius"] ** 3) / 8 + 1) * self.w.depth
                if self.alive_est + est > self.capacity - self.headroom:
                    break  # memory admission: this and later requests wait for releases
                self.alive_est += est
                edits.append(r)
                taken.append(i)
                touched |= r["chunks"]
            else:
                if held_back or len(gets) >= self.max_g:
                    break
                gets.append((r, len(edits)))
                taken.append(i)
        return edits, gets, taken

    # -- staging and launch ----------------------------------------------------------------------------
    def launch(self, edits, gets):
        """Queues a wave: its edits as one batched apply, then its gets (each a (request, cut) pair),
        with the edited chunks' roots held for the gets that must not see every edit."""
        w, torch = self.w, self.torch
        P = lambda t: C.c_void_p(t.data_ptr())  # noqa: E731
        hs = self.hset[self.parity]
        self.parity ^= 1
        ni = 0
        hold = bool(edits) and any(cut < len(edits) for _, cut in gets)
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
            hold = hold and ni > 0
            if ni:
                hn = hs["np"]
                np.take(w.trees.view(np.int32), hn["items"][:ni], out=hn["item_trees"][:ni])
                if hold:  # each item's chunk belongs to exactly one of the wave's edits: its rank
                    rank_of = {c: k for k, e in enumerate(edits) for c in e["chunks"]}
                    hn["ranks"][:ni] = [rank_of[int(c)] for c in hn["items"][:ni]]
                cp = self.copies[hs["k"]]
                hb = 4 * ni if hold else 0
                cp["bytes"][:] = (4 * ni, 4 * nr, 4 * nr, nr, nr, 16 * nr, hb, hb)
                w.call("copy_to_device_async", 8, cp["dst"].ctypes.data, cp["src"].ctypes.data, cp["bytes"].ctypes.data)
                if hold:
                    w.call("world_hold_async", C.byref(w.wdesc), ni, P(self.d_item_chunks), P(self.d_ranks),
                           P(self.d_held), P(w.old_roots), P(w.edit_rank))
                w.call("apply_groups_async", ni, P(self.d_item_trees), P(self.d_flags), P(self.d_fill), nr,
                       P(self.d_ri), P(self.d_rg), P(self.d_rs), P(self.d_rc), P(self.d_rv), None, w.depth)
        if gets:  # the gets' point sets in one call, then one batched world get each
            ng = len(gets)
            self.points += ng * self.ppg
            self.get_src[:ng] = [self.pool_ptr[g["pool"]] for g, _ in gets]
            w.call("copy_to_device_async", ng, self.get_dst.ctypes.data, self.get_src.ctypes.data,
                   self.get_bytes.ctypes.data)
        for k, (g, cut) in enumerate(gets):
            if hold and cut < len(edits):
                w.call("world_get_at_async", C.byref(w.wdesc), C.c_uint64(self.ppg), P(self.d_pts[k]),
                       P(self.d_found[k]), P(self.d_vals[k]), P(w.old_roots), P(w.edit_rank), cut)
            else:
                w.call("world_get_async", C.byref(w.wdesc), C.c_uint64(self.ppg), P(self.d_pts[k]),
                       P(self.d_found[k]), P(self.d_vals[k]))
        if hold:
            w.call("world_release_async", C.byref(w.wdesc), ni, P(self.d_item_chunks), P(self.d_held), P(w.edit_rank))
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
        pending, results = [], {}  # unserved arrived requests (indices), in arrival order
        lat = np.full(len(reqs), np.nan)
        nxt, served = 0, 0
        inflight = None
        while served < len(reqs) or inflight is not None:
            now = time.perf_counter() - t0
            while nxt < len(reqs) and (not realtime or reqs[nxt]["t"] <= now):
                pending.append(nxt)
                nxt += 1
            wave = None
            if pending:
                if one_by_one:
                    r = reqs[pending[0]]
                    e, g, taken = ([r], [], [0]) if r["kind"] == EDIT else ([], [(r, 0)], [0])
                else:
                    window = pending[:4 * (self.max_e + self.max_g)]
                    e, g, taken = self.form_wave([reqs[j] for j in window])
                if taken:
                    ids = [pending[i] for i in taken]
                    tk = set(taken)
                    last = taken[-1]
                    pending = [p for k, p in enumerate(pending[:last + 1]) if k not in tk] + pending[last + 1:]
                    served += len(ids)
                    get_ids = [j for j in ids if reqs[j]["kind"] != EDIT]
                    wave = (ids, get_ids)
                    ev = self.launch(e, g)
            if inflight is not None:
                ids_, _, ev_ = inflight
                ev_.synchronize()
                done = time.perf_counter() - t0
                for j in ids_:
                    lat[j] = done - reqs[j]["t"] if realtime else 0.0
                self.waves += 1
                if self.waves % 64 == 0:
                    self.w.call("interner_maintain")
                    self.alive_est = self.w.stats().alive_nodes
                inflight = None
            if wave is not None:
                ids, get_ids = wave
                if keep_results and get_ids:
                    ev.synchronize()
                    for k, j in enumerate(get_ids):
                        results[j] = (self.h_found[k].clone().numpy(), self.h_vals[k].clone().numpy())
                inflight = (ids, get_ids, ev)
            elif inflight is None and nxt < len(reqs) and realtime:
                time.sleep(max(0.0, min(0.0005, reqs[nxt]["t"] - (time.perf_counter() - t0))))
        self.w.call("interner_maintain")
        return lat, results
