"""Wave formation of the serving loop (voxelis_gb300/serve.py), on the host only.

A wave is the longest arrival-order prefix of the pending requests made of edits touching pairwise
disjoint chunks followed by gets, so that running each wave's edits as one batched apply and its
gets after them gives the one-by-one results. These tests check that property on seeded traces,
without a GPU: the Server is built without its device buffers.
"""
import types

import numpy as np

from voxelis_gb300.serve import EDIT, GET, Server, make_trace, sphere_chunks


def fake_world(nx=16, ny=2, nz=16, depth=6):
    return types.SimpleNamespace(nx=nx, ny=ny, nz=nz, depth=depth, side=1 << depth)


def host_server(world, max_e=512, max_g=64, capacity=1 << 40, headroom=0, alive=0):
    s = object.__new__(Server)
    s.w = world
    s.max_e, s.max_g = max_e, max_g
    s.capacity, s.headroom, s.alive_est = capacity, headroom, alive
    return s


def waves_of(server, reqs):
    out, start = [], 0
    while start < len(reqs):
        e, g, end = server.form_wave(reqs, start)
        assert end > start, "no progress"
        out.append((start, end, e, g))
        start = end
    return out


def test_sphere_chunks_cover_the_clipped_bounding_box():
    w = fake_world(nx=4, ny=2, nz=4, depth=4)  # 16-voxel chunks, world 64 x 32 x 64
    assert sphere_chunks(w, (8, 8, 8), 3) == frozenset({0})
    # straddles x = 16 and z = 16: four chunks of the bottom layer
    assert sphere_chunks(w, (16, 4, 16), 2) == frozenset({0, 1, 4, 5})
    # clipped at the world's edge; entirely outside gives nothing
    assert sphere_chunks(w, (0, 0, 0), 5) == frozenset({0})
    assert sphere_chunks(w, (-20, 0, 0), 3) == frozenset()


def test_waves_are_contiguous_and_keep_arrival_order():
    w = fake_world()
    reqs, _ = make_trace(w, rate=5000.0, duration=0.2, seed=7, points_per_get=16)
    waves = waves_of(host_server(w), reqs)
    assert waves[0][0] == 0 and waves[-1][1] == len(reqs)
    for (s0, e0, _, _), (s1, _, _, _) in zip(waves, waves[1:]):
        assert e0 == s1
    for s, e, edits, gets in waves:
        got = edits + gets
        assert [id(r) for r in got] == [id(r) for r in reqs[s:e]]  # edits first, then gets
        assert all(r["kind"] == EDIT for r in edits) and all(r["kind"] == GET for r in gets)


def test_wave_edits_touch_disjoint_chunks_and_waves_are_maximal():
    w = fake_world(nx=4, ny=1, nz=4)  # few chunks: overlaps are frequent
    reqs, _ = make_trace(w, rate=20000.0, duration=0.1, seed=11, points_per_get=16)
    waves = waves_of(host_server(w, max_e=64, max_g=8), reqs)
    for s, e, edits, gets in waves:
        seen = set()
        for r in edits:
            assert not (r["chunks"] & seen)
            seen |= r["chunks"]
        if e < len(reqs):  # the next request could not have joined this wave
            nxt = reqs[e]
            if nxt["kind"] == EDIT:
                assert gets or (nxt["chunks"] & seen) or len(edits) == 64
            else:
                assert len(gets) == 8


def test_admission_holds_edits_until_headroom_returns():
    w = fake_world()
    reqs, _ = make_trace(w, rate=5000.0, duration=0.05, seed=3, points_per_get=16)
    first_edit = next(i for i, r in enumerate(reqs) if r["kind"] == EDIT)
    s = host_server(w, capacity=1000, headroom=0, alive=1000)  # no free nodes at all
    e, g, end = s.form_wave(reqs, first_edit)
    assert e == [] and g == [] and end == first_edit
    s.alive_est, s.capacity = 0, 1 << 30  # releases came back, and room for a radius-12 sphere
    e, g, end = s.form_wave(reqs, first_edit)
    assert e and e[0] is reqs[first_edit] and end > first_edit
    assert s.alive_est > 0  # the admitted edits' estimate is charged


def test_one_by_one_order_is_preserved_for_edits_after_gets():
    w = fake_world()
    c = (10, 10, 10)
    mk = lambda kind, **kw: dict(kind=kind, t=0.0, **kw)  # noqa: E731
    reqs = [mk(EDIT, center=c, radius=2, value=1, chunks=sphere_chunks(w, c, 2)),
            mk(GET, pool=0),
            mk(EDIT, center=(200, 10, 200), radius=2, value=0, chunks=sphere_chunks(w, (200, 10, 200), 2))]
    waves = waves_of(host_server(w), reqs)
    # the get must not see the second edit, even though their chunks are disjoint
    assert [(s, e) for s, e, _, _ in waves] == [(0, 2), (2, 3)]
    assert np.array_equal([len(x[2]) for x in waves], [1, 1])
