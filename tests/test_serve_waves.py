"""Wave formation of the serving loop (voxelis_gb300/serve.py), on the host only.

A wave takes pending requests in arrival order: edits whose chunks are disjoint from the wave's other
edits and from every edit held back before them, and gets (each with its cut, the number of the
wave's edits that arrived before it) until a get follows a held-back edit. Running the wave's edits
as one batched apply and reading each get's chunks at the root before any edit at or after its cut
gives the one-by-one results. These tests check that on seeded traces, without a GPU: the Server is
built without its device buffers.
"""
import types

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
    """Waves as the serving loop forms them when every request is already pending: a list of
    (requests served, edits, gets with cuts) per wave."""
    pending, out = list(range(len(reqs))), []
    while pending:
        window = pending[:4 * (server.max_e + server.max_g)]
        e, g, taken = server.form_wave([reqs[j] for j in window])
        assert taken, "no progress"
        ids = [pending[i] for i in taken]
        tk = set(taken)
        pending = [p for k, p in enumerate(pending) if k not in tk]
        out.append((ids, e, g))
    return out


def test_sphere_chunks_cover_the_clipped_bounding_box():
    w = fake_world(nx=4, ny=2, nz=4, depth=4)  # 16-voxel chunks, world 64 x 32 x 64
    assert sphere_chunks(w, (8, 8, 8), 3) == frozenset({0})
    # straddles x = 16 and z = 16: four chunks of the bottom layer
    assert sphere_chunks(w, (16, 4, 16), 2) == frozenset({0, 1, 4, 5})
    # clipped at the world's edge; entirely outside gives nothing
    assert sphere_chunks(w, (0, 0, 0), 5) == frozenset({0})
    assert sphere_chunks(w, (-20, 0, 0), 3) == frozenset()


def _check_one_by_one_semantics(reqs, waves):
    served = [j for ids, _, _ in waves for j in ids]
    assert sorted(served) == list(range(len(reqs)))  # every request exactly once
    pos = {id(r): k for k, r in enumerate(reqs)}
    applied = []  # edits in the order the device applies them (wave by wave, rank by rank)
    for ids, edits, gets in waves:
        seen = set()
        for r in edits:  # one batched apply: pairwise disjoint chunks
            assert not (r["chunks"] & seen)
            seen |= r["chunks"]
        assert [pos[id(r)] for r in edits] == sorted(pos[id(r)] for r in edits)  # ranks in arrival order
        for g, cut in gets:  # the get sees the earlier waves' edits and the first `cut` of this one
            visible = {pos[id(r)] for r in applied} | {pos[id(r)] for r in edits[:cut]}
            assert visible == {k for k in range(pos[id(g)]) if reqs[k]["kind"] == EDIT}
        applied += edits
    by_chunk = {}
    for r in applied:  # each chunk's edits are applied in arrival order
        for c in r["chunks"]:
            by_chunk.setdefault(c, []).append(pos[id(r)])
    assert all(v == sorted(v) for v in by_chunk.values())


def test_waves_give_the_one_by_one_results():
    w = fake_world()
    reqs, _ = make_trace(w, rate=5000.0, duration=0.2, seed=7, points_per_get=16)
    _check_one_by_one_semantics(reqs, waves_of(host_server(w), reqs))


def test_crowded_chunks_hold_edits_back_in_order():
    w = fake_world(nx=4, ny=1, nz=4)  # few chunks: conflicts are frequent
    reqs, _ = make_trace(w, rate=20000.0, duration=0.1, seed=11, points_per_get=16)
    waves = waves_of(host_server(w, max_e=64, max_g=8), reqs)
    _check_one_by_one_semantics(reqs, waves)
    assert len(waves) < len(reqs) / 2  # a backlog forms multi-request waves


def test_a_backlog_forms_large_waves():
    w = fake_world(nx=64, ny=4, nz=64)  # the served world's chunk grid
    reqs, _ = make_trace(w, rate=20000.0, duration=0.2, seed=5, points_per_get=16)
    waves = waves_of(host_server(w), reqs)
    _check_one_by_one_semantics(reqs, waves)
    assert len(reqs) / len(waves) > 20  # gets no longer end a wave


def test_admission_holds_edits_until_headroom_returns():
    w = fake_world()
    reqs, _ = make_trace(w, rate=5000.0, duration=0.05, seed=3, points_per_get=16)
    first_edit = next(i for i, r in enumerate(reqs) if r["kind"] == EDIT)
    s = host_server(w, capacity=1000, headroom=0, alive=1000)  # no free nodes at all
    e, g, taken = s.form_wave(reqs[first_edit:])
    assert e == [] and g == [] and taken == []
    s.alive_est, s.capacity = 0, 1 << 30  # releases came back, and room for a radius-12 sphere
    e, g, taken = s.form_wave(reqs[first_edit:])
    assert e and e[0] is reqs[first_edit] and taken[0] == 0
    assert s.alive_est > 0  # the admitted edits' estimate is charged


def test_a_get_between_edits_sees_only_the_earlier_one():
    w = fake_world()
    c = (10, 10, 10)
    mk = lambda kind, **kw: dict(kind=kind, t=0.0, **kw)  # noqa: E731
    reqs = [mk(EDIT, center=c, radius=2, value=1, chunks=sphere_chunks(w, c, 2)),
            mk(GET, pool=0),
            mk(EDIT, center=(200, 10, 200), radius=2, value=0, chunks=sphere_chunks(w, (200, 10, 200), 2)),
            mk(EDIT, center=c, radius=3, value=5, chunks=sphere_chunks(w, c, 3)),
            mk(GET, pool=1)]
    waves = waves_of(host_server(w), reqs)
    # one wave holds the two edits of different chunks and the get between them (cut 1); the third
    # edit shares the first one's chunk and is held back, so the last get waits with it
    ids, edits, gets = waves[0]
    assert ids == [0, 1, 2] and [g[1] for g in gets] == [1]
    assert [x[0] for x in waves[1:]] == [[3, 4]]
    _check_one_by_one_semantics(reqs, waves)
