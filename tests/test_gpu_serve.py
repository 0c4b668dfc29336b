"""The serving loop returns, for every request, what executing the requests one by one in arrival
order returns: identical get results per request and an identical final DAG, whether a request ran
alone or batched into a wave with others. With every request pending at once (a deep backlog) the
waves mix edits and gets, so gets read the chunks edited after them at held roots."""
import numpy as np
import pytest

from voxelis_gb300 import workloads as W
from voxelis_gb300.serve import EDIT, Server, World, make_trace

pytestmark = pytest.mark.gpu


def make_world(gpu_lib):
    w = World(4, 2, 4, 5, budget=256 << 20, lib=gpu_lib)
    grids = W.dune_world_chunks(4, 4, depth=5, seed=77)
    w.build_terrain(grids, np.arange(16))  # the bottom chunk layer (cy = 0) holds the terrain
    return w


@pytest.mark.parametrize("max_edits,rate", [(1 << 10, 5000.0), (3, 5000.0), (1 << 10, 40000.0)])
def test_served_results_equal_one_by_one(gpu_lib, max_edits, rate):
    wa, wb = make_world(gpu_lib), make_world(gpu_lib)
    reqs, pool = make_trace(wa, rate=rate, duration=0.06, seed=5, points_per_get=4096, points_pool=4)
    assert sum(r["kind"] == EDIT for r in reqs) > 100
    sa = Server(wa, pool, max_wave_edits=max_edits, max_wave_gets=8)
    sb = Server(wb, pool)
    _, res_mix = sa.run(reqs, realtime=False, keep_results=True)
    _, res_alone = sb.run(reqs, realtime=False, keep_results=True, one_by_one=True)
    assert sa.waves < sb.waves == len(reqs)
    if max_edits > 3:
        assert sa.waves * 4 < len(reqs)  # gets do not end waves
    assert set(res_mix) == set(res_alone)
    for j in res_alone:
        np.testing.assert_array_equal(res_mix[j][0], res_alone[j][0])
        np.testing.assert_array_equal(res_mix[j][1], res_alone[j][1])
    from voxelis_gb300.api import export_canonical as export

    ca, cb = export(wa.lib, wa.h, wa.trees), export(wb.lib, wb.h, wb.trees)
    for k in ca:
        np.testing.assert_array_equal(ca[k], cb[k])
    assert wa.stats().alive_nodes == wb.stats().alive_nodes
    wa.close()
    wb.close()


def test_realtime_loop_reports_latencies(gpu_lib):
    w = make_world(gpu_lib)
    reqs, pool = make_trace(w, rate=2000.0, duration=0.25, seed=9, points_per_get=4096, points_pool=4)
    s = Server(w, pool)
    lat, _ = s.run(reqs, realtime=True)
    assert np.all(np.isfinite(lat)) and np.all(lat >= 0)
    assert s.waves <= len(reqs)
    w.close()
