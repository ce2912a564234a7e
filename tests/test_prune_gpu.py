"""Row pruning in the face walk (AM_OPT_PRUNE_ROWS): the walk that scans only
the rows whose line can meet the face gives the same regions, in the same
order, with the same polygons bit for bit, as the walk over every row."""
import numpy as np
import pytest

from analyticmesh_gb300 import _lib, engine, workloads as wl

pytestmark = pytest.mark.gpu

CASES = {
    "sphere": (lambda: wl.sphere(), 0.0, 0),
    "perturbed48x3": (lambda: wl.geometric([48, 48, 48], 12, perturb=0.05), 0.0, 0),
    "skips24x4": (lambda: wl.geometric([24, 24, 24, 24], 9, skips=[[0], [1, 1, 0], [1, 0, 1], [0]],
                                       tm_shapes=[[0, 0], [24, 3]]), 0.0, 0),
    "deep_sample": (lambda: wl.deep(), wl.DEEP_ISO, 200000),
    "large_skip_sample": (lambda: wl.large_skip(), 0.0, 150000),
}


@pytest.mark.parametrize("form", ["float32", "mixed", "float64"])
@pytest.mark.parametrize("name", list(CASES))
def test_pruned_walk_gives_the_same_faces(name, form):
    factory, iso, limit = CASES[name]
    if form == "float64" and limit:
        pytest.skip("the float64 form of the wide networks is checked on the small cases")
    m = factory()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=512, seed=3, iso=iso)
    out = {}
    for prune in (0, 1):
        eng = engine.Engine(form, net.nodes, net.arc_table, net.num_extra)
        eng.set_option(_lib.AM_OPT_PRUNE_ROWS, prune)
        if limit:
            eng.set_option(_lib.AM_OPT_MAX_REGIONS, limit)
        try:
            eng.run_net(net, st, pt, iso)
        except _lib.AmError as ex:
            assert limit and ex.status == _lib.AM_ERR_CAPACITY, str(ex)
        out[prune] = eng.regions()
        eng.close()
    a, b = out[0], out[1]
    assert a.num == b.num and a.num > 1000
    assert np.array_equal(a.bits, b.bits)
    assert np.array_equal(a.nverts, b.nverts)
    assert np.array_equal(a.status, b.status)
    assert np.array_equal(a.edges, b.edges)
    assert np.array_equal(a.verts.view(np.int64), b.verts.view(np.int64))
