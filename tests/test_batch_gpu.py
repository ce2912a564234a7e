"""Batched marching (am_run_batch): several networks of different widths,
depths and skip layouts march side by side, each on its own engine; every
network's regions come out exactly as in a standalone run of the same
engine (the kernels' results do not depend on the grid sizes the batch uses)."""
import numpy as np
import pytest

from analyticmesh_gb300 import _lib, engine, workloads as wl

pytestmark = pytest.mark.gpu

MODELS = [
    lambda: wl.geometric([32, 32], 101, perturb=0.01),
    lambda: wl.geometric([64] * 4, 102, perturb=0.01),
    lambda: wl.geometric([20, 50, 20, 80, 20], 13, skips=[[0], [1, 1, 0], [1, 1, 1], [0], [0]],
                         tm_shapes=[[0, 0], [80, 20]]),
    lambda: wl.geometric([128] * 3, 104, perturb=0.01),
    lambda: wl.geometric([64] * 5, 15, perturb=0.01, skips=[[0], [0], [1, 0, 0], [0], [0]], tm_shapes=[[64, 3]]),
]


@pytest.mark.parametrize("form", ["mixed", "float32"])
def test_batch_matches_standalone_runs(form):
    nets, sts, pts = [], [], []
    for i, f in enumerate(MODELS):
        m = f()
        nets.append(wl.net_arrays(m))
        st, pt = wl.seeds_for(m, init_num=128, seed=20 + i)
        sts.append(st)
        pts.append(pt)
    engines = [engine.Engine(form, n.nodes, n.arc_table, n.num_extra) for n in nets]
    wall = engine.run_batch(engines, nets, sts, pts)
    assert wall > 0
    for i, (eng, net) in enumerate(zip(engines, nets)):
        alone = engine.march(net, sts[i], pts[i], form)
        a, b = eng.regions(), alone.regions()
        assert eng.stats()["num_regions"] == alone.stats()["num_regions"] > 0, i
        assert np.array_equal(a.bits, b.bits), i
        assert np.array_equal(a.nverts, b.nverts), i
        assert np.array_equal(a.verts, b.verts), i
        alone.close()
    # results stay usable per engine
    mesh = engines[0].combine()
    assert len(mesh.faces) > 0
    for e in engines:
        e.close()


def test_batch_rejects_an_engine_twice():
    m = wl.geometric([32, 32], 101)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=64, seed=1)
    eng = engine.Engine("float32", net.nodes, net.arc_table, 0)
    with pytest.raises(_lib.AmError):
        engine.run_batch([eng, eng], [net, net], [st, st], [pt, pt])
    eng.close()


def test_batched_configuration_networks_against_float64():
    """Networks of the batched configuration (64 networks, seeds 100..163;
    here the small ones, so that their FP64 marches stay short) marched as
    one mixed-precision batch: each against its own FP64 march, every
    difference explained as in the single-network parity tests."""
    from test_parity_gpu import assert_explained

    pick = [2, 3, 12, 13, 55, 57]
    models = wl.batched(64, 100)
    nets, sts, pts = [], [], []
    for i in pick:
        m = models[i]
        nets.append(wl.net_arrays(m))
        st, pt = wl.seeds_for(m, init_num=1024, seed=100 + i)
        sts.append(st)
        pts.append(pt)
    engines = [engine.Engine("mixed", n.nodes, n.arc_table, n.num_extra) for n in nets]
    engine.run_batch(engines, nets, sts, pts)
    for k, (eng, net) in enumerate(zip(engines, nets)):
        f64 = engine.march(net, sts[k], pts[k], "float64")
        assert eng.stats()["num_faces"] > 0
        assert_explained(eng.regions(), f64.regions(), True, True)
        rep = eng.error_report(0)
        assert rep["max_abs_f"] <= 1e-5, (pick[k], rep)
        f64.close()
        eng.close()
