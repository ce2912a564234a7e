"""Failure detection through the C ABI, all of it made on the host: no GPU
fault, trap or hang is provoked.

* a region hash table fixed too small for the run -> AM_ERR_TABLE_FULL at the
  probe bound (the reference's try_insert spins forever there,
  backend/inc/hash.h:56-64), and the engine marches normally afterwards;
* device error bits written into the control block by the test hook
  AM_OPT_INJECT_ERROR (a tensor-core pipeline wait that ran out, kErrWait)
  -> the run fails with AM_ERR_CUDA, in the graph-driven and the host-driven
  loop;
* NaN / infinite parameters -> AM_ERR_INVALID_ARGUMENT before any wave;
* a face polygon with more vertices than the polygon capacity (32) ->
  counted in num_truncated, the run completes.
"""
import math

import numpy as np
import pytest

from analyticmesh_gb300 import _lib, engine, workloads as wl
from oracle import compare as CM

pytestmark = pytest.mark.gpu


def _small():
    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    return net, st, pt


def _region_set(eng):
    return CM.region_keys(eng.regions())


@pytest.mark.parametrize("form", ["float32", "mixed"])
def test_fixed_table_too_small_reports_table_full_and_engine_recovers(form):
    net, st, pt = _small()
    ref = engine.march(net, st, pt, form)
    want = _region_set(ref)
    assert len(want) > 600
    ref.close()
    eng = engine.Engine(form, net.nodes, net.arc_table, net.num_extra)
    eng.set_option(_lib.AM_OPT_TABLE_SLOTS, 256)  # fewer slots than the run's regions
    with pytest.raises(_lib.AmError) as ex:
        eng.run_net(net, st, pt)
    assert ex.value.status == _lib.AM_ERR_TABLE_FULL, str(ex.value)
    # a fixed table with room, then the automatic one: the same regions
    eng.set_option(_lib.AM_OPT_TABLE_SLOTS, 1 << 16)
    eng.run_net(net, st, pt)
    assert _region_set(eng) == want
    eng.set_option(_lib.AM_OPT_TABLE_SLOTS, 0)
    eng.run_net(net, st, pt)
    assert _region_set(eng) == want
    eng.close()


@pytest.mark.parametrize("graph", [1, 0], ids=["graph_loop", "host_loop"])
@pytest.mark.parametrize("form", ["float32", "mixed"])
def test_device_wait_timeout_bit_fails_the_run(form, graph):
    net, st, pt = _small()
    eng = engine.Engine(form, net.nodes, net.arc_table, net.num_extra)
    eng.set_option(_lib.AM_OPT_GRAPH, graph)
    eng.run_net(net, st, pt)
    want = _region_set(eng)
    eng.set_option(_lib.AM_OPT_INJECT_ERROR, _lib.ERR_WAIT)
    with pytest.raises(_lib.AmError) as ex:
        eng.run_net(net, st, pt)
    assert ex.value.status == _lib.AM_ERR_CUDA
    assert "wait" in str(ex.value)
    # no result is left behind by the failed run
    L = _lib.lib()
    assert L.am_combine_mesh(eng.h, 1.0, None) == _lib.AM_ERR_NO_RESULT
    # the other bits decode to their own statuses
    for bit, status in ((_lib.ERR_TABLE_FULL, _lib.AM_ERR_TABLE_FULL), (_lib.ERR_CAPACITY, _lib.AM_ERR_CAPACITY),
                        (_lib.ERR_NONFINITE, _lib.AM_ERR_INVALID_ARGUMENT)):
        eng.set_option(_lib.AM_OPT_INJECT_ERROR, bit)
        with pytest.raises(_lib.AmError) as ex:
            eng.run_net(net, st, pt)
        assert ex.value.status == status
    eng.set_option(_lib.AM_OPT_INJECT_ERROR, 0)
    eng.run_net(net, st, pt)
    assert _region_set(eng) == want
    eng.close()


@pytest.mark.parametrize("form", ["float32", "float64", "mixed"])
@pytest.mark.parametrize("where", ["weight", "bias", "first_layer"])
def test_non_finite_parameters_are_rejected(form, where):
    net, st, pt = _small()
    W = [w.copy() for w in net.W]
    B = [b.copy() for b in net.b]
    if where == "weight":
        W[1][3, 5] = np.nan
    elif where == "bias":
        B[2][0] = np.inf
    else:
        W[0][7, 1] = -np.inf
    eng = engine.Engine(form, net.nodes, net.arc_table, net.num_extra)
    with pytest.raises(_lib.AmError) as ex:
        eng.run(W, B, st, pt)
    assert ex.value.status == _lib.AM_ERR_INVALID_ARGUMENT
    assert "NaN" in str(ex.value)
    eng.run_net(net, st, pt)  # the same engine, clean parameters
    assert eng.stats()["num_faces"] > 0
    eng.close()


def _polygon_40():
    """3 -> 41 -> 1 whose central region's face is a regular 40-gon: units
    0..39 are relu(cos t_k x + sin t_k y - 1) (inactive inside the unit
    40-gon), unit 40 is relu(z + 2), f = h_40 + sum_k h_k - 2, so f = z there
    and the face plane z = 0 meets the 40 planes in a 40-gon.  A box of six
    extra constraints (|x|, |y|, |z| <= 3) bounds the outer regions."""
    t = 2 * math.pi * np.arange(40) / 40
    W0 = np.zeros((41, 3))
    W0[:40, 0], W0[:40, 1] = np.cos(t), np.sin(t)
    W0[40, 2] = 1.0
    b0 = np.concatenate([-np.ones(40), [2.0]])
    W1 = np.ones((1, 41))
    b1 = np.array([-2.0])
    we = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], float)
    be = -3.0 * np.ones(6)
    net = wl.NetArrays(nodes=[3, 41, 1], W=[W0, W1], b=[b0, b1], arc_table=np.zeros((1, 1), np.int32), tms=[],
                       w_extra=we, b_extra=be)
    pts = np.array([[0.2, 0.1, 0.0], [-0.3, 0.25, 0.0]])
    z = pts @ W0.T + b0
    return net, (z > 0).astype(np.uint8), pts


@pytest.mark.parametrize("form", ["float32", "float64"])
def test_polygon_beyond_vertex_capacity_is_truncated(form):
    net, st, pt = _polygon_40()
    eng = engine.march(net, st, pt, form)
    s = eng.stats()
    assert s["num_truncated"] >= 1, s
    assert s["max_polygon_verts"] == _lib.vert_capacity() == 32
    reg = eng.regions()
    central = np.nonzero((reg.start == -1) & (reg.status == 3))[0]  # kTruncated
    assert len(central) == 1
    # its 32 vertices lie on the 40-gon: |v| = 1 / cos(pi / 40), z = 0
    v = reg.verts[central[0], :32]
    np.testing.assert_allclose(np.linalg.norm(v[:, :2], axis=1), 1 / math.cos(math.pi / 40), atol=1e-5)
    np.testing.assert_allclose(v[:, 2], 0.0, atol=1e-6)
    eng.close()
