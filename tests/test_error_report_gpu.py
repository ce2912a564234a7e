"""The per-result error report (am_error_report): max |f(v)| and the largest
vertex error against FP64, checked against a numpy FP64 forward pass of the
network at the same vertices and against the float64 form's own vertices."""
import numpy as np
import pytest

from analyticmesh_gb300 import _lib, engine, workloads as wl

from test_engine_gpu import f_at

pytestmark = pytest.mark.gpu

# the report's bounds per form: |f(v)| and vertex error against FP64 (the
# FP32 forms' vertex error is bounded by their worst-conditioned vertex)
BOUND = {"float32": (1e-5, 1e-3), "mixed": (1e-5, 1e-3), "float64": (1e-10, 1e-8)}


@pytest.mark.parametrize("form", ["float32", "mixed", "float64"])
def test_error_report_of_the_sphere(form):
    m = wl.sphere()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=1024, seed=1)
    eng = engine.march(net, st, pt, form)
    s = eng.stats()
    rep = eng.error_report(0)  # every region
    closed = s["num_faces"] - s["num_truncated"] - s["num_open"]
    assert rep["faces"] >= closed > 0, (rep, s)
    assert rep["vertices"] >= 3 * rep["faces"]
    assert rep["vertices_singular"] <= rep["vertices"] // 1000
    assert rep["max_abs_f"] <= BOUND[form][0], rep
    assert rep["max_vertex_err"] <= BOUND[form][1], rep
    s2 = eng.stats()
    assert s2["max_abs_f"] == rep["max_abs_f"] and s2["error_faces"] == rep["faces"]
    # the same quantity from a numpy FP64 forward pass of the whole network
    reg = eng.regions()
    ok = (reg.nverts >= 3) & (reg.status == 0)
    v = np.concatenate([reg.verts[i, :reg.nverts[i]] for i in np.nonzero(ok)[0]])
    fnp = np.abs(f_at(net, v)).max()
    assert fnp <= BOUND[form][0], fnp
    # the report evaluates each face's affine piece, numpy the whole network:
    # equal at a vertex inside its region, within rounding of a vertex just
    # outside it
    assert abs(fnp - rep["max_abs_f"]) <= max(10 * BOUND[form][0] / 1e4, 0.5 * fnp), (fnp, rep)
    # a sample: no larger than the whole
    rs = eng.error_report(500)
    assert 0 < rs["faces"] <= 500 and rs["max_abs_f"] <= rep["max_abs_f"]
    eng.close()


def test_error_report_needs_a_result():
    net = wl.net_arrays(wl.geometric([16, 16], 1))
    eng = engine.Engine("float32", net.nodes, net.arc_table, 0)
    with pytest.raises(_lib.AmError) as ex:
        eng.error_report(10)
    assert ex.value.status == _lib.AM_ERR_NO_RESULT
    eng.close()
