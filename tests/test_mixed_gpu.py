"""The mixed-precision form (tensor-core bf16x3 composition, FP64 vertex
solves and near-zero predicates) against the FP64 oracle: every region only
one side visited is faceless or a sliver, the common faces agree within 1e-5
or their conditioning, every vertex on the zero level set."""
import numpy as np
import pytest

from analyticmesh_gb300 import engine, workloads as wl
from oracle import compare as CM
from oracle import oracle as O

from test_engine_gpu import f_at
from test_parity_gpu import assert_explained, common_faces_agree

pytestmark = pytest.mark.gpu

NETS = {
    "plain48x3": (lambda: wl.geometric([48, 48, 48], 12, perturb=0.05), 256),
    "odd_widths": (lambda: wl.geometric([20, 50, 20, 80, 20], 13, skips=[[0], [1, 1, 0], [1, 1, 1], [0], [0]],
                                        tm_shapes=[[0, 0], [80, 20]]), 256),
    "skips24x4": (lambda: wl.geometric([24, 24, 24, 24], 9, skips=[[0], [1, 1, 0], [1, 0, 1], [0]],
                                       tm_shapes=[[0, 0], [24, 3]]), 256),
    "wide256x3": (lambda: wl.geometric([256, 256, 256], 14, perturb=0.02), 256),
    "input_skip": (lambda: wl.geometric([64] * 5, 15, perturb=0.01, skips=[[0], [0], [1, 0, 0], [0], [0]],
                                        tm_shapes=[[64, 3]]), 256),
}


@pytest.mark.parametrize("name", list(NETS))
def test_mixed_against_fp64_oracle(name):
    factory, nseed = NETS[name]
    m = factory()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=nseed, seed=7)
    eng = engine.march(net, st, pt, "mixed")
    reg = eng.regions()
    o64 = O.run_oracle(net, st, pt, dtype="float64")
    # every region only one side visited is faceless or a sliver there, and
    # the common faces agree within 1e-5 or their conditioning
    # (test_parity_gpu)
    assert_explained(reg, o64, True, False, max_diff=max(4, reg.num // 2000))
    common_faces_agree(reg, o64, True, False, eng)
    v = np.concatenate([reg.verts[i, :reg.nverts[i]] for i in range(reg.num) if reg.nverts[i] >= 3])
    assert np.abs(f_at(net, v)).max() <= 1e-5
    eng.close()


@pytest.mark.parametrize("name", ["extra_16x2_f32", "iso_16x2_f32"])
def test_mixed_with_extra_constraints_and_iso(name):
    """The mixed form with the reference's extra half-space constraints (a box
    clip) and a non-zero level, on the golden fixtures' networks and seeds."""
    from golden_io import load

    g = load(name)
    net, st, pt, iso = g["net"], g["states"], g["points"], g["iso"]
    eng = engine.march(net, st, pt, "mixed", iso=iso)
    reg = eng.regions()
    o64 = O.run_oracle(net, st, pt, iso=iso, dtype="float64")
    assert_explained(reg, o64, True, False, max_diff=4)
    common_faces_agree(reg, o64, True, False, eng)
    v = np.concatenate([reg.verts[i, :reg.nverts[i]] for i in range(reg.num) if reg.nverts[i] >= 3])
    assert np.abs(f_at(net, v) - iso).max() <= 1e-5
    if net.num_extra:
        # every vertex inside the clip box (w . v + b <= 0 up to rounding)
        assert (v @ net.w_extra.T + net.b_extra).max() <= 1e-5
    eng.close()
