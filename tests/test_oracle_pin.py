"""The oracle (C restatement of the reference loop) against the reference's
own loop: bit-exact per-region records and welded meshes.

* golden fixtures (always): outputs of the reference's own code, generated by
  tests/golden/make_golden.py;
* live (when the reference CPU build is available): fresh seeded networks.
"""
import numpy as np
import pytest

from analyticmesh_gb300 import workloads as wl
from oracle import compare as CM
from oracle import oracle as O

from golden_io import load, names


@pytest.mark.parametrize("name", names())
def test_oracle_matches_golden(name):
    g = load(name)
    regions, mesh = O.run_oracle(g["net"], g["states"], g["points"], iso=g["iso"], flip=g["flip"], dtype=g["dtype"],
                                 combine=(1.0, [0.0, 0.0, 0.0]))
    assert CM.exact_records(regions, g["regions"]) == []
    assert CM.exact_mesh(mesh, g["mesh"])


def test_golden_fixtures_present():
    assert len(names()) >= 7


def test_fnv_known_answers():
    lib = O.oracle_lib()
    # FNV-1a / FNV-1 32-bit of the empty string and of "a" (published test vectors)
    import ctypes
    empty = (ctypes.c_uint8 * 1)()
    a = (ctypes.c_uint8 * 1)(ord("a"))
    assert lib.amo_fnv1a(empty, 0) == 0x811C9DC5
    assert lib.amo_fnv1a(a, 1) == 0xE40C292C
    assert lib.amo_fnv1(a, 1) == 0x050C5D7E


def test_get_i_j_enumeration():
    lib = O.oracle_lib()
    import ctypes
    i, j = ctypes.c_int(), ctypes.c_int()
    got = []
    for x in range(12):
        lib.amo_get_i_j(x, 100, ctypes.byref(i), ctypes.byref(j))
        got.append((i.value, j.value))
    # anti-diagonals of i + j, i > j (kernel.h:607-622)
    assert got == [(1, 0), (2, 0), (2, 1), (3, 0), (3, 1), (4, 0), (3, 2), (4, 1), (5, 0), (4, 2), (5, 1), (6, 0)]


_live = pytest.mark.skipif(not O.ref_available(), reason="reference CPU build unavailable")


@_live
@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("factory", [
    lambda: wl.geometric([32, 32], 7),
    lambda: wl.geometric([20, 20, 20], 8, perturb=0.05),
    lambda: wl.geometric([24, 24, 24, 24], 9, skips=[[0], [1, 1, 0], [1, 0, 1], [0]], tm_shapes=[[0, 0], [24, 3]]),
], ids=["plain", "perturbed", "skips"])
def test_oracle_matches_reference_live(factory, dtype):
    m = factory()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    ro, mo = O.run_oracle(net, st, pt, dtype=dtype, combine=(2.0, [0.1, -0.2, 0.3]))
    rr, mr = O.run_ref(net, st, pt, dtype=dtype, combine=(2.0, [0.1, -0.2, 0.3]))
    assert CM.exact_records(ro, rr) == []
    assert CM.exact_mesh(mo, mr)


@_live
@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_oracle_matches_reference_live_level_flip_extra_and_hidden_transform(dtype):
    """The iso level, the inside-out flip, extra constraints (three planes of
    a box corner) and a transform between hidden layers of uneven widths, all
    in one run."""
    m = wl.geometric([20, 50, 20, 80, 20], 13, skips=[[0], [1, 1, 0], [1, 1, 1], [0], [0]],
                     tm_shapes=[[0, 0], [80, 20]])
    we = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0]], float) + 1e-8
    be = np.array([-0.2, -0.3, -0.1])
    net = wl.net_arrays(m, we, be)
    st, pt = wl.seeds_for(m, init_num=128, seed=12, iso=0.05, w_extra=we, b_extra=be)
    kw = dict(iso=0.05, flip=True, dtype=dtype, combine=(1.5, [0.0, 0.1, -0.1]))
    ro, mo = O.run_oracle(net, st, pt, **kw)
    rr, mr = O.run_ref(net, st, pt, **kw)
    assert ro.num > 0
    assert CM.exact_records(ro, rr) == []
    assert CM.exact_mesh(mo, mr)


def test_oracle_seed_independence_and_deduplication():
    """A connected surface: one seed reaches every region; seeds given three
    times in shuffled order keep one of each state."""
    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    full = O.run_oracle(net, st, pt)
    one = O.run_oracle(net, st[:1], pt[:1])
    idx = np.random.default_rng(0).permutation(np.concatenate([np.arange(len(st))] * 3))
    dup = O.run_oracle(net, st[idx], pt[idx])
    keys = lambda r: set(map(bytes, r.bits))
    assert keys(one) == keys(full) == keys(dup)
    assert dup.seeds_kept == full.seeds_kept == len(np.unique(st, axis=0))


@_live
def test_oracle_matches_reference_live_on_repeated_seeds():
    m = wl.geometric([24, 24], 21)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=64, seed=2)
    idx = np.random.default_rng(1).permutation(np.concatenate([np.arange(len(st))] * 2))
    ro = O.run_oracle(net, st[idx], pt[idx])
    rr = O.run_ref(net, st[idx], pt[idx])
    assert CM.exact_records(ro, rr) == []


@_live
@pytest.mark.parametrize("name", names())
def test_golden_fixtures_are_the_references_output(name):
    """Provenance of the committed fixtures: the reference's own loop, run
    again on each fixture's inputs, gives its records and mesh bit for bit."""
    g = load(name)
    regions, mesh = O.run_ref(g["net"], g["states"], g["points"], iso=g["iso"], flip=g["flip"], dtype=g["dtype"],
                              combine=(1.0, [0.0, 0.0, 0.0]))
    assert CM.exact_records(regions, g["regions"]) == []
    assert CM.exact_mesh(mesh, g["mesh"])
