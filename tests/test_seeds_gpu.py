"""Seed handling on the GPU: the region set of a connected surface does not
depend on the seeds (one seed reaches every region), and repeated seed
states are de-duplicated as the reference's STATES de-duplicates them
(backend/inc/states.h:147-218)."""
import numpy as np
import pytest

from analyticmesh_gb300 import engine, workloads as wl

pytestmark = pytest.mark.gpu


def _keys(reg):
    return set(map(bytes, reg.bits))


@pytest.mark.parametrize("form", ["float32", "mixed"])
def test_one_seed_and_repeated_seeds_reach_the_same_regions(form):
    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    full = engine.march(net, st, pt, form)
    want = _keys(full.regions())
    assert full.stats()["num_seeds"] == len(np.unique(st, axis=0))

    one = engine.march(net, st[:1], pt[:1], form)
    assert _keys(one.regions()) == want and one.stats()["num_seeds"] == 1

    idx = np.random.default_rng(0).permutation(np.concatenate([np.arange(len(st))] * 3))
    dup = engine.march(net, st[idx], pt[idx], form)
    assert _keys(dup.regions()) == want
    assert dup.stats()["num_seeds"] == full.stats()["num_seeds"]
    assert dup.stats()["num_regions"] == full.stats()["num_regions"]
    for e in (full, one, dup):
        e.close()
