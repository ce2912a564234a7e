"""The order-free comparison the GPU parity tests use (oracle/compare.py),
checked against a per-region restatement of its definition on perturbed
copies of an oracle run: rotated and reversed vertex cycles, moved, NaN and
infinite vertices, changed vertex counts, dropped and repeated regions."""
import copy

import numpy as np
import pytest

from analyticmesh_gb300 import workloads as wl
from oracle import compare as CM
from oracle import oracle as O


def _polygons(r, min_verts):
    out = {}
    for i in range(r.num):
        n = int(r.nverts[i])
        if n >= min_verts:
            out[r.bits[i].tobytes()] = np.asarray(r.verts[i, :n], dtype=np.float64)
    return out


def _report_by_definition(a, b, tol):
    ka, kb = {x.tobytes() for x in a.bits}, {x.tobytes() for x in b.bits}
    pa, pb = _polygons(a, 1), _polygons(b, 1)
    common = set(pa) & set(pb)
    mm = beyond = 0
    worst = 0.0
    for k in common:
        if pa[k].shape != pb[k].shape:
            mm += 1
            continue
        with np.errstate(invalid="ignore"):
            d = CM.cycle_distance(pa[k], pb[k])
        beyond += (not np.isfinite(d)) or d > tol
        if np.isfinite(d):
            worst = max(worst, d)
    return dict(regions_a=len(ka), regions_b=len(kb), regions_only_a=len(ka - kb), regions_only_b=len(kb - ka),
                faces_a=sum(p.shape[0] >= 3 for p in pa.values()), faces_b=sum(p.shape[0] >= 3 for p in pb.values()),
                common_polygons=len(common), faces_count_mismatch=mm, faces_beyond_tol=int(beyond), max_diff=worst)


def _canonical_by_definition(a, b, tol):
    ka, kb = {x.tobytes() for x in a.bits}, {x.tobytes() for x in b.bits}
    pa, pb = _polygons(a, 3), _polygons(b, 3)
    common = set(pa) & set(pb)
    with np.errstate(invalid="ignore"):
        d = [CM.cycle_distance(pa[k], pb[k]) for k in common]
    return dict(regions_a=len(ka), regions_b=len(kb), only_a=len(ka - kb), only_b=len(kb - ka), faces_a=len(pa),
                faces_b=len(pb), faces_only_a=len(set(pa) - set(pb)), faces_only_b=len(set(pb) - set(pa)),
                faces_mismatch=sum(x > tol for x in d), max_vertex_diff=max(d) if d else 0.0)


def _clean_by_definition(r):
    ok = np.zeros(r.num, bool)
    for i in range(r.num):
        nt = int(r.ntab[i])
        t = r.tab[i, :nt]
        ok[i] = nt >= 4 and t[0] == t[nt - 1] and (t >= 0).all()
    return ok


@pytest.fixture(scope="module")
def base():
    m = wl.geometric([24, 24], 3)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=64, seed=1)
    return O.run_oracle(net, st, pt, dtype="float64")


def _perturbed(base, rng):
    b = copy.deepcopy(base)
    R = b.num
    for i in rng.choice(R, size=R // 5, replace=False):
        n = int(b.nverts[i])
        if n > 0:
            cyc = np.roll(b.verts[i, :n].copy(), rng.integers(n), axis=0)
            b.verts[i, :n] = cyc[::-1] if rng.random() < 0.5 else cyc
    for i in rng.choice(R, size=5, replace=False):
        b.verts[i, 0, rng.integers(3)] += rng.choice([1e-7, 1e-4, np.nan, np.inf])
    for i in rng.choice(R, size=3, replace=False):
        b.nverts[i] = max(0, int(b.nverts[i]) - int(rng.integers(0, 3)))
    keep = np.sort(rng.choice(R, size=R - 7, replace=False))
    order = np.concatenate([keep, rng.choice(keep, size=4)])
    for k in ("bits", "nverts", "verts", "ntab", "tab", "mid", "start"):
        setattr(b, k, getattr(b, k)[order])
    return b


@pytest.mark.parametrize("trial", range(6))
def test_comparison_matches_its_definition(base, trial):
    rng = np.random.default_rng(trial)
    b = _perturbed(base, rng)
    for tol in (1e-5, 1e-3):
        for x, y in ((base, b), (b, base)):
            assert CM.parity_report(x, y, tol) == _report_by_definition(x, y, tol)
            assert CM.canonical(x, y, tol) == _canonical_by_definition(x, y, tol)
    assert np.array_equal(CM.clean_walks(b), _clean_by_definition(b))


def test_identical_runs_compare_clean(base):
    r = CM.parity_report(base, base)
    assert r["regions_only_a"] == r["regions_only_b"] == 0
    assert r["faces_count_mismatch"] == r["faces_beyond_tol"] == 0 and r["max_diff"] == 0.0
