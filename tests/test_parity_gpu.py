"""Region-set parity on the benchmark configurations, with every difference
explained.

Two exact runs of Analytic Marching visit the same regions.  Floating-point
runs differ only where the arithmetic cannot decide: at near-degenerate
vertices, where several constraint planes meet within rounding of one point,
a walk may see a zero-length edge (merged at FP_SAME_EPS, no neighbour) where
another sees a tiny one (and spawns a sliver region), or a walk may not close.
The tests below compare the engine with the reference's own loop (compiled
for the CPU, oracle/_ref, run single-threaded so that its racy choices are
made in thread order) and the forms with each other, and require that every
region visited by one run only is, in the run that visited it, faceless or a
sliver (area below 1e-10, or an edge shorter than 1e-5) --
oracle/compare.py:classify_regions -- and that the faces of the common
regions agree within 1e-5 except where one of the two is such a sliver.
"""
import numpy as np
import pytest

from analyticmesh_gb300 import engine, workloads as wl
from oracle import compare as CM
from oracle import oracle as O

from golden_io import load

pytestmark = pytest.mark.gpu

TOL = 1e-5


def assert_explained(a, b, a_engine=True, b_engine=True, max_diff=None):
    """Every region of one run only is faceless or a sliver there; returns
    the counts."""
    oa, ob = CM.region_difference(a, b)
    ca = CM.classify_regions(a, oa, a_engine)
    cb = CM.classify_regions(b, ob, b_engine)
    assert ca["other"] == 0 and cb["other"] == 0, (ca, cb)
    if max_diff is not None:
        assert len(oa) + len(ob) <= max_diff, (len(oa), len(ob))
    return len(oa), len(ob), ca, cb


def face_condition(eng, reg, rid):
    """Largest condition number of the 3x3 systems (two edge planes and the
    face plane, normalised rows) that give region rid's vertices."""
    rows, eq = eng.region_rows(int(rid), 1)
    rows, eq = rows[0], eq[0]
    n = int(reg.nverts[rid])
    worst = 1.0
    for i in range(n):
        a, b = int(reg.edges[rid, (i - 1) % n]), int(reg.edges[rid, i])
        if a < 0 or b < 0:
            return np.inf
        A = np.stack([rows[a, :3], rows[b, :3], eq[:3]])
        A = A / np.linalg.norm(A, axis=1, keepdims=True)
        worst = max(worst, float(np.linalg.cond(A)))
    return worst


def _drop_collinear(P, eps=1e-5):
    """The polygon without vertices where it turns by less than eps radians
    (a vertex on the straight edge between its neighbours, up to the
    rounding of FP32 planes)."""
    n = len(P)
    keep = []
    for i in range(n):
        u, v = P[i] - P[i - 1], P[(i + 1) % n] - P[i]
        if np.linalg.norm(np.cross(u, v)) > eps * max(np.linalg.norm(u) * np.linalg.norm(v), 1e-300):
            keep.append(i)
    return P[keep]


def common_faces_agree(a, b, a_engine=True, b_engine=True, eng=None):
    """Common regions with a face in both runs: same polygon within TOL (up
    to rotation / orientation), except (i) where either is a sliver -- a
    vertex merge at FP_SAME_EPS may differ -- or (ii), given the engine
    `eng` that produced run a, where the difference is within what FP32-
    level constraint rows (relative accuracy ~1e-6) allow at the face's
    worst-conditioned vertex: d <= 3e-6 * cond (a vertex solve amplifies the
    rows' error by the system's condition number).  Regions whose walk did not
    close in either run are counted apart.  Returns the counts."""
    sa, sb, ra, rb = CM._matched(a, b, 3)
    d, count_differs = CM._pair_distances(a, b, ra, rb)
    bad = np.nonzero(count_differs | ~(d <= TOL))[0]
    out = {"compared": int(len(ra)), "sliver": 0, "ill_conditioned": 0}
    failed = lambda r, i, is_engine: is_engine and int(r.status[i]) != 0
    out["failed_walk"] = 0
    out["collinear"] = 0
    for j in bad:
        if failed(a, ra[j], a_engine) or failed(b, rb[j], b_engine):
            out["failed_walk"] += 1  # a walk that did not close: no face to compare
            continue
        if count_differs[j]:  # the same polygon with a vertex on a straight edge in one of them?
            pa = _drop_collinear(np.asarray(a.verts[ra[j], :int(a.nverts[ra[j]])], np.float64))
            pb = _drop_collinear(np.asarray(b.verts[rb[j], :int(b.nverts[rb[j]])], np.float64))
            if len(pa) == len(pb) and CM.cycle_distance(pa, pb) <= TOL:
                out["collinear"] += 1
                continue
        ga = CM.region_geometry(a, ra[j], a_engine)
        gb = CM.region_geometry(b, rb[j], b_engine)
        small = lambda g: g[1] < 1e-10 or g[2] < TOL
        if small(ga) or small(gb):
            out["sliver"] += 1
            continue
        assert eng is not None and not count_differs[j], (int(ra[j]), ga, gb, float(d[j]))
        kappa = face_condition(eng, a, ra[j])
        assert d[j] <= 3e-6 * kappa, (int(ra[j]), ga, gb, float(d[j]), kappa)
        out["ill_conditioned"] += 1
    return out


def test_sphere_float32_against_the_reference_float32_loop():
    """Config 2 (3-[128]x4-1): the engine's FP32 form against the reference's
    own FP32 loop."""
    m = wl.sphere()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=1024, seed=1)
    eng = engine.march(net, st, pt, "float32")
    reg = eng.regions()
    ref = O.run_ref(net, st, pt, dtype="float32", threads=1)
    na, nb, _, _ = assert_explained(reg, ref, True, False, max_diff=20)
    c = common_faces_agree(reg, ref, True, False, eng)
    assert c["compared"] > 260000 and c["sliver"] + c["ill_conditioned"] <= 200, c
    eng.close()


@pytest.mark.parametrize("pair", [("float64", "ref64"), ("mixed", "float64"), ("float32", "float64")])
def test_sphere_forms_agree(pair):
    """Config 2: the float64 form is the reference's FP64 loop region for
    region; the mixed and the plain FP32 forms differ from it only by
    explained regions (between themselves they differ by the union of the
    two: the plain form's FP32 vertices add merge differences of their own)."""
    m = wl.sphere()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=1024, seed=1)
    runs, engines = {}, []
    for name in pair:
        if name == "ref64":
            runs[name] = (O.run_ref(net, st, pt, dtype="float64", threads=1), False)
        else:
            eng = engine.march(net, st, pt, name)
            runs[name] = (eng.regions(), True)
            engines.append(eng)
    (a, ae), (b, be) = runs[pair[0]], runs[pair[1]]
    na, nb, _, _ = assert_explained(a, b, ae, be, max_diff=20)
    c = common_faces_agree(a, b, ae, be, engines[0])
    if pair == ("float64", "ref64"):  # the same regions and the same faces
        assert na == 0 and nb == 0 and c["sliver"] + c["ill_conditioned"] == 0, c
    for e in engines:
        e.close()


def test_polytope_float32_against_the_reference_golden_run():
    """Config 1 (3-14-1 polytope, N(0, 1e-7) noise): the noise leaves the
    fourteen planes in seven nearly coincident pairs, so most regions are
    1e-7-thin slabs, where FP32 walks can fail; the faces that are not agree
    with the reference's own FP32 run (the golden fixture), and every vertex
    of a closed walk lies on the exact surface sum_k |a_k . x| = 2."""
    g = load("polytope_f32")
    eng = engine.march(g["net"], g["states"], g["points"], "float32")
    reg, gold = eng.regions(), g["regions"]
    assert_explained(reg, gold, True, False)
    dirs = np.array([[1, 1, 1], [0, 1, 1], [1, 0, 1], [1, 1, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    on_surface = lambda V: (np.abs(np.abs(V @ dirs.T).sum(1) - 2.0)).max() < TOL
    ok = [i for i in range(reg.num) if reg.nverts[i] >= 3 and reg.status[i] == 0]
    assert len(ok) >= 40
    assert on_surface(np.concatenate([reg.verts[i, :reg.nverts[i]] for i in ok]))
    # common faces: the same polygon within 1e-5, or -- where a slab's
    # planes cut it differently in the two FP32 runs -- ours a piece of the
    # exact surface; the reference's FP32 walk itself leaves a vertex off the
    # surface on some of these (counted, a handful at most)
    sa, sb, ra, rb = CM._matched(reg, gold, 3)
    d, count_differs = CM._pair_distances(reg, gold, ra, rb)
    assert len(ra) >= 20
    same = ref_off = 0
    for j in range(len(ra)):
        if not count_differs[j] and d[j] <= TOL:
            same += 1
            continue
        if reg.status[ra[j]] != 0:
            continue
        assert on_surface(reg.verts[ra[j], :reg.nverts[ra[j]]]), int(ra[j])
        ref_off += not on_surface(gold.verts[rb[j], :gold.nverts[rb[j]]])
    assert same >= len(ra) // 2, (same, len(ra))
    assert ref_off <= 3, ref_off
    eng.close()


def test_deep_mixed_against_float64():
    """Config 3 (3-[256]x6-1 + N(0, 0.02) at level 0.35, 1.35 M regions): the
    mixed form against the float64 form, every difference explained."""
    m = wl.deep()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=1024, seed=1, iso=wl.DEEP_ISO)
    out = {}
    for form in ("mixed", "float64"):
        eng = engine.march(net, st, pt, form, iso=wl.DEEP_ISO)
        out[form] = eng.regions()
        if form == "mixed":
            rep = eng.error_report(20000)
            assert rep["max_abs_f"] <= TOL, rep
        eng.close()
    na, nb, _, _ = assert_explained(out["mixed"], out["float64"], max_diff=1000)
    assert out["float64"].num > 1300000


def _boundary_edges(mesh):
    import collections
    cnt = collections.Counter()
    owner = {}
    for fi, f in enumerate(mesh.faces):
        for a, b in zip(f, f[1:] + f[:1]):
            e = (min(a, b), max(a, b))
            cnt[e] += 1
            owner[e] = fi
    return [(e, owner[e]) for e, c in cnt.items() if c != 2]


@pytest.mark.parametrize("form", ["float64", "float32", "mixed"])
def test_sphere_mesh_is_watertight(form):
    """The topological weld of config 2: in FP64 every edge is shared by
    exactly two faces.  In the FP32-level forms an edge that is not either
    has, in its own face or in the neighbour across its plane, a face that is
    a sliver or has an edge shorter than 1e-5 (one walk merged two vertices
    closer than FP_SAME_EPS and the other did not), or it is closed
    geometrically: its end points are vertices of the neighbour's face within
    1e-5, named there by another plane (a vertex where a fourth plane passes
    within rounding)."""
    m = wl.sphere()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=1024, seed=1)
    eng = engine.march(net, st, pt, form)
    mesh = eng.combine()
    reg = eng.regions()
    bad = _boundary_edges(mesh)
    if form == "float64":
        assert bad == []
    else:
        assert len(bad) <= 1e-3 * len(mesh.faces)
        face_region = np.nonzero(reg.nverts >= 3)[0]
        keys = {bytes(k): i for i, k in enumerate(CM._row_keys(reg.bits))}
        small = lambda r: (lambda g: g[0] < 3 or g[1] < 1e-10 or g[2] < TOL or int(reg.status[r]) != 0)(
            CM.region_geometry(reg, r, True))
        unexplained = []
        for (va, vb), fi in bad:
            r = int(face_region[fi])
            if small(r):
                continue
            # the edge's plane: the one both vertices of the face lie on
            n = int(reg.nverts[r])
            ids = list(mesh.faces[fi])
            i = next(j for j in range(n) if {ids[j], ids[(j + 1) % n]} == {va, vb})
            k = int(reg.edges[r, i])
            if k >= reg.N:  # an extra constraint: no neighbour
                unexplained.append((r, i, "extra"))
                continue
            nb = reg.bits[r].copy()
            nb[k >> 5] ^= np.uint32(1 << (k & 31))
            j = keys.get(bytes(nb.view(np.uint8)))
            if j is None or small(j):
                continue
            # geometrically closed: both end points are vertices of the
            # neighbour's face too, only named by other planes (a vertex
            # where a fourth plane passes within rounding)
            Vn = reg.verts[j, :int(reg.nverts[j])]
            ends = [reg.verts[r, i], reg.verts[r, (i + 1) % n]]
            if all(np.abs(Vn - p).max(axis=1).min() <= TOL for p in ends):
                continue
            unexplained.append((r, i, j))
        assert unexplained == [], unexplained[:10]
    eng.close()
