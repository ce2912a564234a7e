"""Comparison of marching results -- TEST INFRASTRUCTURE ONLY.

Two levels:
* ``exact_records``: record-by-record equality of two runs that process
  regions in the same order (the oracle against the reference's own loop run
  single-threaded).  Only the valid prefix of each region's vertex list and
  edge table is compared; the buffers behind it hold stale data.
* ``canonical``: order-free comparison for runs with different processing
  orders (the CUDA engine against the oracle): the set of regions (activation
  bit strings), and per region its polygon as a cycle of vertices, matched up
  to rotation and orientation within a tolerance.
"""
from __future__ import annotations

import dataclasses

import numpy as np


def exact_records(a, b, vert_tol=0.0):
    """Returns a list of human-readable differences (empty = identical)."""
    out = []
    if a.num != b.num:
        return ["region count %d != %d" % (a.num, b.num)]
    if not np.array_equal(a.bits, b.bits):
        out.append("region order / states differ")
    for k in ("nverts", "ntab", "start"):
        bad = np.where(getattr(a, k) != getattr(b, k))[0]
        if len(bad):
            out.append("%s differs at %d regions (first %d)" % (k, len(bad), bad[0]))
    ntab = np.minimum(a.ntab, b.ntab)
    cols = np.arange(a.tab.shape[1])[None, :]
    valid = cols < ntab[:, None]
    bad = np.where(((a.tab != b.tab) & valid).any(1))[0]
    if len(bad):
        out.append("edge tables differ at %d regions (first %d)" % (len(bad), bad[0]))
    nv = np.minimum(a.nverts, b.nverts)
    vmask = (np.arange(a.verts.shape[1])[None, :] < nv[:, None])[..., None]
    if _differ(np.where(vmask, a.verts, 0.0), np.where(vmask, b.verts, 0.0), vert_tol):
        out.append("vertices differ")
    if _differ(a.mid, b.mid, vert_tol):
        out.append("seed points differ")
    return out


def _differ(x, y, tol):
    """NaN-aware: NaN matches NaN (the reference itself emits NaN vertices
    for singular systems, see kernel.h:729-795 where NaN passes the test)."""
    with np.errstate(invalid="ignore"):
        if tol == 0.0:
            return not np.array_equal(x, y, equal_nan=True)
        return not np.allclose(x, y, rtol=0.0, atol=tol, equal_nan=True)


def exact_mesh(a, b):
    """Welded meshes: identical vertex arrays (NaN-aware) and face lists."""
    return (a.verts.shape == b.verts.shape and not _differ(a.verts, b.verts, 0.0)
            and [list(map(int, f)) for f in a.faces] == [list(map(int, f)) for f in b.faces])


def _key(bits_row):
    return bits_row.tobytes()


def _row_keys(bits):
    """One opaque (void) value per region: its packed activation bits."""
    b = np.ascontiguousarray(bits)
    width = max(1, b.shape[1] * b.itemsize) if b.ndim == 2 else 1
    if b.ndim != 2 or b.shape[0] == 0 or b.shape[1] == 0:
        return np.zeros(b.shape[0] if b.ndim else 0, dtype=np.dtype((np.void, width)))
    return b.view(np.dtype((np.void, width))).ravel()


def _last_of_each(keys, mask):
    """Indices of the rows selected by ``mask``, one per distinct key (the
    last occurrence, as a dict built in row order keeps), in key order."""
    idx = np.nonzero(mask)[0]
    if idx.size == 0:
        return idx
    rev = idx[::-1]
    _, first = np.unique(keys[rev], return_index=True)
    return rev[first]


@dataclasses.dataclass
class Polygons:
    """region key -> (V, 3) polygon, plus the key order."""

    faces: dict

    @classmethod
    def from_regions(cls, r, min_verts=3):
        faces = {}
        for i in range(r.num):
            n = int(r.nverts[i])
            if n >= min_verts:
                faces[_key(r.bits[i])] = np.asarray(r.verts[i, :n], dtype=np.float64)
        return cls(faces)


def cycle_distance(p, q):
    """Smallest max-abs distance between two vertex cycles over all
    rotations and both orientations (inf when the lengths differ)."""
    if p.shape != q.shape:
        return float("inf")
    best = float("inf")
    n = p.shape[0]
    for cand in (q, q[::-1]):
        for s in range(n):
            d = float(np.abs(p - np.roll(cand, -s, axis=0)).max())
            if d < best:
                best = d
    return best


def _cycle_distances(P, Q):
    """cycle_distance for m pairs of n-vertex cycles at once: P, Q (m, n, 3)."""
    n = P.shape[1]
    best = np.full(P.shape[0], np.inf)
    with np.errstate(invalid="ignore"):
        for cand in (Q, Q[:, ::-1]):
            for s in range(n):
                d = np.abs(P - np.roll(cand, -s, axis=1)).max(axis=(1, 2))
                best = np.where(d < best, d, best)  # a NaN distance never wins, as in cycle_distance
    return best


def _matched(a, b, min_verts):
    """Polygons of both runs (regions with >= min_verts vertices, one per
    key) and the pairs with the same key: (sel_a, sel_b, ra, rb)."""
    ka, kb = _row_keys(a.bits), _row_keys(b.bits)
    sa = _last_of_each(ka, np.asarray(a.nverts) >= min_verts)
    sb = _last_of_each(kb, np.asarray(b.nverts) >= min_verts)
    _, ia, ib = np.intersect1d(ka[sa], kb[sb], assume_unique=True, return_indices=True)
    return sa, sb, sa[ia], sb[ib]


def _pair_distances(a, b, ra, rb):
    """cycle_distance of every matched pair (inf where the vertex counts differ)."""
    na = np.asarray(a.nverts)[ra].astype(np.int64)
    nb = np.asarray(b.nverts)[rb].astype(np.int64)
    d = np.full(ra.size, np.inf)
    for n in np.unique(na[na == nb]):
        m = (na == n) & (nb == n)
        d[m] = _cycle_distances(np.asarray(a.verts[ra[m], :n], dtype=np.float64),
                                np.asarray(b.verts[rb[m], :n], dtype=np.float64))
    return d, na != nb


def _key_sets(a, b):
    ua, ub = np.unique(_row_keys(a.bits)), np.unique(_row_keys(b.bits))
    return (ua.size, ub.size, np.setdiff1d(ua, ub, assume_unique=True).size,
            np.setdiff1d(ub, ua, assume_unique=True).size)


def region_keys(r):
    """The set of activation states a run visited (bytes of the packed bits)."""
    return frozenset(bytes(k) for k in np.unique(_row_keys(r.bits)))


def canonical(a_regions, b_regions, tol=1e-5):
    """Order-free comparison.  Returns a dict of counts."""
    na_, nb_, only_a, only_b = _key_sets(a_regions, b_regions)
    sa, sb, ra, rb = _matched(a_regions, b_regions, 3)
    d, _ = _pair_distances(a_regions, b_regions, ra, rb)
    return dict(regions_a=na_, regions_b=nb_, only_a=only_a, only_b=only_b,
                faces_a=int(sa.size), faces_b=int(sb.size), faces_only_a=int(sa.size - ra.size),
                faces_only_b=int(sb.size - rb.size), faces_mismatch=int((d > tol).sum()),
                max_vertex_diff=float(d.max()) if d.size else 0.0)


def clean_walks(r):
    """Mask of oracle / reference records whose walk closed without a
    rejected pivot or merge (tab = [s, ..., s], no negative entries)."""
    nt = np.asarray(r.ntab).astype(np.int64)
    tab = np.asarray(r.tab)
    if nt.size == 0:
        return np.zeros(0, bool)
    cols = np.arange(tab.shape[1])[None, :]
    negative = ((tab < 0) & (cols < nt[:, None])).any(1)
    last = tab[np.arange(nt.size), np.clip(nt - 1, 0, tab.shape[1] - 1)]
    return (nt >= 4) & (tab[:, 0] == last) & ~negative


def parity_report(a, b, tol=1e-5):
    """Order-free comparison split into combinatorial and numeric parts.

    regions_only_a / _b: activation states visited by one side only;
    faces_count_mismatch: common regions whose polygons have different
    vertex counts (combinatorial disagreement); faces_beyond_tol: same
    count but some vertex further than tol after the best rotation /
    orientation; max_diff over all common faces of equal size."""
    na_, nb_, only_a, only_b = _key_sets(a, b)
    sa, sb, ra, rb = _matched(a, b, 1)
    d, count_differs = _pair_distances(a, b, ra, rb)
    same = ~count_differs
    fin = np.isfinite(d) & same
    return dict(regions_a=na_, regions_b=nb_, regions_only_a=only_a, regions_only_b=only_b,
                faces_a=int((np.asarray(a.nverts)[sa] >= 3).sum()), faces_b=int((np.asarray(b.nverts)[sb] >= 3).sum()),
                common_polygons=int(ra.size), faces_count_mismatch=int(count_differs.sum()),
                faces_beyond_tol=int((same & (~np.isfinite(d) | (d > tol))).sum()),
                max_diff=float(d[fin].max()) if fin.any() else 0.0)


def region_geometry(r, i, engine_record=True):
    """(vertex count, polygon area, shortest edge, length of the edge on the
    region's start plane or nan) of region record i -- the engine's records
    carry the plane of every edge, the oracle's only the pivot table."""
    n = int(r.nverts[i])
    if n < 3:
        return n, 0.0, 0.0, float("nan")
    V = np.asarray(r.verts[i, :n], dtype=np.float64)
    e = np.linalg.norm(np.roll(V, -1, axis=0) - V, axis=1)
    c = V.mean(0)
    area = 0.5 * float(np.linalg.norm(np.cross(V - c, np.roll(V, -1, axis=0) - c).sum(0)))
    sedge = float("nan")
    st = int(r.start[i])
    if engine_record and st >= 0:
        on = np.nonzero(np.asarray(r.edges[i, :n]) == st)[0]
        if on.size:
            sedge = float(e[on].min())
    return n, area, float(e.min()), sedge


def classify_regions(r, idx, engine_record=True, length_eps=1e-5, area_eps=1e-10):
    """Why a region can be found by one run and not by another: counts of
    the records idx of run r by category -- "no_face" (fewer than 3
    vertices, or a walk that did not close), "sliver" (area below area_eps or
    an edge shorter than length_eps: a face at a near-degenerate vertex,
    whose neighbours depend on merge decisions at FP_SAME_EPS), "entry" (its
    edge on the start plane, the one its parent shared, is shorter than
    length_eps), or "other"."""
    out = {"no_face": 0, "sliver": 0, "entry": 0, "other": 0}
    others = []
    for i in idx:
        n, area, emin, sedge = region_geometry(r, i, engine_record)
        bad_status = engine_record and hasattr(r, "status") and int(r.status[i]) != 0
        if n < 3 or bad_status:
            out["no_face"] += 1
        elif area < area_eps or emin < length_eps:
            out["sliver"] += 1
        elif sedge == sedge and sedge < length_eps:
            out["entry"] += 1
        else:
            out["other"] += 1
            others.append(int(i))
    out["other_ids"] = others[:20]
    return out


def region_difference(a, b):
    """Record indices (one per key) of the regions only a visited and only b visited."""
    ka, kb = _row_keys(a.bits), _row_keys(b.bits)
    ua, ia = np.unique(ka, return_index=True)
    ub, ib = np.unique(kb, return_index=True)
    return ia[~np.isin(ua, ub)], ib[~np.isin(ub, ua)]
