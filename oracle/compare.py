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


def canonical(a_regions, b_regions, tol=1e-5):
    """Order-free comparison.  Returns a dict of counts."""
    ka = {_key(x) for x in a_regions.bits}
    kb = {_key(x) for x in b_regions.bits}
    pa = Polygons.from_regions(a_regions).faces
    pb = Polygons.from_regions(b_regions).faces
    common = set(pa) & set(pb)
    worst = 0.0
    bad = 0
    for k in common:
        d = cycle_distance(pa[k], pb[k])
        worst = max(worst, d)
        if d > tol:
            bad += 1
    return dict(regions_a=len(ka), regions_b=len(kb), only_a=len(ka - kb), only_b=len(kb - ka),
                faces_a=len(pa), faces_b=len(pb), faces_only_a=len(set(pa) - set(pb)),
                faces_only_b=len(set(pb) - set(pa)), faces_mismatch=bad, max_vertex_diff=worst)


def clean_walks(r):
    """Mask of oracle / reference records whose walk closed without a
    rejected pivot or merge (tab = [s, ..., s], no negative entries)."""
    ok = np.zeros(r.num, bool)
    for i in range(r.num):
        nt = int(r.ntab[i])
        t = r.tab[i, :nt]
        ok[i] = nt >= 4 and t[0] == t[nt - 1] and (t >= 0).all()
    return ok


def parity_report(a, b, tol=1e-5):
    """Order-free comparison split into combinatorial and numeric parts.

    regions_only_a / _b: activation states visited by one side only;
    faces_count_mismatch: common regions whose polygons have different
    vertex counts (combinatorial disagreement); faces_beyond_tol: same
    count but some vertex further than tol after the best rotation /
    orientation; max_diff over all common faces of equal size."""
    ka = {x.tobytes() for x in a.bits}
    kb = {x.tobytes() for x in b.bits}
    pa = Polygons.from_regions(a, min_verts=1).faces
    pb = Polygons.from_regions(b, min_verts=1).faces
    common = set(pa) & set(pb)
    count_mm = beyond = 0
    worst = 0.0
    for k in common:
        if pa[k].shape != pb[k].shape:
            count_mm += 1
            continue
        d = cycle_distance(pa[k], pb[k])
        if not np.isfinite(d) or d > tol:
            beyond += 1
        if np.isfinite(d):
            worst = max(worst, d)
    fa = sum(1 for k in pa if pa[k].shape[0] >= 3)
    fb = sum(1 for k in pb if pb[k].shape[0] >= 3)
    return dict(regions_a=len(ka), regions_b=len(kb), regions_only_a=len(ka - kb), regions_only_b=len(kb - ka),
                faces_a=fa, faces_b=fb, common_polygons=len(common), faces_count_mismatch=count_mm,
                faces_beyond_tol=beyond, max_diff=worst)
