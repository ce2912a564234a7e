"""CUDA engine parity through the C ABI (GPU tests).

The engine processes regions in a different order from the reference (FIFO
chunks instead of LIFO batches of 1024) and builds each face polygon by ray
shooting instead of a sorted candidate scan, so the comparison is order-free
(oracle/compare.py:canonical): identical region sets (activation bit
strings) and, per region, the same polygon up to rotation within 1e-5.
"""
import numpy as np
import pytest
import torch

from analyticmesh_gb300 import _lib, engine, workloads as wl
from oracle import compare as CM
from oracle import oracle as O

from golden_io import load, names

pytestmark = pytest.mark.gpu

TOL = {"float32": 1e-5, "float64": 1e-9}


def f_at(net, pts):
    """FP64 forward pass of the network at pts (N, 3)."""
    x = np.asarray(pts, np.float64)
    srcs = {}
    n_lin = len(net.nodes) - 1
    for i in range(n_lin):
        srcs[i] = x
        y = x @ net.W[i].T + net.b[i]
        if i >= 1:
            row = net.arc_table[i - 1]
            for c in range(int(row[0])):
                src, t = int(row[1 + 2 * c]), int(row[2 + 2 * c])
                tm = net.tms[t]
                y = y + (srcs[src] if tm.size == 0 else srcs[src] @ tm.T)
        x = np.maximum(y, 0.0) if i < n_lin - 1 else y
    return x[:, 0]


def _golden_cases():
    # fixtures where every reference walk closed cleanly; on skips_12x4 the
    # reference's walk breaks down (86% of regions hit the rejected-pivot
    # path, kernel.h:1189) and only pins the oracle
    return [n for n in names() if not n.startswith("polytope") and not n.startswith("skips")]


@pytest.mark.parametrize("name", _golden_cases())
def test_engine_matches_reference_golden(name):
    g = load(name)
    assert CM.clean_walks(g["regions"]).all()
    eng = engine.march(g["net"], g["states"], g["points"], g["dtype"], iso=g["iso"], flip_insideout=g["flip"])
    reg = eng.regions()
    c = CM.parity_report(reg, g["regions"], tol=TOL[g["dtype"]])
    # same regions, same polygons combinatorially
    assert c["regions_only_a"] == 0 and c["regions_only_b"] == 0, c
    assert c["faces_count_mismatch"] == 0, c
    # numerically: within the tolerance, or within what the face's
    # worst-conditioned vertex allows (test_parity_gpu.common_faces_agree)
    if g["dtype"] == "float32":
        from test_parity_gpu import common_faces_agree
        common_faces_agree(reg, g["regions"], True, False, eng)
    else:
        assert c["faces_beyond_tol"] == 0, c
    eng.close()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("factory,nseed", [
    (lambda: wl.geometric([32, 32], 7), 128),
    (lambda: wl.geometric([48, 48, 48], 12, perturb=0.05), 256),
    (lambda: wl.geometric([24, 24, 24, 24], 9, skips=[[0], [1, 1, 0], [1, 0, 1], [0]], tm_shapes=[[0, 0], [24, 3]]), 256),
], ids=["plain", "perturbed", "skips"])
def test_engine_matches_oracle(factory, nseed, dtype):
    m = factory()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=nseed, seed=3)
    eng = engine.march(net, st, pt, dtype)
    reg = eng.regions()
    ref = O.run_oracle(net, st, pt, dtype=dtype)
    c = CM.parity_report(reg, ref, tol=TOL[dtype])
    assert c["regions_only_a"] == 0 and c["regions_only_b"] == 0, c
    # polygons that differ combinatorially must be ones the oracle's walk did
    # not close cleanly (near-degenerate vertex merges)
    clean = CM.clean_walks(ref)
    assert c["faces_count_mismatch"] <= (~clean).sum(), c
    assert c["faces_beyond_tol"] <= max(1, c["common_polygons"] // 500), c
    # every vertex on the zero level set
    v = np.concatenate([reg.verts[i, :reg.nverts[i]] for i in range(reg.num) if reg.nverts[i] >= 3])
    assert np.abs(f_at(net, v)).max() <= (1e-5 if dtype == "float32" else 1e-10)
    eng.close()


def test_output_skip_connections_are_composed():
    # a skip into the output layer (the reference ignores it, process.h:42)
    m = wl.geometric([20, 20, 20], 31, skips=[[0], [0], [1, 1, 0]], tm_shapes=[[1, 20]])
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=4)
    eng = engine.march(net, st, pt, "float64")
    reg = eng.regions()
    assert reg.num > 0
    v = np.concatenate([reg.verts[i, :reg.nverts[i]] for i in range(reg.num) if reg.nverts[i] >= 3])
    assert np.abs(f_at(net, v)).max() <= 1e-10
    eng.close()


def test_polytope_known_answer():
    """3 -> 14 -> 1: f = sum_k |a_k . x| - 2 over 7 directions; every mesh
    vertex lies on that surface and every edge is shared by two faces."""
    m = wl.polytope()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=256, seed=5)
    eng = engine.march(net, st, pt, "float64")
    mesh = eng.combine()
    assert len(mesh.face_sizes) > 0
    dirs = np.array([[1, 1, 1], [0, 1, 1], [1, 0, 1], [1, 1, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    f = np.abs(mesh.verts @ dirs.T).sum(1) - 2.0
    assert np.abs(f).max() < 1e-5
    eng.close()


def _quantised_weld(reg, mul):
    """numpy restatement of the quantised weld on the engine's own polygons."""
    index = {}
    verts = []
    faces = []
    for r in range(reg.num):
        n = int(reg.nverts[r])
        ids = []
        for i in range(n):
            key = tuple(int(np.float32(c) * np.float32(mul)) for c in reg.verts[r, i])
            if key not in index:
                index[key] = len(verts)
                verts.append(reg.verts[r, i])
            ids.append(index[key])
        if n >= 3:
            faces.append(ids)
    return np.array(verts), faces


def test_mesh_combine_quantised_weld():
    from analyticmesh_gb300 import _lib
    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    eng = engine.march(net, st, pt, "float32")
    eng.set_option(_lib.AM_OPT_WELD, 1)
    mesh = eng.combine(scale=2.0, center=(0.1, -0.2, 0.3))
    v, f = _quantised_weld(eng.regions(), 1e6)
    assert mesh.verts.shape == v.shape
    assert mesh.faces == f
    np.testing.assert_allclose(mesh.verts, v * 2.0 + np.array([0.1, -0.2, 0.3]), atol=1e-6)
    eng.close()


def test_host_and_device_inputs_agree():
    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    e1 = engine.march(net, st, pt, "float32")
    dev = torch.device("cuda")
    e2 = engine.Engine("float32", net.nodes, net.arc_table, 0)
    e2.run([torch.tensor(w, dtype=torch.float32, device=dev) for w in net.W],
           [torch.tensor(b, dtype=torch.float32, device=dev) for b in net.b],
           torch.tensor(st, dtype=torch.bool, device=dev), torch.tensor(pt, dtype=torch.float32, device=dev))
    r1, r2 = e1.regions(), e2.regions()
    assert np.array_equal(r1.bits, r2.bits) and np.array_equal(r1.nverts, r2.nverts)
    e1.close()
    e2.close()


@pytest.mark.parametrize("form", ["float32", "mixed", "float64"])
@pytest.mark.parametrize("chunk", [0, 700])
def test_graph_loop_matches_host_loop(form, chunk):
    """The device-driven wave loop (one CUDA graph with a conditional while
    node) gives the same regions, in the same order, as the host-driven loop;
    a small chunk forces many waves, multi-tile launches and relaunches of
    the graph after the region store grows."""
    m = wl.sphere() if form != "float64" else wl.geometric([48, 48, 48], 5)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=256, seed=3)
    out = {}
    for graph in (0, 1):
        eng = engine.Engine(form, net.nodes, net.arc_table, net.num_extra)
        eng.set_option(_lib.AM_OPT_GRAPH, graph)
        if chunk:
            eng.set_option(_lib.AM_OPT_CHUNK, chunk)
        eng.run_net(net, st, pt)
        out[graph] = (eng.stats(), eng.regions())
        eng.close()
    (s0, r0), (s1, r1) = out[0], out[1]
    assert s0["num_regions"] == s1["num_regions"] and s0["num_faces"] == s1["num_faces"]
    assert s0["chunks"] == s1["chunks"]
    assert np.array_equal(r0.bits, r1.bits)
    assert np.array_equal(r0.nverts, r1.nverts)
    assert np.array_equal(r0.verts, r1.verts)


def test_region_limit_stops_and_keeps_results():
    """AM_OPT_MAX_REGIONS: the run stops after the wave that passes the limit,
    returns AM_ERR_CAPACITY, and the regions found so far stay queryable."""
    m = wl.geometric([64, 64], 21, perturb=0.01)
    net = wl.net_arrays(m)
    # four seeds: the search spreads over many waves
    st, pt = wl.seeds_for(m, init_num=128, seed=4)
    st, pt = st[:4], pt[:4]
    full = engine.march(net, st, pt, "float32")
    total, seeds = full.stats()["num_regions"], full.stats()["num_seeds"]
    full.close()
    limit = 200
    assert seeds <= 4 and limit < total // 4
    for graph in (0, 1):
        eng = engine.Engine("float32", net.nodes, net.arc_table, 0)
        eng.set_option(_lib.AM_OPT_GRAPH, graph)
        eng.set_option(_lib.AM_OPT_MAX_REGIONS, limit)
        with pytest.raises(_lib.AmError, match="region limit"):
            eng.run_net(net, st, pt)
        got = eng.stats()["num_regions"]
        assert limit < got < total
        rows, eq = eng.region_rows(0, 100)
        assert np.isfinite(rows).all() and np.isfinite(eq).all()
        eng.close()


@pytest.mark.parametrize("form", ["mixed", "float32"])
def test_warps_per_face_give_the_same_faces(form):
    """AM_OPT_FACE_WARPS: one warp per face, or 2, 4, 8 warps splitting the
    walk's scan over the rows -- the same regions, faces and vertices."""
    m = wl.geometric([256, 256, 256], 14, perturb=0.02)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=7)
    out = {}
    for G in (1, 2, 4, 8):
        eng = engine.march(net, st, pt, form, options={_lib.AM_OPT_FACE_WARPS: G})
        r = eng.regions()
        out[G] = (eng.stats()["num_regions"], r.bits.copy(), r.nverts.copy(), r.verts.copy(), r.edges.copy())
        eng.close()
    for G in (2, 4, 8):
        assert out[G][0] == out[1][0], G
        for a, b in zip(out[G][1:], out[1][1:]):
            assert np.array_equal(a, b), G


def test_autotune_chooses_options_and_keeps_results():
    """am_autotune: sample runs pick the composition tile and the warps per
    face; the marching afterwards gives the same regions as the defaults, and
    a second engine of the same architecture takes the remembered choice."""
    m = wl.geometric([256, 256], 5, perturb=0.01)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=2)
    ref = engine.march(net, st, pt, "mixed")
    want = ref.regions().bits.copy()
    ref.close()
    eng = engine.Engine("mixed", net.nodes, net.arc_table, 0)
    tile, warps = engine.autotune(eng, net, st, pt, sample_regions=3000)
    assert tile in (1, 2) and warps in (1, 2, 4, 8)
    eng.run_net(net, st, pt)
    assert np.array_equal(eng.regions().bits, want)
    eng.close()
    again = engine.Engine("mixed", net.nodes, net.arc_table, 0)
    assert engine.autotune(again, net, st, pt, sample_regions=3000) == (tile, warps)
    again.close()


def _outward_fraction(mesh):
    """Share of faces whose right-hand normal points away from the origin
    (the sphere-like surfaces here enclose it)."""
    V = mesh.verts
    dots = []
    for f in mesh.faces:
        P = V[f]
        c = P.mean(0)
        n = np.cross(P - c, np.roll(P, -1, 0) - c).sum(0)
        dots.append(n @ c)
    return float((np.array(dots) > 0).mean())


@pytest.mark.parametrize("form", ["float32", "mixed"])
def test_face_orientation_and_flip_insideout(form):
    """Faces run counter-clockwise about the gradient, so their normals point
    outward as the reference orients them (correctNormalDirection,
    kernel.h:1325-1385); flip_insideout reverses every face."""
    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    meshes = {}
    for flip in (False, True):
        eng = engine.march(net, st, pt, form, flip_insideout=flip)
        meshes[flip] = eng.combine()
        frac = _outward_fraction(meshes[flip])
        assert (frac > 0.999) if not flip else (frac < 0.001), (flip, frac)
        eng.close()
    a, b = meshes[False], meshes[True]
    # faces come in region order: face i of the flipped mesh is face i reversed
    assert len(a.faces) == len(b.faces)
    for fa, fb in zip(a.faces, b.faces):
        assert len(fa) == len(fb)
        np.testing.assert_allclose(a.verts[fa[::-1]], b.verts[fb], rtol=0, atol=1e-6)
