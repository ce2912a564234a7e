"""The package's public entry point ``AnalyticMarching(model, ...)`` (the
reference's backend/main.py:335-559) on the GPU, used the way the reference's
examples use it: a network built with ``MLP(...)`` or loaded with
``load_model``, marched, its mesh returned and written as a PLY; and the
voxel mode (backend/main.py:475-556)."""
import numpy as np
import pytest
import torch

from analyticmesh_gb300 import MLP, AnalyticMarching, load_model, save_model, workloads as wl
from analyticmesh_gb300.main import read_ply

pytestmark = pytest.mark.gpu

# |f(v)| bounds per form: FP64 vertices, and the gate of the FP32-input forms
F_TOL = {torch.float64: 1e-9, "mixed": 1e-5, torch.float32: 1e-5}


def _f64(net, pts):
    """FP64 forward pass of a plain MLP (no skips) at pts (n, 3)."""
    x = np.asarray(pts, np.float64)
    n_lin = len(net.W)
    for i in range(n_lin):
        x = x @ net.W[i].T + net.b[i]
        if i < n_lin - 1:
            x = np.maximum(x, 0.0)
    return x[:, 0]


def _check_mesh(verts, faces):
    verts = np.asarray(verts)
    assert verts.ndim == 2 and verts.shape[1] == 3 and len(faces) > 0
    assert all(len(f) >= 3 for f in faces)
    idx = np.concatenate([np.asarray(f) for f in faces])
    assert idx.min() >= 0 and idx.max() < len(verts)


@pytest.mark.parametrize("dtype", [torch.float64, "mixed"], ids=["float64", "mixed"])
def test_saved_and_loaded_network_marches_and_writes_its_mesh(tmp_path, dtype):
    torch.manual_seed(3)
    model = MLP(nodes=[3, 48, 48, 1], arc_table=[[0]] * 2, arc_tm_shape=[], geometric_radius=0.5,
                enable_print=False)
    onnx_path = str(tmp_path / "sphere.onnx")
    save_model(model, onnx_path)
    loaded = load_model(onnx_path)
    net = wl.net_arrays(loaded)  # float64 copies of the float32 parameters
    ply = str(tmp_path / "sphere.ply")
    out = AnalyticMarching(loaded, ply, dtype=dtype, generator=torch.Generator().manual_seed(4))
    for key in ("init_point_time", "init_cuda_time", "am_time", "export_time", "vertices", "faces", "stats"):
        assert key in out
    verts, faces = np.asarray(out["vertices"]), out["faces"]
    _check_mesh(verts, faces)
    assert len(faces) == out["stats"]["num_faces"]
    assert np.abs(_f64(net, verts)).max() <= F_TOL[dtype]
    # the PLY holds the returned mesh (float32 vertices, polygons)
    pv, pf = read_ply(ply)
    assert pv.shape == verts.shape
    np.testing.assert_allclose(pv, verts, rtol=0, atol=1e-6)
    assert [list(map(int, f)) for f in pf] == [list(map(int, f)) for f in faces]


def _poly_area(p):
    """Area of a planar polygon (k, 3)."""
    if len(p) < 3:
        return 0.0
    c = np.cross(p[1:-1] - p[0], p[2:] - p[0])
    return 0.5 * np.linalg.norm(c.sum(0))


def _clip_box(p, lo, hi):
    """A convex polygon (k, 3) clipped to the box [lo, hi] (Sutherland-Hodgman)."""
    for ax in range(3):
        for sgn, lim in ((1.0, hi[ax]), (-1.0, lo[ax])):
            if len(p) == 0:
                return p
            d = sgn * (p[:, ax] - lim)  # <= 0 inside
            out = []
            for i in range(len(p)):
                a, b, da, db = p[i], p[(i + 1) % len(p)], d[i], d[(i + 1) % len(p)]
                if da <= 0:
                    out.append(a)
                if (da < 0 < db) or (db < 0 < da):
                    out.append(a + (b - a) * (da / (da - db)))
            p = np.asarray(out).reshape(-1, 3)
    return p


def test_voxel_mode_meshes_the_surface_inside_each_voxel():
    """Voxel mode marches all occupied voxels in one batched run, each with
    its 6 faces as extra constraints: every vertex is on the level set, and a
    voxel's mesh covers the part of the whole surface inside that voxel --
    its area is the area of the whole marching's mesh clipped to the voxel
    (a voxel may miss a piece of the surface that holds none of its seeds,
    and then has less, never more)."""
    model = wl.geometric([32, 32], 7)
    net = wl.net_arrays(model)
    vs = 0.25
    out = AnalyticMarching(model, None, dtype=torch.float64, voxel_configs={"voxel_size": vs},
                           generator=torch.Generator().manual_seed(2))
    verts, faces = np.asarray(out["vertices"]), out["faces"]
    _check_mesh(verts, faces)
    assert np.abs(_f64(net, verts)).max() <= F_TOL[torch.float64]
    boxes = out["voxel_boxes"]
    assert out["stats"]["voxels"] == len(boxes) > 1
    assert out["stats"]["num_faces"] == len(faces)
    whole = AnalyticMarching(model, None, dtype=torch.float64, generator=torch.Generator().manual_seed(2))
    wv = np.asarray(whole["vertices"])
    wpolys = [wv[np.asarray(f)] for f in whole["faces"]]
    wlo = np.array([p.min(0) for p in wpolys])
    whi = np.array([p.max(0) for p in wpolys])
    vpolys = [verts[np.asarray(f)] for f in faces]
    cent = np.array([p.mean(0) for p in vpolys])
    agree, total_v, total_w = 0, 0.0, 0.0
    for lo in boxes:
        hi = lo + vs
        # the voxel's own faces (centroids inside the box)
        inside = np.all((cent >= lo - 1e-9) & (cent <= hi + 1e-9), axis=1)
        a_vox = sum(_poly_area(vpolys[i]) for i in np.where(inside)[0])
        near = np.where(np.all((whi >= lo) & (wlo <= hi), axis=1))[0]
        a_whole = sum(_poly_area(_clip_box(wpolys[i], lo, hi)) for i in near)
        assert a_vox <= a_whole * (1 + 1e-6) + 1e-12, (lo, a_vox, a_whole)
        agree += abs(a_vox - a_whole) <= 1e-6 * max(a_whole, 1e-6)
        total_v += a_vox
        total_w += a_whole
    assert agree >= 0.9 * len(boxes), (agree, len(boxes))
    assert total_v >= 0.97 * total_w


def test_export_triangles_and_double_vertices(tmp_path):
    """ExportMesh's other layouts (backend/inc/polymesh.h:350-423): triangle
    fans instead of polygons, float64 instead of float32 vertices."""
    from analyticmesh_gb300 import engine

    m = wl.geometric([32, 32], 7)
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=11)
    eng = engine.march(net, st, pt, "float64")
    mesh = eng.combine(scale=2.0, center=(0.5, 0.0, -1.0))
    path = str(tmp_path / "tri.ply")
    eng.export(path, is_polymesh=False, is_float32=False)
    pv, pf = read_ply(path)
    assert pv.dtype == np.float64 and np.array_equal(pv, mesh.verts)
    fans = [[int(f[0]), int(f[j + 1]), int(f[j + 2])] for f in mesh.faces for j in range(len(f) - 2)]
    assert [list(map(int, f)) for f in pf] == fans
    eng.close()


def test_reference_call_sequence_through_the_cuam_drop_in(tmp_path):
    """The reference's own sequence of backend/main.py:376-472 with
    ``from analyticmesh_gb300 import cuam as cuamlib`` in place of
    ``build.cuam``: the same tensor preparation (bool states and points moved
    to the CPU and back, int32 CPU arc table, jittered extra constraints),
    Destroy at re-initialisation, Init, AnalyticMarching, CombineMesh,
    ExportMesh; the PLY written is the marching's welded mesh."""
    from analyticmesh_gb300 import cuam as cuamlib
    from analyticmesh_gb300.seeds import dichotomy

    model = wl.geometric([32, 32], 7).cuda().eval()
    net = wl.net_arrays(model)
    dtype = torch.float64
    w_ex, b_ex = torch.zeros([0, 3]), torch.zeros([0])
    points = dichotomy(model, 0.0, init_num=256, generator=torch.Generator().manual_seed(5), device="cuda")
    with torch.no_grad():
        model(points, requires_outputs_list=True)
        states = torch.cat([(s > 0) for s in model.outputs_list], dim=1)
        model.outputs_list = []
    info = model.get_info()
    arc_table = info["arc_table"].to(dtype=torch.int32).cpu()
    weights = [w.to(dtype=dtype).cuda() for w in info["weights"]]
    biases = [b.to(dtype=dtype).cuda() for b in info["biases"]]
    states = states.to(dtype=torch.bool).cpu()
    points = points.to(dtype=dtype).cpu()
    arc_tm = [t.to(dtype=dtype).cuda() for t in info["arc_tm"]]
    w_extra = w_ex.to(dtype=dtype).cuda()
    b_extra = b_ex.to(dtype=dtype).cuda()
    w_extra += 1e-8
    faces = []
    for rep in range(2):  # the second pass re-initialises as after an architecture change
        if rep:
            cuamlib.Destroy()
        cuamlib.Init(float_type="float64", nodesnum=model.nodes, arc_table=arc_table, num_extra_constraints=0)
        cuamlib.AnalyticMarching(weights=weights, biases=biases, states=states.cuda(), points=points.cuda(),
                                 arc_tm=arc_tm, w_extra_constraints=w_extra, b_extra_constraints=b_extra, iso=0.0,
                                 flip_insideout=False)
        mesh = cuamlib.CombineMesh(scale=1.0, center=[0.0, 0.0, 0.0])
        ply = str(tmp_path / ("m%d.ply" % rep))
        cuamlib.ExportMesh(file_path=ply, is_polymesh=True, is_float32=False)
        pv, pf = read_ply(ply)
        assert np.array_equal(pv, mesh.verts)
        assert [list(map(int, f)) for f in pf] == [list(map(int, f)) for f in mesh.faces]
        assert np.abs(_f64(net, pv)).max() <= F_TOL[torch.float64]
        faces.append(len(pf))
    cuamlib.Destroy()
    assert faces[0] == faces[1] > 0
