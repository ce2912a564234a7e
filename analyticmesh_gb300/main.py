"""``AnalyticMarching(model, ...)``: the reference's Python entry point
(backend/main.py:335-559) on the GB300 engine.

Same arguments and the same sequence -- seed points on the surface, their
activation states from a forward pass, network info, ``cuam.Init`` when the
architecture changes, ``AnalyticMarching``, ``CombineMesh``, ``ExportMesh`` --
and the same timing keys.  The returned dict also carries the mesh
(``vertices``, ``faces``) and the marching statistics; the reference returns
timings only and leaves the mesh in the PLY file.  ``dtype`` additionally
accepts ``"mixed"`` (tensor-core composition, float32 inputs).
"""
from __future__ import annotations

import copy
import os
import tempfile
import time

import numpy as np
import torch

from . import cuam
from .seeds import dichotomy, gradient_descent, sphere_tracing
from .utils import get_boundary

SPHERE_TRACING_DICT = {
    "method": "sphere_tracing",
    "args": {"init_num": 1024, "step_size_max": 1.0, "step_size_mul": 0.5, "step_size_min": 1e-3,
             "init_ball_radius": 1.0, "avg_eps": 1e-3, "hist_len": 100, "corr_min": 0.1, "time_out": 60},
}
GRADIENT_DESCENT_DICT = {
    "method": "gradient_descent",
    "args": {"init_num": 1024, "lr_max": 1e-2, "lr_mul": 0.3, "lr_min": 1e-5, "corr_min": 0.1, "hist_len": 100,
             "loss_type": "l1", "optimizer_type": "adam", "accept_bad": True, "init_ball_radius": 1.0,
             "batch_mul": 2, "avg_eps": 1e-3, "time_out": 60},
}
DICHOTOMY_DICT = {
    "method": "dichotomy",
    "args": {"init_num": 1024, "try_pts_num": 4096, "init_ball_radius": 1.0, "iter_max": 100, "avg_eps": 1e-3,
             "time_out": 60, "provided_surfpts": None, "provided_surfstd": None},
}
VOXEL_DICT = {"voxel_size": 0.1}

CONSTRAINTS_JITTER = 1e-8  # backend/main.py:381, added to extra constraint normals
_ENVIRONMENT = ""


def _float_type(dtype):
    if isinstance(dtype, str):
        return dtype
    return "float64" if dtype == torch.float64 else "float32"


def AnalyticMarching(model, save_ply_path="mesh.ply", iso=0.0, scale=1.0, center=(0.0, 0.0, 0.0),
                     w_extra_constraints_=None, b_extra_constraints_=None, init_configs=None, save_polymesh=True,
                     save_float32_verts=True, flip_insideout=False, dtype=torch.float64, voxel_configs=None,
                     generator=None):
    """Mesh the zero (iso) level set of ``model`` exactly.

    Returns ``{"init_point_time", "init_cuda_time", "am_time", "export_time",
    "vertices", "faces", "stats"}``; writes ``save_ply_path`` unless it is None.
    In voxel mode (``voxel_configs``) every occupied voxel is marched with its
    6 faces as extra constraints, all voxels at once (one batched run), and
    the sub-meshes are concatenated; ``stats`` then sums the voxels' counts
    and ``voxel_boxes`` holds the occupied voxels' lower corners.
    """
    global _ENVIRONMENT
    init_configs = copy.deepcopy(init_configs if init_configs is not None else DICHOTOMY_DICT)
    w_ex = torch.zeros([0, 3]) if w_extra_constraints_ is None else torch.as_tensor(w_extra_constraints_).float()
    b_ex = torch.zeros([0]) if b_extra_constraints_ is None else torch.as_tensor(b_extra_constraints_).float()
    assert w_ex.shape[0] == b_ex.shape[0]
    num_extra = w_ex.shape[0] + (0 if voxel_configs is None else 6)
    ft = _float_type(dtype)
    tt = torch.float64 if ft == "float64" else torch.float32
    dev = torch.device("cuda")

    model = model.to(dev).eval()
    for p in model.parameters():
        p.requires_grad_(False)
    args = dict(init_configs["args"])
    args["w_extra_constraints"] = w_ex
    args["b_extra_constraints"] = b_ex
    out = {}
    t0 = time.time()
    method = {"dichotomy": dichotomy, "sphere_tracing": sphere_tracing, "gradient_descent": gradient_descent}
    if init_configs["method"] not in method:
        raise ValueError("No such %s" % init_configs["method"])
    points = method[init_configs["method"]](model, iso, generator=generator, device=dev, **args)
    out["init_point_time"] = time.time() - t0

    with torch.no_grad():  # states = pre-activation > 0 (backend/main.py:407-411)
        model(points, requires_outputs_list=True)
        states = torch.cat([(s > 0) for s in model.outputs_list], dim=1)
        model.outputs_list = []
    info = model.get_info()
    arc_table = info["arc_table"].to(torch.int32).cpu()
    weights = [w.to(dtype=tt, device=dev).contiguous() for w in info["weights"]]
    biases = [b.to(dtype=tt, device=dev).contiguous() for b in info["biases"]]
    arc_tm = [t.to(dtype=tt, device=dev).contiguous() for t in info["arc_tm"]]
    w_extra = (w_ex.to(dtype=tt, device=dev) + CONSTRAINTS_JITTER).contiguous()
    b_extra = b_ex.to(dtype=tt, device=dev).contiguous()
    points = points.to(dtype=tt).contiguous()
    states = states.to(torch.bool).contiguous()

    env = "float_type = %s\nnodesnum = %s\narc_table = %s\nextra = %d" % (ft, model.nodes, arc_table.tolist(),
                                                                          num_extra)
    t0 = time.time()
    if env != _ENVIRONMENT or cuam.engine() is None:
        cuam.Destroy()
        cuam.Init(float_type=ft, nodesnum=model.nodes, arc_table=arc_table, num_extra_constraints=num_extra)
        _ENVIRONMENT = env
        out["init_cuda_time"] = time.time() - t0
    else:
        out["init_cuda_time"] = 0.0

    if voxel_configs is None:
        t0 = time.time()
        cuam.AnalyticMarching(weights=weights, biases=biases, states=states, points=points, arc_tm=arc_tm,
                              w_extra_constraints=w_extra, b_extra_constraints=b_extra, iso=iso,
                              flip_insideout=flip_insideout)
        torch.cuda.synchronize()
        out["am_time"] = time.time() - t0
        t0 = time.time()
        mesh = cuam.CombineMesh(scale=scale, center=list(center))
        if save_ply_path is not None:
            cuam.ExportMesh(file_path=save_ply_path, is_polymesh=save_polymesh, is_float32=save_float32_verts)
        out["export_time"] = time.time() - t0
        out["vertices"] = mesh.verts
        out["faces"] = mesh.faces
        out["stats"] = cuam.engine().stats()
        return out

    # voxel mode (backend/main.py:475-556): every occupied voxel is marched
    # with the voxel's 6 faces as extra constraints -- here all voxels at
    # once, one engine each, in one am_run_batch (the reference loops over
    # the voxels one marching after the other); sub-meshes concatenated
    from . import engine as _engine

    vs = float(voxel_configs["voxel_size"])
    idx3 = torch.floor(points.double() / vs).long()
    imin = idx3.min(0).values
    idx3 = idx3 - imin
    dim = idx3.max(0).values + 1
    idx1 = idx3[:, 0] * dim[1] * dim[2] + idx3[:, 1] * dim[2] + idx3[:, 2]
    engines, nets, sts, pts, lows = [], [], [], [], []
    arc_np = arc_table.numpy()
    for cell in torch.unique(idx1).tolist():
        sel = torch.where(idx1 == cell)[0]
        c0 = cell // int(dim[1] * dim[2])
        c1 = (cell % int(dim[1] * dim[2])) // int(dim[2])
        c2 = cell % int(dim[2])
        lo = [(int(imin[0]) + c0) * vs, (int(imin[1]) + c1) * vs, (int(imin[2]) + c2) * vs]
        lows.append(lo)
        w_b, b_b = get_boundary("cube", min_vert=lo, max_vert=[x + vs for x in lo])
        w_all = torch.cat([w_b.to(dtype=tt, device=dev) + CONSTRAINTS_JITTER, w_extra]).contiguous()
        b_all = torch.cat([b_b.to(dtype=tt, device=dev), b_extra]).contiguous()
        nets.append(type("VoxelNet", (), dict(W=weights, b=biases, tms=arc_tm, w_extra=w_all, b_extra=b_all)))
        sts.append(states[sel].to(torch.uint8).contiguous())
        pts.append(points[sel].contiguous())
        engines.append(_engine.Engine(ft, model.nodes, arc_np, num_extra))
    t0 = time.time()
    _engine.run_batch(engines, nets, sts, pts, iso, flip_insideout)
    torch.cuda.synchronize()
    out["am_time"] = time.time() - t0
    t0 = time.time()
    all_v, all_f, nv = [], [], 0
    stats = {}
    for e in engines:
        m = e.combine(scale=scale, center=tuple(center))
        all_v.append(m.verts)
        all_f.extend([[i + nv for i in f] for f in m.faces])
        nv += len(m.verts)
        for k, v in e.stats().items():
            if k.startswith("num_") or k.startswith("mesh_num"):
                stats[k] = stats.get(k, 0) + v
        e.close()
    verts = np.concatenate(all_v) if all_v else np.zeros((0, 3))
    if save_ply_path is not None:
        write_ply(save_ply_path, verts, all_f, save_polymesh, save_float32_verts)
    stats["voxels"] = len(engines)
    out["export_time"] = time.time() - t0
    out["voxel_boxes"] = np.asarray(lows, np.float64).reshape(-1, 3)  # lower corners; edge voxel_size
    out["vertices"] = verts
    out["faces"] = all_f
    out["stats"] = stats
    return out


def write_ply(path, verts, faces, polymesh=True, float32=True):
    """Binary little-endian PLY in the reference's layout (polymesh.h:350-423)."""
    verts = np.asarray(verts)
    tris = faces if polymesh else [[f[0], f[j + 1], f[j + 2]] for f in faces for j in range(len(f) - 2)]
    ty = "float" if float32 else "double"
    with open(path, "wb") as fh:
        fh.write(("ply\nformat binary_little_endian 1.0\nelement vertex %d\nproperty %s x\nproperty %s y\n"
                  "property %s z\nelement face %d\nproperty list uchar int vertex_index\nend_header\n"
                  % (len(verts), ty, ty, ty, len(tris))).encode())
        fh.write(verts.astype("<f4" if float32 else "<f8").tobytes())
        for f in tris:
            fh.write(np.uint8(len(f)).tobytes())
            fh.write(np.asarray(f, "<i4").tobytes())


def read_ply(path):
    """Reads the binary PLY files written above / by ExportMesh."""
    with open(path, "rb") as fh:
        head = b""
        while not head.endswith(b"end_header\n"):
            head += fh.readline()
        lines = head.decode().splitlines()
        nv = int([l for l in lines if l.startswith("element vertex")][0].split()[-1])
        nf = int([l for l in lines if l.startswith("element face")][0].split()[-1])
        ty = "<f4" if "property float x" in lines else "<f8"
        verts = np.frombuffer(fh.read(nv * 3 * np.dtype(ty).itemsize), ty).reshape(nv, 3)
        faces = []
        for _ in range(nf):
            n = fh.read(1)[0]
            faces.append(list(np.frombuffer(fh.read(4 * n), "<i4")))
    return verts, faces
