"""Loader for the golden fixtures in tests/golden (see make_golden.py)."""
import glob
import os

import numpy as np

from analyticmesh_gb300.workloads import NetArrays
from oracle.oracle import Mesh, Regions, VERT_MAX

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    """The marching fixtures (seeds_*.npz hold seed-point fixtures instead)."""
    all_ = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    return [n for n in all_ if not n.startswith("seeds_")]


def load(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as f:
        z = {k: f[k] for k in f.files}  # NpzFile decompresses on every access
    nodes = [int(x) for x in z["nodes"]]
    n_lin = len(nodes) - 1
    net = NetArrays(nodes=nodes, W=[z["W%d" % i] for i in range(n_lin)], b=[z["b%d" % i] for i in range(n_lin)],
                    arc_table=z["arc_table"], tms=[z["tm%d" % i] for i in range(int(z["n_tm"]))],
                    w_extra=z["w_extra"], b_extra=z["b_extra"])
    nvs, nts, rv, rt = z["r_nverts"], z["r_ntab"], z["r_verts"], z["r_tab"]
    R = nvs.shape[0]
    verts = np.zeros((R, VERT_MAX, 3))
    tab = np.zeros((R, VERT_MAX + 1), np.int32)
    vo = to = 0
    for i in range(R):
        nv, nt = int(nvs[i]), int(nts[i])
        verts[i, :nv] = rv[vo:vo + nv]
        tab[i, :nt] = rt[to:to + nt]
        vo += nv
        to += nt
    N = sum(nodes[1:-1])
    regions = Regions(N=N, bits=z["r_bits"], nverts=z["r_nverts"], verts=verts, ntab=z["r_ntab"], tab=tab,
                      mid=z["r_mid"], start=z["r_start"])
    faces, o = [], 0
    fidx = z["m_fidx"]
    for L in z["m_flen"]:
        faces.append(list(fidx[o:o + L]))
        o += int(L)
    mesh = Mesh(verts=z["m_verts"], faces=faces)
    return dict(net=net, states=z["states"], points=z["points"], iso=float(z["iso"]), flip=bool(z["flip"]),
                dtype=str(z["dtype"]), regions=regions, mesh=mesh)
