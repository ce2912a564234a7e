"""Generate the golden fixtures: the reference's own marching loop (compiled
for the CPU by oracle/build_ref.py from the reference checkout, run with one
thread so every racy choice is settled in thread-index order) on small seeded
networks.  Each .npz holds the inputs and the reference's per-region records
and welded mesh.

    python tests/golden/make_golden.py

The reference checkout must be present (it is not on the GPU machine; the
fixtures are committed so the tests run without it).
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from analyticmesh_gb300 import workloads as wl  # noqa: E402
from oracle import oracle as O  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def cases():
    """(name, model factory, seeds, dtype, extra constraints, iso, flip)"""
    box = (np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0]], float) + 1e-8, np.array([-0.2, -0.3, -0.1]))
    return [
        ("polytope_f32", wl.polytope, 256, "float32", None, 0.0, False),
        ("polytope_f64", wl.polytope, 256, "float64", None, 0.0, False),
        ("plain_16x2_f32", lambda: wl.geometric([16, 16], 21), 64, "float32", None, 0.0, False),
        ("plain_16x3_f64", lambda: wl.geometric([16] * 3, 22), 64, "float64", None, 0.0, True),
        ("skips_12x4_f32", lambda: wl.geometric([12, 12, 12, 12], 23, skips=[[0], [1, 1, 0], [1, 0, 1], [0]],
                                                tm_shapes=[[0, 0], [12, 3]]), 64, "float32", None, 0.0, False),
        ("extra_16x2_f32", lambda: wl.geometric([16, 16], 24), 64, "float32", box, 0.0, False),
        ("iso_16x2_f32", lambda: wl.geometric([16, 16], 25), 64, "float32", None, 0.1, False),
    ]


def pack_regions(r):
    nv = r.nverts.astype(np.int32)
    nt = r.ntab.astype(np.int32)
    verts = np.concatenate([r.verts[i, :max(nv[i], 0)] for i in range(r.num)] or [np.zeros((0, 3))])
    tab = np.concatenate([r.tab[i, :nt[i]] for i in range(r.num)] or [np.zeros(0, np.int32)])
    return dict(r_bits=r.bits, r_nverts=nv, r_verts=verts, r_ntab=nt, r_tab=tab.astype(np.int32), r_mid=r.mid,
                r_start=r.start)


def main():
    for name, mk, nseed, dt, extra, iso, flip in cases():
        m = mk()
        net = wl.net_arrays(m)
        if extra is not None:
            net.w_extra, net.b_extra = extra
        st, pt = wl.seeds_for(m, init_num=nseed, seed=5, iso=iso, w_extra=net.w_extra if extra is not None else None,
                              b_extra=net.b_extra if extra is not None else None)
        regions, mesh = O.run_ref(net, st, pt, iso=iso, flip=flip, dtype=dt, combine=(1.0, [0.0, 0.0, 0.0]))
        fl = np.array([len(f) for f in mesh.faces], np.int32)
        fidx = np.concatenate([np.asarray(f, np.int32) for f in mesh.faces] or [np.zeros(0, np.int32)])
        arrs = dict(nodes=np.asarray(net.nodes, np.int32), arc_table=net.arc_table, w_extra=net.w_extra,
                    b_extra=net.b_extra, states=st, points=pt, iso=np.float64(iso), flip=np.int32(flip),
                    dtype=np.array(dt), m_verts=mesh.verts, m_flen=fl, m_fidx=fidx, **pack_regions(regions))
        for i, (w, b) in enumerate(zip(net.W, net.b)):
            arrs["W%d" % i] = w
            arrs["b%d" % i] = b
        for i, t in enumerate(net.tms):
            arrs["tm%d" % i] = t
        arrs["n_tm"] = np.int32(len(net.tms))
        out = os.path.join(HERE, name + ".npz")
        np.savez_compressed(out, **arrs)
        print("%-16s regions=%5d faces=%5d verts=%5d  %6.1f KB" % (name, regions.num, len(mesh.faces),
                                                                   len(mesh.verts), os.path.getsize(out) / 1024))


if __name__ == "__main__":
    main()
