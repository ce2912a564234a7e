"""ctypes front end of the CPU parity checkers -- TEST INFRASTRUCTURE ONLY.

``run_oracle`` drives the C restatement (oracle/am_oracle.c), ``run_ref``
drives the reference's own loop compiled for the CPU (oracle/_ref).  Both
return ``Regions``: one record per popped region, in processing order.
Only tests/, __graft_entry__.smoke() and bench.py's CPU legs use this module.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
import os

import numpy as np

from . import build_ref

VERT_MAX = 20


@dataclasses.dataclass
class Regions:
    N: int
    bits: np.ndarray      # (R, words) uint32
    nverts: np.ndarray    # (R,)
    verts: np.ndarray     # (R, VERT_MAX, 3) float64
    ntab: np.ndarray      # (R,)
    tab: np.ndarray       # (R, VERT_MAX + 1)
    mid: np.ndarray       # (R, 3)
    start: np.ndarray     # (R,)
    seeds_kept: int = -1

    @property
    def num(self) -> int:
        return int(self.nverts.shape[0])


@dataclasses.dataclass
class Mesh:
    verts: np.ndarray     # (V, 3)
    faces: list           # list of index lists


class _amo_net(C.Structure):
    _fields_ = [
        ("n_lin", C.c_int), ("nodes", C.POINTER(C.c_int)), ("W", C.POINTER(C.c_void_p)), ("b", C.POINTER(C.c_void_p)),
        ("arc_table", C.POINTER(C.c_int)), ("arc_cols", C.c_int), ("n_tm", C.c_int), ("tm", C.POINTER(C.c_void_p)),
        ("tm_shape", C.POINTER(C.c_int)), ("E", C.c_int), ("w_extra", C.c_void_p), ("b_extra", C.c_void_p),
        ("output_skips", C.c_int),
    ]


_ORACLE = None
_REF = None


def oracle_lib():
    global _ORACLE
    if _ORACLE is None:
        path = build_ref.ORACLE_SO
        if not os.path.exists(path):
            build_ref.build_oracle()
        lib = C.CDLL(path)
        lib.amo_run_f32.restype = C.c_int
        lib.amo_run_f64.restype = C.c_int
        lib.amo_fnv1a.restype = C.c_uint32
        lib.amo_fnv1.restype = C.c_uint32
        lib.amo_combine.argtypes = [C.c_void_p, C.c_double, C.POINTER(C.c_double)]
        for n in ("amo_num_regions", "amo_state_len", "amo_num_seeds_kept", "amo_mesh_num_verts", "amo_mesh_num_faces"):
            getattr(lib, n).argtypes = [C.c_void_p]
        lib.amo_get_regions.argtypes = [C.c_void_p] + [C.c_void_p] * 7
        lib.amo_get_mesh.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        lib.amo_free.argtypes = [C.c_void_p]
        lib.amo_set_region_budget.argtypes = [C.c_long]
        _ORACLE = lib
    return _ORACLE


def ref_available() -> bool:
    try:
        return ref_lib() is not None
    except Exception:
        return False


def ref_lib():
    global _REF
    if _REF is None:
        path = build_ref.REF_SO
        if not os.path.exists(path):
            path = build_ref.build_ref()
            if path is None:
                return None
        lib = C.CDLL(path)
        lib.amref_run.restype = C.c_int
        lib.amref_combine.argtypes = [C.c_double, C.POINTER(C.c_double)]
        lib.amref_get_regions.argtypes = [C.c_void_p] * 7
        lib.amref_get_mesh.argtypes = [C.c_void_p, C.c_void_p]
        lib.amref_export.argtypes = [C.c_char_p, C.c_int, C.c_int]
        lib.amref_last_seconds.restype = C.c_double
        lib.amref_set_region_budget.argtypes = [C.c_long]
        _REF = lib
    return _REF


class _Packed:
    """Keeps the numpy buffers alive for one call."""

    def __init__(self, net, dtype):
        npt = np.float64 if dtype == "float64" else np.float32
        self.npt = npt
        self.nodes = np.ascontiguousarray(net.nodes, dtype=np.int32)
        self.W = [np.ascontiguousarray(w, dtype=npt) for w in net.W]
        self.b = [np.ascontiguousarray(x, dtype=npt) for x in net.b]
        self.arc = np.ascontiguousarray(net.arc_table, dtype=np.int32)
        if self.arc.ndim != 2 or self.arc.shape[1] == 0:
            self.arc = np.zeros((len(net.nodes) - 2, 1), dtype=np.int32)
        self.tms = [np.ascontiguousarray(t, dtype=npt) if t.size else np.zeros(1, dtype=npt) for t in net.tms]
        self.tm_shape = np.ascontiguousarray([s for t in net.tms for s in t.shape] or [0], dtype=np.int32)
        self.we = np.ascontiguousarray(net.w_extra, dtype=npt).reshape(-1) if net.num_extra else np.zeros(3, dtype=npt)
        self.be = np.ascontiguousarray(net.b_extra, dtype=npt).reshape(-1) if net.num_extra else np.zeros(1, dtype=npt)
        self.Wp = (C.c_void_p * len(self.W))(*[w.ctypes.data for w in self.W])
        self.bp = (C.c_void_p * len(self.b))(*[x.ctypes.data for x in self.b])
        self.tmp = (C.c_void_p * max(1, len(self.tms)))(*([t.ctypes.data for t in self.tms] or [None]))
        self.n_tm = len(net.tms)
        self.E = net.num_extra


def _inputs(states, points, npt):
    st = np.ascontiguousarray(states, dtype=np.uint8)
    pt = np.ascontiguousarray(points, dtype=npt)
    assert st.ndim == 2 and pt.shape == (st.shape[0], 3)
    return st, pt


def _alloc_regions(R, N):
    words = (N + 31) // 32
    return dict(bits=np.zeros((R, words), np.uint32), nverts=np.zeros(R, np.int32),
                verts=np.zeros((R, VERT_MAX, 3), np.float64), ntab=np.zeros(R, np.int32),
                tab=np.zeros((R, VERT_MAX + 1), np.int32), mid=np.zeros((R, 3), np.float64), start=np.zeros(R, np.int32))


def _ptrs(d):
    return [d[k].ctypes.data for k in ("bits", "nverts", "verts", "ntab", "tab", "mid", "start")]


def run_oracle(net, states, points, iso=0.0, flip=False, dtype="float32", output_skips=False, combine=None,
               region_budget=0):
    """Run the restatement.  ``combine=(scale, center)`` also welds the mesh.
    ``region_budget`` stops the loop at the end of the first batch that
    reaches that many regions (timed samples; 0 = run to completion)."""
    lib = oracle_lib()
    p = _Packed(net, dtype)
    st, pt = _inputs(states, points, p.npt)
    cn = _amo_net(len(net.nodes) - 1, p.nodes.ctypes.data_as(C.POINTER(C.c_int)), p.Wp, p.bp,
                  p.arc.ctypes.data_as(C.POINTER(C.c_int)), p.arc.shape[1], p.n_tm, p.tmp,
                  p.tm_shape.ctypes.data_as(C.POINTER(C.c_int)), p.E, p.we.ctypes.data, p.be.ctypes.data,
                  1 if output_skips else 0)
    res = C.c_void_p()
    fn = lib.amo_run_f64 if dtype == "float64" else lib.amo_run_f32
    lib.amo_set_region_budget(int(region_budget))
    try:
        rc = fn(C.byref(cn), st.ctypes.data_as(C.c_void_p), pt.ctypes.data_as(C.c_void_p), st.shape[0],
                C.c_double(iso), 1 if flip else 0, C.byref(res))
    finally:
        lib.amo_set_region_budget(0)
    if rc != 0:
        raise RuntimeError("oracle run failed: %d" % rc)
    try:
        R = lib.amo_num_regions(res)
        N = lib.amo_state_len(res)
        d = _alloc_regions(R, N)
        lib.amo_get_regions(res, *_ptrs(d))
        regions = Regions(N=N, seeds_kept=lib.amo_num_seeds_kept(res), **d)
        mesh = None
        if combine is not None:
            scale, center = combine
            c3 = (C.c_double * 3)(*center)
            lib.amo_combine(res, C.c_double(scale), c3)
            mesh = _read_mesh(lib.amo_mesh_num_verts(res), lib.amo_mesh_num_faces(res),
                              lambda v, f: lib.amo_get_mesh(res, v, f))
    finally:
        lib.amo_free(res)
    return (regions, mesh) if combine is not None else regions


def _read_mesh(nv, nf, getter):
    v = np.zeros((max(nv, 1), 3), np.float64)
    f = np.zeros((max(nf, 1), 1 + VERT_MAX), np.int32)
    getter(v.ctypes.data, f.ctypes.data)
    faces = [list(f[i, 1:1 + f[i, 0]]) for i in range(nf)]
    return Mesh(verts=v[:nv].copy(), faces=faces)


def run_ref(net, states, points, iso=0.0, flip=False, dtype="float32", combine=None, export=None, threads=1,
            region_budget=0, timing=None):
    """Run the reference's own loop on the CPU.  ``threads=1`` executes every
    launch in thread-index order (deterministic, the parity setting);
    ``export=(path, poly, f32)`` writes its PLY after combining;
    ``region_budget`` stops the loop after that many regions (timed samples);
    ``timing`` (a dict) receives the wall time of the marching call."""
    lib = ref_lib()
    if lib is None:
        raise RuntimeError("reference CPU build unavailable")
    lib.amref_set_threads(int(threads))
    lib.amref_set_region_budget(int(region_budget))
    p = _Packed(net, dtype)
    st, pt = _inputs(states, points, p.npt)
    rc = lib.amref_run(1 if dtype == "float64" else 0, len(net.nodes) - 1, p.nodes.ctypes.data_as(C.c_void_p), p.Wp,
                       p.bp, p.arc.ctypes.data_as(C.c_void_p), p.arc.shape[1], p.n_tm, p.tmp,
                       p.tm_shape.ctypes.data_as(C.c_void_p), p.E, C.c_void_p(p.we.ctypes.data),
                       C.c_void_p(p.be.ctypes.data), st.ctypes.data_as(C.c_void_p), pt.ctypes.data_as(C.c_void_p),
                       st.shape[0], C.c_double(iso), 1 if flip else 0)
    if rc != 0:
        raise RuntimeError("reference run failed: %d" % rc)
    if timing is not None:
        timing["am_seconds"] = lib.amref_last_seconds()
    R = lib.amref_num_regions()
    N = lib.amref_state_len()
    d = _alloc_regions(R, N)
    lib.amref_get_regions(*_ptrs(d))
    regions = Regions(N=N, **d)
    mesh = None
    if combine is not None:
        scale, center = combine
        lib.amref_combine(C.c_double(scale), (C.c_double * 3)(*center))
        mesh = _read_mesh(lib.amref_mesh_num_verts(), lib.amref_mesh_num_faces(), lambda v, f: lib.amref_get_mesh(v, f))
        if export is not None:
            path, poly, f32 = export
            lib.amref_export(path.encode(), 1 if poly else 0, 1 if f32 else 0)
    lib.amref_destroy()
    return (regions, mesh) if combine is not None else regions
