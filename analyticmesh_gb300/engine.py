"""Handle-based Python front end of the C ABI.

``Engine`` owns one ``am_engine`` (include/analyticmesh_gb300.h).  Array
arguments may be numpy arrays or torch tensors on the CPU or the GPU; they
are passed to the library as raw pointers and must stay alive for the call,
which this class takes care of.
"""
from __future__ import annotations

import ctypes as C
import dataclasses
from typing import List, Optional, Sequence

import numpy as np

from . import _lib

FLOAT_TYPES = ("float32", "float64", "mixed")


def _np_dtype(float_type: str):
    return np.float64 if float_type == "float64" else np.float32


class _Keep:
    """Collects the buffers whose pointers were handed to the library."""

    def __init__(self):
        self.objs = []

    def ptr(self, x, dtype):
        import torch

        if x is None:
            return None
        if isinstance(x, torch.Tensor):
            want = torch.float64 if dtype == np.float64 else (torch.float32 if dtype == np.float32 else None)
            if dtype == np.uint8:
                want = torch.uint8
            t = x.detach()
            if t.dtype == torch.bool and want == torch.uint8:
                t = t.to(torch.uint8)
            if want is not None and t.dtype != want:
                t = t.to(want)
            t = t.contiguous()
            self.objs.append(t)
            return t.data_ptr() if t.numel() else None
        a = np.ascontiguousarray(x, dtype=dtype)
        self.objs.append(a)
        return a.ctypes.data if a.size else None

    def ptr_array(self, xs, dtype):
        ps = [self.ptr(x, dtype) for x in xs]
        arr = (C.c_void_p * max(1, len(ps)))(*(ps or [None]))
        self.objs.append(arr)
        return arr


@dataclasses.dataclass
class Regions:
    """Per-region records in region-id order."""

    N: int
    bits: np.ndarray      # (R, words) uint32
    nverts: np.ndarray    # (R,)
    verts: np.ndarray     # (R, VMAX, 3)
    edges: np.ndarray     # (R, VMAX)
    status: np.ndarray    # (R,)
    mid: np.ndarray       # (R, 3)
    start: np.ndarray     # (R,)

    @property
    def num(self) -> int:
        return int(self.nverts.shape[0])


@dataclasses.dataclass
class Mesh:
    verts: np.ndarray     # (V, 3) float64
    face_sizes: np.ndarray
    face_indices: np.ndarray

    @property
    def faces(self) -> List[List[int]]:
        out, o = [], 0
        for n in self.face_sizes:
            out.append(list(self.face_indices[o:o + n]))
            o += int(n)
        return out


class Engine:
    """One marching engine: ``Init`` + repeated ``run`` calls."""

    def __init__(self, float_type: str, nodesnum: Sequence[int], arc_table, num_extra_constraints: int = 0):
        if float_type not in FLOAT_TYPES:
            raise ValueError("float_type is either float32, float64 or mixed")
        self.float_type = float_type
        self.nodes = [int(n) for n in nodesnum]
        arc = np.ascontiguousarray(np.asarray(arc_table, dtype=np.int32).reshape(len(self.nodes) - 2, -1))
        if arc.shape[1] == 0:
            arc = np.zeros((len(self.nodes) - 2, 1), np.int32)
        self.arc = arc
        self.E = int(num_extra_constraints)
        self.N = int(sum(self.nodes[1:-1]))
        L = _lib.lib()
        h = C.c_void_p()
        nodes = np.ascontiguousarray(self.nodes, dtype=np.int32)
        rc = L.am_init(C.byref(h), float_type.encode(), nodes.ctypes.data_as(C.POINTER(C.c_int32)), len(self.nodes),
                       arc.ctypes.data_as(C.POINTER(C.c_int32)), arc.shape[0], arc.shape[1], self.E)
        _lib.check(rc)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            _lib.lib().am_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, option: int, value: int):
        _lib.check(_lib.lib().am_set_option(self.h, option, int(value)), self.h)

    def run(self, weights, biases, states, points, arc_tm=(), w_extra=None, b_extra=None, iso=0.0,
            flip_insideout=False, stream=None):
        dt = _np_dtype(self.float_type)
        k = _Keep()
        wp = k.ptr_array(weights, dt)
        bp = k.ptr_array(biases, dt)
        sp = k.ptr(states, np.uint8)
        pp = k.ptr(points, dt)
        shapes = np.ascontiguousarray([s for t in arc_tm for s in tuple(t.shape)] or [0], dtype=np.int32)
        tp = k.ptr_array(arc_tm, dt)
        we = k.ptr(w_extra, dt) if self.E else None
        be = k.ptr(b_extra, dt) if self.E else None
        S = int(states.shape[0])
        st = None
        if stream is not None:
            st = getattr(stream, "cuda_stream", stream)
        rc = _lib.lib().am_analytic_marching(self.h, wp, bp, sp, pp, S, tp,
                                             shapes.ctypes.data_as(C.POINTER(C.c_int32)), len(arc_tm), we, be,
                                             float(iso), 1 if flip_insideout else 0, st)
        _lib.check(rc, self.h)
        return self.stats()

    def run_net(self, net, states, points, iso=0.0, flip_insideout=False, stream=None):
        """Run on a ``workloads.NetArrays``."""
        return self.run(net.W, net.b, states, points, net.tms, net.w_extra, net.b_extra, iso, flip_insideout, stream)

    def stats(self) -> dict:
        s = _lib.AmStats()
        _lib.check(_lib.lib().am_get_stats(self.h, C.byref(s)), self.h)
        return s.as_dict()

    def error_report(self, sample_regions: int = 4096) -> dict:
        """am_error_report: max |f(v)| and the largest vertex error of the
        last result against FP64, over ``sample_regions`` evenly spaced
        regions (0: all)."""
        r = _lib.AmErrorReport()
        _lib.check(_lib.lib().am_error_report(self.h, int(sample_regions), C.byref(r)), self.h)
        return r.as_dict()

    def combine(self, scale=1.0, center=(0.0, 0.0, 0.0)) -> Mesh:
        c3 = (C.c_double * 3)(*[float(x) for x in center])
        L = _lib.lib()
        _lib.check(L.am_combine_mesh(self.h, float(scale), c3), self.h)
        s = self.stats()
        V, F, I = s["mesh_num_verts"], s["mesh_num_faces"], s["mesh_num_indices"]
        v = np.zeros((max(V, 1), 3), np.float64)
        fs = np.zeros(max(F, 1), np.int32)
        fi = np.zeros(max(I, 1), np.int32)
        _lib.check(L.am_get_mesh(self.h, v.ctypes.data, fs.ctypes.data, fi.ctypes.data), self.h)
        return Mesh(verts=v[:V], face_sizes=fs[:F], face_indices=fi[:I])

    def export(self, path: str, is_polymesh=True, is_float32=True):
        _lib.check(_lib.lib().am_export_mesh(self.h, path.encode(), 1 if is_polymesh else 0, 1 if is_float32 else 0),
                   self.h)

    def region_rows(self, first: int, count: int):
        """Constraint rows (count, ALL, 4) and face planes (count, 4) of
        regions [first, first + count), recomposed on the device."""
        ALL = self.N + self.E
        rows = np.zeros((count, ALL, 4))
        eq = np.zeros((count, 4))
        _lib.check(_lib.lib().am_region_rows(self.h, int(first), int(count), rows.ctypes.data, eq.ctypes.data), self.h)
        return rows, eq

    def regions(self) -> Regions:
        s = self.stats()
        R = int(s["num_regions"])
        VM = _lib.vert_capacity()
        W = (self.N + 31) // 32
        d = dict(bits=np.zeros((R, W), np.uint32), nverts=np.zeros(R, np.int32), verts=np.zeros((R, VM, 3)),
                 edges=np.zeros((R, VM), np.int32), status=np.zeros(R, np.int8), mid=np.zeros((R, 3)),
                 start=np.zeros(R, np.int32))
        _lib.check(_lib.lib().am_get_regions(self.h, d["bits"].ctypes.data, d["nverts"].ctypes.data,
                                             d["verts"].ctypes.data, d["edges"].ctypes.data, d["status"].ctypes.data,
                                             d["mid"].ctypes.data, d["start"].ctypes.data), self.h)
        return Regions(N=self.N, **d)


def _fill_run_args(a, k, eng, net, st, pt, iso, flip_insideout):
    """One am_run_args record for network ``net`` on engine ``eng``; ``k``
    keeps the converted arrays alive."""
    dt = _np_dtype(eng.float_type)
    a.weights = C.cast(k.ptr_array(net.W, dt), C.c_void_p)
    a.biases = C.cast(k.ptr_array(net.b, dt), C.c_void_p)
    a.states = k.ptr(st, np.uint8)
    a.points = k.ptr(pt, dt)
    a.num_points = int(st.shape[0])
    shapes = np.ascontiguousarray([s for t in net.tms for s in tuple(t.shape)] or [0], dtype=np.int32)
    k.objs.append(shapes)
    a.arc_tm = C.cast(k.ptr_array(net.tms, dt), C.c_void_p)
    a.arc_tm_shapes = shapes.ctypes.data
    a.num_arc_tm = len(net.tms)
    a.w_extra = k.ptr(net.w_extra, dt) if eng.E else None
    a.b_extra = k.ptr(net.b_extra, dt) if eng.E else None
    a.iso = float(iso)
    a.flip_insideout = 1 if flip_insideout else 0


def autotune(eng, net, states, points, iso=0.0, flip_insideout=False, sample_regions=65536):
    """am_autotune: choose the composition tile and the warps per face for
    this engine's architecture from sample runs; returns (tile, warps)."""
    k = _Keep()
    a = _lib.AmRunArgs()
    _fill_run_args(a, k, eng, net, states, points, iso, flip_insideout)
    chosen = (C.c_int32 * 2)()
    _lib.check(_lib.lib().am_autotune(eng.h, C.byref(a), int(sample_regions), chosen), eng.h)
    return int(chosen[0]), int(chosen[1])


def run_batch(engines, nets, states_list, points_list, iso=0.0, flip_insideout=False):
    """am_run_batch: march every network at once, each on its engine (made
    for that network); returns the device wall time in ms.  Inputs may be
    numpy arrays or tensors, on the host or the device."""
    n = len(engines)
    if not (len(nets) == len(states_list) == len(points_list) == n) or n == 0:
        raise ValueError("one network, state set and point set per engine")
    k = _Keep()
    args = (_lib.AmRunArgs * n)()
    for i, (eng, net, st, pt) in enumerate(zip(engines, nets, states_list, points_list)):
        _fill_run_args(args[i], k, eng, net, st, pt, iso, flip_insideout)
    handles = (C.c_void_p * n)(*[e.h for e in engines])
    wall = C.c_double(0.0)
    rc = _lib.lib().am_run_batch(handles, args, n, C.byref(wall))
    if rc != 0:
        bad = next((e for e in engines if _lib.lib().am_last_error(e.h)), engines[0])
        _lib.check(rc, bad.h)
    return wall.value


def march(net, states, points, float_type="float32", iso=0.0, flip_insideout=False, chunk=None, phase_timing=False,
          options=None):
    """One-shot: Init + AnalyticMarching on a ``workloads.NetArrays``; returns
    the engine.  ``options``: further {AM_OPT_*: value} set before the run."""
    eng = Engine(float_type, net.nodes, net.arc_table, net.num_extra)
    if chunk:
        eng.set_option(_lib.AM_OPT_CHUNK, chunk)
    if phase_timing:
        eng.set_option(_lib.AM_OPT_PHASE_TIMING, 1)
    for opt, value in (options or {}).items():
        eng.set_option(opt, value)
    eng.run_net(net, states, points, iso, flip_insideout)
    return eng
