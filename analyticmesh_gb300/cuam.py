"""Drop-in for the reference's compiled module ``build.cuam``
(backend/src/cuam.cpp:186-217, imported by backend/main.py:13).

Same five functions, same keyword names, same call order:
``Init -> AnalyticMarching -> CombineMesh -> ExportMesh``, ``Destroy`` at
re-initialisation or exit.  Argument checks follow cuam.cpp:58-184 and raise
``RuntimeError`` as its TORCH_CHECKs do; calls out of order raise instead of
printing and returning.  Behind them is one engine of the C ABI
(include/analyticmesh_gb300.h), like the reference's global singleton
(backend/src/cuam_kernel.cu:23).
"""
from __future__ import annotations

import torch

from . import engine as _engine

_ENGINE = None
_FLOAT_TYPE = ""
_NODES = []
_ARC = None


def _check(cond, msg):
    if not cond:
        raise RuntimeError(msg)


def Init(float_type, nodesnum, arc_table, num_extra_constraints):
    """cuam.cpp:58-95.  float_type: "float32" | "float64" (and "mixed", the
    tensor-core form with float32 inputs)."""
    global _ENGINE, _FLOAT_TYPE, _NODES, _ARC
    _check(float_type in ("float32", "float64", "mixed"), "Error: `float_type` is either `float32` or `float64`!")
    nodes = [int(n) for n in nodesnum]
    _check(nodes[0] == 3 and nodes[-1] == 1 and len(nodes) >= 3, "nodesnum must be [3, ..., 1] with >= 3 entries")
    _check(isinstance(arc_table, torch.Tensor) and not arc_table.is_cuda, "arc_table must be a CPU tensor")
    _check(arc_table.dim() == 2 and arc_table.size(0) == len(nodes) - 2, "arc_table must have len(nodesnum) - 2 rows")
    _check(arc_table.size(1) >= 1 and (arc_table.size(1) + 1) % 2 == 0, "arc_table width must be odd")
    _check(arc_table.dtype == torch.int32, "arc_table must be int32")
    for r in range(arc_table.size(0)):
        _check(1 + 2 * int(arc_table[r, 0]) <= arc_table.size(1), "arc_table row has more connections than columns")
    _check(int(num_extra_constraints) >= 0, "num_extra_constraints must be >= 0")
    if _ENGINE is not None:
        _ENGINE.close()
    _ENGINE = _engine.Engine(float_type, nodes, arc_table.numpy(), int(num_extra_constraints))
    _FLOAT_TYPE, _NODES, _ARC = float_type, nodes, arc_table.clone()


def AnalyticMarching(weights, biases, states, points, arc_tm, w_extra_constraints, b_extra_constraints, iso,
                     flip_insideout):
    """cuam.cpp:97-184: tensors CUDA, contiguous, of the Init float type."""
    _check(_ENGINE is not None, "Environment must be initialized first!")
    tt = torch.float64 if _FLOAT_TYPE == "float64" else torch.float32
    _check(len(weights) == len(biases) == len(_NODES) - 1, "weights / biases do not match nodesnum")
    n = 0
    for i, (w, b) in enumerate(zip(weights, biases)):
        for t in (w, b):
            _check(t.is_cuda and t.is_contiguous(), "weights / biases must be contiguous CUDA tensors")
            _check(t.dtype == tt, "weights / biases must match float_type")
        _check(w.dim() == 2 and b.dim() == 1 and w.size(0) == b.size(0), "weight / bias shapes")
        _check(w.size(0) == _NODES[i + 1], "weight rows must match nodesnum")
        if i:
            _check(w.size(1) == weights[i - 1].size(0), "consecutive weights do not chain")
        n += w.size(0)
    _check(weights[0].size(1) == 3 and weights[-1].size(0) == 1, "input must be 3-D and output scalar")
    n -= 1
    _check(states.is_cuda and states.is_contiguous() and states.dim() == 2, "states must be a contiguous CUDA matrix")
    _check(states.size(0) >= 1 and states.size(1) == n and states.dtype == torch.bool, "states must be bool (S, N)")
    _check(points.is_cuda and points.is_contiguous() and points.dim() == 2, "points must be a contiguous CUDA matrix")
    _check(points.size(0) == states.size(0) and points.size(1) == 3 and points.dtype == tt, "points must be (S, 3)")
    for tm in arc_tm:
        _check(tm.is_cuda and tm.is_contiguous() and tm.dim() == 2 and tm.dtype == tt, "arc_tm tensors")
    for t in (w_extra_constraints, b_extra_constraints):
        _check(t.is_cuda and t.is_contiguous(), "extra constraints must be contiguous CUDA tensors")
    _check(w_extra_constraints.dim() == 2 and w_extra_constraints.size(1) == 3, "w_extra_constraints must be (E, 3)")
    _check(b_extra_constraints.dim() == 1 and w_extra_constraints.size(0) == b_extra_constraints.size(0),
           "b_extra_constraints must be (E,)")
    _check(w_extra_constraints.size(0) == _ENGINE.E, "extra constraint count differs from Init")
    _ENGINE.run(list(weights), list(biases), states, points, list(arc_tm), w_extra_constraints, b_extra_constraints,
                float(iso), bool(flip_insideout), stream=torch.cuda.current_stream())


def CombineMesh(scale, center):
    """cuam_kernel.cu:185-200: weld, index, vertex * scale + center."""
    _check(_ENGINE is not None, "AnalyticMarching must be done first!")
    return _ENGINE.combine(float(scale), [float(c) for c in center])


def ExportMesh(file_path, is_polymesh, is_float32):
    """cuam_kernel.cu:205-246 (binary little-endian PLY)."""
    _check(_ENGINE is not None, "CombineMesh must be done first!")
    _ENGINE.export(str(file_path), bool(is_polymesh), bool(is_float32))


def Destroy():
    """cuam_kernel.cu:153-179."""
    global _ENGINE, _FLOAT_TYPE
    if _ENGINE is None:
        return
    _ENGINE.close()
    _ENGINE = None
    _FLOAT_TYPE = ""


def engine():
    """The engine behind the module (stats, regions, the welded mesh)."""
    return _ENGINE
