"""Host-side pieces that need no GPU: the model, helpers, the C ABI
library's exports, argument checks of the cuam drop-in."""
import ctypes as C
import os
import re

import numpy as np
import pytest
import torch

import analyticmesh_gb300 as am
from analyticmesh_gb300 import _lib, cuam, workloads as wl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    header = open(os.path.join(ROOT, "include", "analyticmesh_gb300.h")).read()
    names = set(re.findall(r"\b(am_[a-z0-9_]+)\s*\(", header))
    assert len(names) >= 14
    for n in sorted(names):
        assert hasattr(L, n), n


def test_strerror_and_status_codes():
    L = _lib.lib()
    assert L.am_strerror(0) == b"ok"
    assert b"argument" in L.am_strerror(1)
    assert L.am_vert_capacity() >= 20


def test_init_validates_like_the_reference():
    L = _lib.lib()
    h = C.c_void_p()
    nodes = np.array([3, 16, 1], np.int32)
    arc = np.zeros((1, 1), np.int32)
    i32 = C.POINTER(C.c_int32)
    assert L.am_init(C.byref(h), b"float16", nodes.ctypes.data_as(i32), 3, arc.ctypes.data_as(i32), 1, 1, 0) == 1
    bad = np.array([2, 16, 1], np.int32)
    assert L.am_init(C.byref(h), b"float32", bad.ctypes.data_as(i32), 3, arc.ctypes.data_as(i32), 1, 1, 0) == 1
    assert L.am_init(C.byref(h), b"float32", nodes.ctypes.data_as(i32), 3, arc.ctypes.data_as(i32), 1, 2, 0) == 1
    # a zero-width hidden layer, a negative extra-constraint count, a skip from a
    # later layer, a row with more connections than columns: all rejected
    # before anything touches a device
    zero = np.array([3, 16, 0, 1], np.int32)
    arc2 = np.zeros((2, 1), np.int32)
    assert L.am_init(C.byref(h), b"float32", zero.ctypes.data_as(i32), 4, arc2.ctypes.data_as(i32), 2, 1, 0) == 1
    assert L.am_init(C.byref(h), b"float32", nodes.ctypes.data_as(i32), 3, arc.ctypes.data_as(i32), 1, 1, -1) == 1
    deep = np.array([3, 16, 16, 1], np.int32)
    later = np.array([[0, 0, 0], [1, 3, 0]], np.int32)  # into linear 2 from hidden layer 3
    assert L.am_init(C.byref(h), b"float32", deep.ctypes.data_as(i32), 4, later.ctypes.data_as(i32), 2, 3, 0) == 1
    crowded = np.array([[0, 0, 0], [2, 1, 0]], np.int32)  # two connections, room for one
    assert L.am_init(C.byref(h), b"float32", deep.ctypes.data_as(i32), 4, crowded.ctypes.data_as(i32), 2, 3, 0) == 1
    assert not h.value


def test_cuam_rejects_bad_arguments():
    with pytest.raises(RuntimeError):
        cuam.Init("float16", [3, 8, 1], torch.zeros(1, 1, dtype=torch.int32), 0)
    with pytest.raises(RuntimeError):
        cuam.Init("float32", [3, 8, 1], torch.zeros(1, 1, dtype=torch.int64), 0)
    with pytest.raises(RuntimeError):
        cuam.AnalyticMarching([], [], None, None, [], None, None, 0.0, False)


def test_mlp_forward_matches_reference_dataflow():
    m = wl.geometric([8, 8, 8], 3, skips=[[0], [1, 1, 0], [1, 0, 1]], tm_shapes=[[0, 0], [1, 3]])
    x = torch.randn(5, 3)
    # explicit restatement of backend/model.py:101-123
    h1 = torch.relu(m.linears[0](x))
    h2 = torch.relu(m.linears[1](h1))
    h3 = torch.relu(m.linears[2](h2) + h1)
    y = m.linears[3](h3) + m.tms[1](x)
    torch.testing.assert_close(m(x), y)
    info = m.get_info()
    assert info["arc_table"].tolist() == [[0, 0, 0], [1, 1, 0], [1, 0, 1]]


def test_geometric_init_and_helpers():
    m = am.MLP([3, 64, 64, 1], [[0], [0]], [], geometric_radius=0.5)
    assert m.linears[-1].bias.item() == -0.5
    w, b = am.get_boundary("cube", min_vert=(-1, -2, -3), max_vert=(1, 2, 3))
    pts = torch.tensor([[0.0, 0.0, 0.0], [1.5, 0.0, 0.0]])
    inside = ((pts @ w.t() + b) < 0).all(1)
    assert inside.tolist() == [True, False]
    assert am.estimate_am_time(m) > 0


def test_ply_roundtrip(tmp_path):
    from analyticmesh_gb300.main import read_ply, write_ply
    v = np.random.rand(5, 3)
    f = [[0, 1, 2], [1, 2, 3, 4]]
    p = str(tmp_path / "m.ply")
    write_ply(p, v, f, polymesh=True, float32=False)
    v2, f2 = read_ply(p)
    np.testing.assert_array_equal(v, v2)
    assert [list(map(int, x)) for x in f2] == f
    write_ply(p, v, f, polymesh=False, float32=True)
    v3, f3 = read_ply(p)
    assert len(f3) == 3 and np.allclose(v3, v, atol=1e-6)


def test_batch_and_option_argument_checks():
    """Host-side validation that needs no device: am_run_batch with no
    engines, am_set_option without an engine."""
    L = _lib.lib()
    wall = C.c_double(0.0)
    assert L.am_run_batch(None, None, 1, C.byref(wall)) == 1          # AM_ERR_INVALID_ARGUMENT
    handles = (C.c_void_p * 1)(None)
    args = (_lib.AmRunArgs * 1)()
    assert L.am_run_batch(handles, args, 0, C.byref(wall)) == 1      # count < 1
    assert L.am_run_batch(handles, args, 1, C.byref(wall)) == 2      # AM_ERR_NOT_INITIALIZED
    L.am_set_option.argtypes = [C.c_void_p, C.c_int, C.c_int64]
    assert L.am_set_option(None, _lib.AM_OPT_MAX_REGIONS, 10) == 2
    assert L.am_set_option(None, _lib.AM_OPT_FACE_WARPS, 2) == 2
    assert L.am_autotune(None, args, 1000, None) == 2                 # AM_ERR_NOT_INITIALIZED


def test_reference_main_calls_bind_to_the_cuam_drop_in():
    """Every ``cuamlib.X(...)`` call in the reference's backend/main.py (read
    as text from the reference checkout, when present) binds to the drop-in's
    function of that name: same names, same keyword arguments."""
    import ast
    import inspect

    from oracle import build_ref

    path = os.path.join(build_ref.REF_ROOT, "backend", "main.py")
    if not os.path.exists(path):
        pytest.skip("reference checkout not present")
    tree = ast.parse(open(path).read())
    calls = [n for n in ast.walk(tree) if isinstance(n, ast.Call) and isinstance(n.func, ast.Attribute)
             and isinstance(n.func.value, ast.Name) and n.func.value.id == "cuamlib"]
    assert {c.func.attr for c in calls} == {"Init", "AnalyticMarching", "CombineMesh", "ExportMesh", "Destroy"}
    for c in calls:
        fn = getattr(cuam, c.func.attr)
        inspect.signature(fn).bind(*[None] * len(c.args), **{k.arg: None for k in c.keywords})
