"""The composition entry point that allocates nothing
(am_compose_rows_noalloc), checked against the engine's own composition of
the same regions (am_region_rows) on two calls in a row, and independently
against an FP64 composition in numpy (a network of mixed widths included),
plus its argument checks.

Named to be collected last: it must pass both in a fresh process and after
every other test has used the library on the same device.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from analyticmesh_gb300 import _lib, engine, workloads as wl
from test_compose_gpu import compose_fp64, rel_err

# same kernel and the same FP32 weights on both sides: the rows agree to
# rounding of the input conversion at most
RTOL = 1e-6


def _unpack(bits, N):
    """(R, words) uint32 keys -> (R, N) uint8 states, bit b of word w = unit 32 w + b."""
    R, W = bits.shape
    b = (bits[:, :, None] >> np.arange(32, dtype=np.uint32)[None, None, :]) & 1
    return b.reshape(R, W * 32)[:, :N].astype(np.uint8)


def _call(nodes, Ws, Bs, states, iso, rows, eq):
    L = _lib.lib()
    n = len(nodes)
    nodes_c = (C.c_int32 * n)(*nodes)
    wp = (C.c_void_p * (n - 1))(*[w.data_ptr() for w in Ws])
    bp = (C.c_void_p * (n - 1))(*[b.data_ptr() for b in Bs])
    return L.am_compose_rows_noalloc(nodes_c, n, wp, bp, C.c_void_p(states.data_ptr()), int(states.shape[0]),
                                     C.c_double(iso), C.c_void_p(rows.data_ptr()), C.c_void_p(eq.data_ptr()),
                                     C.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.gpu
def test_noalloc_rows_match_engine_twice_in_a_row():
    model = wl.sphere(1)  # 3 -> 128 x 4 -> 1
    net = wl.net_arrays(model)
    states, pts = wl.seeds_for(model, 256)
    iso = 0.01
    eng = engine.march(net, states, pts, "float32", iso=iso)
    reg = eng.regions()
    assert reg.num >= 4000, reg.num
    N = sum(net.nodes[1:-1])
    dev = torch.device("cuda")
    Ws = [torch.tensor(w, dtype=torch.float32, device=dev).contiguous() for w in net.W]
    Bs = [torch.tensor(b, dtype=torch.float32, device=dev).contiguous() for b in net.b]

    # a large call, then a smaller one over other regions: the second runs on
    # scratch that still holds the first call's contents
    for first, count in ((0, 3000), (3000, 1000)):
        ref_rows, ref_eq = eng.region_rows(first, count)
        st = torch.from_numpy(_unpack(reg.bits[first:first + count], N)).to(dev)
        rows = torch.full((count, N, 4), float("nan"), dtype=torch.float32, device=dev)
        eq = torch.full((count, 4), float("nan"), dtype=torch.float32, device=dev)
        assert _call(net.nodes, Ws, Bs, st, iso, rows, eq) == 0
        torch.cuda.synchronize()
        got_rows, got_eq = rows.double().cpu().numpy(), eq.double().cpu().numpy()
        np.testing.assert_allclose(got_rows, ref_rows, rtol=RTOL, atol=RTOL * np.abs(ref_rows).max())
        np.testing.assert_allclose(got_eq, ref_eq, rtol=RTOL, atol=RTOL * np.abs(ref_eq).max())
    eng.close()


@pytest.mark.gpu
def test_noalloc_rejects_work_beyond_its_scratch():
    model = wl.sphere(1)
    net = wl.net_arrays(model)
    dev = torch.device("cuda")
    Ws = [torch.tensor(w, dtype=torch.float32, device=dev).contiguous() for w in net.W]
    Bs = [torch.tensor(b, dtype=torch.float32, device=dev).contiguous() for b in net.b]
    small = torch.zeros((1, 512), dtype=torch.uint8, device=dev)
    rows = torch.zeros((1, 512, 4), dtype=torch.float32, device=dev)
    eq = torch.zeros((1, 4), dtype=torch.float32, device=dev)
    L = _lib.lib()
    n = len(net.nodes)
    args = [(C.c_int32 * n)(*net.nodes), n, (C.c_void_p * (n - 1))(*[w.data_ptr() for w in Ws]),
            (C.c_void_p * (n - 1))(*[b.data_ptr() for b in Bs]), C.c_void_p(small.data_ptr())]
    # 200000 regions x 16 key words exceed the 8 MiB scratch: rejected before
    # any buffer is touched
    rc = L.am_compose_rows_noalloc(*args, 200000, C.c_double(0.0), C.c_void_p(rows.data_ptr()),
                                   C.c_void_p(eq.data_ptr()), None)
    assert rc == 8  # AM_ERR_CAPACITY
    assert L.am_compose_rows_noalloc(*args, 0, C.c_double(0.0), C.c_void_p(rows.data_ptr()),
                                     C.c_void_p(eq.data_ptr()), None) == 1  # AM_ERR_INVALID_ARGUMENT: count < 1


@pytest.mark.gpu
@pytest.mark.parametrize("factory", [lambda: wl.sphere(1), lambda: wl.geometric([64, 96], 21, perturb=0.02)],
                         ids=["sphere", "widths_64_96"])
def test_noalloc_rows_match_fp64_composition(factory):
    """Independent of the engine: FP32 rows within FP32 accuracy of an FP64
    composition of the same regions (the per-layer offsets of a network whose
    hidden widths differ included)."""
    model = factory()
    net = wl.net_arrays(model)
    states, pts = wl.seeds_for(model, 128, seed=5)
    eng = engine.march(net, states, pts, "float32")
    reg = eng.regions()
    count = min(reg.num, 2000)
    N = sum(net.nodes[1:-1])
    dev = torch.device("cuda")
    Ws = [torch.tensor(w, dtype=torch.float32, device=dev).contiguous() for w in net.W]
    Bs = [torch.tensor(b, dtype=torch.float32, device=dev).contiguous() for b in net.b]
    st = torch.from_numpy(_unpack(reg.bits[:count], N)).to(dev)
    rows = torch.empty((count, N, 4), dtype=torch.float32, device=dev)
    eq = torch.empty((count, 4), dtype=torch.float32, device=dev)
    assert _call(net.nodes, Ws, Bs, st, 0.0, rows, eq) == 0
    torch.cuda.synchronize()
    # the FP64 reference composes the FP32 weights exactly
    net32 = wl.NetArrays(nodes=net.nodes, W=[w.astype(np.float32).astype(np.float64) for w in net.W],
                         b=[b.astype(np.float32).astype(np.float64) for b in net.b], arc_table=net.arc_table,
                         tms=net.tms, w_extra=net.w_extra, b_extra=net.b_extra)
    ref_rows, ref_eq = compose_fp64(net32, reg.bits[:count])
    # the SIMT FP32 composition's accuracy: up to ~1.4e-5 of a row's scale
    # where its terms cancel (measured on the sphere's 4-layer rows)
    assert rel_err(rows.double().cpu().numpy(), ref_rows) <= 5e-5
    assert rel_err(eq.double().cpu().numpy(), ref_eq) <= 5e-5
    eng.close()


@pytest.mark.gpu
def test_noalloc_rejects_misaligned_outputs():
    model = wl.geometric([32, 32], 3)
    net = wl.net_arrays(model)
    dev = torch.device("cuda")
    Ws = [torch.tensor(w, dtype=torch.float32, device=dev).contiguous() for w in net.W]
    Bs = [torch.tensor(b, dtype=torch.float32, device=dev).contiguous() for b in net.b]
    st = torch.zeros((4, 64), dtype=torch.uint8, device=dev)
    buf = torch.zeros(4 * 64 * 4 + 4, dtype=torch.float32, device=dev)
    eq = torch.zeros((4, 4), dtype=torch.float32, device=dev)
    L = _lib.lib()
    n = len(net.nodes)
    args = [(C.c_int32 * n)(*net.nodes), n, (C.c_void_p * (n - 1))(*[w.data_ptr() for w in Ws]),
            (C.c_void_p * (n - 1))(*[b.data_ptr() for b in Bs]), C.c_void_p(st.data_ptr()), 4, C.c_double(0.0)]
    # rows four bytes past a 16-byte boundary
    assert L.am_compose_rows_noalloc(*args, C.c_void_p(buf.data_ptr() + 4), C.c_void_p(eq.data_ptr()),
                                     None) == _lib.AM_ERR_INVALID_ARGUMENT
    assert L.am_compose_rows_noalloc(*args, C.c_void_p(buf.data_ptr()), C.c_void_p(eq.data_ptr() + 4),
                                     None) == _lib.AM_ERR_INVALID_ARGUMENT
    # aligned: accepted
    assert L.am_compose_rows_noalloc(*args, C.c_void_p(buf.data_ptr()), C.c_void_p(eq.data_ptr()), None) == 0
    torch.cuda.synchronize()
