"""Composition accuracy: constraint rows of the SIMT fp32 path and of the
tensor-core (three-term bf16 split) path against an FP64 composition of the
same regions in numpy (the reference's fill_constraints,
backend/inc/process.h:18-193, with connections into the output layer)."""
import numpy as np
import pytest

from analyticmesh_gb300 import _lib, engine, workloads as wl

pytestmark = pytest.mark.gpu


def compose_fp64(net, bits, iso=0.0):
    """rows (R, N + E, 4) sign-flipped, eq (R, 4) for packed keys."""
    N = net.state_len
    nodes = net.nodes
    n_lin = len(nodes) - 1
    R = bits.shape[0]
    s = np.zeros((R, N), np.float64)
    for k in range(N):
        s[:, k] = (bits[:, k >> 5] >> np.uint32(k & 31)) & 1
    hoff = [0, 0]
    for h in range(1, n_lin):
        hoff.append(hoff[-1] + nodes[h])
    A = {}  # hidden layer h -> (R, n_h, 4) unflipped affine maps
    A[1] = np.broadcast_to(np.concatenate([net.W[0], net.b[0][:, None]], 1), (R, nodes[1], 4)).copy()
    X = lambda h: A[h] * s[:, hoff[h]:hoff[h] + nodes[h], None]
    out = None
    for i in range(1, n_lin):
        y = np.einsum("mk,rkc->rmc", net.W[i], X(i))
        y[:, :, 3] += net.b[i]
        row = net.arc_table[i - 1]
        for c in range(int(row[0])):
            src, t = int(row[1 + 2 * c]), int(row[2 + 2 * c])
            tm = net.tms[t]
            if src == 0:
                if tm.size == 0:
                    y[:, :3, :3] += np.eye(3)
                else:
                    y[:, :, :3] += tm
            else:
                y += X(src) if tm.size == 0 else np.einsum("mk,rkc->rmc", tm, X(src))
        if i < n_lin - 1:
            A[i + 1] = y
        else:
            out = y[:, 0, :]
    rows = np.concatenate([A[h] for h in range(1, n_lin)], 1)
    rows = rows * (1 - 2 * s)[:, :, None]
    if net.num_extra:
        ex = np.concatenate([net.w_extra, net.b_extra[:, None]], 1)
        rows = np.concatenate([rows, np.broadcast_to(ex, (R, net.num_extra, 4))], 1)
    out = out.copy()
    out[:, 3] -= iso
    return rows, out


def rel_err(rows, ref):
    scale = np.abs(ref[..., :3]).sum(-1) + np.abs(ref[..., 3])
    return (np.abs(rows - ref).max(-1) / np.maximum(scale, 1e-30)).max()


@pytest.mark.parametrize("factory", [
    lambda: wl.sphere(),
    lambda: wl.geometric([20, 50, 20, 80, 20], 13, skips=[[0], [1, 1, 0], [1, 1, 1], [0], [0]], tm_shapes=[[0, 0], [80, 20]]),
    lambda: wl.geometric([256, 256, 256], 14, perturb=0.02),
    lambda: wl.geometric([64] * 5, 15, perturb=0.01, skips=[[0], [0], [1, 0, 0], [0], [0]], tm_shapes=[[64, 3]]),
    lambda: wl.geometric([512] * 3, 16, perturb=0.01),
], ids=["sphere", "odd_widths", "wide256", "input_skip", "wide512_kmajor"])
def test_tensor_core_rows_match_fp32_accuracy(factory):
    m = factory()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=7)
    errs = {}
    for form in ("float32", "mixed"):
        eng = engine.march(net, st, pt, form)
        total = eng.stats()["num_regions"]
        n = min(total, 300)
        rows, eq = eng.region_rows(0, n)
        # a larger launch uses wider tensor-core tiles: same rows bit for bit
        big = min(total, 6000)
        rows_b, eq_b = eng.region_rows(0, big)
        assert np.array_equal(rows_b[:n], rows) and np.array_equal(eq_b[:n], eq), form
        bits = eng.regions().bits[:big]
        ref_rows, ref_eq = compose_fp64(net, bits)
        errs[form] = (rel_err(rows_b, ref_rows), rel_err(eq_b, ref_eq))
        eng.close()
    # fp32-level rows and face planes from the tensor cores
    assert errs["mixed"][0] <= max(4 * errs["float32"][0], 2e-6), errs
    assert errs["mixed"][1] <= max(4 * errs["float32"][1], 2e-6), errs


@pytest.mark.parametrize("factory", [
    lambda: wl.geometric([256, 256, 256], 14, perturb=0.02),
    lambda: wl.geometric([512] * 3, 16, perturb=0.01),
    lambda: wl.geometric([20, 50, 20, 80, 20], 13, skips=[[0], [1, 1, 0], [1, 1, 1], [0], [0]], tm_shapes=[[0, 0], [80, 20]]),
    lambda: wl.geometric([64] * 5, 15, perturb=0.01, skips=[[0], [0], [1, 0, 0], [0], [0]], tm_shapes=[[64, 3]]),
], ids=["wide256", "wide512", "odd_widths_tc_skip", "input_skip"])
def test_streamed_and_resident_operand_tiles_agree(factory):
    """The tensor-core composition with the operand resident in shared memory
    for all layers, with the operand rebuilt per 64-deep block from the rows
    just written, and the latter with each layer's M tiles in two passes:
    same rows, same face planes, same regions, bit for bit."""
    m = factory()
    net = wl.net_arrays(m)
    st, pt = wl.seeds_for(m, init_num=128, seed=7)
    out = {}
    for tile in (1, 2, 3):
        try:
            eng = engine.march(net, st, pt, "mixed", options={_lib.AM_OPT_COMPOSE_TILE: tile})
        except RuntimeError as e:  # the resident tile of a 512-wide net may not fit
            assert tile == 1 and "does not fit" in str(e), e
            continue
        s = eng.stats()
        n = min(s["num_regions"], 4000)
        rows, eq = eng.region_rows(0, n)
        out[tile] = (s["num_regions"], s["num_faces"], eng.regions().bits[:n], rows, eq)
        eng.close()
    assert 2 in out and 3 in out
    for other in (1, 3):  # the resident tile, and the streamed tile in two M passes
        if other not in out:
            continue
        a, b = out[other], out[2]
        assert a[0] == b[0] and a[1] == b[1]
        assert np.array_equal(a[2], b[2])
        assert np.array_equal(a[3].view(np.int64), b[3].view(np.int64))
        assert np.array_equal(a[4].view(np.int64), b[4].view(np.int64))
    ref_rows, ref_eq = compose_fp64(net, out[2][2])
    assert rel_err(out[2][3], ref_rows) <= 1e-5
    assert rel_err(out[2][4], ref_eq) <= 1e-5
