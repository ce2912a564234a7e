"""ONNX codec (save_model / load_model, the reference's backend/onnx_io.py)
on the protobuf wire format: round trips of plain and skip-connected MLPs,
the graph form the reference's parser expects, and the reference's shipped
network examples/chair.onnx (3 -> 60 x 4 -> 1) when the reference is present."""
import os

import numpy as np
import pytest
import torch

from analyticmesh_gb300 import load_model, onnx_io, save_model, workloads as wl
from oracle import build_ref

# the reference checkout (AM_REFERENCE_ROOT): its shipped network, when present
CHAIR = os.path.join(build_ref.REF_ROOT, "examples", "chair.onnx")


@pytest.mark.parametrize("factory", [
    lambda: wl.geometric([32, 32], 1),
    lambda: wl.geometric([20, 50, 20, 80, 20], 13, skips=[[0], [1, 1, 0], [1, 1, 1], [0], [0]],
                         tm_shapes=[[0, 0], [80, 20]]),
    lambda: wl.geometric([64] * 5, 15, perturb=0.01, skips=[[0], [0], [1, 0, 0], [0], [0]], tm_shapes=[[64, 3]]),
    lambda: wl.geometric([16, 16, 16], 4, skips=[[0], [1, 1, 0], [0]], tm_shapes=[[0, 0]]),
], ids=["plain", "hidden_skips", "input_transform", "identity"])
def test_round_trip(tmp_path, factory):
    m = factory()
    path = str(tmp_path / "m.onnx")
    save_model(m, path)
    m2 = load_model(path)
    assert m2.nodes == m.nodes and m2.arc_table == m.arc_table and m2.arc_tm_shape == m.arc_tm_shape
    x = torch.randn(256, 3, generator=torch.Generator().manual_seed(0))
    with torch.no_grad():
        assert torch.equal(m(x), m2(x))
    # bytes input as well
    with open(path, "rb") as fh:
        m3 = load_model(fh.read())
    with torch.no_grad():
        assert torch.equal(m(x), m3(x))


def test_graph_form_matches_the_reference_parser():
    m = wl.geometric([20, 50, 20], 3, skips=[[0], [1, 1, 0], [0]], tm_shapes=[[0, 0]])
    g = onnx_io._parse(onnx_io._parse(onnx_io.model_bytes(m))[7][0][1])
    ops = [onnx_io._str(onnx_io._parse(n), 4) for _, n in g[1]]
    assert ops == ["Gemm", "Relu", "Gemm", "Relu", "Gemm", "Add", "Relu", "Gemm"]
    gemm = onnx_io._parse(g[1][0][1])
    attrs = onnx_io._decode_attrs(gemm)
    assert attrs == {"alpha": 1.0, "beta": 1.0, "transB": 1}
    # the graph output is produced by the last node
    assert onnx_io._strs(onnx_io._parse(g[1][-1][1]), 2) == ["output"]


def test_rejects_unsupported_graphs():
    with pytest.raises(ValueError):
        load_model(b"\x0a\x02hi")  # no graph
    with pytest.raises(ValueError):
        load_model("no/such/file.onnx")


@pytest.mark.skipif(not os.path.exists(CHAIR), reason="reference checkout not present")
def test_reference_chair_network():
    m = load_model(CHAIR)
    assert m.nodes == [3, 60, 60, 60, 60, 1] and m.arc_table == [[0]] * 4 and m.arc_tm_shape == []
    for p in m.parameters():
        assert torch.isfinite(p).all()
    # a closed level set: the function changes sign inside [-1, 1]^3
    g = torch.Generator().manual_seed(1)
    with torch.no_grad():
        f = m(torch.rand(4096, 3, generator=g) * 2 - 1)
    assert (f < 0).any() and (f > 0).any()
    # and survives a round trip through the writer bit for bit
    m2 = load_model(onnx_io.model_bytes(m))
    x = torch.rand(512, 3, generator=g)
    with torch.no_grad():
        assert torch.equal(m(x), m2(x))


class _TwoLayer(torch.nn.Module):
    """A hand-written ReLU network, saved the way the reference's examples
    save theirs (any module, not only MLP)."""

    def __init__(self, width=14):
        super().__init__()
        g = torch.Generator().manual_seed(5)
        self.first = torch.nn.Linear(3, width)
        self.second = torch.nn.Linear(width, 1)
        with torch.no_grad():
            for p in self.parameters():
                p.copy_(torch.randn(p.shape, generator=g))

    def forward(self, x):
        return self.second(torch.relu(self.first(x)))


class _Skipped(torch.nn.Module):
    """Identity skip between hidden layers and a bias-free transform of the
    input added before the third layer's ReLU."""

    def __init__(self):
        super().__init__()
        g = torch.Generator().manual_seed(6)
        self.a = torch.nn.Linear(3, 24)
        self.b = torch.nn.Linear(24, 24)
        self.c = torch.nn.Linear(24, 16)
        self.t = torch.nn.Linear(3, 16, bias=False)
        self.out = torch.nn.Linear(16, 1)
        with torch.no_grad():
            for p in self.parameters():
                p.copy_(torch.randn(p.shape, generator=g) * 0.5)

    def forward(self, x):
        h1 = torch.nn.functional.relu(self.a(x))
        h2 = (self.b(h1) + h1).relu()
        h3 = torch.relu(self.c(h2) + self.t(x))
        return self.out(h3)


@pytest.mark.parametrize("factory", [
    _TwoLayer,
    lambda: torch.nn.Sequential(torch.nn.Linear(3, 32), torch.nn.ReLU(), torch.nn.Linear(32, 32), torch.nn.ReLU(),
                                torch.nn.Linear(32, 1)),
    _Skipped,
], ids=["hand_written", "sequential", "skips_and_transform"])
def test_any_relu_module_saves_and_loads_as_mlp(tmp_path, factory):
    torch.manual_seed(0)
    m = factory().eval()
    path = str(tmp_path / "net.onnx")
    save_model(m, path)
    mlp = load_model(path)
    x = torch.randn(512, 3, generator=torch.Generator().manual_seed(1))
    with torch.no_grad():
        want, got = m(x), mlp(x)
    assert got.shape == want.shape
    assert torch.allclose(got, want, rtol=1e-6, atol=1e-6), (got - want).abs().max()
    if factory is _Skipped:
        assert mlp.nodes == [3, 24, 24, 16, 1]
        assert mlp.arc_table == [[1, 1, 0], [1, 0, 1], [0]] and mlp.arc_tm_shape == [[0, 0], [16, 3]]


def test_save_model_rejects_non_mlp_modules(tmp_path):
    class Smooth(torch.nn.Module):
        def __init__(self):
            super().__init__()
            self.l = torch.nn.Linear(3, 1)

        def forward(self, x):
            return torch.sigmoid(self.l(x))

    with pytest.raises(ValueError):
        save_model(Smooth(), str(tmp_path / "s.onnx"))
