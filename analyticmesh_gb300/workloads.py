"""Seeded synthetic networks for the benchmark configurations, and the plain
array form (``NetArrays``) every marcher in this repository consumes.

Configurations (all ReLU, fp32 weights):
  polytope   3 -> 14 -> 1, the 14 fixed directions of the reference's
             examples/2_polytope.py, b1 = -2, N(0, 1e-7) noise (seed 0)
  sphere     3 -> [128] x 4 -> 1, geometric init r = 0.5 (seed 1)
  deep       3 -> [256] x 6 -> 1, geometric init + N(0, 0.02) (seed 2)
  batched    64 networks, seeds 100..163, width in {32..512}, depth in {2..8},
             geometric init + N(0, 0.01)
  large_skip 3 -> [512] x 8 -> 1, the input added into the layer-4 input
             through a 512 x 3 transform, r = 0.6, + N(0, 0.01) (seed 3)
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np
import torch

from .model import MLP
from .seeds import dichotomy


@dataclasses.dataclass
class NetArrays:
    """A network as plain arrays (float64 master copy)."""

    nodes: List[int]
    W: List[np.ndarray]
    b: List[np.ndarray]
    arc_table: np.ndarray          # (L-1, cols) int32, rows = len(nodes) - 2
    tms: List[np.ndarray]          # (0, 0) for identity
    w_extra: np.ndarray            # (E, 3)
    b_extra: np.ndarray            # (E,)

    @property
    def state_len(self) -> int:
        return int(sum(self.nodes[1:-1]))

    @property
    def num_extra(self) -> int:
        return int(self.w_extra.shape[0])

    @property
    def has_output_skips(self) -> bool:
        return int(self.arc_table[-1, 0]) > 0 if self.arc_table.shape[0] else False


def net_arrays(model: MLP, w_extra=None, b_extra=None) -> NetArrays:
    info = model.get_info()
    f = lambda t: t.detach().cpu().double().numpy().copy()
    we = np.zeros((0, 3)) if w_extra is None else np.asarray(w_extra, dtype=np.float64).reshape(-1, 3)
    be = np.zeros((0,)) if b_extra is None else np.asarray(b_extra, dtype=np.float64).reshape(-1)
    return NetArrays(nodes=list(model.nodes), W=[f(w) for w in info["weights"]], b=[f(x) for x in info["biases"]],
                     arc_table=info["arc_table"].numpy().astype(np.int32), tms=[f(t) for t in info["arc_tm"]],
                     w_extra=we, b_extra=be)


def _perturb(model: MLP, std: float, g: torch.Generator, hidden_only=True):
    with torch.no_grad():
        n = model.num_of_linears
        for i, lin in enumerate(model.linears):
            if hidden_only and i == n - 1:
                continue
            lin.weight.add_(torch.randn(lin.weight.shape, generator=g) * std)
            lin.bias.add_(torch.randn(lin.bias.shape, generator=g) * std)


def _last_layer(model: MLP, radius: float, g: torch.Generator, std=1e-4):
    with torch.no_grad():
        lin = model.linears[-1]
        n = model.nodes[-2]
        lin.weight.copy_(math.sqrt(math.pi) / math.sqrt(n) + std * torch.randn(lin.weight.shape, generator=g))
        lin.bias.fill_(-radius)


def polytope(seed: int = 0) -> MLP:
    dirs = torch.tensor([[1, 1, 1], [-1, -1, -1], [0, 1, 1], [0, -1, -1], [1, 0, 1], [-1, 0, -1], [1, 1, 0],
                         [-1, -1, 0], [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]],
                        dtype=torch.float32)
    g = torch.Generator().manual_seed(seed)
    m = MLP([3, 14, 1], [[0]], [], initialization=None, enable_print=False)
    noise = lambda x: x + torch.randn(x.shape, generator=g) * 1e-7
    with torch.no_grad():
        m.linears[0].weight.copy_(noise(dirs))
        m.linears[0].bias.copy_(noise(torch.zeros(14)))
        m.linears[1].weight.copy_(noise(torch.ones(1, 14)))
        m.linears[1].bias.copy_(noise(torch.tensor([-2.0])))
    return m


def geometric(widths, seed: int, radius: float = 0.5, perturb: float = 0.0, skips=None, tm_shapes=None) -> MLP:
    """Geometric (SAL) init with an explicit generator; optional N(0, perturb)
    on every hidden weight and bias."""
    g = torch.Generator().manual_seed(seed)
    nodes = [3] + list(widths) + [1]
    arc = skips if skips is not None else [[0] for _ in range(len(nodes) - 2)]
    m = MLP(nodes, arc, tm_shapes or [], initialization="geometric", geometric_radius=radius, generator=g)
    _last_layer(m, radius, g)
    for t, shape in zip(m.tms, tm_shapes or []):
        if isinstance(t, torch.nn.Linear):
            with torch.no_grad():
                t.weight.copy_(torch.randn(t.weight.shape, generator=g) * (math.sqrt(2) / math.sqrt(shape[0])))
    if perturb:
        _perturb(m, perturb, g)
        with torch.no_grad():
            for t in m.tms:
                if isinstance(t, torch.nn.Linear):
                    t.weight.add_(torch.randn(t.weight.shape, generator=g) * perturb)
    return m


def sphere(seed: int = 1) -> MLP:
    return geometric([128] * 4, seed, radius=0.5)


def deep(seed: int = 2) -> MLP:
    return geometric([256] * 6, seed, radius=0.5, perturb=0.02)


# The perturbation lifts the deep network above zero on the whole unit ball
# (f grows with the radius from ~0.01 at the centre to ~0.75 at radius 1); its
# level set at DEEP_ISO is a closed irregular surface near radius 0.5.
DEEP_ISO = 0.35


def large_skip(seed: int = 3) -> MLP:
    # the input added into linear layer 4 (after hidden layer 4): the
    # concatenation [h4 | x] of width 515 as W4 h4 + W4_x x
    skips = [[0], [0], [0], [1, 0, 0], [0], [0], [0], [0]]
    return geometric([512] * 8, seed, radius=0.6, perturb=0.01, skips=skips, tm_shapes=[[512, 3]])


def batched(count: int = 64, first_seed: int = 100) -> List[MLP]:
    out = []
    for s in range(first_seed, first_seed + count):
        r = np.random.default_rng(s)
        width = int(r.choice([32, 64, 128, 256, 512]))
        depth = int(r.integers(2, 9))
        out.append(geometric([width] * depth, s, radius=0.5, perturb=0.01))
    return out


def seeds_for(model: MLP, init_num: int = 1024, seed: int = 1234, iso: float = 0.0, w_extra=None, b_extra=None,
              device="cpu", **kw):
    """Dichotomy seed points and their activation states.  States are taken
    from a float64 forward pass.  Returns (states uint8 (S, N), points float64 (S, 3)).
    ``device`` runs the network there (the samples come from a CPU generator)."""
    g = torch.Generator().manual_seed(seed)
    model = _float_copy(model).to(device).eval()
    we = None if w_extra is None else torch.as_tensor(w_extra, dtype=torch.float32)
    be = None if b_extra is None else torch.as_tensor(b_extra, dtype=torch.float32)
    pts = dichotomy(model, iso, init_num=init_num, generator=g, w_extra_constraints=we, b_extra_constraints=be,
                    device=device, **kw)
    md = _double_copy(model).to(device)
    with torch.no_grad():
        z = md.pre_activations(pts.double())
    return (z > 0).cpu().numpy().astype(np.uint8), pts.double().cpu().numpy()


def _float_copy(model: MLP) -> MLP:
    m = MLP(model.nodes, model.arc_table, model.arc_tm_shape, initialization=None, enable_print=False)
    m.load_state_dict(model.state_dict())
    return m.float()


def _double_copy(model: MLP) -> MLP:
    m = MLP(model.nodes, model.arc_table, model.arc_tm_shape, initialization=None, enable_print=False)
    m.load_state_dict({k: v.cpu() for k, v in model.state_dict().items()})
    return m.double()
