"""ReLU MLP with additive skip connections -- the network family Analytic
Marching meshes.

Mirrors the reference's ``MLP`` (backend/model.py:5-148): same constructor
arguments, same ``arc_table`` / ``arc_tm_shape`` conventions, same
``geometric`` (SAL) initialisation, same forward pass and ``get_info()``.
"""
from __future__ import annotations

import math

import torch


class MLP(torch.nn.Module):
    """``nodes``: widths including the 3-D input and the scalar output, e.g.
    ``[3, 128, 128, 1]``.

    ``arc_table[i]`` lists the additive connections into linear layer ``i+1``:
    ``[count, src_0, tm_0, src_1, tm_1, ...]`` where ``src`` is the index of
    the source (0 = network input, k = output of hidden layer k) and ``tm``
    indexes ``arc_tm_shape``; a ``[0, 0]`` shape is the identity.
    (backend/model.py:19-36)
    """

    def __init__(self, nodes, arc_table, arc_tm_shape, initialization="geometric", geometric_radius=1.0,
                 enable_print=True, generator=None):
        super().__init__()
        self.nodes = list(nodes)
        self.arc_table = [list(a) for a in arc_table]
        self.arc_tm_shape = [list(s) for s in arc_tm_shape]
        self.geometric_radius = geometric_radius
        if len(self.arc_table) != len(self.nodes) - 2:
            raise ValueError("len(arc_table) must equal len(nodes) - 2")

        self.num_of_linears = len(self.nodes) - 1
        self.linears = torch.nn.ModuleList()
        for i in range(self.num_of_linears):
            lin = torch.nn.Linear(self.nodes[i], self.nodes[i + 1], bias=True)
            if initialization is not None:
                with torch.no_grad():
                    if initialization == "kaiming":
                        std = math.sqrt(2.0 / self.nodes[i])
                        lin.weight.normal_(0.0, std, generator=generator)
                        lin.bias.zero_()
                    elif initialization == "geometric":  # SAL init, backend/model.py:63-70
                        if i != self.num_of_linears - 1:
                            lin.weight.normal_(0.0, math.sqrt(2.0) / math.sqrt(self.nodes[i + 1]), generator=generator)
                            lin.bias.zero_()
                        else:
                            lin.weight.fill_(math.sqrt(math.pi) / math.sqrt(self.nodes[i]))
                            lin.bias.fill_(-self.geometric_radius)
                    else:
                        raise ValueError("no such initialization: %s" % initialization)
            elif i == 0 and enable_print:
                print("Warning: Initialization strategy for MLP is not specified.")
            self.linears.append(lin)

        self.tms = torch.nn.ModuleList()
        for shape in self.arc_tm_shape:
            if shape[0] == 0 and shape[1] == 0:
                self.tms.append(torch.nn.Identity())
            else:  # default torch.nn.Linear init, as backend/model.py:91
                self.tms.append(torch.nn.Linear(shape[1], shape[0], bias=False))

        self.srcs = {}
        for arc in self.arc_table:
            for j in range(arc[0]):
                self.srcs[arc[1 + 2 * j]] = None
        self.outputs_list = []

    def forward(self, x, requires_outputs_list=False):
        """Same dataflow as backend/model.py:101-123; with
        ``requires_outputs_list`` the hidden activations are kept (their
        pre-ReLU signs give the activation state)."""
        if requires_outputs_list:
            self.outputs_list = []
        srcs = {}
        for i in range(self.num_of_linears):
            if i in self.srcs:
                srcs[i] = x
            x = self.linears[i](x)
            if i >= 1:
                arc = self.arc_table[i - 1]
                for j in range(arc[0]):
                    x = x + self.tms[arc[2 + 2 * j]](srcs[arc[1 + 2 * j]])
            if i != self.num_of_linears - 1:
                if requires_outputs_list:
                    self.outputs_list.append(x)
                x = torch.relu(x)
        return x

    def pre_activations(self, x):
        """Hidden pre-activations concatenated: (P, N).  The activation state
        is ``pre_activations(x) > 0`` (backend/main.py:407-411 takes
        ``relu(z) > 0``, the same predicate)."""
        self.forward(x, requires_outputs_list=True)
        out = torch.cat(self.outputs_list, dim=1)
        self.outputs_list = []
        return out

    def get_info(self):
        """weights, biases, transform matrices and the padded int32 arc table
        (backend/model.py:125-148)."""
        weights = [l.weight for l in self.linears]
        biases = [l.bias for l in self.linears]
        arc_tm = []
        for tm in self.tms:
            arc_tm.append(torch.zeros([0, 0]) if isinstance(tm, torch.nn.Identity) else tm.weight)
        width = max([len(a) for a in self.arc_table] + [1])
        arc_table = torch.zeros([len(self.arc_table), width], dtype=torch.int32)
        for r, arc in enumerate(self.arc_table):
            for c, val in enumerate(arc):
                arc_table[r, c] = val
        return {"weights": weights, "biases": biases, "arc_tm": arc_tm, "arc_table": arc_table}

    @property
    def state_len(self) -> int:
        return int(sum(self.nodes[1:-1]))
