"""``save_model`` / ``load_model``: the ONNX files of the reference's
backend/onnx_io.py:11-285, without the ``onnx`` package.

The reference exports with ``torch.onnx.export`` and parses the graph's
printable form back into an ``MLP``.  Here both directions work on the
protobuf wire format directly, for the subset of ONNX an MLP needs:

* ``Gemm`` (alpha = beta = 1, transB = 1) per linear layer, ``Relu`` after
  every hidden one;
* skip connections as ``Add(main, src)`` (identity) or
  ``Add(main, MatMul(src, T))`` with ``T`` the transform transposed, or
  ``MatMul(src, Transpose(T, perm=[1, 0]))`` -- the forms the reference
  accepts (backend/onnx_io.py:100-125, 166-212);
* float32 (or float64) initializers, stored as ``raw_data`` or ``float_data``.

The field numbers below are those of the public ``onnx.proto`` schema
(ModelProto, GraphProto, NodeProto, AttributeProto, TensorProto,
ValueInfoProto, TypeProto, TensorShapeProto); the file format has to match
for the files to interchange.
"""
from __future__ import annotations

import os
import struct
from typing import Dict, List, Tuple

import numpy as np
import torch

from .model import MLP

# --------------------------------------------------------------------------
# protobuf wire format

_VARINT, _I64, _LEN, _I32 = 0, 1, 2, 5


def _varint(n: int) -> bytes:
    n &= (1 << 64) - 1
    out = bytearray()
    while True:
        b = n & 0x7F
        n >>= 7
        if n:
            out.append(b | 0x80)
        else:
            out.append(b)
            return bytes(out)


def _key(field: int, wt: int) -> bytes:
    return _varint((field << 3) | wt)


def _f_int(field: int, v: int) -> bytes:
    return _key(field, _VARINT) + _varint(v)


def _f_bytes(field: int, b: bytes) -> bytes:
    return _key(field, _LEN) + _varint(len(b)) + b


def _f_str(field: int, s: str) -> bytes:
    return _f_bytes(field, s.encode())


def _f_float(field: int, v: float) -> bytes:
    return _key(field, _I32) + struct.pack("<f", v)


def _read_varint(buf: bytes, pos: int) -> Tuple[int, int]:
    shift = 0
    v = 0
    while True:
        if pos >= len(buf):
            raise ValueError("truncated varint")
        b = buf[pos]
        pos += 1
        v |= (b & 0x7F) << shift
        if not b & 0x80:
            return v, pos
        shift += 7
        if shift > 70:
            raise ValueError("varint too long")


def _parse(buf: bytes) -> Dict[int, List[Tuple[int, object]]]:
    """field number -> [(wire type, value)] of one message (value: int or bytes)."""
    out: Dict[int, List[Tuple[int, object]]] = {}
    pos = 0
    while pos < len(buf):
        k, pos = _read_varint(buf, pos)
        field, wt = k >> 3, k & 7
        if wt == _VARINT:
            v, pos = _read_varint(buf, pos)
        elif wt == _I64:
            v = buf[pos:pos + 8]
            pos += 8
        elif wt == _LEN:
            n, pos = _read_varint(buf, pos)
            v = buf[pos:pos + n]
            pos += n
        elif wt == _I32:
            v = buf[pos:pos + 4]
            pos += 4
        else:
            raise ValueError("unsupported wire type %d" % wt)
        if pos > len(buf):
            raise ValueError("truncated message")
        out.setdefault(field, []).append((wt, v))
    return out


def _ints(fields, f) -> List[int]:
    """repeated int64, packed or not."""
    vals: List[int] = []
    for wt, v in fields.get(f, []):
        if wt == _LEN:
            p = 0
            while p < len(v):
                x, p = _read_varint(v, p)
                vals.append(x)
        else:
            vals.append(v)
    return [x - (1 << 64) if x >= 1 << 63 else x for x in vals]


def _str(fields, f, default="") -> str:
    v = fields.get(f)
    return v[-1][1].decode() if v else default


def _strs(fields, f) -> List[str]:
    return [v.decode() for _, v in fields.get(f, [])]


# --------------------------------------------------------------------------
# ONNX messages

_FLOAT, _DOUBLE = 1, 11  # TensorProto.DataType


def _tensor(name: str, a: np.ndarray) -> bytes:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = b"".join(_f_int(1, d) for d in a.shape)  # dims
    b += _f_int(2, _FLOAT)                        # data_type
    b += _f_str(8, name)                          # name
    b += _f_bytes(9, a.astype("<f4").tobytes())   # raw_data
    return b


def _value_info(name: str, shape) -> bytes:
    dims = b"".join(_f_bytes(1, _f_int(1, d)) for d in shape)  # Dimension.dim_value
    tensor_type = _f_int(1, _FLOAT) + _f_bytes(2, dims)         # elem_type, shape
    return _f_str(1, name) + _f_bytes(2, _f_bytes(1, tensor_type))


def _node(op: str, inputs, outputs, name: str, attrs: bytes = b"") -> bytes:
    b = b"".join(_f_str(1, s) for s in inputs) + b"".join(_f_str(2, s) for s in outputs)
    return b + _f_str(3, name) + _f_str(4, op) + attrs


def _attr_float(name: str, v: float) -> bytes:
    return _f_bytes(5, _f_str(1, name) + _f_float(2, v) + _f_int(20, 1))  # type FLOAT


def _attr_int(name: str, v: int) -> bytes:
    return _f_bytes(5, _f_str(1, name) + _f_int(3, v) + _f_int(20, 2))  # type INT


def _decode_tensor(buf: bytes) -> Tuple[str, np.ndarray]:
    f = _parse(buf)
    dims = _ints(f, 1)
    dtype = _ints(f, 2)[0] if 2 in f else _FLOAT
    name = _str(f, 8)
    if dtype not in (_FLOAT, _DOUBLE):
        raise ValueError("initializer %s: unsupported data type %d" % (name, dtype))
    npdt = "<f4" if dtype == _FLOAT else "<f8"
    if 9 in f:
        a = np.frombuffer(f[9][-1][1], dtype=npdt).astype(np.float64 if dtype == _DOUBLE else np.float32)
    else:
        field, code, size = (4, "f", 4) if dtype == _FLOAT else (10, "d", 8)
        vals: List[float] = []
        for wt, v in f.get(field, []):
            if wt == _LEN:
                vals.extend(struct.unpack("<%d%s" % (len(v) // size, code), v))
            else:
                vals.append(struct.unpack("<" + code, v)[0])
        a = np.asarray(vals, dtype=np.float32 if dtype == _FLOAT else np.float64)
    n = int(np.prod(dims)) if dims else 1
    if a.size != n:
        raise ValueError("initializer %s: %d values for dims %s" % (name, a.size, dims))
    return name, a.reshape(dims)


def _decode_attrs(node_fields) -> Dict[str, object]:
    out: Dict[str, object] = {}
    for _, ab in node_fields.get(5, []):
        a = _parse(ab)
        name = _str(a, 1)
        atype = _ints(a, 20)[0] if 20 in a else 0
        if atype == 1 or (atype == 0 and 2 in a):
            out[name] = struct.unpack("<f", a[2][-1][1])[0]
        elif atype == 2 or (atype == 0 and 3 in a):
            out[name] = _ints(a, 3)[-1]
        elif atype == 7 or (atype == 0 and 8 in a):
            out[name] = _ints(a, 8)
        else:
            out[name] = None
    return out


# --------------------------------------------------------------------------
# MLP <-> graph

def _graph_bytes(model: MLP) -> bytes:
    nodes, nodes_b, inits = model.nodes, [], []
    n_lin = len(nodes) - 1
    aux = {0: "input"}  # layer index -> tensor name (0 = input, h = output of hidden layer h)
    tm_names = {}
    x = "input"
    for i in range(n_lin):
        W = model.linears[i].weight.detach().cpu().numpy()
        b = model.linears[i].bias.detach().cpu().numpy()
        inits.append(_tensor("linears.%d.weight" % i, W))
        inits.append(_tensor("linears.%d.bias" % i, b))
        out = "gemm_%d" % i
        nodes_b.append(_node("Gemm", [x, "linears.%d.weight" % i, "linears.%d.bias" % i], [out], "Gemm_%d" % i,
                             _attr_float("alpha", 1.0) + _attr_float("beta", 1.0) + _attr_int("transB", 1)))
        x = out
        if i >= 1:
            row = model.arc_table[i - 1]
            for j in range(row[0]):
                src, t = row[1 + 2 * j], row[2 + 2 * j]
                if list(model.arc_tm_shape[t]) == [0, 0]:
                    term = aux[src]
                else:
                    tname = "tms.%d.weight_t" % t
                    if t not in tm_names:
                        T = model.tms[t].weight.detach().cpu().numpy()
                        inits.append(_tensor(tname, T.T))
                        tm_names[t] = tname
                    term = "matmul_%d_%d" % (i, j)
                    nodes_b.append(_node("MatMul", [aux[src], tname], [term], "MatMul_%d_%d" % (i, j)))
                out = "add_%d_%d" % (i, j)
                nodes_b.append(_node("Add", [x, term], [out], "Add_%d_%d" % (i, j)))
                x = out
        if i < n_lin - 1:
            out = "relu_%d" % (i + 1)
            nodes_b.append(_node("Relu", [x], [out], "Relu_%d" % (i + 1)))
            x = out
            aux[i + 1] = out
    # the last node writes the graph output
    last = nodes_b[-1]
    nodes_b[-1] = last.replace(_f_str(2, x), _f_str(2, "output"), 1)
    g = b"".join(_f_bytes(1, n) for n in nodes_b)
    g += _f_str(2, "analytic_mlp")
    g += b"".join(_f_bytes(5, t) for t in inits)
    g += _f_bytes(11, _value_info("input", (1, 3)))
    g += _f_bytes(12, _value_info("output", (1, 1)))
    return g


def _is_relu(n) -> bool:
    import torch.nn.functional as F

    if n.op == "call_function":
        return n.target in (torch.relu, F.relu, torch.relu_)
    if n.op == "call_method":
        return n.target in ("relu", "relu_")
    return False


def _is_add(n) -> bool:
    import operator

    if n.op == "call_function":
        return n.target in (operator.add, operator.iadd, torch.add)
    return n.op == "call_method" and n.target in ("add", "add_")


def _traced_graph_bytes(module: torch.nn.Module) -> bytes:
    """The ONNX graph of any torch module whose forward is a ReLU MLP:
    ``nn.Linear`` layers, ReLUs after the hidden ones, and additive skip
    connections (an identity, or a bias-free ``nn.Linear`` transform of an
    earlier layer's output).  The reference exports such a module with
    ``torch.onnx.export`` (backend/onnx_io.py:255-258; examples/2_polytope.py
    saves a hand-written module that way); here the forward is traced with
    ``torch.fx`` and written in the node forms ``load_model`` reads back:
    ``Gemm`` per layer, ``Relu``, ``Add``, ``MatMul`` by the transposed
    transform."""
    import torch.fx as fx

    try:
        gm = fx.symbolic_trace(module)
    except Exception as exc:
        raise ValueError("save_model: the module's forward cannot be traced (%s)" % exc) from exc
    nodes = list(gm.graph.nodes)
    placeholders = [n for n in nodes if n.op == "placeholder"]
    outs = [n for n in nodes if n.op == "output"]
    if len(placeholders) != 1 or len(outs) != 1 or not isinstance(outs[0].args[0], fx.Node):
        raise ValueError("save_model: expected a module with one input tensor and one output tensor")
    result = outs[0].args[0]

    def linear_of(n):
        if n.op == "call_module":
            mod = gm.get_submodule(n.target)
            if isinstance(mod, torch.nn.Linear):
                return mod
        return None

    def is_main(n):
        lin = linear_of(n)
        return (lin is not None and lin.bias is not None) or _is_add(n)

    def is_transform(n):
        # a bias-free linear added onto the main path: a skip transform
        lin = linear_of(n)
        if lin is None or lin.bias is not None or len(n.users) != 1:
            return False
        user = next(iter(n.users))
        return _is_add(user) and any(is_main(a) for a in user.args if isinstance(a, fx.Node) and a is not n)

    name = {placeholders[0]: "input"}
    body, inits = [], []
    for n in nodes:
        if n.op in ("placeholder", "output"):
            continue
        out = "output" if n is result else n.name
        args = [a for a in n.args if isinstance(a, fx.Node)]
        lin = linear_of(n)
        if lin is not None:
            if len(args) != 1:
                raise ValueError("save_model: unsupported call of %s" % n.target)
            W = lin.weight.detach().cpu().float().numpy()
            if is_transform(n):
                inits.append(_tensor(n.name + ".weight_t", W.T))
                body.append(_node("MatMul", [name[args[0]], n.name + ".weight_t"], [out], n.name))
            else:
                b = lin.bias.detach().cpu().float().numpy() if lin.bias is not None else np.zeros(W.shape[0], np.float32)
                inits.append(_tensor(n.name + ".weight", W))
                inits.append(_tensor(n.name + ".bias", b))
                body.append(_node("Gemm", [name[args[0]], n.name + ".weight", n.name + ".bias"], [out], n.name,
                                  _attr_float("alpha", 1.0) + _attr_float("beta", 1.0) + _attr_int("transB", 1)))
        elif _is_relu(n) or (n.op == "call_module" and isinstance(gm.get_submodule(n.target), torch.nn.ReLU)):
            if len(args) != 1:
                raise ValueError("save_model: unsupported call of %s" % n.target)
            body.append(_node("Relu", [name[args[0]]], [out], n.name))
        elif _is_add(n):
            if len(args) != 2 or len(n.args) != 2 or n.kwargs:
                raise ValueError("save_model: only two-operand additions are supported")
            body.append(_node("Add", [name[args[0]], name[args[1]]], [out], n.name))
        else:
            raise ValueError("save_model: unsupported operation %s %s (a ReLU MLP uses nn.Linear, ReLU and "
                             "additions only)" % (n.op, n.target))
        name[n] = out
    if not body:
        raise ValueError("save_model: the module computes nothing")
    g = b"".join(_f_bytes(1, nb) for nb in body)
    g += _f_str(2, "analytic_mlp")
    g += b"".join(_f_bytes(5, t) for t in inits)
    g += _f_bytes(11, _value_info("input", (1, 3)))
    g += _f_bytes(12, _value_info("output", (1, 1)))
    return g


def model_bytes(model: torch.nn.Module) -> bytes:
    """The ONNX ModelProto of ``model`` (ir_version 8, opset 17): an ``MLP``,
    or any module whose forward is a ReLU MLP of ``nn.Linear`` layers."""
    graph = _graph_bytes(model) if isinstance(model, MLP) else _traced_graph_bytes(model)
    m = _f_int(1, 8)                                        # ir_version
    m += _f_str(2, "analyticmesh_gb300")                    # producer_name
    m += _f_bytes(7, graph)                                 # graph
    m += _f_bytes(8, _f_str(1, "") + _f_int(2, 17))         # opset_import
    return m


def save_model(model: torch.nn.Module, model_path: str) -> None:
    """Write ``model`` as an ONNX file (backend/onnx_io.py:255-258): an
    ``MLP``, or any module whose forward is a ReLU MLP (``nn.Linear`` layers,
    ReLU, additive skips), as the reference's examples save them."""
    with open(model_path, "wb") as fh:
        fh.write(model_bytes(model))


def _mlp_from_graph(gbuf: bytes) -> MLP:
    g = _parse(gbuf)
    inits = dict(_decode_tensor(t) for _, t in g.get(5, []))
    flows = []
    for _, nb in g.get(1, []):
        n = _parse(nb)
        flows.append(dict(op=_str(n, 4), inputs=_strs(n, 1), outputs=_strs(n, 2), attrs=_decode_attrs(n)))
    graph_inputs = [_str(_parse(v), 1) for _, v in g.get(11, [])]
    graph_inputs = [s for s in graph_inputs if s not in inits]  # older exporters list initializers too
    outputs = [_str(_parse(v), 1) for _, v in g.get(12, [])]
    if len(graph_inputs) != 1 or len(outputs) != 1:
        raise ValueError("expected one graph input and one output")
    x_in, y_out = graph_inputs[0], outputs[0]
    producer = {}
    for f in flows:
        if f["op"] not in ("Gemm", "Relu", "MatMul", "Add", "Transpose"):
            raise ValueError("unsupported operator %s" % f["op"])
        for o in f["outputs"]:
            producer[o] = f
        if f["op"] == "Gemm":
            a = f["attrs"]
            if a.get("alpha", 1.0) != 1.0 or a.get("beta", 1.0) != 1.0 or a.get("transB", 0) != 1:
                raise ValueError("Gemm must have alpha = beta = 1 and transB = 1")
        if f["op"] == "Transpose" and list(f["attrs"].get("perm", [1, 0])) != [1, 0]:
            raise ValueError("Transpose must have perm = [1, 0]")

    gemms = [f for f in flows if f["op"] == "Gemm"]
    relus = [f for f in flows if f["op"] == "Relu"]
    if len(relus) != len(gemms) - 1:
        raise ValueError("expected a Relu after every hidden Gemm")
    weights = [np.asarray(inits[f["inputs"][1]]) for f in gemms]
    biases = [np.asarray(inits[f["inputs"][2]]) for f in gemms]
    if weights[0].shape[1] != 3 or weights[-1].shape[0] != 1:
        raise ValueError("the network must map R^3 to R")
    nodes = [3] + [w.shape[0] for w in weights]
    aux = [x_in] + [r["outputs"][0] for r in relus] + [y_out]

    consumers: Dict[str, List[dict]] = {}
    for f in flows:
        for s in f["inputs"]:
            consumers.setdefault(s, []).append(f)

    def dst_of(t: str) -> int:
        # follow the value forward to the next Relu output or the graph output
        while t not in aux[1:]:
            nxt = [f for f in consumers.get(t, []) if f["op"] in ("Add", "Relu")]
            if not nxt:
                raise ValueError("dangling value %s" % t)
            t = nxt[0]["outputs"][0]
        return aux.index(t)

    def weight_of(name: str) -> np.ndarray:
        # a MatMul right operand: an initializer (transform transposed) or
        # Transpose(transform)
        if name in inits:
            return np.asarray(inits[name]).T
        f = producer.get(name)
        if f is not None and f["op"] == "Transpose" and f["inputs"][0] in inits:
            return np.asarray(inits[f["inputs"][0]])
        raise ValueError("MatMul operand %s is not a constant" % name)

    arc_table = [[0] for _ in range(len(nodes) - 2)]
    tm_keys, tm_mats = [], []
    for f in flows:
        if f["op"] != "Add":
            continue
        dst = dst_of(f["outputs"][0])
        src = tm = None
        for a in f["inputs"]:
            p = producer.get(a)
            if p is not None and p["op"] in ("Gemm", "Add"):
                continue  # the main path
            if p is not None and p["op"] == "MatMul":
                src_name, key = p["inputs"][0], p["inputs"][1]
                mat = weight_of(key)
            else:
                src_name, key, mat = a, "identity", None
            if src_name not in aux[:-1]:
                raise ValueError("skip source %s is not a layer output" % src_name)
            src = aux.index(src_name)
            if key not in tm_keys:
                tm_keys.append(key)
                tm_mats.append(mat)
            tm = tm_keys.index(key)
        if src is None or dst < 2:
            raise ValueError("unrecognised Add")
        row = arc_table[dst - 2]
        row[0] += 1
        row.extend([src, tm])
    arc_tm_shape = [[0, 0] if m is None else list(m.shape) for m in tm_mats]

    model = MLP(nodes, arc_table, arc_tm_shape, initialization=None, enable_print=False)
    with torch.no_grad():
        for i in range(len(weights)):
            model.linears[i].weight.copy_(torch.as_tensor(weights[i], dtype=torch.float32))
            model.linears[i].bias.copy_(torch.as_tensor(biases[i], dtype=torch.float32))
        for t, m in enumerate(tm_mats):
            if m is not None:
                model.tms[t].weight.copy_(torch.as_tensor(m, dtype=torch.float32))
    return model


def load_model(model_file_str) -> MLP:
    """An ``MLP`` from an ONNX file path or its bytes (backend/onnx_io.py:261-285)."""
    if isinstance(model_file_str, (bytes, bytearray)):
        buf = bytes(model_file_str)
    elif isinstance(model_file_str, str) and os.path.exists(model_file_str):
        with open(model_file_str, "rb") as fh:
            buf = fh.read()
    else:
        raise ValueError("unknown model_file_str = %r" % (model_file_str,))
    m = _parse(buf)
    if 7 not in m:
        raise ValueError("not an ONNX model (no graph)")
    return _mlp_from_graph(m[7][-1][1])
