"""Compute graph / `.qx` programme (mirror of src/compute_graph/{compute_graph,tensor_cache}.jl).

`build_compute_graph(tnc, plan, bond_groups)` (compute_graph.jl:15-98) emits the command list
the executor runs: `load` per tensor (:25-29), `output` per output tensor (:32-35), `view`
per tensor touching each sliced bond group with chained `_s` names (:39-58), `ncon` per plan
step with labels from `contraction_indices` (:61-74), outer-product joins of disconnected
parts (:77-90) and `save` of the root (:94).  Commands are emitted in post-order of the
compute tree (children before parents, first operand first), like the reference's DSL
example in docs/src/users_guide.md:73-90.

`TensorCache` (tensor_cache.jl:6-111) deduplicates leaf data: same shape and max |a - b| <
eps(Float64) -> the existing `data_<k>` key.
"""
from __future__ import annotations

from collections import OrderedDict
from dataclasses import dataclass, field

import numpy as np

from .planning import HyperNet, contraction_indices, hyper_network, mock_contract

__all__ = ["TensorCache", "Load", "View", "Output", "Ncon", "Save", "ComputeGraph",
           "build_compute_graph"]


class TensorCache:
    """Unique leaf tensors keyed `data_<k>` (tensor_cache.jl:6-69)."""

    def __init__(self, label: str = "data_"):
        self.label = label
        self.tensors: dict = {}          # shape tuple -> [(key, flat data)]
        self.key_dim_map: "OrderedDict[str, tuple]" = OrderedDict()
        self.id_val = 1

    def _next(self) -> str:
        k = f"{self.label}{self.id_val}"
        self.id_val += 1
        return k

    def push(self, data) -> str:
        data = np.asarray(data, dtype=np.complex128)
        dim = tuple(data.shape)
        flat = data.reshape(-1, order="F")
        eps = np.finfo(np.float64).eps
        if dim not in self.tensors:
            key = self._next()
            self.tensors[dim] = [(key, flat.copy())]
            self.key_dim_map[key] = dim
            return key
        for key, other in self.tensors[dim]:
            if np.max(np.abs(flat - other)) < eps if flat.size else True:
                return key
        key = self._next()
        self.tensors[dim].append((key, flat.copy()))
        self.key_dim_map[key] = dim
        return key

    def __getitem__(self, key: str) -> np.ndarray:
        if key not in self.key_dim_map:
            raise KeyError(f"No symbol {key} in cache")
        dim = self.key_dim_map[key]
        for k, flat in self.tensors[dim]:
            if k == key:
                return flat.reshape(dim, order="F")
        raise KeyError(key)

    def __len__(self):
        return len(self.key_dim_map)

    def to_dict(self) -> "OrderedDict[str, np.ndarray]":
        return OrderedDict((k, self[k]) for k in self.key_dim_map)


@dataclass
class Load:
    name: str
    data: str
    dims: tuple


@dataclass
class View:
    name: str
    src: str
    var: str          # "v<i>"
    pos: int          # 1-based rank position
    dim: int


@dataclass
class Output:
    name: str
    qubit: int        # 1-based
    dim: int


@dataclass
class Ncon:
    name: str
    c_labels: tuple   # () for a scalar
    a: str
    a_labels: tuple
    b: str
    b_labels: tuple


@dataclass
class Save:
    label: str
    name: str


@dataclass
class ComputeGraph:
    """The programme (commands in executable order) and its leaf data table."""
    commands: list
    data: "OrderedDict[str, np.ndarray]"
    metadata: dict = field(default_factory=dict)
    num_qubits: int = 0

    @property
    def ncons(self):
        return [c for c in self.commands if isinstance(c, Ncon)]

    @property
    def num_slices(self) -> int:
        vs = {}
        for c in self.commands:
            if isinstance(c, View):
                vs[c.var] = c.dim
        n = 1
        for d in vs.values():
            n *= d
        return n

    def __len__(self):
        """Nodes of the compute tree (load/output, view, ncon, save), like `length(cg.root)`."""
        return len(self.commands)


def _local_labels(lc, la, lb):
    """Number labels 1.. in order of first appearance in (a, b); c/a/b label tuples."""
    num = OrderedDict()
    for l in list(la) + list(lb):
        if l not in num:
            num[l] = len(num) + 1
    return tuple(num[l] for l in lc), tuple(num[l] for l in la), tuple(num[l] for l in lb)


def build_compute_graph(tnc, plan, bond_groups=None) -> ComputeGraph:
    """Programme for contracting `tnc` along `plan`, slicing `bond_groups` (lists of plain
    index ids) -- restated from src/compute_graph/compute_graph.jl:15-98."""
    tnc = tnc.copy()
    tn = tnc.tn
    net = hyper_network(tnc)
    tc = TensorCache()
    nodes: dict = {}          # name -> (command, children names)
    for t in list(tn.tensors):
        data = tn.reduced_data(t)
        key = tc.push(data)
        nodes[t] = (Load(t, key, tuple(data.shape)), [])
    for i, o in enumerate(tnc.output_tensors, start=1):
        nodes[o] = (Output(o, i, tn.reduced_data(o).shape[0]), [])
    changed: dict = {}
    if bond_groups:
        for i, bg in enumerate(bond_groups, start=1):
            var = f"v{i}"
            lab = tn.root(bg[0])
            dim = tn.dims[bg[0]]
            related = [t for t, ls in net.tensors.items() if lab in ls]
            for t in related:
                new = f"{t}_s"
                pos = net.tensors[t].index(lab) + 1
                nodes[new] = (View(new, t, var, pos, dim), [t])
                # rename t -> new in the planning state
                net.tensors = OrderedDict((new if k == t else k, v) for k, v in net.tensors.items())
                net._names.add(new)
                changed[t] = new
    parent: dict = {}
    for (a, b, c) in plan:
        while a in changed:
            a = changed[a]
        while b in changed:
            b = changed[b]
        lc, la, lb = contraction_indices(net, a, b)
        nc, na, nb = _local_labels(lc, la, lb)
        nodes[c] = (Ncon(c, nc, a, na, b, nb), [a, b])
        parent[a] = c; parent[b] = c
        mock_contract(net, a, b, c)
    for name, (_, ch) in list(nodes.items()):
        for x in ch:
            parent[x] = name
    roots = [n for n in nodes if n not in parent]
    cur = roots[0]
    for other in roots[1:]:
        lc, la, lb = contraction_indices(net, cur, other)
        nc, na, nb = _local_labels(lc, la, lb)
        new = net.next_tensor_id()
        while new in nodes:
            new = net.next_tensor_id()
        nodes[new] = (Ncon(new, nc, cur, na, other, nb), [cur, other])
        parent[cur] = new; parent[other] = new
        mock_contract(net, cur, other, new)
        cur = new
    root = cur
    # post-order emission
    commands = []
    stack = [(root, False)]
    while stack:
        name, done = stack.pop()
        cmd, ch = nodes[name]
        if done or not ch:
            commands.append(cmd)
            continue
        stack.append((name, True))
        for x in reversed(ch):
            stack.append((x, False))
    commands.append(Save("output", root))
    used = OrderedDict()
    for c in commands:
        if isinstance(c, Load):
            used[c.data] = tc[c.data]
    data = OrderedDict((k, tc[k]) for k in tc.key_dim_map if k in used)
    return ComputeGraph(commands, data, num_qubits=tnc.qubits)
