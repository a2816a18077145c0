"""Tensor network circuits (mirror of QXTns' TensorNetworkCircuit as used by src/tn_conversion.jl).

QXTns is un-vendored; this restates what the reference's call sites rely on:
  - `TensorNetworkCircuit(n)`, `push!(tnc, qubits, data; decompose)` (tn_conversion.jl:10-18),
    `add_input!` / `add_output!` with a bitstring of '0','1','+','-' (docs/src/basics.md:55-64;
    src/simulation.jl:88), `length(tnc)`, `qubits(tnc)`, `bonds`, `tensor_data`.
  - hyperindices: indices tied by diagonal structure form one hyperedge
    (docs/src/features.md:5-11); a tensor's data is reduced to one axis per tied group and
    its ncon labels are the groups (`hyperindices(tnc, t, all_indices=true)`,
    src/compute_graph/compute_graph.jl:46-48).
  - `decompose=true` splits a two-qubit gate into two rank-3 tensors joined by a bond
    (tn_conversion.jl:10-18, docs/src/features.md).  A gate that is block diagonal in one
    qubit (controlled gates) is split as sum_c |c><c| (x) U_c, which makes the control half
    a fully tied delta; any other gate is split by SVD of the (o1,i1) x (o2,i2) matrix,
    keeping the numerically non-zero singular values.

Tensor index order: one-qubit gate (out, in); two-qubit gate (out1, out2, in1, in2);
decomposed halves (out_q, in_q, bond); input/output tensors one index.
"""
from __future__ import annotations

from collections import OrderedDict

import numpy as np

from . import circuits as _circ

__all__ = ["TensorNetworkCircuit", "TensorNetwork", "QXTensor", "convert_to_tnc"]

_DIAG_TOL = 0.0          # exact zeros define diagonal structure (gate matrices are exact)
_SVD_RTOL = 1e-12


class QXTensor:
    __slots__ = ("indices", "data")

    def __init__(self, indices, data):
        self.indices = list(indices)
        self.data = np.asarray(data, dtype=np.complex128)
        if self.data.ndim != len(self.indices):
            raise ValueError("tensor rank does not match its index count")


class TensorNetwork:
    """Tensors keyed by symbol name, plain index ids with dims, and a union-find of tied indices."""

    def __init__(self):
        self.tensors: "OrderedDict[str, QXTensor]" = OrderedDict()
        self.dims: dict = {}
        self._parent: dict = {}
        self._next_index = 1
        self._next_tensor = 1

    # ---- ids -------------------------------------------------------------------------
    def new_index(self, dim: int) -> int:
        i = self._next_index
        self._next_index += 1
        self.dims[i] = int(dim)
        self._parent[i] = i
        return i

    def next_tensor_id(self) -> str:
        """Next unused tensor symbol `t<k>` (QXTns `next_tensor_id!`)."""
        while f"t{self._next_tensor}" in self.tensors:
            self._next_tensor += 1
        name = f"t{self._next_tensor}"
        self._next_tensor += 1
        return name

    # ---- hyperedges ------------------------------------------------------------------
    def root(self, i: int) -> int:
        p = self._parent
        while p[i] != i:
            p[i] = p[p[i]]
            i = p[i]
        return i

    def tie(self, i: int, j: int):
        ri, rj = self.root(i), self.root(j)
        if ri != rj:
            if self.dims[ri] != self.dims[rj]:
                raise ValueError("cannot tie indices of different dimension")
            self._parent[max(ri, rj)] = min(ri, rj)

    def groups(self, name: str) -> list:
        """Groups of the tensor's indices tied together, in order of first occurrence
        (QXTns `hyperindices(tn, t, all_indices=true)`)."""
        out, seen = [], {}
        for ix in self.tensors[name].indices:
            r = self.root(ix)
            if r in seen:
                out[seen[r]].append(ix)
            else:
                seen[r] = len(out)
                out.append([ix])
        return out

    def labels(self, name: str) -> list:
        """Hyperedge labels (union-find roots) of the tensor, one per group."""
        return [self.root(g[0]) for g in self.groups(name)]

    def reduced_data(self, name: str, data=None) -> np.ndarray:
        """Tensor data (or `data` of the same shape, e.g. a derivative of it) with each tied
        group reduced to its diagonal (one axis per group)."""
        t = self.tensors[name]
        if data is not None:
            t = QXTensor(t.indices, data)
        grp = self.groups(name)
        pos = {ix: k for k, ix in enumerate(t.indices)}
        if all(len(g) == 1 for g in grp):
            return t.data
        letters = "abcdefghijklmnopqrstuvwxyz"
        sub_in = [""] * len(t.indices)
        sub_out = ""
        for gi, g in enumerate(grp):
            for ix in g:
                sub_in[pos[ix]] = letters[gi]
            sub_out += letters[gi]
        return np.einsum("".join(sub_in) + "->" + sub_out, t.data).copy()

    def hyperedges(self) -> "OrderedDict[int, list]":
        """Hyperedge label -> tensor names touching it (each name once), by label id."""
        he: "OrderedDict[int, list]" = OrderedDict()
        for name in self.tensors:
            for lab in self.labels(name):
                he.setdefault(lab, [])
                if name not in he[lab]:
                    he[lab].append(name)
        return OrderedDict(sorted(he.items()))

    def bonds(self) -> list:
        """Plain index ids used by at least one tensor."""
        s = set()
        for t in self.tensors.values():
            s.update(t.indices)
        return sorted(s)

    def tensors_with_index(self, ix: int) -> list:
        return [n for n, t in self.tensors.items() if ix in t.indices]

    def __len__(self):
        return len(self.tensors)

    def __contains__(self, name):
        return name in self.tensors

    def add_tensor(self, indices, data, name=None) -> str:
        name = name or self.next_tensor_id()
        if name in self.tensors:
            raise ValueError(f"tensor {name} exists")
        self.tensors[name] = QXTensor(indices, data)
        for ix, d in zip(indices, np.shape(data)):
            if self.dims[ix] != d:
                raise ValueError("data shape does not match index dims")
        return name

    def detect_ties(self, name: str):
        """Tie every pair of the tensor's equal-dimension indices on which its data is diagonal."""
        t = self.tensors[name]
        r = t.data.ndim
        for a in range(r):
            for b in range(a + 1, r):
                if t.data.shape[a] != t.data.shape[b]:
                    continue
                if self.root(t.indices[a]) == self.root(t.indices[b]):
                    continue
                d = t.data.shape[a]
                moved = np.moveaxis(t.data, (a, b), (0, 1))
                off = ~np.eye(d, dtype=bool)
                if np.all(np.abs(moved[off]) <= _DIAG_TOL):
                    self.tie(t.indices[a], t.indices[b])

    def copy(self) -> "TensorNetwork":
        n = TensorNetwork()
        n.tensors = OrderedDict((k, QXTensor(v.indices, v.data)) for k, v in self.tensors.items())
        n.dims = dict(self.dims)
        n._parent = dict(self._parent)
        n._next_index = self._next_index
        n._next_tensor = self._next_tensor
        return n


def _decompose_two_qubit(m4: np.ndarray):
    """Split a 4x4 gate into halves A[o1,i1,b] (first qubit) and B[o2,i2,b] (second qubit).

    Returns (A, B, tie_first, tie_second): tie_X says that half is a delta over (o, i, b)."""
    t = m4.reshape(2, 2, 2, 2, order="F")          # t[o1,o2,i1,i2]
    # block diagonal in the second qubit: t[:,o2,:,i2] == 0 for o2 != i2  -> control = q2
    ctrl2 = all(np.all(t[:, o2, :, i2] == 0) for o2 in range(2) for i2 in range(2) if o2 != i2)
    ctrl1 = all(np.all(t[o1, :, i1, :] == 0) for o1 in range(2) for i1 in range(2) if o1 != i1)
    if ctrl2:
        a = np.stack([t[:, c, :, c] for c in range(2)], axis=2)       # a[o1,i1,c]
        b = np.zeros((2, 2, 2), dtype=np.complex128)
        for c in range(2):
            b[c, c, c] = 1.0
        return a, b, False, True
    if ctrl1:
        b = np.stack([t[c, :, c, :] for c in range(2)], axis=2)       # b[o2,i2,c]
        a = np.zeros((2, 2, 2), dtype=np.complex128)
        for c in range(2):
            a[c, c, c] = 1.0
        return a, b, True, False
    mat = t.transpose(0, 2, 1, 3).reshape(4, 4, order="F")            # rows (o1,i1), cols (o2,i2)
    u, s, vh = np.linalg.svd(mat)
    r = int(np.sum(s > _SVD_RTOL * s[0]))
    sq = np.sqrt(s[:r])
    a = (u[:, :r] * sq).reshape(2, 2, r, order="F")
    b = (sq[:, None] * vh[:r, :]).T.reshape(2, 2, r, order="F")
    return a, b, False, False


class TensorNetworkCircuit:
    """Mirror of QXTns' TensorNetworkCircuit: a tensor network plus per-qubit input and
    output (open) index ids."""

    def __init__(self, qubits: int):
        self.tn = TensorNetwork()
        self.qubits = int(qubits)
        self.input_indices = [self.tn.new_index(2) for _ in range(self.qubits)]
        self.output_indices = list(self.input_indices)
        self.input_tensors: list = []
        self.output_tensors: list = []

    def __len__(self):
        return len(self.tn)

    def keys(self):
        return list(self.tn.tensors.keys())

    def copy(self) -> "TensorNetworkCircuit":
        c = TensorNetworkCircuit.__new__(TensorNetworkCircuit)
        c.tn = self.tn.copy()
        c.qubits = self.qubits
        c.input_indices = list(self.input_indices)
        c.output_indices = list(self.output_indices)
        c.input_tensors = list(self.input_tensors)
        c.output_tensors = list(self.output_tensors)
        return c

    def tensor_data(self, name: str, consider_hyperindices: bool = True) -> np.ndarray:
        return self.tn.reduced_data(name) if consider_hyperindices else self.tn.tensors[name].data

    def push(self, qubits, data, decompose: bool = False) -> list:
        """Append a gate (`push!(tnc, qubits, data; decompose)`); returns the new tensor names."""
        tn = self.tn
        data = np.asarray(data, dtype=np.complex128)
        qs = [int(q) - 1 for q in qubits]
        if len(qs) == 1:
            q = qs[0]
            o = tn.new_index(2)
            name = tn.add_tensor([o, self.output_indices[q]], data)
            self.output_indices[q] = o
            tn.detect_ties(name)
            return [name]
        if len(qs) != 2 or data.shape != (4, 4):
            raise ValueError("only one- and two-qubit gates are supported")
        q1, q2 = qs
        o1, o2 = tn.new_index(2), tn.new_index(2)
        i1, i2 = self.output_indices[q1], self.output_indices[q2]
        if not decompose:
            name = tn.add_tensor([o1, o2, i1, i2], data.reshape(2, 2, 2, 2, order="F"))
            self.output_indices[q1], self.output_indices[q2] = o1, o2
            tn.detect_ties(name)
            return [name]
        a, b, tie1, tie2 = _decompose_two_qubit(data)
        bond = tn.new_index(a.shape[2])
        na = tn.add_tensor([o1, i1, bond], a)
        nb = tn.add_tensor([o2, i2, bond], b)
        self.output_indices[q1], self.output_indices[q2] = o1, o2
        if tie1:
            tn.tie(o1, i1); tn.tie(o1, bond)
        if tie2:
            tn.tie(o2, i2); tn.tie(o2, bond)
        tn.detect_ties(na)
        tn.detect_ties(nb)
        return [na, nb]

    def _boundary(self, which: str, bitstring):
        if bitstring is None:
            bitstring = "0" * self.qubits
        if len(bitstring) != self.qubits:
            raise ValueError("bitstring length must equal the number of qubits")
        names = []
        idx = self.input_indices if which == "in" else self.output_indices
        for q, ch in enumerate(bitstring):
            names.append(self.tn.add_tensor([idx[q]], basis_vector(ch)))
        return names

    def add_input(self, bitstring=None):
        """`add_input!`: rank-1 tensor per qubit on its input index (default all '0')."""
        if self.input_tensors:
            raise ValueError("inputs already added")
        self.input_tensors = self._boundary("in", bitstring)

    def add_output(self, bitstring=None):
        """`add_output!`: rank-1 tensor per qubit on its output index (default all '0')."""
        if self.output_tensors:
            raise ValueError("outputs already added")
        self.output_tensors = self._boundary("out", bitstring)

    def add_output_subset(self, qubits):
        """Output tensors on the listed qubits (1-based) only; the others stay open, so the
        contraction yields a 2^k tensor per bitstring (k open qubits).  Output i of the
        programme is qubits[i-1]; bitstrings carry one character per listed qubit."""
        if self.output_tensors:
            raise ValueError("outputs already added")
        self.output_tensors = [self.tn.add_tensor([self.output_indices[q - 1]], basis_vector("0"))
                               for q in qubits]

    def set_output(self, bitstring: str):
        """Replace the data of the existing output tensors with another bitstring's vectors."""
        for q, ch in enumerate(bitstring):
            self.tn.tensors[self.output_tensors[q]].data = basis_vector(ch)

    def open_labels(self) -> set:
        """Hyperedge labels with a dangling plain index (an unterminated circuit wire)."""
        count: dict = {}
        for t in self.tn.tensors.values():
            for ix in t.indices:
                count[ix] = count.get(ix, 0) + 1
        wires = set(self.input_indices) | set(self.output_indices)
        return {self.tn.root(ix) for ix, c in count.items() if c == 1 and ix in wires}


def basis_vector(ch: str) -> np.ndarray:
    """Output/input vector for a bitstring character (docs/src/basics.md:55-64):
    '0' -> |0>, '1' -> |1>, '+' -> (|0>+|1>)/sqrt 2, '-' -> (|0>-|1>)/sqrt 2."""
    r = 1.0 / np.sqrt(2.0)
    table = {"0": [1.0, 0.0], "1": [0.0, 1.0], "+": [r, r], "-": [r, -r]}
    if ch not in table:
        raise ValueError(f"bitstring character {ch!r} not in '01+-'")
    return np.array(table[ch], dtype=np.complex128)


def convert_to_tnc(circ, *, input=None, output=None, no_input=False, no_output=False,
                   decompose=False) -> TensorNetworkCircuit:
    """Circuit -> TensorNetworkCircuit (src/tn_conversion.jl:30-39, `_convert_to_tnc` :10-18)."""
    tnc = TensorNetworkCircuit(circ.num_qubits)
    tnc.gate_tensors = []
    for g in circ.circ_ops:
        names = tnc.push(_circ.gate_qubits(g), _circ.gate_matrix(g), decompose=decompose)
        tnc.gate_tensors.append((g, names))
    if not no_input:
        tnc.add_input(input)
    if not no_output:
        tnc.add_output(output)
    return tnc
