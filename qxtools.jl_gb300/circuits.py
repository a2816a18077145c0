"""Circuits: gate matrices and circuit builders (mirror of src/circuits/circuits.jl).

The reference wraps QXZoo (un-vendored): `create_test_circuit` (circuits.jl:17-23),
`create_ghz_circuit` (:30-37), `create_qft_circuit` (:44-50), `create_rqc_circuit` (:61-67,
QXZoo.RQC.create_RQC), `gate_matrix` (:74-76, ComplexF64 matrix) and `gate_qubits` (:83-90,
`[target, ctrl]` for two-qubit gates).  QXZoo is not available, so the random circuit here
is this package's own seeded generator of the family the benchmark configurations name:
per cycle one single-qubit gate per qubit drawn uniformly from {sqrt(X), sqrt(Y), sqrt(W)}
without repeating the qubit's previous draw, then fSim(theta, phi) on one of four
nearest-neighbour coupler patterns, cycling A B C D C D A B.  Its amplitudes are not
comparable with QXZoo's `create_RQC` output (parity with that generator is unpinned).

Qubits are numbered from 1 like the reference.  For a gate on qubits [q1, q2] the matrix
row/column index is bit(q1) + 2*bit(q2) (Julia column-major reshape), so the first listed
qubit is the fastest index; for CX that is the target, as in the reference's
docs/src/basics.md:38-45.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "Gate", "Circuit", "gates",
    "create_test_circuit", "create_ghz_circuit", "create_qft_circuit", "create_rqc_circuit",
    "create_parametrised_circuit", "gate_matrix", "gate_qubits",
]

_S2 = 1.0 / math.sqrt(2.0)


def _sqrt_involution(g: np.ndarray) -> np.ndarray:
    """Principal square root of a Hermitian involution G (G^2 = I): (I+G)/2 + i(I-G)/2."""
    i2 = np.eye(2, dtype=np.complex128)
    return (i2 + g) / 2 + 1j * (i2 - g) / 2


class gates:
    """Gate matrices (ComplexF64, row = output basis state, column = input)."""
    I = np.eye(2, dtype=np.complex128)
    X = np.array([[0, 1], [1, 0]], dtype=np.complex128)
    Y = np.array([[0, -1j], [1j, 0]], dtype=np.complex128)
    Z = np.array([[1, 0], [0, -1]], dtype=np.complex128)
    H = np.array([[1, 1], [1, -1]], dtype=np.complex128) * _S2
    W = (X + Y) * _S2
    SX = _sqrt_involution(X)
    SY = _sqrt_involution(Y)
    SW = _sqrt_involution(W)
    # two-qubit gates, index bit(q1) + 2*bit(q2); CX/CZ listed as [target, control]
    CX = np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 0, 1], [0, 0, 1, 0]],
                  dtype=np.complex128).T
    CZ = np.diag([1, 1, 1, -1]).astype(np.complex128)

    @staticmethod
    def rz(theta: float) -> np.ndarray:
        return np.diag([np.exp(-0.5j * theta), np.exp(0.5j * theta)]).astype(np.complex128)

    @staticmethod
    def rx(theta: float) -> np.ndarray:
        c, s = math.cos(theta / 2), math.sin(theta / 2)
        return np.array([[c, -1j * s], [-1j * s, c]], dtype=np.complex128)

    @staticmethod
    def fsim(theta: float, phi: float) -> np.ndarray:
        c, s = math.cos(theta), math.sin(theta)
        return np.array([[1, 0, 0, 0],
                         [0, c, -1j * s, 0],
                         [0, -1j * s, c, 0],
                         [0, 0, 0, np.exp(-1j * phi)]], dtype=np.complex128)

    @staticmethod
    def cphase(phi: float) -> np.ndarray:
        return np.diag([1, 1, 1, np.exp(1j * phi)]).astype(np.complex128)


@dataclass
class Gate:
    """One gate call: name, qubits (1-based; [target, ctrl] for controlled gates), matrix.

    `params` carries the angles of parametrised gates (Rz, Rx, fSim) so gradients can be
    chained to them; `param_ids` names the circuit parameter each angle comes from."""
    name: str
    qubits: list
    matrix: np.ndarray
    params: tuple = ()
    param_ids: tuple = ()


@dataclass
class Circuit:
    """Mirror of the fields the reference reads from a QXZoo `Circ`: `num_qubits` and
    `circ_ops` (docs/src/circuits.md:16-24)."""
    num_qubits: int
    circ_ops: list = field(default_factory=list)
    num_params: int = 0

    def add(self, name, qubits, matrix, params=(), param_ids=()):
        for q in qubits:
            if not 1 <= q <= self.num_qubits:
                raise ValueError(f"qubit {q} out of range 1..{self.num_qubits}")
        self.circ_ops.append(Gate(name, list(qubits), np.asarray(matrix, dtype=np.complex128),
                                  tuple(params), tuple(param_ids)))
        return self


def gate_matrix(gate: Gate) -> np.ndarray:
    """ComplexF64 matrix of a gate (circuits.jl:74-76)."""
    return np.asarray(gate.matrix, dtype=np.complex128)


def gate_qubits(gate: Gate) -> list:
    """Qubits a gate acts on, `[target, ctrl]` for two-qubit gates (circuits.jl:83-90)."""
    return list(gate.qubits)


def create_test_circuit() -> Circuit:
    """3-qubit GHZ preparation: H on 1, CX 1->2, CX 2->3 (circuits.jl:17-23)."""
    return create_ghz_circuit(3)


def create_ghz_circuit(n: int) -> Circuit:
    """n-qubit GHZ preparation (circuits.jl:30-37)."""
    c = Circuit(n)
    c.add("h", [1], gates.H)
    for i in range(1, n):
        c.add("cx", [i + 1, i], gates.CX)       # [target, control]
    return c


def create_qft_circuit(n: int) -> Circuit:
    """Quantum Fourier transform on n qubits followed by CX(1,2), CX(2,3) like circuits.jl:44-50.

    Textbook QFT: H then controlled phases 2*pi/2^k, no final swaps."""
    c = Circuit(n)
    for j in range(1, n + 1):
        c.add("h", [j], gates.H)
        for k in range(j + 1, n + 1):
            c.add("cphase", [j, k], gates.cphase(2 * math.pi / 2 ** (k - j + 1)))
    if n >= 2:
        c.add("cx", [2, 1], gates.CX)
    if n >= 3:
        c.add("cx", [3, 2], gates.CX)
    return c


def _coupler_patterns(rows: int, cols: int) -> dict:
    """Four nearest-neighbour coupler patterns of a rows x cols grid; qubit (r, c) -> r*cols+c+1.

    A: horizontal pairs starting at an even column, B: horizontal at odd column,
    C: vertical pairs starting at an even row, D: vertical at odd row."""
    q = lambda r, c: r * cols + c + 1
    pats = {k: [] for k in "ABCD"}
    for r in range(rows):
        for c in range(cols - 1):
            pats["A" if c % 2 == 0 else "B"].append((q(r, c), q(r, c + 1)))
    for r in range(rows - 1):
        for c in range(cols):
            pats["C" if r % 2 == 0 else "D"].append((q(r, c), q(r + 1, c)))
    return pats


RQC_PATTERN_ORDER = "ABCDCDAB"


def create_rqc_circuit(rows: int, cols: int, depth: int, seed=None, *, final_h: bool = False,
                       theta: float = math.pi / 2, phi: float = math.pi / 6) -> Circuit:
    """Seeded random quantum circuit on a rows x cols grid (stand-in for circuits.jl:61-67).

    Each of `depth` cycles: a single-qubit gate on every qubit, uniform over
    {sqrt(X), sqrt(Y), sqrt(W)} with no repeat of the qubit's previous gate, then
    fSim(theta, phi) on the couplers of pattern ABCDCDAB[cycle % 8].  `final_h` appends a
    Hadamard layer.  Seeded with numpy's PCG64 (`seed=None` -> 0)."""
    rng = np.random.Generator(np.random.PCG64(0 if seed is None else int(seed)))
    n = rows * cols
    c = Circuit(n)
    one_q = [("sx", gates.SX), ("sy", gates.SY), ("sw", gates.SW)]
    prev = [-1] * n
    pats = _coupler_patterns(rows, cols)
    fs = gates.fsim(theta, phi)
    for cyc in range(depth):
        for qi in range(n):
            choices = [k for k in range(3) if k != prev[qi]]
            k = choices[int(rng.integers(len(choices)))]
            prev[qi] = k
            c.add(one_q[k][0], [qi + 1], one_q[k][1])
        for (a, b) in pats[RQC_PATTERN_ORDER[cyc % len(RQC_PATTERN_ORDER)]]:
            c.add("fsim", [a, b], fs, params=(theta, phi))
    if final_h:
        for qi in range(n):
            c.add("h", [qi + 1], gates.H)
    return c


def create_parametrised_circuit(rows: int, cols: int, layers: int, seed=None) -> Circuit:
    """Parametrised grid circuit: per layer Rz(t)*Rx(t) on every qubit, then fSim(t, p) on
    the couplers of pattern ABCDCDAB[layer % 8].  Every angle is its own parameter, drawn
    uniformly from [0, 2*pi) with numpy's PCG64(seed)."""
    rng = np.random.Generator(np.random.PCG64(0 if seed is None else int(seed)))
    n = rows * cols
    c = Circuit(n)
    pats = _coupler_patterns(rows, cols)
    pid = 0
    angles = []
    for layer in range(layers):
        for qi in range(n):
            tx = float(rng.uniform(0, 2 * math.pi)); angles.append(tx)
            c.add("rx", [qi + 1], gates.rx(tx), params=(tx,), param_ids=(pid,)); pid += 1
            tz = float(rng.uniform(0, 2 * math.pi)); angles.append(tz)
            c.add("rz", [qi + 1], gates.rz(tz), params=(tz,), param_ids=(pid,)); pid += 1
        for (a, b) in pats[RQC_PATTERN_ORDER[layer % len(RQC_PATTERN_ORDER)]]:
            th = float(rng.uniform(0, 2 * math.pi)); ph = float(rng.uniform(0, 2 * math.pi))
            angles += [th, ph]
            c.add("fsim", [a, b], gates.fsim(th, ph), params=(th, ph), param_ids=(pid, pid + 1))
            pid += 2
    c.num_params = pid
    c.angles = np.array(angles)
    return c
