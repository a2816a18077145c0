"""Gradients of amplitude losses with respect to gate angles.

The executor's reverse-mode pass (qxg_gradient) returns dL/d conj(T) for every leaf tensor T of the
programme.  For a real loss and a gate tensor T(theta):

    dL/dtheta = 2 Re sum_elements conj(dL/d conj T) * dT/dtheta

with dT/dtheta the analytic derivative of the gate matrix, reshaped and reduced over tied
(hyperindex) groups exactly like the leaf data itself.  Parametrised two-qubit gates are kept
whole (decompose=False) so their leaf is the gate matrix itself.
"""
from __future__ import annotations

import math

import numpy as np

from .compute_graph import build_compute_graph
from .executor import Executor, Programme
from .planning import contraction_scheme, native_contraction_scheme
from .tnc import convert_to_tnc

__all__ = ["gate_derivatives", "ParametrisedCircuitLoss"]


def gate_derivatives(gate) -> list:
    """Analytic derivatives dM/dtheta of a parametrised gate matrix, one per parameter."""
    name = gate.name
    if name == "rz":
        (t,) = gate.params
        return [np.diag([-0.5j * np.exp(-0.5j * t), 0.5j * np.exp(0.5j * t)]).astype(np.complex128)]
    if name == "rx":
        (t,) = gate.params
        c, s = math.cos(t / 2), math.sin(t / 2)
        return [np.array([[-s / 2, -0.5j * c], [-0.5j * c, -s / 2]], dtype=np.complex128)]
    if name == "fsim":
        t, p = gate.params
        c, s = math.cos(t), math.sin(t)
        dt = np.array([[0, 0, 0, 0], [0, -s, -1j * c, 0], [0, -1j * c, -s, 0], [0, 0, 0, 0]], dtype=np.complex128)
        dp = np.zeros((4, 4), dtype=np.complex128)
        dp[3, 3] = -1j * np.exp(-1j * p)
        return [dt, dp]
    raise ValueError(f"no derivative for gate {name!r}")


def chain_rule_tables(terms, layout):
    """Index tables of the chain rule to the parameters: for terms (parameter id, load instruction,
    dT/dtheta as an array of the leaf's shape) and the gradient vector's layout (instruction ->
    (offset, shape), `Executor.leaf_slices`), element e of the concatenation is entry idx[e] of the
    flat gradient vector times dt[e] (column-major, as the leaves are laid out), added into
    parameter pid[e].  Returns (idx, dt, pid)."""
    idx, dtv, pid = [], [], []
    for p, instr, dt in terms:
        o, shape = layout[instr]
        n = int(np.prod(shape)) if shape else 1
        idx.append(np.arange(o, o + n))
        dtv.append(np.asarray(dt, dtype=np.complex128).reshape(-1, order="F"))
        pid.append(np.full(n, p))
    if not idx:
        return np.zeros(0, dtype=np.int64), np.zeros(0, dtype=np.complex128), np.zeros(0, dtype=np.int64)
    return np.concatenate(idx), np.concatenate(dtv), np.concatenate(pid)


def apply_chain_rule(gvec, tables, num_params):
    """dL/dtheta = 2 Re sum conj(dL/d conj T) dT/dtheta for every parameter, from the flat leaf
    gradient vector and chain_rule_tables."""
    idx, dt, pid = tables
    w = 2.0 * np.real(np.conj(gvec[idx]) * dt)
    return np.bincount(pid, weights=w, minlength=num_params)[:num_params]


class ParametrisedCircuitLoss:
    """L(theta) = sum over bitstrings of |<x|C(theta)|0>|^2 and dL/dtheta on the GPU.

    The circuit is converted without decomposition, planned (with `nslice` sliced bonds; by the
    Python stand-in for FlowCutter, or by the library's planner with planner="native") and compiled
    once; each evaluation runs one reverse-mode pass per (slice batch, bitstring batch)."""

    def __init__(self, circ, nslice: int = 0, seed: int = 1, time: int = 1, precision: str = "fp64",
                 width_cap: float | None = None, beta: int = 1, planner: str = "python", **opts):
        self.circ = circ
        self.tnc = convert_to_tnc(circ, decompose=False)
        if planner == "native":
            groups, plan, _ = native_contraction_scheme(self.tnc, num=nslice, seed=seed, trials=8 * time,
                                                        batched=self.tnc.output_tensors, beta=beta)
        elif planner == "python":
            groups, plan, _ = contraction_scheme(self.tnc, nslice, seed=seed, time=time, width_cap=width_cap,
                                                 batched=self.tnc.output_tensors, beta=beta)
        else:
            raise ValueError(f"planner {planner!r}: python or native")
        self.graph = build_compute_graph(self.tnc, plan, groups)
        self.programme = Programme.from_graph(self.graph)
        self.executor = Executor(self.programme, precision=precision, **opts)
        load_instr = {}
        for i, r in enumerate(self.programme.instrs):
            if int(r[0]) == 1:
                load_instr[int(r[1])] = i
        # (parameter id, load instruction, reduced dT/dtheta) for every parametrised gate
        self.terms = []
        for gate, names in self.tnc.gate_tensors:
            if not gate.param_ids:
                continue
            if len(names) != 1:
                raise ValueError("parametrised gates must not be decomposed")
            name = names[0]
            instr = load_instr[self.programme.tensor_ids[name]]
            shape = self.tnc.tn.tensors[name].data.shape
            for pid, dm in zip(gate.param_ids, gate_derivatives(gate)):
                full = dm.reshape(shape, order="F")
                self.terms.append((pid, instr, self.tnc.tn.reduced_data(name, full)))
        self.num_params = circ.num_params
        # the chain rule as one gather over the flat gradient vector
        self._chain = chain_rule_tables(self.terms, self.executor.leaf_slices())

    def loss_and_grad(self, bitstrings, slices=None):
        amps, gvec = self.executor.gradient(bitstrings, slices=slices, flat=True)
        loss = float(np.sum(np.abs(amps) ** 2))
        # L = sum |a|^2 with amp_bar = a; dL/dtheta = 2 Re sum conj(dL/d conj T) dT/dtheta
        return loss, apply_chain_rule(gvec, self._chain, self.num_params), amps

    def loss(self, bitstrings) -> float:
        return float(np.sum(np.abs(self.executor.amplitudes(bitstrings)) ** 2))

    def close(self):
        self.executor.close()
