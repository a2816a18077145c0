"""Seeded synthetic workloads of the benchmark configurations (random grid circuits).

Each workload is a `.qx` programme built the way generate_simulation_files builds one
(src/simulation.jl:52-77: convert_to_tnc with decomposition, contraction_scheme, then
build_compute_graph) plus a seeded list of bitstrings (the `.yml` List method).  The planner
runs 8 x `time` seeded greedy trials (default time 16) and, among plans whose largest
intermediate (times the bitstring batch where it depends on the outputs) is at most 2^32
elements, keeps the one with the shortest estimated time (plan_cost: per step the longer of
FLOPs at 1e14/s and Complex64 bytes at 5e12/s).  Plans are
deterministic for (name, seed, time).  Generated programmes are cached under _build/workloads/
(the planner takes seconds to a minute).

  rqc_4x4_d10          4x4 grid, 10 cycles, unsliced, 64 bitstrings (the CPU-runnable case)
  rqc_6x6_d14_s4       6x6 grid, 14 cycles, 4 sliced bonds, 256 bitstrings (library planner)
  rqc_5x5_d12_open6    5x5 grid, 12 cycles, 6 qubits open (2^6 amplitudes per bitstring),
                       64 bitstrings of the other 19 qubits -> 4096 amplitudes (library planner)
  rqc_3x4_d8_s3        3x4 grid, 8 cycles, 3 sliced bonds, 64 bitstrings (parity size)
  rqc_6x6_d14_w28      the same circuit sliced until every intermediate has at most 2^28 elements
                       (8 bonds, 256 slices; 4 GiB per ComplexF64 intermediate instead of the
                       64 GiB of the 4-bond plan's largest), 256 bitstrings (library planner)
  rqc_7x7_d10_w22      7x7 grid, 10 cycles, sliced until every intermediate has at most 2^22
                       elements (8 slices), 1024 bitstrings (library planner): the 7x7 precision
                       case at a depth one GPU finishes; at 16 cycles every balanced split of the
                       network cuts all 49 qubit wires and no plan comes near 2^28 elements with
                       2^10 slices

Workloads marked "library planner" are planned by qxg_plan_contraction (recursive hypergraph
bisection and random-greedy trees, subtree reconfiguration, greedy slicing; `plan_time` x 8 trees)
with the bitstring batch in its step model; the others by the Python stand-in for FlowCutter.
"""
from __future__ import annotations

import hashlib
import json
from pathlib import Path

import numpy as np

from . import dsl as _dsl
from .circuits import create_parametrised_circuit, create_rqc_circuit
from .compute_graph import build_compute_graph
from .executor import Programme
from .planning import contraction_scheme, hyper_network, native_contraction_scheme, plan_cost
from .simulation import amplitudes_uniform
from .tnc import convert_to_tnc

__all__ = ["WORKLOADS", "build_workload"]

WORKLOADS = {
    "rqc_4x4_d10": dict(rows=4, cols=4, depth=10, nslice=0, open=0, nbits=64),
    "rqc_6x6_d14_s4": dict(rows=6, cols=6, depth=14, nslice=4, open=0, nbits=256, planner="native"),
    # library planner, plan seed 18, 32 trees: 675k amplitudes/s on a GB300 against 524k for the
    # fastest plan of a seed search with the Python stand-in
    "rqc_5x5_d12_open6": dict(rows=5, cols=5, depth=12, nslice=0, open=6, nbits=64, plan_time=4, plan_seed=18,
                              planner="native"),
    "rqc_3x4_d8_s3": dict(rows=3, cols=4, depth=8, nslice=3, open=0, nbits=64),
    "rqc_6x6_d14_w28": dict(rows=6, cols=6, depth=14, nslice=4, max_log2=28, open=0, nbits=256, planner="native"),
    "rqc_7x7_d10_w22": dict(rows=7, cols=7, depth=10, nslice=0, max_log2=22, open=0, nbits=1024, planner="native"),
    # parametrised: per layer Rx(t) Rz(t) on every qubit + fSim(t, p) on one coupler pattern;
    # 840 angles; two-qubit gates kept whole so each gate is one differentiable leaf
    # library planner (2^34.9 FLOPs per bitstring against 2^37.1 for the stand-in's plan): the
    # gradient takes 3.5x the forward time against 4.5x
    "param_5x5_l12": dict(rows=5, cols=5, depth=12, nslice=0, open=0, nbits=256, parametrised=True, plan_time=4,
                          plan_seed=14, planner="native"),
}

_CACHE = Path(__file__).resolve().parent / "_build" / "workloads"
_PLANNER_VERSION = 3          # bump when the planner's choices change (invalidates the cache)
WIDTH_CAP = 32.0              # log2 elements, bitstring batch included: plans within it rank by
                              # plan_cost's estimated time


def _key(name, spec, seed, time):
    h = hashlib.sha1(json.dumps([name, spec, seed, time, _PLANNER_VERSION, WIDTH_CAP],
                                sort_keys=True).encode()).hexdigest()[:12]
    return f"{name}_{h}"


def build_workload(name: str, seed: int = 1, time: int | None = None, cache: bool = True,
                   plan_seed: int | None = None, planner: str | None = None):
    """-> (Programme, bitstrings, info dict).  Deterministic for (name, seed, time, plan seed).
    `seed` draws the circuit and the bitstrings; the planner's seed is `plan_seed`, else the
    workload's pinned "plan_seed" (the best of a seed search under plan_cost's ranking), else
    `seed`; `time` (8 x time greedy trials) defaults to the workload's "plan_time", else 16.
    `planner` ("python" or "native") overrides the workload's planner."""
    spec = dict(WORKLOADS[name])
    if plan_seed is not None:
        spec["plan_seed"] = int(plan_seed)
    if planner is not None:
        if planner not in ("python", "native"):
            raise ValueError(f"planner {planner!r}: python or native")
        spec["planner"] = planner
    if time is None:
        time = spec.get("plan_time", 16)
    key = _key(name, spec, seed, time)
    qx, npz, meta_p = (_CACHE / f"{key}.qx", _CACHE / f"{key}.npz", _CACHE / f"{key}.json")
    if cache and qx.exists() and npz.exists() and meta_p.exists():
        cmds, _ = _dsl.read_qx(str(qx))
        info = json.loads(meta_p.read_text())
        prog = Programme.from_commands(cmds, _dsl.read_data(str(npz)), info["nqubits"])
        return prog, info["bitstrings"], info
    if spec.get("parametrised"):
        circ = create_parametrised_circuit(spec["rows"], spec["cols"], spec["depth"], seed=seed)
    else:
        circ = create_rqc_circuit(spec["rows"], spec["cols"], spec["depth"], seed=seed)
    n = circ.num_qubits
    tnc = convert_to_tnc(circ, decompose=not spec.get("parametrised"), no_output=True)
    if spec["open"]:
        rng = np.random.Generator(np.random.PCG64(seed + 1000))
        open_q = sorted(int(x) + 1 for x in rng.choice(n, size=spec["open"], replace=False))
        out_q = [q for q in range(1, n + 1) if q not in open_q]
    else:
        open_q, out_q = [], list(range(1, n + 1))
    tnc.add_output_subset(out_q)
    if spec.get("planner") == "native":
        groups, plan, meta = native_contraction_scheme(tnc, num=spec["nslice"], seed=spec.get("plan_seed", seed),
                                                       max_log2=spec.get("max_log2"), trials=8 * time,
                                                       batched=tnc.output_tensors, beta=spec["nbits"])
    else:
        groups, plan, meta = contraction_scheme(tnc, spec["nslice"], seed=spec.get("plan_seed", seed), time=time,
                                                width_cap=WIDTH_CAP, batched=tnc.output_tensors, beta=spec["nbits"])
    graph = build_compute_graph(tnc, plan, groups)
    nq = len(out_q)
    prog = Programme.from_commands(graph.commands, graph.data, nq)
    bits = list(amplitudes_uniform(nq, seed, spec["nbits"]))
    net = hyper_network(tnc)
    sl = [tnc.tn.root(g[0]) for g in groups]
    pc = plan_cost(net, plan, sl, tnc.output_tensors, spec["nbits"])
    info = dict(name=name, spec=spec, seed=seed, nqubits=nq, open_qubits=open_q, bitstrings=bits,
                num_slices=prog.num_slices, plan_steps=len(plan), max_log2=pc["max_log2"],
                flops_per_slice=pc["flops"], flops_per_bitstring=pc["flops"] * prog.num_slices,
                amplitudes_per_bitstring=2 ** len(open_q), plan_seed=spec.get("plan_seed", seed),
                est_seconds_per_pass=pc["time"], max_log2_batched=pc["max_log2_batched"], metadata=meta)
    if cache:
        _CACHE.mkdir(parents=True, exist_ok=True)
        _dsl.write_qx(graph, str(qx), metadata=meta)
        _dsl.write_data(graph.data, str(npz))
        meta_p.write_text(json.dumps(info, default=str))
    return prog, bits, info
