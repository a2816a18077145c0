"""Simulation API (mirror of src/simulation.jl and src/outputs.jl), executed on the GPU.

  - `amplitudes_all(n)` (simulation.jl:14-16), `amplitudes_uniform(n, seed, k)` (:24-28; seeded
    with numpy's PCG64 instead of Julia's MersenneTwister, so the draws differ from Julia's);
  - `single_amplitude(tnc, plan, bitstring)` (:86-91): the reference copies the network, binds
    the output tensors to the bitstring and contracts along the plan on the CPU.  Here the
    network and plan are compiled once into a `.qx` programme (build_compute_graph) whose output
    tensors are `output` commands, and each call runs that programme on the GPU in ComplexF64;
  - `run_simulation(circ; num_amplitudes, seed)` (:102-133);
  - `generate_simulation_files(circ, prefix, nslice; ...)` (:52-77) writing `.qx`, leaf data
    (`.npz` with `data_<k>` keys in place of `.jld2`) and `.yml`;
  - `generate_parameter_file` (:149-155) and `output_params_dict` (src/outputs.jl:47-78);
  - `execute(dsl, input, param, output; max_amplitudes, max_slices)`: the call qxrun.jl makes
    into QXContexts (bin/qxrun.jl:83-87) for the `List` output method, on the GPU.
"""
from __future__ import annotations

import itertools
import math
from collections import OrderedDict

import numpy as np

from . import dsl as _dsl
from .compute_graph import build_compute_graph
from .executor import Executor, Programme
from .planning import contraction_scheme, flow_cutter_contraction_plan
from .tnc import convert_to_tnc

__all__ = ["amplitudes_all", "amplitudes_uniform", "single_amplitude", "run_simulation",
           "generate_simulation_files", "generate_parameter_file", "output_params_dict",
           "execute", "compile_programme"]


def amplitudes_all(qubits: int):
    """All 2^n bitstrings in counting order, most significant bit first, like the reference's
    `bitstring(x-1)[end-n+1:end]`."""
    return (format(x, f"0{qubits}b") if qubits else "" for x in range(2 ** qubits))


def amplitudes_uniform(qubits: int, seed, number_amplitudes: int):
    """`number_amplitudes` uniformly random bitstrings (with replacement), seeded."""
    rng = np.random.Generator(np.random.PCG64(0 if seed is None else int(seed)))

    def gen():
        for _ in range(number_amplitudes):
            bits = rng.integers(0, 2, size=qubits)
            yield "".join("01"[b] for b in bits)
    return gen()


def compile_programme(tnc, plan, bond_groups=None) -> Programme:
    """`.qx` programme of `tnc` along `plan` with output tensors as `output` commands."""
    net = tnc
    if not tnc.output_tensors:
        net = tnc.copy()
        net.add_output()
    graph = build_compute_graph(net, plan, bond_groups)
    return Programme.from_graph(graph)


def _cached_executor(tnc, plan, precision="fp64") -> Executor:
    cache = tnc.__dict__.setdefault("_qxg_cache", {})
    key = (tuple(tuple(p) for p in plan), precision)
    if key not in cache:
        cache[key] = Executor(compile_programme(tnc, plan), precision=precision)
    return cache[key]


def single_amplitude(tnc, plan, amplitude=None, precision: str = "fp64") -> complex:
    """Amplitude <amplitude|C|input> of the network along `plan` (simulation.jl:86-91).
    `amplitude=None` -> all zeros, like `add_output!(tnc, nothing)`."""
    if amplitude is None:
        amplitude = "0" * tnc.qubits
    ex = _cached_executor(tnc, plan, precision)
    return complex(ex.amplitudes([amplitude])[0, 0])


def run_simulation(circ, num_amplitudes=None, seed=None, precision: str = "fp64") -> "OrderedDict[str, complex]":
    """Amplitudes of all bitstrings (<= 30 qubits) or `num_amplitudes` random ones
    (simulation.jl:102-133); all bitstrings go to the GPU in one call."""
    tnc = convert_to_tnc(circ)
    plan = flow_cutter_contraction_plan(tnc, hypergraph=True, time=1)
    if num_amplitudes is None and tnc.qubits > 30:
        num_amplitudes = 1000
    if num_amplitudes is None:
        bits = list(amplitudes_all(tnc.qubits))
    else:
        bits = list(amplitudes_uniform(tnc.qubits, seed, num_amplitudes))
    bits = list(OrderedDict.fromkeys(bits))
    ex = _cached_executor(tnc, plan, precision)
    amps = ex.amplitudes(bits)[:, 0]
    return OrderedDict((b, complex(a)) for b, a in zip(bits, amps))


def output_params_dict(num_qubits: int, num_outputs: int = 10, output_method: str = "List", seed=None,
                       M: float = 0.0001, fix_M: bool = False, bitstrings=None) -> "OrderedDict":
    """`output:` block parameters (src/outputs.jl:47-78)."""
    out = OrderedDict()
    out["method"] = output_method
    params = OrderedDict()
    if output_method == "Rejection":
        params["num_qubits"] = num_qubits
        params["M"] = M
        params["fix_M"] = fix_M
        params["seed"] = seed
        params["num_samples"] = num_outputs
    elif output_method == "List":
        if bitstrings is None:
            bitstrings = list(amplitudes_uniform(num_qubits, seed, num_outputs))
        else:
            num_outputs = len(bitstrings)
        params["num_samples"] = num_outputs
        params["bitstrings"] = list(bitstrings)
    elif output_method == "Uniform":
        params["num_qubits"] = num_qubits
        params["num_samples"] = num_outputs
        params["seed"] = seed
    else:
        raise ValueError(f'Output method "{output_method}" not supported')
    out["params"] = params
    return out


def generate_parameter_file(filename_prefix: str, output_parameters):
    _dsl.write_yml(OrderedDict([("output", output_parameters)]), f"{filename_prefix}.yml")


def generate_simulation_files(circ, output_prefix: str = "simulation_input", number_bonds_to_slice: int = 2,
                              decompose: bool = True, seed=None, output_args=None, time: int = 1,
                              hypergraph: bool = True, score_function: str = "tree_trimming",
                              max_log2=None):
    """Write `<prefix>.qx`, `<prefix>.npz` (leaf data) and `<prefix>.yml` (simulation.jl:52-77)."""
    tnc = convert_to_tnc(circ, decompose=decompose)
    fc_seed = -1 if seed is None else seed
    groups, plan, meta = contraction_scheme(tnc, number_bonds_to_slice, seed=fc_seed, time=time,
                                            hypergraph=hypergraph, score_function=score_function,
                                            max_log2=max_log2)
    graph = build_compute_graph(tnc, plan, groups)
    _dsl.write_qx(graph, f"{output_prefix}.qx", metadata=meta)
    _dsl.write_data(graph.data, f"{output_prefix}.npz")
    if output_args is None:
        output_args = output_params_dict(tnc.qubits)
    generate_parameter_file(output_prefix, output_args)
    return graph


def load_programme(dsl_file: str, input_file: str | None = None) -> Programme:
    """Programme from `.qx` text and its leaf data file."""
    commands, _ = _dsl.read_qx(dsl_file)
    if input_file is None:
        input_file = dsl_file[:-3] + ".npz" if dsl_file.endswith(".qx") else dsl_file + ".npz"
    data = _dsl.read_data(input_file)
    from .compute_graph import Output
    nq = max([c.qubit for c in commands if isinstance(c, Output)], default=0)
    return Programme.from_commands(commands, data, nq)


def execute(dsl_file: str, input_file=None, param_file=None, output_file=None, max_amplitudes=None,
            max_slices=None, precision: str = "fp64", nqubits=None) -> "OrderedDict[str, np.ndarray]":
    """Run a `.qx` programme for the `.yml` List bitstrings (QXContexts.execute as called by
    bin/qxrun.jl:83-87): `max_amplitudes` / `max_slices` truncate the bitstring list and the
    slice range like qxrun's `--number-amplitudes` / `--number-slices`."""
    prog = load_programme(dsl_file, input_file)
    if nqubits is not None:
        prog.nqubits = nqubits
    if param_file is None:
        param_file = dsl_file[:-3] + ".yml" if dsl_file.endswith(".qx") else dsl_file + ".yml"
    params = _dsl.read_yml(param_file)["output"]
    if params["method"] != "List":
        raise NotImplementedError(f"output method {params['method']} (only List runs on the GPU executor)")
    bits = list(params["params"]["bitstrings"])
    if max_amplitudes is not None:
        bits = bits[:max_amplitudes]
    if bits and prog.nqubits < len(bits[0]):
        prog.nqubits = len(bits[0])
    ex = Executor(prog, precision=precision)
    ns = ex.num_slices
    s1 = ns if max_slices is None else min(ns, max_slices)
    res = ex.amplitudes(bits, slices=(0, s1))
    out = OrderedDict((b, r if r.size > 1 else complex(r[0])) for b, r in zip(bits, res))
    if output_file:
        np.savez(output_file, bitstrings=np.array(bits), amplitudes=res)
    ex.close()
    return out
