"""GB300-native executor for QXTools' contraction hot path (host-side mirror of the Julia API).

The directory name is not a Python identifier; it is loaded as the package `qxtools_gb300`
(see `load()` in __graft_entry__.py at the repository root).  The compute path is the C-ABI
library `_build/libqxgpu.so` (include/qxgpu.h); this package builds programmes for it and mirrors
the reference's API: convert_to_tnc, flow_cutter_contraction_plan, contraction_scheme,
build_compute_graph, single_amplitude, run_simulation, generate_simulation_files.
"""
from . import circuits, compute_graph, dsl, planning, tnc
from .circuits import (Circuit, Gate, create_ghz_circuit, create_parametrised_circuit,
                       create_qft_circuit, create_rqc_circuit, create_test_circuit, gate_matrix,
                       gate_qubits, gates)
from .compute_graph import (ComputeGraph, Load, Ncon, Output, Save, TensorCache, View,
                            build_compute_graph)
from .executor import Executor, Programme, QXGError, load_library, ncon_device
from .planning import (HyperNet, contraction_indices, contraction_scheme, convert_to_graph,
                       convert_to_line_graph, flow_cutter_contraction_plan,
                       greedy_contraction_plan, hyper_network, min_fill,
                       min_fill_contraction_plan, native_contraction_scheme, native_plan, netcon,
                       order_to_contraction_plan, plan_cost)
from .simulation import (amplitudes_all, amplitudes_uniform, compile_programme, execute,
                         generate_parameter_file, generate_simulation_files, output_params_dict,
                         run_simulation, single_amplitude)
from .tnc import TensorNetwork, TensorNetworkCircuit, basis_vector, convert_to_tnc
from . import gradients, replicas, sampling, simulation, workloads

__version__ = "0.1.0"
