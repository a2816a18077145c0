"""The library's host-side producers of the path, run on the device.

* A `.qx` text read by the library's own parser (qxg_parse_qx, through Programme.from_qx_text)
  runs on the GPU and matches the oracle on the programme built directly from the command list.
* A plan from the library's planner (qxg_plan_contraction, through native_contraction_scheme),
  sliced, runs on the GPU and matches the oracle.
* The Rejection output method (src/outputs.jl:57-62) draws its candidates' amplitudes from the GPU
  executor in batches: the accepted samples' amplitudes are the oracle's, and the samples follow
  |amplitude|^2 (their mean of 2^n |a|^2 is near 2, the Porter-Thomas value, against 1 for
  uniform draws).

Tolerances as in test_gpu_parity.py: FP64 <= 1e-12 per amplitude (below 1e-6 of the largest
amplitude, 1e-12 of the largest absolutely).
"""
import numpy as np
import pytest

from test_gpu_parity import FP64_TOL, rel_err

pytestmark = pytest.mark.gpu


def _rqc_graph(q, rows, cols, depth, seed, nslice):
    circ = q.create_rqc_circuit(rows, cols, depth, seed=seed)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, _ = q.contraction_scheme(tnc, nslice, seed=seed, time=1)
    return q.build_compute_graph(tnc, plan, groups)


@pytest.mark.parametrize("precision", ["fp64", "split_tf32"])
def test_programme_parsed_by_the_library_runs_on_gpu(q, gpu_lib, oracle, precision):
    graph = _rqc_graph(q, 3, 4, 8, seed=3, nslice=2)
    direct = q.Programme.from_graph(graph)
    text = q.dsl.format_qx(graph)
    parsed = q.Programme.from_qx_text(text, graph.data)
    assert parsed.nqubits == direct.nqubits and parsed.num_slices == direct.num_slices == 4
    bits = list(q.amplitudes_uniform(12, 4, 24))
    with q.Executor(parsed, precision=precision) as ex:
        got = ex.amplitudes(bits)[:, 0]
    ref = oracle.run_programme(direct, bits, nthreads=8)[:, 0]
    if precision == "fp64":
        assert rel_err(got, ref) <= FP64_TOL
    else:
        assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= 1e-5


def test_plan_from_the_library_planner_runs_on_gpu(q, gpu_lib, oracle):
    circ = q.create_rqc_circuit(4, 4, 8, seed=5)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, meta = q.native_contraction_scheme(tnc, num=2, seed=2, trials=16, greedy_trials=4)
    assert len(groups) == 2 and len(plan) == len(tnc.tn.tensors) - 1
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))
    assert prog.num_slices >= 4
    bits = list(q.amplitudes_uniform(16, 6, 32))
    with q.Executor(prog) as ex:
        got = ex.amplitudes(bits)[:, 0]
    ref = oracle.run_programme(prog, bits, nthreads=8)[:, 0]
    assert rel_err(got, ref) <= FP64_TOL


def test_rejection_sampling_over_gpu_amplitude_batches(q, gpu_lib, oracle):
    graph = _rqc_graph(q, 3, 3, 8, seed=7, nslice=0)
    prog = q.Programme.from_graph(graph)
    n = 9
    with q.Executor(prog) as ex:
        samples, amps, stats = q.sampling.rejection_sample(ex, n, 600, seed=11, batch=128)
    assert len(samples) == 600 and stats["accepted"] == 600
    assert stats["M"] > 1.0                     # empirical supremum of 2^n p(x)
    ref = oracle.run_programme(prog, samples[:64], nthreads=8)[:, 0]
    assert rel_err(amps[:64], ref) <= FP64_TOL
    # samples follow p(x) = |a|^2: E_p[2^n p(x)] = 2^n sum p^2, which is ~2 for this circuit,
    # while bitstrings drawn uniformly average 1
    all_bits = [format(i, f"0{n}b") for i in range(2 ** n)]
    p_all = np.abs(oracle.run_programme(prog, all_bits, nthreads=8)[:, 0]) ** 2
    expected = 2 ** n * float(np.sum(p_all ** 2))
    got = 2 ** n * float(np.mean(np.abs(amps) ** 2))
    assert abs(np.sum(p_all) - 1.0) < 1e-10
    assert abs(got - expected) < 0.25 * expected, (got, expected)
    assert got > 1.4
