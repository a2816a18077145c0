"""Output methods (List / Uniform / Rejection) on a stand-in executor backed by the CPU oracle:
the sampling logic is host code; the GPU executor is exercised by the GPU tests."""
import numpy as np


class OracleExecutor:
    def __init__(self, prog, oracle):
        self.prog, self.oracle = prog, oracle

    def amplitudes(self, bits):
        return self.oracle.run_programme(self.prog, list(bits), nthreads=2)


def _ghz4(q, oracle):
    tnc = q.convert_to_tnc(q.create_ghz_circuit(4), decompose=True)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    return OracleExecutor(q.compile_programme(tnc, plan), oracle)


def test_rejection_sampling_ghz(q, oracle):
    ex = _ghz4(q, oracle)
    samples, amps, stats = q.sampling.rejection_sample(ex, 4, 200, M=1e-4, seed=3, batch=64)
    assert len(samples) == 200
    assert set(samples) <= {"0000", "1111"}
    frac = samples.count("0000") / len(samples)
    assert 0.35 < frac < 0.65
    assert np.allclose(np.abs(amps), 1 / np.sqrt(2))
    assert stats["M"] >= 8.0 - 1e-9               # empirical supremum: p(x) 2^n = 0.5 * 16


def test_fixed_M_frugal_sampling_keeps_M(q, oracle):
    ex = _ghz4(q, oracle)
    _, _, stats = q.sampling.rejection_sample(ex, 4, 20, M=16.0, fix_M=True, seed=1, batch=32)
    assert stats["M"] == 16.0 and stats["accepted"] == 20


def test_output_methods_dispatch(q, oracle):
    ex = _ghz4(q, oracle)
    p = q.output_params_dict(4, 3, bitstrings=["0000", "1111", "0101"])
    bits, amps = q.sampling.run_output_method(ex, p, 4)
    assert bits == ["0000", "1111", "0101"] and abs(amps[2]) < 1e-15
    p = q.output_params_dict(4, 5, output_method="Uniform", seed=2)
    bits, amps = q.sampling.run_output_method(ex, p, 4)
    assert len(bits) == 5 and len(amps) == 5
    p = q.output_params_dict(4, 6, output_method="Rejection", seed=2)
    bits, _ = q.sampling.run_output_method(ex, p, 4)
    assert len(bits) == 6 and set(bits) <= {"0000", "1111"}
