"""Parity at the benchmark configurations' own sizes.

* The 6x6, 14-cycle circuit planned to keep every intermediate within 2^28 elements (256 slices,
  intermediates of 2 GiB in Complex64 and 4 GiB in ComplexF64): the plain FP64 executor on slice 0
  for four bitstrings against the reference's CPU arithmetic (oracle/blas_walk.py: permute +
  zgemm per ncon) on the same slice, within 1e-12 per amplitude.
* The 7x7, 10-cycle benchmark workload (8 slices): FP64 over all slices for four bitstrings
  against the same CPU walk, within 1e-12 per amplitude.
* The 5x5, 12-cycle batching workload (6 open qubits, 2^6 amplitudes per bitstring): the 3xTF32
  executor against the FP64 executor on eight bitstrings, within 1e-5 of the largest amplitude,
  with its per-amplitude error reported.

Per-amplitude tolerance as in test_gpu_parity.py: relative to each amplitude, with amplitudes
below 1e-6 of the largest compared at that floor.
"""
import numpy as np
import pytest

from test_gpu_parity import FP64_TOL, rel_err

pytestmark = pytest.mark.gpu


def test_6x6_d14_sliced_fp64_slice_against_cpu_walk(q, gpu_lib, oracle):
    from oracle import blas_walk
    prog, bits, info = q.workloads.build_workload("rqc_6x6_d14_w28")
    assert info["num_slices"] >= 256 and info["max_log2"] <= 28
    sub = bits[:4]
    with q.Executor(prog, precision="fp64") as ex:
        got = ex.amplitudes(sub, slices=(0, 1))[:, 0]
    ref = blas_walk.run_programme(prog, sub, slices=(0, 1))[:, 0]
    assert rel_err(got, ref) <= FP64_TOL


def test_7x7_d10_fp64_against_cpu_walk(q, gpu_lib, oracle):
    from oracle import blas_walk
    prog, bits, info = q.workloads.build_workload("rqc_7x7_d10_w22")
    sub = bits[:4]
    with q.Executor(prog, precision="fp64") as ex:
        got = ex.amplitudes(sub)[:, 0]
    ref = blas_walk.run_programme(prog, sub)[:, 0]
    assert rel_err(got, ref) <= FP64_TOL


def test_5x5_d12_open6_split_tf32_against_fp64(q, gpu_lib):
    prog, bits, info = q.workloads.build_workload("rqc_5x5_d12_open6")
    sub = bits[:8]
    with q.Executor(prog, precision="fp64") as ex:
        ref = ex.amplitudes(sub)
    with q.Executor(prog, precision="split_tf32") as ex:
        got = ex.amplitudes(sub)
    assert got.shape == (8, 64)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    per_amp = np.abs(got - ref) / np.abs(ref)
    print(f"3xTF32 vs FP64: max {err:.2e} of the largest amplitude; per amplitude median "
          f"{np.median(per_amp):.2e}, max {per_amp.max():.2e}")
    assert err <= 1e-5
    assert np.median(per_amp) <= 1e-5
