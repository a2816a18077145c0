"""The BLAS walk (oracle/blas_walk.py, the timed CPU baseline: permute + zgemm per ncon, as
TensorOperations contracts) pinned against the reference's golden vectors and the C oracle."""
import math

import numpy as np
import pytest

from test_oracle_golden import golden, users_guide_programme


@pytest.fixture(scope="module")
def bw():
    from oracle import blas_walk
    return blas_walk


def test_users_guide_example_golden(q, bw):
    prog, g = users_guide_programme(q)
    for bits, (re, im) in g["amplitudes"].items():
        got = bw.run_programme(prog, [bits])[0, 0]
        assert abs(got - complex(re, im)) < 1e-14, bits
    # slice 1 (v1 = 1, v2 = 0, first variable fastest) alone carries "11"
    assert abs(bw.run_programme(prog, ["11"], slices=(1, 2))[0, 0] - 1 / math.sqrt(2)) < 1e-15


def test_ghz5_all_amplitudes_golden(q, bw):
    g = golden()["ghz5"]
    circ = q.create_ghz_circuit(g["n"])
    tnc = q.convert_to_tnc(circ, decompose=True)
    prog = q.compile_programme(tnc, q.flow_cutter_contraction_plan(tnc, time=1))
    amps = bw.run_programme(prog, list(q.amplitudes_all(g["n"])))[:, 0]
    assert abs(amps[0] - g["value"]) < 1e-14 and abs(amps[-1] - g["value"]) < 1e-14
    assert np.allclose(amps[1:-1], 0, atol=1e-15)


def test_ghz3_state_vector_golden(q, bw):
    g = golden()["ghz3_state"]
    circ = q.create_test_circuit()
    tnc = q.convert_to_tnc(circ, no_output=True, decompose=True)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, q.netcon(tnc)))
    out = bw.run_programme(prog, [""])[0]
    assert out.shape == (8,)
    assert abs(out[0] - g["value"]) < 1e-14 and abs(out[7] - g["value"]) < 1e-14
    assert np.allclose(out[1:7], 0, atol=1e-15)


@pytest.mark.parametrize("decompose,nslice", [(False, 0), (True, 0), (True, 3)])
def test_matches_c_oracle_rqc(q, oracle, bw, decompose, nslice):
    circ = q.create_rqc_circuit(3, 3, 6, seed=13)
    tnc = q.convert_to_tnc(circ, decompose=decompose)
    if nslice:
        groups, plan, _ = q.contraction_scheme(tnc, nslice, seed=4, time=1)
        prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))
        assert prog.num_slices == 2 ** nslice
    else:
        prog = q.compile_programme(tnc, q.flow_cutter_contraction_plan(tnc, time=1))
    bits = list(q.amplitudes_uniform(9, 7, 6)) + ["+-01+-01+"]
    ref = oracle.run_programme(prog, bits)[:, 0]
    got = bw.run_programme(prog, bits)[:, 0]
    assert np.max(np.abs(got - ref)) < 1e-14


def test_open_qubits_batch_matches_c_oracle(q, oracle, bw):
    """Output tensor of 2^3 amplitudes (three qubits left open), as the batching workloads."""
    circ = q.create_rqc_circuit(3, 3, 5, seed=21)
    tnc = q.convert_to_tnc(circ, decompose=True, no_output=True)
    tnc.add_output_subset([1, 2, 3, 5, 6, 8])
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan))
    bits = list(q.amplitudes_uniform(6, 3, 4))
    ref = oracle.run_programme(prog, bits, out_size=8)
    got = bw.run_programme(prog, bits)
    assert got.shape == ref.shape
    assert np.max(np.abs(got - ref)) < 1e-14


def test_ncon_hyper_scalar_and_lone_labels(bw):
    """Batched (hyper) labels, a scalar operand, a label summed within one operand and a label
    repeated within one operand, each against numpy.einsum."""
    rng = np.random.default_rng(5)
    z = lambda *s: rng.standard_normal(s) + 1j * rng.standard_normal(s)
    A, B = z(2, 3, 4, 2), z(4, 2, 5)
    C, f = bw.ncon(A, [1, 2, 3, 4], B, [3, 4, 6], [6, 1, 2])
    assert np.allclose(C, np.einsum("abcd,cdf->fab", A, B), atol=1e-13)
    assert f == 8.0 * 5 * 2 * 3 * 4 * 2
    A, B = z(2, 3, 4), z(3, 4, 5)
    C, _ = bw.ncon(A, [1, 2, 3], B, [2, 3, 4], [2, 1, 4])      # label 2 batched, 3 summed
    assert np.allclose(C, np.einsum("abc,bcd->bad", A, B), atol=1e-13)
    s = np.array(2.0 - 1.0j)
    C, _ = bw.ncon(s, [], A, [1, 2, 3], [3, 1, 2])
    assert np.allclose(C, s * A.transpose(2, 0, 1))
    C, _ = bw.ncon(A, [1, 2, 3], z(5), [7], [1, 7])             # 2 and 3 summed within A alone
    assert C.shape == (2, 5)
    D = z(3, 3, 2)
    C, _ = bw.ncon(D, [1, 1, 2], z(2), [2], [1])               # diagonal of a repeated label
    assert C.shape == (3,)


def test_timed_sample_stops_at_deadline(q, bw):
    circ = q.create_rqc_circuit(3, 3, 5, seed=2)
    tnc = q.convert_to_tnc(circ, decompose=True)
    prog = q.compile_programme(tnc, q.flow_cutter_contraction_plan(tnc, time=1))
    fl, sec, done = bw.run_timed(prog, "0" * 9, 60.0)
    assert done and fl > 0 and sec > 0
    fl0, _, done0 = bw.run_timed(prog, "0" * 9, 0.0)
    assert not done0 and fl0 == 0.0
    assert bw.blas_threads() >= 1


def test_threaded_gather_matches_numpy(bw):
    """The threaded permute-copy on views above the size where it takes over from numpy:
    bit permutations of a rank-16 tensor, a sliced view (size-1 axis, offset start), a
    permutation of a permuted view and axes that merge into longer runs."""
    rng = np.random.default_rng(11)
    x = (rng.standard_normal(2 ** 16) + 1j * rng.standard_normal(2 ** 16)).reshape((2,) * 16)
    for seed in range(4):
        p = np.random.default_rng(seed).permutation(16)
        v = x.transpose(p)
        assert np.array_equal(bw._contiguous(v), np.ascontiguousarray(v))
    idx = [slice(None)] * 16
    idx[5] = slice(1, 2)
    v = x[tuple(idx)].transpose(list(range(15, -1, -1)))
    assert v.size >= bw._GATHER_MIN and np.array_equal(bw._contiguous(v), np.ascontiguousarray(v))
    y = x.reshape(4, 64, 256).transpose(2, 0, 1)
    w = y.transpose(1, 2, 0)[:, 3:40, :].transpose(2, 1, 0)
    assert np.array_equal(bw._contiguous(w), np.ascontiguousarray(w))
    c = x.reshape(2 ** 8, 2 ** 8)
    assert bw._contiguous(c) is c
