"""The CPU oracle pinned against the reference's golden vectors and independent checks.

Golden fixtures come from the reference's own documents and tests (tests/golden/make_golden.py):
the DSL example of docs/src/users_guide.md (views, chained views, batched ncon, scalar save,
sum over 4 slices), the GHZ-3 state vector (test/test_tn_conversion.jl:39) and GHZ-5 amplitudes
(test/test_simulation.jl:17-25).  Beyond those, the oracle is checked against a second
restatement (numpy einsum per command) and a state-vector simulation of the circuit.
"""
import json
import math
from collections import OrderedDict
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


def golden():
    return json.loads((GOLD / "golden.json").read_text())


def users_guide_programme(q):
    g = golden()["users_guide_ghz2"]
    cmds, ver = q.dsl.parse_qx((GOLD / "users_guide_ghz2.qx").read_text())
    assert ver == "0.4.0"
    data = OrderedDict((k, np.array([complex(*x) for x in v]).reshape(g["data_dims"][k], order="F"))
                       for k, v in g["data"].items())
    return q.Programme.from_commands(cmds, data, g["nqubits"]), g


def einsum_run(prog, bitstring, slice_id):
    """Second restatement of the DSL semantics with numpy.einsum (small cases only)."""
    from qxtools_gb300.tnc import basis_vector
    T = {}
    vdims = {}
    for r in prog.instrs:
        if r[0] == 2:
            vdims[int(r[3])] = int(r[5])
    vals, s = {}, slice_id
    for v in sorted(vdims):
        vals[v] = s % vdims[v]
        s //= vdims[v]
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    result = None
    for r in prog.instrs:
        op, dst, a, b, pos, dim, nc, na, nb, off = (int(x) for x in r)
        if op == 1:
            T[dst] = prog.data[a]
        elif op == 2:
            x = np.take(T[a], [vals[b]], axis=pos)
            T[dst] = x
        elif op == 3:
            T[dst] = basis_vector(bitstring[a])
        elif op == 4:
            lab = prog.labels[off:off + nc + na + nb]
            lc, la, lb = lab[:nc], lab[nc:nc + na], lab[nc + na:]
            m = {}
            for l in list(la) + list(lb):
                m.setdefault(int(l), letters[len(m)])
            spec = "".join(m[int(l)] for l in la) + "," + "".join(m[int(l)] for l in lb) + "->" + \
                "".join(m[int(l)] for l in lc)
            T[dst] = np.einsum(spec, T[a], T[b])
        elif op == 5:
            result = T[a]
    return np.asarray(result).reshape(-1, order="F")


def statevector(circ):
    """Dense state-vector simulation; index = sum_q bit_q 2^(q-1) (qubit 1 fastest)."""
    n = circ.num_qubits
    psi = np.zeros((2,) * n, dtype=np.complex128, order="F")
    psi[(0,) * n] = 1.0
    for g in circ.circ_ops:
        qs = [x - 1 for x in g.qubits]
        if len(qs) == 1:
            psi = np.moveaxis(np.tensordot(g.matrix, psi, axes=([1], [qs[0]])), 0, qs[0])
        else:
            u = g.matrix.reshape(2, 2, 2, 2, order="F")   # u[o1,o2,i1,i2]
            psi = np.tensordot(u, psi, axes=([2, 3], qs))
            psi = np.moveaxis(psi, [0, 1], qs)
    return psi


def amp_from_sv(psi, bitstring):
    return psi[tuple(int(c) for c in bitstring)]


def test_users_guide_example_golden(q, oracle):
    prog, g = users_guide_programme(q)
    assert prog.num_slices == 4
    for bits, (re, im) in g["amplitudes"].items():
        got = oracle.run_programme(prog, [bits])[0, 0]
        assert abs(got - complex(re, im)) < 1e-14, bits


def test_users_guide_slices_are_partial_sums(q, oracle):
    prog, g = users_guide_programme(q)
    total = oracle.run_programme(prog, ["11"], slices=(0, 4))[0, 0]
    parts = sum(oracle.run_programme(prog, ["11"], slices=(s, s + 1))[0, 0] for s in range(4))
    assert abs(total - parts) < 1e-15
    # slice id -> (v1, v2) with v1 fastest.  v1 is the control wire, v2 the target's input
    # wire (fed by |0>): only v1 = 1, v2 = 0 (slice 1) contributes to "11"
    assert abs(oracle.run_programme(prog, ["11"], slices=(1, 2))[0, 0] - 1 / math.sqrt(2)) < 1e-15
    for s in (0, 2, 3):
        assert abs(oracle.run_programme(prog, ["11"], slices=(s, s + 1))[0, 0]) < 1e-15


def test_users_guide_matches_einsum(q, oracle):
    prog, _ = users_guide_programme(q)
    for bits in ["00", "01", "10", "11", "+0", "-1", "++"]:
        ref = sum(einsum_run(prog, bits, s)[0] for s in range(4))
        assert abs(oracle.run_programme(prog, [bits])[0, 0] - ref) < 1e-14


def test_ghz3_state_vector_golden(q, oracle):
    g = golden()["ghz3_state"]
    for decompose in (False, True):
        circ = q.create_test_circuit()
        tnc = q.convert_to_tnc(circ, no_output=True, decompose=decompose)
        for plan in (q.flow_cutter_contraction_plan(tnc, time=1), q.min_fill_contraction_plan(tnc),
                     q.netcon(tnc)):
            prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan))
            out = oracle.run_programme(prog, [""], out_size=8)[0]
            ref = np.zeros(8)
            ref[[i - 1 for i in g["nonzero_1based"]]] = g["value"]
            # the saved tensor's axes follow the result labels; for GHZ only 000 and 111 are nonzero
            assert np.allclose(np.sort(np.abs(out)), np.sort(ref), atol=1e-14)
            assert abs(out[0] - g["value"]) < 1e-14 and abs(out[7] - g["value"]) < 1e-14


def test_ghz5_all_amplitudes_golden(q, oracle):
    g = golden()["ghz5"]
    circ = q.create_ghz_circuit(g["n"])
    tnc = q.convert_to_tnc(circ, decompose=True)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.compile_programme(tnc, plan)
    bits = list(q.amplitudes_all(g["n"]))
    assert len(bits) == g["num_results"]
    amps = oracle.run_programme(prog, bits)[:, 0]
    assert abs(amps[0] - g["value"]) < 1e-14 and abs(amps[-1] - g["value"]) < 1e-14
    assert np.allclose(amps[1:-1], 0, atol=1e-15)


@pytest.mark.parametrize("decompose", [False, True])
def test_oracle_matches_statevector(q, oracle, decompose):
    circ = q.create_rqc_circuit(3, 3, 5, seed=11)
    psi = statevector(circ)
    tnc = q.convert_to_tnc(circ, decompose=decompose)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.compile_programme(tnc, plan)
    bits = list(q.amplitudes_uniform(9, 5, 16))
    amps = oracle.run_programme(prog, bits, nthreads=4)[:, 0]
    ref = np.array([amp_from_sv(psi, b) for b in bits])
    assert np.max(np.abs(amps - ref)) < 1e-13


def test_oracle_norm_4x4_small_depth(q, oracle):
    """Sum over all 2^n |amp|^2 = 1 (unitarity) on a 3x4 circuit."""
    circ = q.create_rqc_circuit(3, 4, 4, seed=2)
    tnc = q.convert_to_tnc(circ, decompose=True)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.compile_programme(tnc, plan)
    amps = oracle.run_programme(prog, list(q.amplitudes_all(12)), nthreads=8)[:, 0]
    assert abs(np.sum(np.abs(amps) ** 2) - 1.0) < 1e-12


def test_sliced_sum_equals_unsliced(q, oracle):
    circ = q.create_rqc_circuit(3, 3, 6, seed=3)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, meta = q.contraction_scheme(tnc, 3, seed=4, time=1)
    assert len(groups) == 3
    sliced = q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))
    unsliced = q.Programme.from_graph(q.build_compute_graph(tnc, plan))
    assert sliced.num_slices == 2 ** 3
    bits = list(q.amplitudes_uniform(9, 1, 6))
    a = oracle.run_programme(sliced, bits)[:, 0]
    b = oracle.run_programme(unsliced, bits)[:, 0]
    assert np.max(np.abs(a - b)) < 1e-14


def test_different_plans_same_amplitudes(q, oracle):
    circ = q.create_rqc_circuit(2, 4, 6, seed=5)
    tnc = q.convert_to_tnc(circ, decompose=True)
    net = q.hyper_network(tnc)
    p1 = q.greedy_contraction_plan(net, seed=1)
    p2 = q.greedy_contraction_plan(net, seed=2, temperature=0.3)
    p3 = q.min_fill_contraction_plan(tnc, hypergraph=True)
    bits = list(q.amplitudes_uniform(8, 9, 8))
    res = [oracle.run_programme(q.compile_programme(tnc, p), bits)[:, 0] for p in (p1, p2, p3)]
    assert np.max(np.abs(res[0] - res[1])) < 1e-14
    assert np.max(np.abs(res[0] - res[2])) < 1e-14


def test_oracle_einsum_on_random_sliced_programme(q, oracle):
    circ = q.create_rqc_circuit(2, 3, 4, seed=8)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, _ = q.contraction_scheme(tnc, 2, seed=2, time=1)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))
    for bits in ["010101", "+-01+-"]:
        ref = sum(einsum_run(prog, bits, s)[0] for s in range(prog.num_slices))
        assert abs(oracle.run_programme(prog, [bits])[0, 0] - ref) < 1e-14


def test_oracle_rejects_bad_programme(q, oracle):
    prog, _ = users_guide_programme(q)
    bad = prog.instrs.copy()
    bad[5, 7] = 3          # ncon label count no longer matches the operand rank
    with pytest.raises(RuntimeError):
        oracle.run(bad, prog.labels, prog.data_rank, prog.data_dims, *prog.data_flat(), 2, ["00"],
                   num_slices=4)
