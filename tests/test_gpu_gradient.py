"""Reverse-mode gradients (qxg_gradient) against a CPU FP64 reference and finite differences.

* Leaf gradients dL/d conj(T) for L = sum_x |amplitude(x)|^2: against a numpy-einsum backprop through
  the same programme (FP64, <= 1e-12 relative to the largest entry).
* Gate-angle gradients of a parametrised circuit: against central finite differences
  (h = 1e-6, FP64 amplitudes) to <= 1e-6 absolute, and sliced == unsliced.
* Complex64 gradients (FP32 and 3xTF32 products) within 1e-4 of the FP64 gradient's largest entry.
"""
import math
from collections import OrderedDict

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
LET = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"


def einsum_backprop(prog, bitstrings):
    """Leaf gradients of L = sum_x |a(x)|^2 by numpy einsum forward + backward (small cases)."""
    from qxtools_gb300.tnc import basis_vector
    vdims = {}
    for r in prog.instrs:
        if r[0] == 2:
            vdims[int(r[3])] = int(r[5])
    nsl = int(np.prod(list(vdims.values()))) if vdims else 1
    grads = {i: np.zeros(prog.data[int(r[2])].shape, dtype=np.complex128)
             for i, r in enumerate(prog.instrs) if r[0] == 1}

    def run(bits, s, seed=None):
        vals, x = {}, s
        for v in sorted(vdims):
            vals[v] = x % vdims[v]
            x //= vdims[v]
        T, how = {}, {}
        root = None
        for i, r in enumerate(prog.instrs):
            op, dst, a, b, pos, dim, nc, na, nb, off = (int(v) for v in r)
            if op == 1:
                T[dst] = prog.data[a]; how[dst] = ("load", i)
            elif op == 2:
                T[dst] = np.take(T[a], [vals[b]], axis=pos); how[dst] = ("view", a, pos, vals[b])
            elif op == 3:
                T[dst] = basis_vector(bits[a]); how[dst] = ("out",)
            elif op == 4:
                lab = [int(l) for l in prog.labels[off:off + nc + na + nb]]
                lc, la, lb = lab[:nc], lab[nc:nc + na], lab[nc + na:]
                sub = lambda ls: "".join(LET[l] for l in ls)
                T[dst] = np.einsum(f"{sub(la)},{sub(lb)}->{sub(lc)}", T[a], T[b])
                how[dst] = ("ncon", a, b, lc, la, lb)
            elif op == 5:
                root = a
        if seed is None:
            return T[root]
        bar = {root: np.full(T[root].shape, seed, dtype=np.complex128)}
        order = [i for i in reversed(range(len(prog.instrs)))]
        for i in order:
            r = prog.instrs[i]
            op, dst = int(r[0]), int(r[1])
            if op == 5 or dst not in bar:
                continue
            h = how[dst]
            if h[0] == "ncon":
                _, a, b, lc, la, lb = h
                sub = lambda ls: "".join(LET[l] for l in ls)
                bar[a] = bar.get(a, 0) + np.einsum(f"{sub(lc)},{sub(lb)}->{sub(la)}", bar[dst], np.conj(T[b]))
                bar[b] = bar.get(b, 0) + np.einsum(f"{sub(la)},{sub(lc)}->{sub(lb)}", np.conj(T[a]), bar[dst])
            elif h[0] == "view":
                _, src, pos, v = h
                full = np.zeros(T[src].shape, dtype=np.complex128)
                idx = [slice(None)] * full.ndim
                idx[pos] = slice(v, v + 1)
                full[tuple(idx)] = bar[dst]
                bar[src] = bar.get(src, 0) + full
            elif h[0] == "load":
                grads[h[1]] += bar[dst]
        return None

    for bits in bitstrings:
        amp = sum(run(bits, s) for s in range(nsl)).reshape(-1)[0]
        for s in range(nsl):
            run(bits, s, seed=amp)
    return grads


def test_leaf_gradients_match_einsum_backprop(q, gpu_lib):
    circ = q.create_rqc_circuit(2, 3, 4, seed=3)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, _ = q.contraction_scheme(tnc, 2, seed=2, time=1)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))
    bits = list(q.amplitudes_uniform(6, 4, 5))
    ref = einsum_backprop(prog, bits)
    with q.Executor(prog, precision="fp64") as ex:
        amps, leaf = ex.gradient(bits)
    scale = max(np.max(np.abs(g)) for g in ref.values())
    for i, g in ref.items():
        assert np.max(np.abs(leaf[i] - g)) <= 1e-12 * scale, i


def test_gradient_over_several_bitstring_batches(q, gpu_lib):
    circ = q.create_rqc_circuit(3, 3, 4, seed=5)
    tnc = q.convert_to_tnc(circ, decompose=True)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.compile_programme(tnc, plan)
    bits = list(q.amplitudes_uniform(9, 1, 19))
    with q.Executor(prog) as ex1, q.Executor(prog, max_bitstring_batch=4) as ex2:
        a1, g1 = ex1.gradient(bits)
        a2, g2 = ex2.gradient(bits)
    assert np.max(np.abs(a1 - a2)) < 1e-14
    for i in g1:
        assert np.max(np.abs(g1[i] - g2[i])) <= 1e-12 * (np.max(np.abs(g1[i])) + 1e-300)


@pytest.mark.parametrize("precision", ["fp64", "split_tf32"])
def test_gradient_graph_replay_matches_eager(q, gpu_lib, precision):
    """With use_graphs the gradient pass is captured on its second run and replayed for later
    passes (5 bitstring batches of 4); three calls in a row give the eager executor's results."""
    circ = q.create_rqc_circuit(3, 3, 4, seed=5)
    tnc = q.convert_to_tnc(circ, decompose=True)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.compile_programme(tnc, plan)
    bits = list(q.amplitudes_uniform(9, 1, 19))
    with q.Executor(prog, precision=precision, max_bitstring_batch=4) as ex1, \
            q.Executor(prog, precision=precision, max_bitstring_batch=4, use_graphs=True) as ex2:
        a1, g1 = ex1.gradient(bits)
        for _ in range(3):
            a2, g2 = ex2.gradient(bits)
            assert np.array_equal(a1, a2)
            for i in g1:
                assert np.array_equal(g1[i], g2[i]), i
        a3 = ex2.amplitudes(bits)                     # the forward still matches after replays
        assert np.max(np.abs(a3[:, 0] - a1[:, 0])) <= 1e-12 * np.max(np.abs(a1))


def _loss(q, circ_fn, angles, bits):
    circ = circ_fn(angles)
    tnc = q.convert_to_tnc(circ, decompose=False)
    plan = q.flow_cutter_contraction_plan(tnc, time=1, seed=1)
    with q.Executor(q.compile_programme(tnc, plan)) as ex:
        return float(np.sum(np.abs(ex.amplitudes(bits)) ** 2))


def _param_circuit(q, rows, cols, layers, seed):
    base = q.create_parametrised_circuit(rows, cols, layers, seed=seed)

    def with_angles(angles):
        c = q.Circuit(base.num_qubits)
        for g in base.circ_ops:
            if g.name == "rx":
                m = q.gates.rx(angles[g.param_ids[0]])
                c.add("rx", g.qubits, m, params=(angles[g.param_ids[0]],), param_ids=g.param_ids)
            elif g.name == "rz":
                m = q.gates.rz(angles[g.param_ids[0]])
                c.add("rz", g.qubits, m, params=(angles[g.param_ids[0]],), param_ids=g.param_ids)
            else:
                th, ph = angles[g.param_ids[0]], angles[g.param_ids[1]]
                c.add("fsim", g.qubits, q.gates.fsim(th, ph), params=(th, ph), param_ids=g.param_ids)
        c.num_params = base.num_params
        return c
    return base, with_angles


def test_angle_gradients_match_finite_differences(q, gpu_lib):
    base, circ_fn = _param_circuit(q, 2, 3, 3, seed=4)
    bits = list(q.amplitudes_uniform(6, 2, 8))
    lossf = q.gradients.ParametrisedCircuitLoss(base, seed=1)
    L, g, _ = lossf.loss_and_grad(bits)
    lossf.close()
    angles = np.array(base.angles)
    assert abs(L - _loss(q, circ_fn, angles, bits)) < 1e-12
    h = 1e-6
    rng = np.random.default_rng(0)
    for pid in rng.choice(base.num_params, size=12, replace=False):
        e = np.zeros_like(angles)
        e[pid] = h
        fd = (_loss(q, circ_fn, angles + e, bits) - _loss(q, circ_fn, angles - e, bits)) / (2 * h)
        assert abs(fd - g[pid]) <= 1e-6, (pid, fd, g[pid])


def test_sliced_gradient_equals_unsliced(q, gpu_lib):
    base, _ = _param_circuit(q, 2, 3, 3, seed=6)
    bits = list(q.amplitudes_uniform(6, 3, 6))
    a = q.gradients.ParametrisedCircuitLoss(base, nslice=0, seed=1)
    b = q.gradients.ParametrisedCircuitLoss(base, nslice=2, seed=1)
    assert b.programme.num_slices >= 4
    La, ga, _ = a.loss_and_grad(bits)
    Lb, gb, _ = b.loss_and_grad(bits)
    a.close(); b.close()
    assert abs(La - Lb) < 1e-13
    assert np.max(np.abs(ga - gb)) <= 1e-12 * np.max(np.abs(ga))


@pytest.mark.parametrize("precision", ["fp32", "split_tf32"])
def test_complex64_gradients_close_to_fp64(q, gpu_lib, precision):
    base, _ = _param_circuit(q, 3, 3, 4, seed=7)
    bits = list(q.amplitudes_uniform(9, 5, 16))
    ref = q.gradients.ParametrisedCircuitLoss(base, seed=1, precision="fp64")
    got = q.gradients.ParametrisedCircuitLoss(base, seed=1, precision=precision)
    _, g64, _ = ref.loss_and_grad(bits)
    _, g32, _ = got.loss_and_grad(bits)
    ref.close(); got.close()
    assert np.max(np.abs(g32 - g64)) <= 1e-4 * np.max(np.abs(g64))
