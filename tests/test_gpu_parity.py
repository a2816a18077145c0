"""GPU executor (libqxgpu through its C ABI) against the CPU FP64 oracle and golden vectors.

Tolerances: the ComplexF64 executor must match the oracle to <= 1e-12 relative error per
amplitude (amplitudes below 1e-6 of the largest are compared absolutely at 1e-12 of the largest);
the Complex64 executors (FP32 arithmetic) to <= 1e-5 relative to the largest amplitude.
"""
import json
import math
from collections import OrderedDict
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
FP64_TOL = 1e-12
FP32_TOL = 1e-5


def rel_err(got, ref):
    got, ref = np.asarray(got).ravel(), np.asarray(ref).ravel()
    scale = np.max(np.abs(ref))
    floor = 1e-6 * scale
    den = np.maximum(np.abs(ref), floor)
    return float(np.max(np.abs(got - ref) / den))


def users_guide(q):
    g = json.loads((GOLD / "golden.json").read_text())["users_guide_ghz2"]
    cmds, _ = q.dsl.parse_qx((GOLD / "users_guide_ghz2.qx").read_text())
    data = OrderedDict((k, np.array([complex(*x) for x in v]).reshape(g["data_dims"][k], order="F"))
                       for k, v in g["data"].items())
    return q.Programme.from_commands(cmds, data, 2), g


@pytest.mark.parametrize("bb,sb", [(0, 0), (1, 1), (2, 1), (1, 2), (4, 4)])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_users_guide_golden_on_gpu(q, gpu_lib, bb, sb, precision):
    prog, g = users_guide(q)
    with q.Executor(prog, precision=precision, max_bitstring_batch=bb, max_slice_batch=sb) as ex:
        bits = list(g["amplitudes"])
        got = ex.amplitudes(bits)[:, 0]
    ref = np.array([complex(*g["amplitudes"][b]) for b in bits])
    tol = 1e-15 if precision == "fp64" else 1e-7
    assert np.max(np.abs(got - ref)) < tol


def test_users_guide_slice_ranges(q, gpu_lib):
    prog, _ = users_guide(q)
    with q.Executor(prog) as ex:
        parts = [ex.amplitudes(["11"], slices=(s, s + 1))[0, 0] for s in range(4)]
        assert abs(parts[1] - 1 / math.sqrt(2)) < 1e-15
        assert max(abs(parts[s]) for s in (0, 2, 3)) < 1e-15
        assert abs(ex.amplitudes(["11"], slices=(0, 2))[0, 0] - 1 / math.sqrt(2)) < 1e-15


def test_ghz3_state_vector_open_outputs(q, gpu_lib, oracle):
    tnc = q.convert_to_tnc(q.create_test_circuit(), no_output=True, decompose=True)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan))
    with q.Executor(prog) as ex:
        out = ex.amplitudes([""])[0]
    assert out.shape == (8,)
    r = 1 / math.sqrt(2)
    assert abs(out[0] - r) < 1e-15 and abs(out[7] - r) < 1e-15
    assert np.max(np.abs(out[1:7])) < 1e-15


def test_ghz5_run_simulation_gpu(q, gpu_lib):
    res = q.run_simulation(q.create_ghz_circuit(5))
    assert len(res) == 32
    r = 1 / math.sqrt(2)
    assert abs(res["00000"] - r) < 1e-14 and abs(res["11111"] - r) < 1e-14


def test_single_amplitude_api(q, gpu_lib, oracle):
    circ = q.create_rqc_circuit(3, 3, 4, seed=2)
    tnc = q.convert_to_tnc(circ)
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.compile_programme(tnc, plan)
    for b in ["000000000", "101010101", "+-01+-01+"]:
        ref = oracle.run_programme(prog, [b])[0, 0]
        assert abs(q.single_amplitude(tnc, plan, b) - ref) <= FP64_TOL * max(abs(ref), 1e-300) + 1e-17


def rqc_programme(q, rows, cols, depth, seed, nslice=0, max_log2=None, decompose=True):
    circ = q.create_rqc_circuit(rows, cols, depth, seed=seed)
    tnc = q.convert_to_tnc(circ, decompose=decompose)
    groups, plan, _ = q.contraction_scheme(tnc, nslice, seed=seed, time=1, max_log2=max_log2)
    return q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))


def test_4x4_depth10_64_bitstrings_fp64(q, gpu_lib, oracle):
    """The 4x4, 10-cycle random circuit, unsliced, 64 seeded bitstrings."""
    prog = rqc_programme(q, 4, 4, 10, seed=1)
    bits = list(q.amplitudes_uniform(16, 1, 64))
    with q.Executor(prog) as ex:
        got = ex.amplitudes(bits)[:, 0]
    ref = oracle.run_programme(prog, bits, nthreads=8)[:, 0]
    assert rel_err(got, ref) <= FP64_TOL


@pytest.mark.parametrize("bb,sb", [(0, 0), (8, 2), (3, 4)])
def test_sliced_rqc_fp64(q, gpu_lib, oracle, bb, sb):
    prog = rqc_programme(q, 3, 4, 8, seed=5, nslice=3)
    assert prog.num_slices >= 8
    bits = list(q.amplitudes_uniform(12, 2, 37))          # not a multiple of the batch
    with q.Executor(prog, max_bitstring_batch=bb, max_slice_batch=sb) as ex:
        got = ex.amplitudes(bits)[:, 0]
        part = ex.amplitudes(bits[:5], slices=(1, 5))[:, 0]
    ref = oracle.run_programme(prog, bits, nthreads=8)[:, 0]
    assert rel_err(got, ref) <= FP64_TOL
    refp = oracle.run_programme(prog, bits[:5], slices=(1, 5), nthreads=8)[:, 0]
    assert rel_err(part, refp) <= FP64_TOL


def test_sliced_rqc_unsliced_agree_on_gpu(q, gpu_lib):
    circ = q.create_rqc_circuit(3, 4, 8, seed=9)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, _ = q.contraction_scheme(tnc, 3, seed=3, time=1)
    bits = list(q.amplitudes_uniform(12, 4, 16))
    with q.Executor(q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))) as ex:
        a = ex.amplitudes(bits)[:, 0]
    with q.Executor(q.Programme.from_graph(q.build_compute_graph(tnc, plan))) as ex:
        b = ex.amplitudes(bits)[:, 0]
    assert rel_err(a, b) <= FP64_TOL


def test_open_qubits_batch_tensor(q, gpu_lib, oracle):
    """Some qubits left open: each bitstring's result is a 2^k tensor."""
    circ = q.create_rqc_circuit(3, 3, 5, seed=4)
    tnc = q.convert_to_tnc(circ, decompose=True, no_output=True)
    keep = [0, 1, 2, 4, 6, 8]                 # qubits with output tensors; 3, 5, 7 stay open
    from qxtools_gb300.tnc import basis_vector
    names = []
    for qi in keep:
        names.append(tnc.tn.add_tensor([tnc.output_indices[qi]], basis_vector("0")))
    tnc.output_tensors = names
    plan = q.flow_cutter_contraction_plan(tnc, time=1)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan))
    prog.nqubits = 6
    bits = list(q.amplitudes_uniform(6, 3, 10))
    with q.Executor(prog) as ex:
        got = ex.amplitudes(bits)
    assert got.shape == (10, 8)
    ref = oracle.run_programme(prog, bits, out_size=8)
    assert rel_err(got, ref) <= FP64_TOL


def test_fp32_executor_error(q, gpu_lib, oracle):
    prog = rqc_programme(q, 3, 4, 8, seed=5, nslice=2)
    bits = list(q.amplitudes_uniform(12, 2, 24))
    with q.Executor(prog, precision="fp32") as ex:
        got = ex.amplitudes(bits)[:, 0]
    ref = oracle.run_programme(prog, bits, nthreads=8)[:, 0]
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= FP32_TOL


def test_padded_dimension_three(q, gpu_lib, oracle):
    """A bond of dimension 3 (not a power of two) is zero-padded on the device."""
    rng = np.random.default_rng(1)
    A = rng.standard_normal((2, 3, 2)) + 1j * rng.standard_normal((2, 3, 2))
    B = rng.standard_normal((3, 2)) + 1j * rng.standard_normal((3, 2))
    text = ("load a data_1 2,3,2\nload b data_2 3,2\nview a_s a v1 2 3\nview b_s b v1 1 3\n"
            "output o1 1 2\noutput o2 2 2\nncon c 1,3 a_s 1,2,3 b_s 2,4\n"
            "ncon d 2 c 1,2 o1 1\nncon e 0 d 1 o2 1\nsave output e\n")
    cmds, _ = q.dsl.parse_qx(text)
    # result label 4 of b_s is dropped from c; make c keep it: rewrite the command
    cmds[6] = q.Ncon("c", (1, 3), "a_s", (1, 2, 3), "b_s", (2, 3))
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", A), ("data_2", B)]), 2)
    assert prog.num_slices == 3
    bits = ["00", "01", "10", "11", "+-"]
    with q.Executor(prog) as ex:
        got = ex.amplitudes(bits)[:, 0]
    ref = oracle.run_programme(prog, bits)[:, 0]
    assert rel_err(got, ref) <= FP64_TOL


def test_invalid_bitstring_rejected(q, gpu_lib):
    prog, _ = users_guide(q)
    with q.Executor(prog) as ex:
        with pytest.raises(q.QXGError) as e:
            ex.amplitudes(["0x"])
        assert e.value.code == -1
        with pytest.raises(q.QXGError):
            ex.amplitudes(["00"], slices=(0, 9))


def test_device_resident_call(q, gpu_lib, oracle):
    import torch
    prog = rqc_programme(q, 3, 3, 6, seed=3, nslice=2)
    bits = list(q.amplitudes_uniform(9, 6, 20))
    raw = torch.tensor(list("".join(bits).encode()), dtype=torch.uint8, device="cuda")
    out = torch.zeros(2 * len(bits), dtype=torch.float64, device="cuda")
    with q.Executor(prog) as ex:
        ex.amplitudes_device(raw.data_ptr(), len(bits), out.data_ptr())
        ex.synchronize()
    got = out.cpu().numpy().view(np.complex128)
    ref = oracle.run_programme(prog, bits)[:, 0]
    assert rel_err(got, ref) <= FP64_TOL


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_ncon_entry_point(q, gpu_lib, precision):
    import torch
    rng = np.random.default_rng(0)
    cases = [
        # (a_labels, a_dims, b_labels, b_dims, c_labels)
        ((1, 2, 3), (2, 4, 2), (3, 4, 2), (2, 2, 4), (1, 4)),          # K = labels 2, 3
        ((1, 2, 3, 5), (2, 2, 2, 2), (5, 2, 6), (2, 2, 4), (6, 3, 1, 2)),   # batched label 2
        ((1,), (8,), (2,), (4,), (2, 1)),                               # outer product
        ((), (), (1, 2), (2, 2), (2, 1)),                                # scalar operand
        (tuple(range(1, 13)), (2,) * 12, (3, 7, 13), (2, 2, 2), tuple([13] + list(range(12, 0, -1)))),
    ]
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    for la, ad, lb, bd, lc in cases:
        A = rng.standard_normal(ad) + 1j * rng.standard_normal(ad) if ad else np.array(1.5 - 0.5j)
        B = rng.standard_normal(bd) + 1j * rng.standard_normal(bd)
        letters = {}
        for l in la + lb:
            letters.setdefault(l, "abcdefghijklmnopqrstuvwxyz"[len(letters)])
        ref = np.einsum("".join(letters[l] for l in la) + "," + "".join(letters[l] for l in lb) + "->" +
                        "".join(letters[l] for l in lc), A, B)
        dA = torch.tensor(np.asarray(A).reshape(-1, order="F"), dtype=cdt, device="cuda")
        dB = torch.tensor(B.reshape(-1, order="F"), dtype=cdt, device="cuda")
        dC = torch.zeros(max(ref.size, 1), dtype=cdt, device="cuda")
        q.ncon_device(precision, dC.data_ptr(), lc, dA.data_ptr(), la, ad, dB.data_ptr(), lb, bd)
        torch.cuda.synchronize()
        got = dC.cpu().numpy().reshape(ref.shape, order="F") if ref.ndim else dC.cpu().numpy()[0]
        tol = 1e-13 if precision == "fp64" else 2e-5
        assert np.max(np.abs(got - ref)) <= tol * max(1.0, np.max(np.abs(ref)))


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_gate_steps_random_layouts(q, gpu_lib, precision):
    """Gate-like contractions (X of 2^14..2^16 elements; Y with 0..5 summed, 0..6 new and 0..2
    batch labels) under random label orders of X, Y and C, conjugation-free: the row forms
    (tiled through shared memory, or one row per thread) against numpy."""
    import torch
    rng = np.random.default_rng(11)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    for case in range(24):
        nk = int(rng.integers(0, 5 if precision == "fp64" else 6))
        nn = int(rng.integers(0, 7))
        nb = int(rng.integers(0, 3))
        nx = int(rng.integers(14, 17))
        if nx - nk + nn > 20:
            nn = 20 - nx + nk
        xl = list(range(1, nx + 1))
        kl, bl, fl = xl[:nk], xl[nk:nk + nb], xl[nk + nb:]
        nl = list(range(100, 100 + nn))
        la = [int(v) for v in rng.permutation(xl)]
        lb = [int(v) for v in rng.permutation(kl + bl + nl)]
        lc = [int(v) for v in rng.permutation(bl + fl + nl)]
        ad, bd = (2,) * len(la), (2,) * len(lb)
        A = rng.standard_normal(ad) + 1j * rng.standard_normal(ad)
        B = rng.standard_normal(bd) + 1j * rng.standard_normal(bd)
        idx = {v: letters[i] for i, v in enumerate(sorted(set(la + lb)))}
        ref = np.einsum("".join(idx[v] for v in la) + "," + "".join(idx[v] for v in lb) + "->" +
                        "".join(idx[v] for v in lc), A, B)
        dA = torch.tensor(A.reshape(-1, order="F"), dtype=cdt, device="cuda")
        dB = torch.tensor(B.reshape(-1, order="F"), dtype=cdt, device="cuda")
        dC = torch.full((ref.size,), float("nan"), dtype=cdt, device="cuda")
        q.ncon_device(precision, dC.data_ptr(), lc, dA.data_ptr(), la, ad, dB.data_ptr(), lb, bd)
        torch.cuda.synchronize()
        got = dC.cpu().numpy().reshape(ref.shape, order="F")
        tol = 1e-13 if precision == "fp64" else 2e-5
        assert np.max(np.abs(got - ref)) <= tol * max(1.0, np.max(np.abs(ref))), (case, nk, nn, nb, nx)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_long_sums_random_layouts(q, gpu_lib, precision):
    """Contractions with few results and a long sum (2^12..2^14 summed terms; 0..4 bits only in
    A, 0..4 only in B, 0..2 in both and in the result; four cases with 2^10-2^11 results per
    batch value) under random label orders: the long sum (per-block FP64 partials added in block
    order, wide results in chunks) against numpy."""
    import torch
    rng = np.random.default_rng(5)
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    for case in range(20):
        nk, na, nb, ng = (int(rng.integers(12, 15)), int(rng.integers(0, 5)), int(rng.integers(0, 5)),
                          int(rng.integers(0, 3)))
        if case >= 16:                      # wide results: 2^10..2^11 values per batch value
            nk, na, nb = 12, 5 + case % 2, 5
        kl = list(range(1, nk + 1))
        al = list(range(100, 100 + na))
        bl = list(range(200, 200 + nb))
        gl = list(range(300, 300 + ng))
        la = [int(v) for v in rng.permutation(al + gl + kl)]
        lb = [int(v) for v in rng.permutation(bl + gl + kl)]
        lc = [int(v) for v in rng.permutation(al + bl + gl)]
        ad, bd = (2,) * len(la), (2,) * len(lb)
        A = rng.standard_normal(ad) + 1j * rng.standard_normal(ad)
        B = rng.standard_normal(bd) + 1j * rng.standard_normal(bd)
        idx = {v: letters[i] for i, v in enumerate(sorted(set(la + lb)))}
        ref = np.einsum("".join(idx[v] for v in la) + "," + "".join(idx[v] for v in lb) + "->" +
                        "".join(idx[v] for v in lc), A, B)
        ref = np.asarray(ref)
        dA = torch.tensor(A.reshape(-1, order="F"), dtype=cdt, device="cuda")
        dB = torch.tensor(B.reshape(-1, order="F"), dtype=cdt, device="cuda")
        dC = torch.full((max(ref.size, 1),), float("nan"), dtype=cdt, device="cuda")
        q.ncon_device(precision, dC.data_ptr(), lc, dA.data_ptr(), la, ad, dB.data_ptr(), lb, bd)
        torch.cuda.synchronize()
        got = dC.cpu().numpy().reshape(ref.shape, order="F") if ref.ndim else dC.cpu().numpy()[0]
        tol = 1e-12 if precision == "fp64" else 2e-5
        assert np.max(np.abs(got - ref)) <= tol * np.sqrt(2.0 ** nk), (case, nk, na, nb, ng)


@pytest.mark.parametrize("precision", ["fp32", "split_tf32"])
def test_graph_branches_match_eager_exactly(q, gpu_lib, precision):
    """Captured passes run independent sub-trees concurrently (graph edges from the launches'
    read/write ranges, the shared scratch serialising tensor-core steps).  Every kernel is
    deterministic, so replays must reproduce the eager first call bit for bit; a missing edge
    shows up as a difference."""
    prog = rqc_programme(q, 4, 4, 10, seed=3)
    bits = list(q.amplitudes_uniform(16, 1, 32))
    with q.Executor(prog, precision=precision, use_graphs=True, max_bitstring_batch=32) as ex:
        first = ex.amplitudes(bits)                           # eager (and autotuning)
        for _ in range(4):                                    # capture, then replays
            assert np.array_equal(ex.amplitudes(bits), first)


@pytest.mark.parametrize("precision", ["fp64", "split_tf32"])
def test_graph_replay_matches_eager(q, gpu_lib, oracle, precision):
    """Passes captured in CUDA graphs and replayed give the eager results, across repeated calls,
    slice ranges, device-resident calls and a plan change (new batch size -> graphs rebuilt)."""
    import torch
    prog = rqc_programme(q, 3, 4, 8, seed=5, nslice=3)
    bits = list(q.amplitudes_uniform(12, 2, 40))
    ref = oracle.run_programme(prog, bits, nthreads=8)[:, 0]
    tol = FP64_TOL if precision == "fp64" else 1e-5
    with q.Executor(prog, precision=precision, use_graphs=True, max_bitstring_batch=16, max_slice_batch=2) as ex:
        # FP64 per amplitude (rel_err); Complex64 relative to the largest amplitude
        err = rel_err if precision == "fp64" else (lambda g, r: np.max(np.abs(g - r)) / np.max(np.abs(r)))
        for _ in range(3):                                   # eager run, capture, replay
            got = ex.amplitudes(bits)[:, 0]
            assert err(got, ref) <= tol
        part = ex.amplitudes(bits[:7], slices=(2, 6))[:, 0]   # smaller batch: new plan
        refp = oracle.run_programme(prog, bits[:7], slices=(2, 6), nthreads=8)[:, 0]
        assert err(part, refp) <= tol
        raw = torch.tensor(list("".join(bits).encode()), dtype=torch.uint8, device="cuda")
        out = torch.zeros(2 * len(bits), dtype=torch.float64, device="cuda")
        for _ in range(2):
            ex.amplitudes_device(raw.data_ptr(), len(bits), out.data_ptr())
            ex.synchronize()
            dev = out.cpu().numpy().view(np.complex128)
            assert err(dev, ref) <= tol
