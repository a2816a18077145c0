"""Split-precision executors (3xBF16 / 3xTF32 products on tcgen05 tensor cores, FP32
accumulation, power-of-two operand scaling, FP64 slice sum) against exact references.

Tolerances (relative to the largest result element): 3xTF32 <= 5e-6, 3xBF16 <= 1e-4 for a single
contraction (FP32 accumulation over up to 2^8 real terms is itself ~1e-6); on whole random-circuit
programmes <= 1e-5 (3xTF32, FP32) and <= 1e-4 (3xBF16) against the FP64 oracle.
"""
import math
from collections import OrderedDict

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = {"split_tf32": 5e-6, "split_bf16": 1e-4, "fp32": 5e-6}


def single_ncon_programme(q, nm, nk, nn, nbatch=0, seed=0, scale=1.0, a_order="mkb", c_order="mnb"):
    """C[m.., n.., b..] = sum_k A[m.., k.., b..] B[k.., n.., b..] with dim-2 labels; a_order
    permutes A's label groups (its lowest address bits: m, k or batch), c_order C's ("i" for
    m and n labels interleaved from the lowest bit)."""
    rng = np.random.default_rng(seed)
    lm = list(range(1, nm + 1))
    lk = list(range(nm + 1, nm + nk + 1))
    ln = list(range(nm + nk + 1, nm + nk + nn + 1))
    lb = list(range(nm + nk + nn + 1, nm + nk + nn + nbatch + 1))
    groups = {"m": lm, "k": lk, "b": lb, "n": ln}
    la = [l for g in a_order for l in groups[g]]
    lbb = lk + ln + lb
    if c_order == "i":
        inter = [l for pair in zip(ln, lm) for l in pair]
        lc = inter + lm[len(ln):] + ln[len(lm):] + lb
    else:
        lc = [l for g in c_order for l in groups[g]]
    A = (rng.standard_normal((2,) * len(la)) + 1j * rng.standard_normal((2,) * len(la))) * scale
    B = (rng.standard_normal((2,) * len(lbb)) + 1j * rng.standard_normal((2,) * len(lbb))) * scale
    cmds = [q.Load("a", "data_1", A.shape), q.Load("b", "data_2", B.shape),
            q.Ncon("c", tuple(lc), "a", tuple(la), "b", tuple(lbb)), q.Save("output", "c")]
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", A), ("data_2", B)]), 0)
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    sub = lambda ls: "".join(letters[l - 1] for l in ls)
    ref = np.einsum(f"{sub(la)},{sub(lbb)}->{sub(lc)}", A, B).reshape(-1, order="F")
    return prog, ref


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16"])
@pytest.mark.parametrize("nm,nk,nn,nb", [(7, 5, 4, 0), (8, 6, 8, 0), (7, 7, 2, 0), (9, 4, 5, 1), (7, 3, 5, 0)])
def test_tensor_core_single_contraction(q, gpu_lib, precision, nm, nk, nn, nb):
    prog, ref = single_ncon_programme(q, nm, nk, nn, nb, seed=nm * 100 + nk * 10 + nn)
    with q.Executor(prog, precision=precision) as ex:
        got = ex.amplitudes([""])[0]
        assert ex.info()["num_steps_tensor_core"] == 1
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err <= TOL[precision], err


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16"])
def test_tensor_core_scaling_tiny_and_huge_values(q, gpu_lib, precision):
    """Operands far from 1 are scaled by powers of two before the split: no underflow/overflow."""
    for scale in (2.0 ** -60, 2.0 ** 50):
        prog, ref = single_ncon_programme(q, 7, 5, 4, seed=3, scale=scale)
        with q.Executor(prog, precision=precision) as ex:
            got = ex.amplitudes([""])[0]
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= TOL[precision], (scale, err)


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16", "fp32"])
def test_split_executor_on_random_circuit(q, gpu_lib, oracle, precision):
    circ = q.create_rqc_circuit(4, 4, 8, seed=21)
    tnc = q.convert_to_tnc(circ, decompose=True, no_output=True)
    tnc.add_output_subset(list(range(1, 11)))          # 6 qubits open: 64 amplitudes per bitstring
    groups, plan, _ = q.contraction_scheme(tnc, 1, seed=2, time=1)
    prog = q.Programme.from_graph(q.build_compute_graph(tnc, plan, groups))
    bits = list(q.amplitudes_uniform(10, 5, 12))
    with q.Executor(prog, precision=precision) as ex:
        got = ex.amplitudes(bits)
    ref = oracle.run_programme(prog, bits, nthreads=8, out_size=64)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    tol = 1e-5 if precision != "split_bf16" else 1e-4
    assert err <= tol, err


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16"])
def test_tensor_core_error_at_large_k(q, gpu_lib, precision):
    """K = 2^9 complex terms (2^10 real terms per accumulator): the error stays at the level of FP32
    accumulation itself (~sqrt(2^10) * 2^-24) because the correction products accumulate apart
    from the main products -- 3xTF32 within 5e-6 of the largest element, 3xBF16 within 5e-5."""
    prog, ref = single_ncon_programme(q, 7, 9, 4, seed=9)
    with q.Executor(prog, precision=precision) as ex:
        got = ex.amplitudes([""])[0]
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"{precision} K=512 error {err:.3e}")
    assert err <= (5e-6 if precision == "split_tf32" else 5e-5), err


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16"])
@pytest.mark.parametrize("nm,nk,nn,nb,order,corder", [(8, 9, 6, 0, "mkb", "mnb"), (7, 3, 7, 1, "mkb", "mnb"),
                                                       (9, 6, 2, 0, "mkb", "mnb"), (7, 6, 6, 0, "kmb", "mnb"),
                                                       (8, 4, 5, 2, "bmk", "mnb"), (8, 5, 6, 1, "kbm", "mnb"),
                                                       (8, 6, 7, 1, "mkb", "nmb"), (9, 5, 6, 0, "kmb", "i"),
                                                       (7, 7, 4, 2, "mkb", "bnm")])
def test_every_tile_variant_matches(q, gpu_lib, precision, nm, nk, nn, nb, order, corder):
    """Each candidate tile variant (X gathered in the GEMM by contiguous segments or by rows, or
    packed into planes first; N tiles of 16/32/64), forced with tc_tuning = k, and the autotuned
    choice give the einsum result within the split tolerance.  Shapes cover K chunks beyond the
    gather ring (nk=9), K below one chunk (nk=3 with 3xBF16), batch bits, N narrower than the
    smallest tile (nn=2), larger operands whose lowest address bits are summed (segments of
    rows and k values interleaved) or batch bits (batch-first tile order, no segment gather), and
    results whose lowest address bits are columns, interleaved rows and columns, or batch bits."""
    prog, ref = single_ncon_programme(q, nm, nk, nn, nb, seed=nm + 7 * nk + 31 * nn, a_order=order, c_order=corder)
    for k in ["auto"] + list(range(1, 13)):
        with q.Executor(prog, precision=precision, tc_tuning=k) as ex:
            got = ex.amplitudes([""])[0]
            info = ex.info()
            desc = ex.explain(2)                 # the ncon command
        assert "tensor-core" in desc, desc
        assert info["num_steps_tensor_core"] == 1
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= TOL[precision], (k, err)
        if k == "auto":                         # fused and planes candidates at least
            assert info["num_steps_tuned"] == 1


@pytest.mark.parametrize("precision", ["fp64", "fp32", "split_tf32"])
@pytest.mark.parametrize("nm,nk,nn", [(2, 16, 2), (7, 14, 6), (0, 15, 3)])
def test_long_sum_small_result(q, gpu_lib, precision, nm, nk, nn):
    """Few results, long sums (the shape of adjoint steps ending in leaf gradients): the split-K
    CUDA-core form and, for (7, 14, 6) in 3xTF32, the tensor cores with K cut into blocks of at
    most 1024 (partials summed in a fixed order) against einsum; FP64 to 1e-12, the Complex64
    modes to 1e-5 of the largest result."""
    prog, ref = single_ncon_programme(q, nm, nk, nn, 0, seed=nm + nk + nn)
    with q.Executor(prog, precision=precision) as ex:
        got = ex.amplitudes([""])[0]
        got2 = ex.amplitudes([""])[0]
        if precision != "split_tf32" or nm < 7:
            assert ex.info()["num_steps_tensor_core"] == 0
        else:                                   # K = 2^14 on the tensor cores: split into blocks
            assert "split-K" in ex.explain(2)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err <= (1e-12 if precision == "fp64" else 1e-5), err
    assert np.array_equal(got, got2)                   # deterministic: fixed partition and order


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16"])
@pytest.mark.parametrize("nm,nk,nn", [(11, 7, 11), (8, 11, 8)])
def test_outer_column_blocks(q, gpu_lib, precision, nm, nk, nn):
    """A planes budget of 1 MiB forces the smaller operand's free columns into blocks looped on
    the host (each block packs its part of Y and runs the GEMM on offset pointers), alone and with
    split K (nk=11); results against einsum within the split tolerance."""
    prog, ref = single_ncon_programme(q, nm, nk, nn, 0, seed=nm * nk + nn)
    for k in ["auto", 1]:
        with q.Executor(prog, precision=precision, tc_tuning=k, tc_plane_budget_mb=1) as ex:
            got = ex.amplitudes([""])[0]
            desc = ex.explain(2)
        assert "n-blocks=" in desc, desc
        err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
        assert err <= TOL[precision], (k, err)


def test_tuning_decisions_carry_over(q, gpu_lib):
    """qxg_program_tuning_get / _set: a second programme preloaded with the first one's decisions
    times no candidate and runs the same variant, with the same result."""
    prog, ref = single_ncon_programme(q, 9, 7, 6, 1, seed=11, a_order="kmb")
    with q.Executor(prog, precision="split_tf32") as ex1:
        got1 = ex1.amplitudes([""])[0]
        text = ex1.tuning()
        desc1 = ex1.explain(2)
        assert ex1.info()["num_steps_tuned"] == 1 and text.count("\n") == 1
    with q.Executor(prog, precision="split_tf32") as ex2:
        ex2.set_tuning(text)
        got2 = ex2.amplitudes([""])[0]
        desc2 = ex2.explain(2)
        assert ex2.info()["num_steps_tuned"] == 0
    variant = lambda d: d.split("tensor-core ")[1].split(" nb=")[0]
    assert variant(desc1) == variant(desc2)
    assert np.array_equal(got1, got2)
    with pytest.raises(q.QXGError):
        q.Executor(prog, precision="split_tf32").set_tuning("zz 1 7 0 0 0\n")


@pytest.mark.parametrize("precision", ["fp32", "split_tf32"])
@pytest.mark.parametrize("nk,na,nb,ng", [(12, 5, 5, 3), (15, 5, 5, 0), (13, 6, 4, 3), (11, 6, 6, 4)])
def test_batched_join_gemm(q, gpu_lib, precision, nk, na, nb, ng):
    """The final-join shape: both operands large (2^20-2^22 elements), 2^4-2^6 free values on
    each side, 2^11-2^15 summed terms and 2^0-2^4 batch values, under random label orders.  It
    runs on the batched small GEMM (the plan's explanation names it), with K cut into ranges whose
    FP64 partials are added in order when there is one batch value; FP32 products with FP64
    accumulation every 512 terms stay within 1e-6 of the largest result of einsum, and a second
    call gives the same bits."""
    rng = np.random.default_rng(nk * 1000 + na * 100 + nb * 10 + ng)
    kl = list(range(1, nk + 1))
    al, bl, gl = list(range(100, 100 + na)), list(range(200, 200 + nb)), list(range(300, 300 + ng))
    la = [int(v) for v in rng.permutation(al + gl + kl)]
    lb = [int(v) for v in rng.permutation(bl + gl + kl)]
    lc = [int(v) for v in rng.permutation(al + bl + gl)]
    A = rng.standard_normal((2,) * len(la)) + 1j * rng.standard_normal((2,) * len(la))
    B = rng.standard_normal((2,) * len(lb)) + 1j * rng.standard_normal((2,) * len(lb))
    cmds = [q.Load("a", "data_1", A.shape), q.Load("b", "data_2", B.shape),
            q.Ncon("c", tuple(lc), "a", tuple(la), "b", tuple(lb)), q.Save("output", "c")]
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", A), ("data_2", B)]), 0)
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    idx = {v: letters[i] for i, v in enumerate(sorted(set(la + lb)))}
    sub = lambda ls: "".join(idx[v] for v in ls)
    ref = np.einsum(f"{sub(la)},{sub(lb)}->{sub(lc)}", A, B).reshape(-1, order="F")
    # split-TF32 programmes send the joins that fit it to the tensor-core join unless told otherwise
    with q.Executor(prog, precision=precision, cuda_core_joins=True) as ex:
        got = ex.amplitudes([""])[0]
        got2 = ex.amplitudes([""])[0]
        assert "batched-gemm" in ex.explain(2), ex.explain(2)
        assert ex.info()["num_steps_tensor_core"] == 0
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err <= 1e-6, err
    assert np.array_equal(got, got2)


def join_programme(q, nk, na, nb, ng, seed, batch_on_top=True):
    """One ncon of the final-join shape, laid out so a raw chunk of the tensor-core join is a TMA
    box: in each operand six summed labels first (the same six in both, in each operand's own
    seeded order), then the free labels in one or two blocks around three other summed labels,
    then the remaining summed labels, and the batch labels last (the highest address bits, as the
    programme's layout rule places them in intermediates).  With batch_on_top=False every label is
    in a random place.  Returns the programme and the einsum result."""
    rng = np.random.default_rng(seed)
    kl = list(range(1, nk + 1))
    al, bl, gl = list(range(100, 100 + na)), list(range(200, 200 + nb)), list(range(300, 300 + ng))
    if batch_on_top:
        perm = lambda xs: [int(v) for v in rng.permutation(xs)] if xs else []
        ks = perm(kl)
        first, rest = ks[:6], ks[6:]

        def lay(free):
            f, r = perm(free), perm(rest)
            split = int(rng.integers(1, len(free) + 1))
            return perm(first) + f[:split] + r[:3] + f[split:] + r[3:] + perm(gl)
        la, lb = lay(al), lay(bl)
    else:
        la = [int(v) for v in rng.permutation(al + gl + kl)]
        lb = [int(v) for v in rng.permutation(bl + gl + kl)]
    lc = [int(v) for v in rng.permutation(al + bl + gl)]
    A = rng.standard_normal((2,) * len(la)) + 1j * rng.standard_normal((2,) * len(la))
    B = rng.standard_normal((2,) * len(lb)) + 1j * rng.standard_normal((2,) * len(lb))
    cmds = [q.Load("a", "data_1", A.shape), q.Load("b", "data_2", B.shape),
            q.Ncon("c", tuple(lc), "a", tuple(la), "b", tuple(lb)), q.Save("output", "c")]
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", A), ("data_2", B)]), 0)
    letters = "abcdefghijklmnopqrstuvwxyzABCDEFGHIJKLMNOPQRSTUVWXYZ"
    idx = {v: letters[i] for i, v in enumerate(sorted(set(la + lb)))}
    sub = lambda ls: "".join(idx[v] for v in ls)
    ref = np.einsum(f"{sub(la)},{sub(lb)}->{sub(lc)}", A, B).reshape(-1, order="F")
    return prog, ref


# (summed bits, free bits of A, free bits of B, batch bits): P = the side with 32 free values (B
# when both have), Q with 8, 16 or 32; one batch value cuts K into ranges (FP64 partials)
JOIN_CASES = [(12, 5, 5, 3), (15, 5, 5, 0), (15, 5, 3, 2), (12, 4, 5, 4), (15, 5, 4, 1)]


@pytest.mark.parametrize("nk,na,nb,ng", JOIN_CASES)
def test_tensor_core_join(q, gpu_lib, nk, na, nb, ng):
    """The tensor-core join (3xTF32, operands split on the fly, FP64 drains every 128 terms):
    within the split-TF32 tolerance of einsum, equal to the CUDA-core batched GEMM within it, and
    the same bits on a second call."""
    prog, ref = join_programme(q, nk, na, nb, ng, seed=nk * 1000 + na * 100 + nb * 10 + ng)
    with q.Executor(prog, precision="split_tf32") as ex:
        got = ex.amplitudes([""])[0]
        got2 = ex.amplitudes([""])[0]
        desc = ex.explain(2)
        assert "tensor-core join" in desc and "copies=tma" in desc, desc
        assert ex.info()["num_steps_tensor_core"] == 1
    with q.Executor(prog, precision="split_tf32", cuda_core_joins=True) as ex:
        cc = ex.amplitudes([""])[0]
        assert "batched-gemm" in ex.explain(2)
    scale = np.max(np.abs(ref))
    err = np.max(np.abs(got - ref)) / scale
    print(f"tensor-core join {nk},{na},{nb},{ng}: {err:.2e} of the largest result; {desc.split('join ')[1][:90]}")
    assert err <= TOL["split_tf32"], err
    assert np.max(np.abs(got - cc)) / scale <= TOL["split_tf32"]
    assert np.array_equal(got, got2)
