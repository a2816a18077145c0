"""qxg_ncon_tc_static: the tensor-core contraction for callers that cannot allocate device memory
(graph-capture code, hosts whose allocator belongs to another runtime, allocation-free loops).

It keeps its scratch in the library's static device array instead of cudaMalloc.  Checked through
the C ABI against the allocating entry point qxg_ncon (Complex64 storage, FP32 arithmetic) on
two calls in a row with different inputs, within the split-precision tolerances used by the
other tests (3xTF32 5e-6, 3xBF16 1e-4 of the largest element), on a plain shape, a split sum
and a shape processed in column blocks; shapes too large for the static array are rejected with
a message, and a programme walk afterwards is not failed by the static calls.  Kept in its own
file so it is collected last.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
TOL = {"split_tf32": 5e-6, "split_bf16": 1e-4}
PREC = {"split_bf16": 1, "split_tf32": 2}


def _declare(lib):
    P = ct.c_void_p
    lib.qxg_ncon_tc_static.argtypes = [ct.c_int32, P, ct.c_int32, ct.POINTER(ct.c_int32), P, ct.c_int32,
                                       ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), P, ct.c_int32,
                                       ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), P]
    lib.qxg_ncon_tc_static.restype = ct.c_int
    return lib


def _arr(x, t):
    a = np.ascontiguousarray(np.asarray(x, dtype=t))
    return a, a.ctypes.data_as(ct.POINTER(ct.c_int32 if t == np.int32 else ct.c_int64))


def _shapes(nm, nk, nn):
    la = list(range(1, nm + 1)) + list(range(100, 100 + nk))
    lb = list(range(100, 100 + nk)) + list(range(200, 200 + nn))
    lc = list(range(1, nm + 1)) + list(range(200, 200 + nn))
    return la, [2] * len(la), lb, [2] * len(lb), lc


def _call(lib, fn, precision, C, lc, A, la, ad, B, lb, bd):
    lc_, plc = _arr(lc, np.int32)
    la_, pla = _arr(la, np.int32)
    lb_, plb = _arr(lb, np.int32)
    ad_, pad = _arr(ad, np.int64)
    bd_, pbd = _arr(bd, np.int64)
    return getattr(lib, fn)(PREC[precision], ct.c_void_p(C.data_ptr()), len(lc), plc, ct.c_void_p(A.data_ptr()),
                            len(la), pla, pad, ct.c_void_p(B.data_ptr()), len(lb), plb, pbd, None)


# (free rows, summed, free columns) as powers of two: a plain tile walk; a summed extent of 2^11,
# cut into K blocks whose partial sums follow the planes in the array; and 2^12 columns by 2^10
# summed, whose planes (64 MiB of 3xTF32 words) are processed in outer column blocks to fit
SHAPES = [(9, 6, 5), (9, 11, 5), (8, 10, 12)]


@pytest.mark.parametrize("precision", ["split_tf32", "split_bf16"])
@pytest.mark.parametrize("shape", SHAPES)
def test_static_scratch_contraction_matches_allocating_entry_point(q, gpu_lib, precision, shape):
    import torch
    lib = _declare(gpu_lib)
    la, ad, lb, bd, lc = _shapes(*shape)
    g = torch.Generator(device="cuda").manual_seed(7)
    for call in range(2):                          # two calls in a row, new inputs each time
        A = torch.randn(2 ** len(la), dtype=torch.complex64, device="cuda", generator=g)
        B = torch.randn(2 ** len(lb), dtype=torch.complex64, device="cuda", generator=g)
        ref = torch.zeros(2 ** len(lc), dtype=torch.complex64, device="cuda")
        got = torch.full_like(ref, float("nan"))
        assert _call(lib, "qxg_ncon", precision, ref, lc, A, la, ad, B, lb, bd) == 0
        rc = _call(lib, "qxg_ncon_tc_static", precision, got, lc, A, la, ad, B, lb, bd)
        assert rc == 0, lib.qxg_last_error().decode()
        torch.cuda.synchronize()
        err = (got - ref).abs().max().item() / ref.abs().max().item()
        assert err <= TOL[precision], (call, err)


def test_static_scratch_rejects_oversized_shapes(q, gpu_lib):
    import torch
    lib = _declare(gpu_lib)
    # a summed extent of 2^16: even one block of 64 columns packs 64 MiB of 3xTF32 planes, more
    # than the static array holds
    la, ad, lb, bd, lc = _shapes(7, 16, 8)
    A = torch.zeros(2 ** len(la), dtype=torch.complex64, device="cuda")
    B = torch.zeros(2 ** len(lb), dtype=torch.complex64, device="cuda")
    C = torch.zeros(2 ** len(lc), dtype=torch.complex64, device="cuda")
    rc = _call(lib, "qxg_ncon_tc_static", "split_tf32", C, lc, A, la, ad, B, lb, bd)
    assert rc == -4
    assert "static scratch" in lib.qxg_last_error().decode()


def test_programme_walk_after_static_calls(q, gpu_lib):
    """The static entry point reports its waits to its own word, so a programme walk on the same
    GPU afterwards reads no stale timeout: a tensor-core programme returns QXG_OK and the right
    result."""
    import torch
    from collections import OrderedDict
    lib = _declare(gpu_lib)
    la, ad, lb, bd, lc = _shapes(9, 6, 5)
    A = torch.randn(2 ** len(la), dtype=torch.complex64, device="cuda")
    B = torch.randn(2 ** len(lb), dtype=torch.complex64, device="cuda")
    C = torch.zeros(2 ** len(lc), dtype=torch.complex64, device="cuda")
    assert _call(lib, "qxg_ncon_tc_static", "split_tf32", C, lc, A, la, ad, B, lb, bd) == 0
    rng = np.random.default_rng(5)
    shape_a, shape_b = (2,) * len(la), (2,) * len(lb)
    An = rng.standard_normal(shape_a) + 1j * rng.standard_normal(shape_a)
    Bn = rng.standard_normal(shape_b) + 1j * rng.standard_normal(shape_b)
    cmds = [q.Load("a", "data_1", An.shape), q.Load("b", "data_2", Bn.shape),
            q.Ncon("c", tuple(lc), "a", tuple(la), "b", tuple(lb)), q.Save("output", "c")]
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", An), ("data_2", Bn)]), 0)
    with q.Executor(prog, precision="split_tf32") as ex:
        got = ex.amplitudes([""])[0]
        assert ex.info()["num_steps_tensor_core"] == 1
    letters = "abcdefghijklmnopqrstuvwxyz"
    ids = {l: letters[i] for i, l in enumerate(sorted(set(la) | set(lb)))}
    sub = lambda ls: "".join(ids[l] for l in ls)
    ref = np.einsum(f"{sub(la)},{sub(lb)}->{sub(lc)}", An, Bn).reshape(-1, order="F")
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= TOL["split_tf32"]
