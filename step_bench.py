#!/usr/bin/env python3
"""Micro-benchmark of single contraction steps through the C ABI (`qxg_ncon`, FP32 CUDA cores).

The named cases are gate steps of the bench workloads, described by the bit layouts the planner
gives them (lowest address bit first): in X, `r` is a row bit (kept in the result), `b` a row
bit that Y also has (a bitstring-batch bit) and `k` a summed bit; in Y, `k` summed, `n` a
result column and `r` a batch bit; in C, `r`/`b` rows and `n` columns.  A trailing `s` on a name
times the adjoint of Y instead (the sum over every row of conj(X) and C: a long sum with a
small result; qxg_ncon does not conjugate, which changes no data movement).  `drop` removes the
highest row bits to shrink a case (for profiler captures).

    python step_bench.py rqc_1161,rqc_1159s [--drop 0] [--reps 10]

Prints one JSON line per case: milliseconds per call and the algorithmic bandwidth
8 (|X| + |Y| + |C|) bytes / time.

Final joins run only inside programmes (the tensor-core join is chosen by the programme compiler):
`--programme` times the JOINS cases as one-ncon split-TF32 programmes through the executor (the
step's own time from the executor's profile), `--cuda-core-joins` on the batched small GEMM.

    python step_bench.py join7x7 --programme [--cuda-core-joins] [--reps 5]
"""
from __future__ import annotations

import argparse
import ctypes as ct
import json
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent

# (X bits, Y bits, C bits) of the planned steps (rqc_5x5_d12_open6 and param_5x5_l12, pinned
# plan seeds, 64 / 256 bitstrings per pass)
CASES = {
    "rqc_1157": ("kkrrrrrrrrkrrrrrrrrrrrrrr", "nknknk", "nnrrrrrrrrnrrrrrrrrrrrrrr"),
    "rqc_1159": ("kbrrbrrrrrrrbrbbrbrrkkrrrrrrr", "nrrrrrrnkkk", "nbrrbrrrrrrrbrbbrbrrnrrrrrrr"),
    "rqc_1161": ("rrkrrrrkrrrrrrrrrrrkrrrrkrrr", "nkkkkn", "rrnrrrrnrrrrrrrrrrrrrrrrrr"),
    "rqc_1162": ("kbkrbrrrrrrkbrbbrbkrrrkrrr", "krrrrrrkknnkk", "nbnrbrrrrrrbrbbrbrrrrrr"),
    "param_1521": ("rrrrrrrrrrrrkrrrrrrkrrrrrr", "nnkk", "rrrrrrrrrrrrnrrrrrrnrrrrrr"),
    "param_1534": ("rrrrrrrrrrkrrrrrkkrrrrrrrrrrrrk", "nnkkkk", "rrrrrrrrrrnrrrrrnrrrrrrrrrrrr"),
    # final joins (the batched small GEMM), with fewer batch / summed bits than the full passes:
    # 7x7 stand-in: 32 x 32 results per batch value, 2^17 summed, 2^5 batch values (2^11 in a pass)
    "join_7x7": ("rrrrbkkrbkkkkbkkkbkkkbkkkkk", "nnnnrkknrkkkkrkkkrkkkrkkkkk", "rrrrbnnnnnrbbbb"),
    # 6x6, 14 cycles: 64 x 16 results per batch value, 2^16 summed (2^22 in a pass), 2^5 batch values
    "join_6x6": ("kbbbbbrkkkrrrkkrrkkkkkkkkkk", "kkkkknnnnrrrrrkkkkkkkkkkk", "bbbbbrrrrrrnnnn"),
}


# Final joins (programme mode): A's, B's and C's index bits from the lowest address bit, as named
# in qxg_program_explain (k summed, m free in A, n free in B, b batch).
_K = ["k%d" % i for i in range(17)]
JOINS = {
    # the 7x7 stand-in's final join (2^17 summed terms, 32 x 32 results per batch value) with 2^5
    # of its 2^11 batch values: 1 GiB per operand
    "join7x7": (_K[:14] + ["m0", "k14", "m1", "m2", "k15", "m3", "m4", "k16"] + ["b%d" % i for i in range(5)],
                "k3,k4,k13,n0,n1,k2,k1,k11,n2,n3,k16,k0,n4,k12,k5,k6,k15,k8,k14,k7,k10,k9".split(",")
                + ["b%d" % i for i in range(5)],
                ["m%d" % i for i in range(5)] + ["n%d" % i for i in range(5)] + ["b%d" % i for i in range(5)]),
}


def run_join(name: str, reps: int, cuda_core_joins: bool):
    """One JOINS case as a one-ncon split-TF32 programme: milliseconds per call of the step."""
    from collections import OrderedDict
    import __graft_entry__ as entry
    q = entry.load()
    a_bits, b_bits, c_bits = JOINS[name]
    lab = {n: i + 1 for i, n in enumerate(sorted(set(a_bits) | set(b_bits)))}
    rng = np.random.default_rng(1)

    def rnd(n):
        x = rng.standard_normal(2 ** n, dtype=np.float32) + 1j * rng.standard_normal(2 ** n, dtype=np.float32)
        return x.astype(np.complex128).reshape((2,) * n)
    A, B = rnd(len(a_bits)), rnd(len(b_bits))
    cmds = [q.Load("a", "data_1", A.shape), q.Load("b", "data_2", B.shape),
            q.Ncon("c", tuple(lab[x] for x in c_bits), "a", tuple(lab[x] for x in a_bits), "b",
                   tuple(lab[x] for x in b_bits)), q.Save("output", "c")]
    prog = q.Programme.from_commands(cmds, OrderedDict([("data_1", A), ("data_2", B)]), 0)
    del A, B
    nbytes = 8 * (2 ** len(a_bits) + 2 ** len(b_bits) + 2 ** len(c_bits))
    with q.Executor(prog, precision="split_tf32", cuda_core_joins=cuda_core_joins) as ex:
        ex.amplitudes([""])
        form = ex.explain(2)
        best = None
        for _ in range(reps):
            ex.profile(True)                # clears the records of the previous call
            ex.amplitudes([""])
            rows, _ = ex.profile_read()
            ms = sum(r["ms"] for r in rows if r["instr"] == 2)
            best = ms if best is None else min(best, ms)
        ex.profile(False)
    print(json.dumps({"case": name, "programme": True, "form": form.split(" c_bits=")[0], "ms": round(best, 4),
                      "gb_s": round(nbytes / best / 1e6, 1)}), flush=True)


def labels(x: str, y: str, c: str, drop: int):
    """ncon labels of X, Y, C for bit strings x, y, c (one binary label per bit)."""
    if drop:
        xi = [i for i, ch in enumerate(x) if ch == "r"]
        for i in sorted(xi[-drop:], reverse=True):
            x = x[:i] + x[i + 1:]
        ci = [i for i, ch in enumerate(c) if ch == "r"]
        for i in sorted(ci[-drop:], reverse=True):
            c = c[:i] + c[i + 1:]
    lx, rows, bats, ks = [], [], [], []
    for ch in x:
        if ch in "rb":
            lab = 1000 + len(rows)
            rows.append(lab)
            lx.append(lab)
            if ch == "b":
                bats.append(lab)
        else:
            lab = 2000 + len(ks)
            ks.append(lab)
            lx.append(lab)
    ly, kj, bj, nj = [], 0, 0, 0
    for ch in y:
        if ch == "k":
            ly.append(ks[kj])
            kj += 1
        elif ch == "r":
            ly.append(bats[bj])
            bj += 1
        else:
            ly.append(3000 + nj)
            nj += 1
    lc, ri, ni = [], 0, 0
    for ch in c:
        if ch in "rb":
            lc.append(rows[ri])
            ri += 1
        else:
            lc.append(3000 + ni)
            ni += 1
    return lx, ly, lc


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("cases", help="comma-separated case names (" + ", ".join(CASES) + "; suffix s: adjoint of Y)")
    ap.add_argument("--drop", type=int, default=0)
    ap.add_argument("--reps", type=int, default=10)
    ap.add_argument("--lib", default=str(HERE / "qxtools.jl_gb300" / "_build" / "libqxgpu.so"))
    ap.add_argument("--programme", action="store_true", help="JOINS cases through the executor")
    ap.add_argument("--cuda-core-joins", action="store_true", help="programme mode: the batched small GEMM")
    args = ap.parse_args()
    if args.programme:
        for name in args.cases.split(","):
            run_join(name, args.reps, args.cuda_core_joins)
        return
    import torch
    lib = ct.CDLL(args.lib)
    P = ct.c_void_p
    lib.qxg_ncon.argtypes = [ct.c_int32, P, ct.c_int32, P, P, ct.c_int32, P, P, P, ct.c_int32, P, P, P]
    lib.qxg_ncon.restype = ct.c_int
    lib.qxg_last_error.restype = ct.c_char_p
    for name in args.cases.split(","):
        ysum = name.endswith("s")
        lx, ly, lc = labels(*CASES[name[:-1] if ysum else name], args.drop)
        if ysum:   # the adjoint of Y: sum over every row of X and C
            ks = [v for v in lx if v not in lc]
            ns = [v for v in lc if v not in lx]
            bs = [v for v in lx if v in ly and v in lc]
            lx, ly, lc = lx, lc, ks + ns + bs
        X = torch.randn(2 ** len(lx), dtype=torch.complex64, device="cuda")
        Y = torch.randn(2 ** len(ly), dtype=torch.complex64, device="cuda")
        C = torch.empty(2 ** len(lc), dtype=torch.complex64, device="cuda")
        arr = lambda v, t: np.ascontiguousarray(np.array(v, dtype=t))
        a_l, a_d = arr(lx, np.int32), arr([2] * len(lx), np.int64)
        b_l, b_d = arr(ly, np.int32), arr([2] * len(ly), np.int64)
        c_l = arr(lc, np.int32)

        def call():
            r = lib.qxg_ncon(3, C.data_ptr(), len(lc), c_l.ctypes.data, X.data_ptr(), len(lx), a_l.ctypes.data,
                             a_d.ctypes.data, Y.data_ptr(), len(ly), b_l.ctypes.data, b_d.ctypes.data, None)
            if r != 0:
                raise RuntimeError(lib.qxg_last_error().decode())

        for _ in range(3):
            call()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(args.reps):
            call()
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.reps
        nbytes = 8 * (X.numel() + Y.numel() + C.numel())
        nk = len([v for v in lx if v in ly and v not in lc])
        flops = 8.0 * C.numel() * 2 ** nk
        print(json.dumps({"case": name, "drop": args.drop, "x_log2": len(lx), "y_log2": len(ly), "c_log2": len(lc),
                          "ms": round(ms, 4), "gb_s": round(nbytes / ms / 1e6, 1),
                          "tflop_s": round(flops / ms / 1e9, 2)}), flush=True)
        del X, Y, C


if __name__ == "__main__":
    main()
