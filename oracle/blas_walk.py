"""BLAS walk of a `.qx` programme: the CPU path's arithmetic as the reference performs it.
TEST INFRASTRUCTURE: imported only by the tests and the benchmark's CPU-baseline legs, as the
timed CPU baseline; the product (libqxgpu) never calls it.

The reference contracts each plan step with TensorOperations "3.1" (Project.toml:33-38, called
through QXTns' `contract_tn!` at src/simulation.jl:89 and `contract_pair!` at
src/compute_graph/compute_graph.jl:65-73).  For BLAS element types TensorOperations' pairwise
contraction permutes both operands into matrix form (free labels x summed labels), multiplies
them with one BLAS GEMM (zgemm for ComplexF64) and permutes the product into the result's label
order.  This module restates that algorithm: the permutations are threaded gathers
(`qxo_permute_copy` in qxoracle.c, OpenMP over every host core, as Strided.jl threads
permutedims) and the product is `np.matmul` (OpenBLAS zgemm, every host core).  Labels in both
operands and the result (hyper-indices) become the GEMM batch.  The command semantics (load /
view / output / ncon / save, docs/src/users_guide.md:93-165) are the same as the C oracle's
(qxoracle.c); tests check the two against each other and against the golden vectors.

Tensors are held as numpy arrays with one axis per label in label order; leaf data is
column-major like Julia's, so it is read with order="F" and the saved tensor is written back
with order="F".
"""
from __future__ import annotations

import ctypes as ct
import os
import time

import numpy as np

OP_LOAD, OP_VIEW, OP_OUTPUT, OP_NCON, OP_SAVE = 1, 2, 3, 4, 5
_R = 1.0 / np.sqrt(2.0)
_BASIS = {"0": (1.0, 0.0), "1": (0.0, 1.0), "+": (_R, _R), "-": (_R, -_R)}


def blas_threads() -> int:
    """Threads numpy's BLAS runs with: OpenBLAS's own count when its library is loaded in this
    process (found by its exported name), else the host's CPU count (OpenBLAS's default)."""
    libs = set()
    try:
        with open("/proc/self/maps") as f:
            for ln in f:
                path = ln.split()[-1]
                base = os.path.basename(path).lower()
                if "openblas" in base and ".so" in base:
                    libs.add(path)
    except OSError:
        pass
    for path in sorted(libs):
        try:
            lib = ct.CDLL(path)
        except OSError:
            continue
        for name in ("scipy_openblas_get_num_threads64_", "scipy_openblas_get_num_threads",
                     "openblas_get_num_threads64_", "openblas_get_num_threads"):
            fn = getattr(lib, name, None)
            if fn is not None:
                fn.restype = ct.c_int
                n = int(fn())
                if n > 0:
                    return n
    return os.cpu_count() or 1


_lib = None
_GATHER_MIN = 1 << 14   # smaller permutations stay in numpy (the call costs more than the copy)


def _oracle_lib():
    global _lib
    if _lib is None:
        from . import oracle
        _lib = oracle.load()
        _lib.qxo_permute_copy.restype = ct.c_int
    return _lib


def _contiguous(x):
    """x (any strided complex128 view) copied into C order by the threaded gather.  Axes of size
    1 are dropped, neighbours that are already contiguous in x are merged, and merged runs longer
    than 64 elements are split into pieces of 64 first."""
    if x.flags.c_contiguous:
        return x
    if x.size < _GATHER_MIN:
        return np.ascontiguousarray(x)
    dims, strides = [], []
    for n, st in zip(x.shape, x.strides):
        if n == 1:
            continue
        st //= x.itemsize
        if dims and strides[-1] == st * n:
            dims[-1] *= n
            strides[-1] = st
        else:
            dims.append(n)
            strides.append(st)
    # long runs are split into pieces of 64 so that the gather's tiles stay small and many
    sd, ss = [], []
    for n, st in zip(dims, strides):
        parts = []
        while n > 64 and n % 64 == 0:
            parts.append((64, st))
            n //= 64
            st *= 64
        parts.append((n, st))
        for n2, st2 in reversed(parts):
            sd.append(n2)
            ss.append(st2)
    dims, strides = sd, ss
    out = np.empty(x.shape, dtype=np.complex128)
    d = np.array(dims, dtype=np.int64)
    s = np.array(strides, dtype=np.int64)
    P = lambda a, t: a.ctypes.data_as(ct.POINTER(t))
    rc = _oracle_lib().qxo_permute_copy(ct.c_void_p(x.ctypes.data), ct.c_void_p(out.ctypes.data),
                                        ct.c_int(len(dims)), P(d, ct.c_int64), P(s, ct.c_int64))
    if rc != 0:
        raise RuntimeError(f"qxo_permute_copy failed with status {rc}")
    return out


def blas_name() -> str:
    """numpy's BLAS as its build configuration names it (e.g. "scipy-openblas 0.3.x")."""
    try:
        d = np.show_config(mode="dicts")["Build Dependencies"]["blas"]
        return f"{d.get('name', '?')} {d.get('version', '')}".strip()
    except Exception:   # older numpy without mode="dicts", or a build without the section
        return "unknown BLAS"


def _leaf(flat, offs, dims_list, i):
    dims = dims_list[i]
    n = int(np.prod(dims)) if len(dims) else 1
    z = flat[2 * offs[i]: 2 * (offs[i] + n)].view(np.complex128)
    return z.reshape(tuple(dims), order="F")


def _sum_lone_labels(T, lt, other, lc):
    """Sum out labels of one operand that appear in neither the other operand nor the result,
    and take diagonals of labels repeated within the operand (the C oracle's strides add up)."""
    labels = list(lt)
    # repeated labels within one operand: keep the diagonal
    while len(set(labels)) != len(labels):
        seen = {}
        for ax, l in enumerate(labels):
            if l in seen:
                T = np.diagonal(T, axis1=seen[l], axis2=ax)   # diagonal moves to the last axis
                labels = [x for k, x in enumerate(labels) if k not in (seen[l], ax)] + [l]
                break
            seen[l] = ax
    lone = [ax for ax, l in enumerate(labels) if l not in other and l not in lc]
    if lone:
        T = T.sum(axis=tuple(lone))
        labels = [l for ax, l in enumerate(labels) if ax not in lone]
    return T, labels


def ncon(A, la, B, lb, lc):
    """C[lc] = sum over labels not in lc of A[la] B[lb], as permute + batched GEMM + permute."""
    A, la = _sum_lone_labels(np.asarray(A), la, set(lb), set(lc))
    B, lb = _sum_lone_labels(np.asarray(B), lb, set(la), set(lc))
    sa, sb, sc = set(la), set(lb), set(lc)
    dim = {l: A.shape[k] for k, l in enumerate(la)}
    for k, l in enumerate(lb):
        if l in dim and dim[l] != B.shape[k]:
            raise ValueError(f"label {l}: dimension {dim[l]} in the first operand, {B.shape[k]} in the second")
        dim[l] = B.shape[k]
    for l in lc:
        if l not in dim:
            raise ValueError(f"result label {l} is in neither operand")
    batch = [l for l in lc if l in sa and l in sb]
    free_a = [l for l in lc if l in sa and l not in sb]
    free_b = [l for l in lc if l in sb and l not in sa]
    summed = [l for l in la if l in sb and l not in sc]
    size = lambda ls: int(np.prod([dim[l] for l in ls])) if ls else 1
    pa = [la.index(l) for l in batch + free_a + summed]
    pb = [lb.index(l) for l in batch + summed + free_b]
    Am = _contiguous(A.transpose(pa)).reshape(size(batch), size(free_a), size(summed))
    Bm = _contiguous(B.transpose(pb)).reshape(size(batch), size(summed), size(free_b))
    Cm = np.matmul(Am, Bm)
    order = batch + free_a + free_b
    C = Cm.reshape(tuple(dim[l] for l in order))
    return C.transpose([order.index(l) for l in lc]), 8.0 * size(lc) * size(summed)


def walk(prog, bitstring: str, slice_id: int = 0, deadline: float | None = None):
    """One walk of the programme for one bitstring and one slice.
    -> (saved tensor flattened column-major or None if stopped, FLOPs of completed steps)."""
    flat, offs = prog.data_flat()
    flat = np.ascontiguousarray(flat, dtype=np.float64)
    ranks = [int(r) for r in prog.data_rank]
    dims_list, o = [], 0
    for r in ranks:
        dims_list.append([int(d) for d in prog.data_dims[o:o + r]])
        o += r
    ins = np.asarray(prog.instrs, dtype=np.int64).reshape(-1, 10)
    labels = np.asarray(prog.labels, dtype=np.int64)
    vdim = {}
    for I in ins:
        if I[0] == OP_VIEW:
            vdim[int(I[3])] = int(I[5])
    vval, s = {}, slice_id
    for j in range(max(vdim) + 1 if vdim else 0):
        vval[j] = s % vdim[j]
        s //= vdim[j]
    last = {}
    for n, I in enumerate(ins):
        if I[0] == OP_VIEW:
            last[int(I[2])] = n
        elif I[0] == OP_NCON:
            last[int(I[2])] = n
            last[int(I[3])] = n
    T, flops = {}, 0.0
    for n, I in enumerate(ins):
        if deadline is not None and time.perf_counter() > deadline:
            return None, flops
        op, dst, a, b, pos, d, nc, na, nb, lo = (int(x) for x in I)
        if op == OP_LOAD:
            T[dst] = _leaf(flat, offs, dims_list, a)
        elif op == OP_VIEW:
            t = T[a]
            idx = [slice(None)] * t.ndim
            idx[pos] = slice(vval[b], vval[b] + 1)
            T[dst] = t[tuple(idx)]
        elif op == OP_OUTPUT:
            if b != 2:
                raise ValueError(f"instruction {n}: output dimension {b}, not 2")
            T[dst] = np.array(_BASIS[bitstring[a]], dtype=np.complex128)
        elif op == OP_NCON:
            l = labels[lo:lo + nc + na + nb].tolist()
            lc, la, lb = l[:nc], l[nc:nc + na], l[nc + na:]
            if T[a].ndim != na or T[b].ndim != nb:
                raise ValueError(f"instruction {n}: operand ranks do not match the labels")
            T[dst], f = ncon(T[a], la, T[b], lb, lc)
            flops += f
        elif op == OP_SAVE:
            return np.asarray(T[a]).reshape(-1, order="F").copy(), flops
        else:
            raise ValueError(f"instruction {n}: unknown op {op}")
        for t in [k for k, v in last.items() if v == n]:
            T.pop(t, None)
    raise ValueError("programme has no save command")


def run_programme(prog, bitstrings, slices=None) -> np.ndarray:
    """Amplitudes summed over the slice range (default: all slices), complex128 (n, out_size),
    like the C oracle's run_programme."""
    if isinstance(bitstrings, str):
        bitstrings = [bitstrings]
    lo, hi = slices if slices is not None else (0, prog.num_slices)
    rows = []
    for x in bitstrings:
        acc = None
        for s in range(lo, hi):
            r, _ = walk(prog, x, s)
            acc = r if acc is None else acc + r
        rows.append(acc)
    return np.stack(rows)


def run_timed(prog, bitstring: str, max_seconds: float, slice_id: int = 0):
    """CPU-baseline sample: one walk (one bitstring, one slice) with BLAS on every host core,
    stopped at the first instruction boundary after `max_seconds`.
    -> (FLOPs of completed contractions, seconds, finished)."""
    t0 = time.perf_counter()
    r, flops = walk(prog, bitstring, slice_id, deadline=t0 + max_seconds)
    return flops, time.perf_counter() - t0, r is not None
