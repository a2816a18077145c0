"""ctypes wrapper of the CPU FP64 oracle (qxoracle.c).  TEST INFRASTRUCTURE: imported only by
the tests, the smoke check and the benchmark's CPU-baseline leg, as the checker.

`run(programme_arrays, bitstrings, slices, nthreads)` executes a `.qx` programme given as the
C ABI's arrays (instructions, labels, leaf shapes and data) on the host cores and returns the
saved tensor per bitstring summed over the slice range, like libqxgpu's qxg_amplitudes.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "qxoracle.c"
    if force or not LIB.exists() or LIB.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)] + (["-B"] if force else []), check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        build()
        _lib = ct.CDLL(str(LIB))
        _lib.qxo_run.restype = ct.c_int
        _lib.qxo_max_threads.restype = ct.c_int
    return _lib


def max_threads() -> int:
    return load().qxo_max_threads()


def run(instrs, labels, data_rank, data_dims, data_flat, data_off, nqubits, bitstrings, slices=None,
        nthreads: int = 0, out_size: int = 1, num_slices: int | None = None) -> np.ndarray:
    """Oracle amplitudes: complex128 array (n, out_size)."""
    lib = load()
    ins = np.ascontiguousarray(instrs, dtype=np.int32)
    lab = np.ascontiguousarray(labels, dtype=np.int32)
    if lab.size == 0:
        lab = np.zeros(1, np.int32)
    dr = np.ascontiguousarray(data_rank, dtype=np.int32)
    dd = np.ascontiguousarray(data_dims, dtype=np.int64)
    if dd.size == 0:
        dd = np.zeros(1, np.int64)
    df = np.ascontiguousarray(data_flat, dtype=np.float64)
    do = np.ascontiguousarray(data_off, dtype=np.int64)
    if isinstance(bitstrings, str):
        bitstrings = [bitstrings]
    bits = "".join(bitstrings).encode("ascii") if nqubits else b"\0" * len(bitstrings)
    n = len(bitstrings)
    if slices is None:
        slices = (0, num_slices if num_slices is not None else 1)
    out = np.zeros(2 * n * out_size, dtype=np.float64)
    P = lambda a, t: a.ctypes.data_as(ct.POINTER(t))
    rc = lib.qxo_run(P(ins, ct.c_int32), ct.c_int(ins.shape[0]), P(lab, ct.c_int32), P(dr, ct.c_int32),
                     P(dd, ct.c_int64), P(do, ct.c_int64), P(df, ct.c_double), ct.c_int(dr.size),
                     ct.c_int(nqubits), ct.c_char_p(bits), ct.c_int(n), ct.c_int64(slices[0]),
                     ct.c_int64(slices[1]), ct.c_int(nthreads), P(out, ct.c_double), ct.c_int64(out_size))
    if rc != 0:
        raise RuntimeError(f"oracle failed with status {rc}")
    return out.view(np.complex128).reshape(n, out_size)


def run_programme(prog, bitstrings, slices=None, nthreads: int = 0, out_size: int = 1) -> np.ndarray:
    """Oracle run of a qxtools_gb300 Programme (duck-typed: instrs, labels, data...)."""
    flat, offs = prog.data_flat()
    return run(prog.instrs, prog.labels, prog.data_rank, prog.data_dims, flat, offs, prog.nqubits,
               bitstrings, slices=slices, nthreads=nthreads, out_size=out_size,
               num_slices=prog.num_slices)


def run_timed(prog, bitstring: str, max_seconds: float, slice_id: int = 0, nthreads: int = 0,
              out_size: int = 1):
    """CPU-baseline sample: one FP64 walk (one bitstring, one slice) using every thread inside
    the contractions, stopped after `max_seconds`.  -> (flops completed, seconds, finished)."""
    lib = load()
    flat, offs = prog.data_flat()
    ins = np.ascontiguousarray(prog.instrs, dtype=np.int32)
    lab = np.ascontiguousarray(prog.labels if prog.labels.size else np.zeros(1), dtype=np.int32)
    dr = np.ascontiguousarray(prog.data_rank, dtype=np.int32)
    dd = np.ascontiguousarray(prog.data_dims, dtype=np.int64)
    do = np.ascontiguousarray(offs, dtype=np.int64)
    df = np.ascontiguousarray(flat, dtype=np.float64)
    out = np.zeros(2 * out_size, dtype=np.float64)
    fl, sec = ct.c_double(0), ct.c_double(0)
    P = lambda a, t: a.ctypes.data_as(ct.POINTER(t))
    rc = lib.qxo_run_timed(P(ins, ct.c_int32), ct.c_int(ins.shape[0]), P(lab, ct.c_int32), P(dr, ct.c_int32),
                           P(dd, ct.c_int64), P(do, ct.c_int64), P(df, ct.c_double), ct.c_int(dr.size),
                           ct.c_int(prog.nqubits), ct.c_char_p(bitstring.encode() or b"\0"), ct.c_int64(slice_id),
                           ct.c_int(nthreads), ct.c_double(max_seconds), P(out, ct.c_double),
                           ct.c_int64(out_size), ct.byref(fl), ct.byref(sec))
    if rc not in (0, 1):
        raise RuntimeError(f"oracle failed with status {rc}")
    return fl.value, sec.value, rc == 0
