"""Output sampling over GPU amplitude batches (the `Rejection` and `Uniform` output methods).

`output_params_dict` (src/outputs.jl:47-78) describes three output methods; QXContexts (un-vendored)
implements them.  `List` is the executor's bitstring list.  Here:

* `rejection_sample`: empirical supremum rejection sampling (docs/src/features.md:68-83) of
  bitstrings x with probability p(x) = |<x|C|0>|^2.  Candidates are drawn uniformly (q(x) = 2^-n),
  their amplitudes are computed on the GPU in batches, and a candidate is accepted with probability
  p(x) 2^n / M.  Unless `fix_M` is set, M is raised to the largest p(x) 2^n seen so far before the
  acceptance test (the empirical supremum); `fix_M` keeps M fixed (frugal rejection sampling).
* `uniform_amplitudes`: amplitudes of `num_samples` uniformly drawn bitstrings (the `Uniform`
  method).

Seeds drive numpy's PCG64, so draws are reproducible here but differ from Julia's.
"""
from __future__ import annotations

import numpy as np

__all__ = ["rejection_sample", "uniform_amplitudes", "run_output_method"]


def _random_bitstrings(rng, n_qubits: int, count: int) -> list:
    bits = rng.integers(0, 2, size=(count, n_qubits))
    return ["".join("01"[b] for b in row) for row in bits]


def uniform_amplitudes(executor, n_qubits: int, num_samples: int, seed=None):
    """(bitstrings, amplitudes) of `num_samples` uniformly drawn bitstrings."""
    rng = np.random.Generator(np.random.PCG64(0 if seed is None else int(seed)))
    bits = _random_bitstrings(rng, n_qubits, num_samples)
    return bits, executor.amplitudes(bits)[:, 0]


def rejection_sample(executor, n_qubits: int, num_samples: int, M: float = 1e-4, fix_M: bool = False,
                     seed=None, batch: int = 256, max_candidates: int | None = None):
    """Draw `num_samples` bitstrings distributed as |amplitude|^2.

    Returns (samples, amplitudes of the samples, statistics dict).  `batch` candidates are
    contracted per GPU call; `max_candidates` bounds the work (default 1000 x num_samples)."""
    rng = np.random.Generator(np.random.PCG64(0 if seed is None else int(seed)))
    dim = 2.0 ** n_qubits
    max_candidates = max_candidates or 1000 * num_samples
    samples, amps = [], []
    drawn = 0
    while len(samples) < num_samples and drawn < max_candidates:
        cand = _random_bitstrings(rng, n_qubits, batch)
        a = executor.amplitudes(cand)[:, 0]
        u = rng.random(batch)
        drawn += batch
        for x, ax, ux in zip(cand, a, u):
            r = (abs(ax) ** 2) * dim           # p(x) / q(x)
            if not fix_M and r > M:
                M = r
            if ux < r / M:
                samples.append(x)
                amps.append(ax)
                if len(samples) == num_samples:
                    break
    stats = {"candidates": drawn, "accepted": len(samples), "M": M,
             "acceptance": len(samples) / max(drawn, 1)}
    return samples, np.array(amps), stats


def run_output_method(executor, params: dict, n_qubits: int):
    """Execute a `.yml` `output:` block (List, Uniform or Rejection) on the GPU executor.
    Returns (bitstrings, amplitudes)."""
    method = params["method"]
    p = params["params"]
    if method == "List":
        bits = list(p["bitstrings"])
        return bits, executor.amplitudes(bits)[:, 0]
    if method == "Uniform":
        return uniform_amplitudes(executor, n_qubits, int(p["num_samples"]), p.get("seed"))
    if method == "Rejection":
        s, a, _ = rejection_sample(executor, n_qubits, int(p["num_samples"]), M=float(p.get("M", 1e-4)),
                                   fix_M=bool(p.get("fix_M", False)), seed=p.get("seed"))
        return s, a
    raise ValueError(f"output method {method!r} not supported")
