#!/usr/bin/env python3
"""Benchmark of the GB300 contraction executor (amplitudes/s and TFLOP/s): the split-precision
batched executor against the plain ComplexF64 GPU executor on the same programme.

Workload (default `rqc_7x7_d10_w22`): a seeded 7x7-grid random circuit (49 qubits), 10 cycles of
{sqrt X, sqrt Y, sqrt W} + fSim(pi/2, pi/6) (pattern ABCDCDAB), two-qubit gates decomposed,
planned by the library's planner and sliced until every intermediate has at most 2^22 elements
(8 slices), compiled into a `.qx` programme as generate_simulation_files does, with 1024 seeded
bitstrings.  It stands in for the 7x7, 16-cycle precision configuration (<= 2^28 elements with
about 2^10 slices), for which no contraction tree exists within that budget: every balanced
split of the 16-cycle network cuts all 49 qubit wires.  Synthetic, seeded data.

A step is one pass of the programme over one batch of bitstrings (`--bits-per-step`, default
all 1024) and all its slices.  `value` times steps of the split-precision executor
(`--precision`, default 3xTF32) with the bitstrings already in HBM (the device entry point
qxg_amplitudes_device); `e2e` times the same steps through the host entry point qxg_amplitudes
with pinned host buffers (bitstrings copied in, amplitudes copied out, every step).  The FP64
arm (`fp64`) runs the plain ComplexF64 executor on the first `--fp64-bits` bitstrings of the
same list, and the line reports the ratio of the two rates and the error of the split arm's
amplitudes against the FP64 ones, per amplitude.  Intermediates exceed L2 (largest intermediate
reported in `config`).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|fp32|split_bf16|split_tf32]
                    [--workload NAME] [--fp64-bits N] [--fp64-steps K] [--no-fp64]
    python bench.py --impl reference ...   # the reference's CPU arithmetic (permute + OpenBLAS
                                           # zgemm per ncon, oracle/blas_walk.py) on the host cores
Under torchrun (N > 1) every rank runs its own replica on its own shard of bitstrings (the
path shards by bitstring with no exchange) and the slowest rank's time is reported.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "amplitudes/s & TFLOP/s: split-prec batched vs FP64 GPU path at <=1e-5 rel err"
UNIT = "amplitudes/s"


def parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="rqc_7x7_d10_w22")
    ap.add_argument("--precision", default="split_tf32", choices=["fp64", "fp32", "split_bf16", "split_tf32"])
    ap.add_argument("--bits-per-step", type=int, default=0, help="bitstrings per step (0: the workload's list)")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--plan-seed", type=int, default=None, help="planner seed (default: the workload's pinned one)")
    ap.add_argument("--planner", default=None, choices=["python", "native"],
                    help="plan with the Python stand-in or the library's planner (default: the workload's)")
    ap.add_argument("--cpu-seconds", type=float, default=20.0, help="CPU-baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64-bits", type=int, default=0,
                    help="bitstrings of the FP64 arm, the first ones of the split arm's list (0: all of them)")
    ap.add_argument("--fp64-steps", type=int, default=1, help="timed steps of the FP64 arm (after one warm-up)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 arm and the error")
    ap.add_argument("--no-graphs", action="store_true", help="launch every kernel eagerly (no CUDA graphs)")
    ap.add_argument("--tuning-file", default=None,
                    help="read the autotuner's decisions from this file if it exists, else write them after warm-up "
                         "(so a profiler run repeats the plain run's variants)")
    ap.add_argument("--tc-tuning", default="auto",
                    help="tensor-core tile variants: 'auto' (timed per step) or candidate number k >= 1")
    ap.add_argument("--gradient", action="store_true",
                    help="only the reverse-mode gradient against the forward pass (parametrised 5x5 circuit)")
    ap.add_argument("--no-gradient", action="store_true",
                    help="leave out the gradient leg of the default line (gradient / forward on the parametrised "
                         "5x5 circuit, with its error against FP64)")
    return ap.parse_args()


# --------------------------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier_max(value: float, ws: int, backend_dev):
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device=backend_dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"qxg_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sms, maxs, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sms.append(float(p[1]))
                maxs.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        self.path.unlink(missing_ok=True)
        if not sms:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        return {"sm_mhz": statistics.median(sms), "sm_max_mhz": max(maxs), "reasons": sorted(reasons),
                "samples": len(sms)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d, "MEASURED_PEAKS.json"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def fp64_peak_tflops(torch, dev) -> float:
    """FP64 peak of this GPU measured here: cuBLAS DGEMM 4096^3 (torch.matmul), best of 5."""
    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    for _ in range(2):
        a @ b
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = max(best, 2 * 4096 ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    return best


def traffic_summary(workload: str, kernel: str, precision: str):
    """DRAM bytes per launch of the dominant kernel from a committed ncu summary, if any."""
    p = ROOT / "profiles" / f"{kernel}_{workload}_{precision}.json"
    if p.exists():
        try:
            d = json.loads(p.read_text())
            return d.get("dram_bytes_per_launch"), d
        except ValueError:
            pass
    return None, None


# --------------------------------------------------------------------------------------------
def cpu_sample(prog, bits, info, seconds: float, start: int = 0):
    """FP64 walks (oracle/blas_walk.py) of (bitstring, slice) pairs in order from bitstring
    `start`, slice 0, until `seconds` have passed; the last walk may stop at an instruction
    boundary.  -> (FLOPs of completed contractions, seconds, walks completed, walks started)."""
    from oracle import blas_walk
    nsl = max(1, int(info["num_slices"]))
    flops, sec, done, started, k = 0.0, 0.0, 0, 0, 0
    while sec < seconds:
        b, sl = bits[(start + k // nsl) % len(bits)], k % nsl
        f, t, fin = blas_walk.run_timed(prog, b, seconds - sec, slice_id=sl)
        flops += f
        sec += t
        done += int(fin)
        started += 1
        k += 1
    return flops, sec, done, started


def cpu_baseline(prog, bits, info, seconds: float):
    """The reference's CPU arithmetic restated (oracle/blas_walk.py: permute + OpenBLAS zgemm per
    ncon, as TensorOperations contracts) on a bounded sample: walks of one bitstring and one slice
    each, in order, with BLAS on every host thread, for `seconds`; the FLOP rate is converted to
    amplitudes/s with the programme's FLOPs per bitstring (all slices)."""
    from oracle import blas_walk
    cores = blas_walk.blas_threads()
    out_size = info["amplitudes_per_bitstring"]
    flops, sec, done, started = cpu_sample(prog, bits, info, seconds)
    rate = flops / max(sec, 1e-9)
    amps = rate / info["flops_per_bitstring"] * out_size
    sample = (f"FP64 walks (threaded permute + {blas_walk.blas_name()} zgemm per ncon) of (bitstring, slice) pairs of "
              f"{info['name']} in order for {sec:.1f} s ({done} walks complete of {started} started, "
              f"{flops:.3e} FLOPs); amplitudes/s = FLOP rate / {info['flops_per_bitstring']:.3e} FLOPs per "
              f"bitstring (all {info['num_slices']} slices) x {out_size} amplitudes per bitstring")
    return {"value": amps, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample,
            "gflops": rate / 1e9, "executed_flops_per_amplitude": info["flops_per_bitstring"] / out_size}


def run_reference(args):
    ws, rank, local = dist_env()
    if ws > 1 and rank != 0:
        return
    import __graft_entry__ as entry
    q = entry.load()
    from oracle import blas_walk
    prog, bits, info = q.workloads.build_workload(args.workload, seed=args.seed, plan_seed=args.plan_seed,
                                                  planner=args.planner)
    cores = blas_walk.blas_threads()
    out_size = info["amplitudes_per_bitstring"]
    # each step is a bounded sample (the whole run stays within a few minutes)
    per = max(1.0, min(args.cpu_seconds, 150.0 / max(1, args.steps + args.warmup)))
    for w in range(args.warmup):
        cpu_sample(prog, bits, info, min(per, 3.0), start=w)
    fl_tot, sec_tot, done, started = 0.0, 0.0, 0, 0
    t0 = time.perf_counter()
    for k in range(args.steps):
        fl, sec, d, st = cpu_sample(prog, bits, info, per, start=k * 7)
        fl_tot += fl
        sec_tot += sec
        done += d
        started += st
    wall = time.perf_counter() - t0
    rate = fl_tot / sec_tot
    value = rate / info["flops_per_bitstring"] * out_size
    sample = (f"each step: {per:.1f} s of FP64 walks of (bitstring, slice) pairs (threaded permute + "
              f"{blas_walk.blas_name()} zgemm per ncon, as TensorOperations contracts; {done} walks complete of "
              f"{started} started over all steps); amplitudes/s = FLOP rate / {info['flops_per_bitstring']:.3e} "
              f"FLOPs per bitstring (all {info['num_slices']} slices) x {out_size} amplitudes")
    cfg = workload_config(info, args, None)
    cfg.update({"precision": "fp64", "executor": "CPU: permute + zgemm per ncon (TensorOperations' algorithm)",
                "threads": cores})
    for k in ("cuda_graphs", "tc_tuning"):
        cfg.pop(k, None)
    cfg["arm"] = "reference CPU arithmetic, restated (oracle/blas_walk.py)"
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": cfg,
            "executed_flops_per_amplitude": info["flops_per_bitstring"] / out_size,
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "tflops": rate / 1e12}
    print(json.dumps(line), flush=True)


def workload_config(info, args, ex_info):
    cfg = {"workload": info["name"], "grid": f"{info['spec']['rows']}x{info['spec']['cols']}",
           "cycles": info["spec"]["depth"], "gate_set": "sqrtX/sqrtY/sqrtW + fSim(pi/2,pi/6), ABCDCDAB",
           "open_qubits": len(info["open_qubits"]), "bitstrings": len(info["bitstrings"]),
           "amplitudes_per_bitstring": info["amplitudes_per_bitstring"], "slices": info["num_slices"],
           "plan_steps": info["plan_steps"], "max_intermediate_log2": info["max_log2"],
           "flops_per_bitstring": info["flops_per_bitstring"], "seed": info["seed"],
           "planner": info["spec"].get("planner", "python"),
           "precision": args.precision, "cuda_graphs": not args.no_graphs,
           "l2": "intermediates larger than L2 (no flush needed)", "arm": "split-precision batched executor"}
    if info["name"] == "rqc_7x7_d10_w22":
        cfg["stands_in_for"] = ("7x7 grid, 16 cycles, every intermediate <= 2^28 elements with about 2^10 slices, 1024 "
                                "amplitudes: at 16 cycles that width target takes more than 2^20 slices and 2^60 FLOPs "
                                "per amplitude, so the 7x7 circuit runs at 10 cycles (<= 2^22 elements, 8 slices)")
    if ex_info:
        cfg.update({"bitstring_batch": ex_info["bitstring_batch"], "slice_batch": ex_info["slice_batch"],
                    "workspace_bytes": ex_info["workspace_bytes"],
                    "tensor_core_steps": ex_info["num_steps_tensor_core"],
                    "fused_gather_steps": ex_info["num_steps_fused"],
                    "autotuned_steps": ex_info["num_steps_tuned"], "tc_tuning": args.tc_tuning})
    return cfg


def error_stats(got, ref, target: float = 1e-5) -> dict:
    """Error of `got` against the FP64 amplitudes `ref`, per amplitude: |got - ref| / |ref| for
    every amplitude (random-circuit amplitudes are never 0; an amplitude below 1e-12 of the
    largest would be compared at that floor), as max / 99th / 90th percentile / median and the
    share within `target`; and normalised by the largest and by the RMS amplitude."""
    import numpy as np
    g, r = np.asarray(got).ravel(), np.asarray(ref).ravel()
    a = np.abs(r)
    floor = 1e-12 * a.max()
    rel = np.abs(g - r) / np.maximum(a, floor)
    rms = float(np.sqrt(np.mean(a ** 2)))
    return {"amplitudes": int(r.size), "per_amplitude_max": float(rel.max()),
            "per_amplitude_p99": float(np.quantile(rel, 0.99)), "per_amplitude_p90": float(np.quantile(rel, 0.90)),
            "per_amplitude_median": float(np.median(rel)),
            "share_within_target": float(np.mean(rel <= target)), "target": target,
            "max_over_largest_amplitude": float(np.abs(g - r).max() / a.max()),
            "max_over_rms_amplitude": float(np.abs(g - r).max() / rms),
            "floor": "amplitudes below 1e-12 of the largest compared at that floor (none here)"
                     if not np.any(a < floor) else "amplitudes below 1e-12 of the largest compared at that floor"}


def fp64_arm(q, prog, bits, out_size, local, dev, stream_of, args):
    """The plain ComplexF64 executor on `bits` of the same programme: one warm-up call, then
    `--fp64-steps` timed steps (CUDA events on the executor's stream, inputs in HBM).
    -> (summary dict, its amplitudes as complex128 (n, out_size))."""
    import numpy as np
    torch = stream_of
    n = len(bits)
    ex = q.Executor(prog, precision="fp64", device=local, use_graphs=not args.no_graphs)
    stream = torch.cuda.ExternalStream(ex.stream, device=dev)
    d_bits = torch.tensor(list("".join(bits).encode()), dtype=torch.uint8, device=dev)
    d_out = torch.zeros(2 * n * out_size, dtype=torch.float64, device=dev)
    nsl = ex.num_slices
    run = lambda: ex.amplitudes_device(d_bits.data_ptr(), n, d_out.data_ptr(), slices=(0, nsl))
    run()
    ex.synchronize()
    steps = max(1, args.fp64_steps)
    torch.cuda.synchronize()
    s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s_ev.record(stream)
    for _ in range(steps):
        run()
    e_ev.record(stream)
    ex.synchronize()
    ms = s_ev.elapsed_time(e_ev)
    inf = ex.info()
    amps = d_out.cpu().numpy().view(np.complex128).reshape(n, out_size).copy()
    ex.close()
    value = n * out_size * steps / (ms * 1e-3)
    return ({"value": value, "unit": UNIT, "bitstrings": n, "amplitudes_per_step": n * out_size, "steps": steps,
             "warmup": 1, "ms_per_step": ms / steps, "dtype": "f64", "precision": "fp64",
             "bitstring_batch": inf["bitstring_batch"], "slice_batch": inf["slice_batch"],
             "note": "same programme, the first bitstrings of the split arm's list; FP64 CUDA-core contractions"},
            amps)


def run_ours(args):
    ws, rank, local = dist_env()
    import torch
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    import __graft_entry__ as entry
    lib_path = ROOT / "qxtools.jl_gb300" / "_build" / "libqxgpu.so"
    if not lib_path.exists():
        entry._load_build_module().build()
    q = entry.load()
    prog, bits, info = q.workloads.build_workload(args.workload, seed=args.seed, plan_seed=args.plan_seed,
                                                  planner=args.planner)
    # default batch: the whole list for the Complex64 paths, 16 bitstrings for the slower FP64 path
    nb = args.bits_per_step or (min(16, len(bits)) if args.precision == "fp64" else len(bits))
    # weak scaling: rank r takes its own shard of bitstrings (regenerated deterministically)
    all_bits = list(q.amplitudes_uniform(info["nqubits"], args.seed + 7919 * rank, nb)) if rank else bits[:nb]
    if len(all_bits) < nb:
        all_bits = (all_bits * math.ceil(nb / len(all_bits)))[:nb]
    out_size = info["amplitudes_per_bitstring"]
    amps_per_step = nb * out_size
    tuning = args.tc_tuning if args.tc_tuning == "auto" else int(args.tc_tuning)
    ex = q.Executor(prog, precision=args.precision, device=local, use_graphs=not args.no_graphs,
                    tc_tuning=tuning)
    stream = torch.cuda.ExternalStream(ex.stream, device=dev)
    d_bits = torch.tensor(list("".join(all_bits).encode()), dtype=torch.uint8, device=dev)
    d_out = torch.zeros(2 * nb * out_size, dtype=torch.float64, device=dev)
    nslice = ex.num_slices

    def step_device():
        ex.amplitudes_device(d_bits.data_ptr(), nb, d_out.data_ptr(), slices=(0, nslice))

    tuning_path = Path(args.tuning_file) if args.tuning_file else None
    if tuning_path is not None and tuning_path.exists():
        ex.set_tuning(tuning_path.read_text())
    for _ in range(args.warmup):
        step_device()
    ex.synchronize()
    if tuning_path is not None and not tuning_path.exists() and rank == 0:
        tuning_path.write_text(ex.tuning())
    ex_info = ex.info()
    # ---- value: device-resident inputs --------------------------------------------------------
    _, launches0 = ex.profile_read()
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s_ev.record(stream)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step_device()
        e_ev.record(stream)
        ex.synchronize()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    ms = s_ev.elapsed_time(e_ev)
    barrier(ws)
    _, launches1 = ex.profile_read()
    ms = barrier_max(ms, ws, dev)
    clocks = clk.summary()
    value = ws * amps_per_step * args.steps / (ms * 1e-3)
    # ---- e2e: host entry point with pinned host buffers ---------------------------------------
    import ctypes as ct
    h_bits = torch.tensor(list("".join(all_bits).encode()), dtype=torch.uint8).pin_memory()
    h_out = torch.zeros(2 * nb * out_size, dtype=torch.float64).pin_memory()
    lib = ex.lib

    def step_host():
        rc = lib.qxg_amplitudes(ex._h, ct.c_char_p(h_bits.data_ptr()), nb, 0, nslice,
                                ct.cast(ct.c_void_p(h_out.data_ptr()), ct.POINTER(ct.c_double)))
        if rc != 0:
            raise RuntimeError(lib.qxg_last_error().decode())

    step_host()
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step_host()
    e2e_s = barrier_max(time.perf_counter() - t0, ws, dev)
    e2e = {"value": ws * amps_per_step * args.steps / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": int(h_bits.numel()), "d2h_bytes_per_step": int(h_out.numel() * 8)}
    # ---- roofline of the dominant kernel: CUDA events on the executor's stream ---------------
    psteps = max(1, min(args.steps, 3))
    ex.profile(True)
    for _ in range(psteps):
        step_device()
    rows, _ = ex.profile_read()
    ex.profile(False)
    by_kind = {}
    for r in rows:
        k = by_kind.setdefault(r["kernel"], {"launches": 0, "ms": 0.0, "flops": 0.0, "bytes": 0.0})
        for f in ("launches", "ms", "flops", "bytes"):
            k[f] += r[f]
    total_ms = sum(v["ms"] for v in by_kind.values())
    dom_name, dom = max(by_kind.items(), key=lambda kv: kv[1]["ms"])
    peaks, peak_src = measured_peaks()
    flops_exec = sum(v["flops"] for v in by_kind.values())
    tflops = flops_exec / (total_ms * 1e-3) / 1e12 if total_ms else 0.0
    kernel_name = dom_name
    # the committed DRAM summaries are named for the kernel class: tc_contract (tensor-core GEMMs),
    # contract_kernel_fp32 (CUDA-core contractions)
    traffic, tsum = traffic_summary(args.workload, {"contract_tc": "tc_contract", "contract_fp32": "contract_kernel_fp32",
                                                    "contract_fp64": "contract_kernel_fp64"}.get(dom_name, dom_name),
                                    args.precision)
    if tsum and "dram_over_algorithmic" in tsum and dom["launches"]:
        # measured on a smaller case: DRAM bytes per algorithmic byte of this kernel class, applied
        # to this run's algorithmic bytes per launch
        traffic = tsum["dram_over_algorithmic"] * dom["bytes"] / dom["launches"]
    if dom_name == "contract_fp64":
        fp64_peak = fp64_peak_tflops(torch, dev)
        ach = dom["flops"] / (dom["ms"] * 1e-3) / 1e12
        roof = {"bound": "fp64", "achieved": ach, "peak": fp64_peak, "unit": "TFLOP/s", "frac": ach / fp64_peak,
                "traffic": traffic, "peak_source": "measured here: cuBLAS DGEMM 4096^3 (no FP64 entry in "
                                                  "MEASURED_PEAKS.json; GB300 FP64 runs on CUDA cores)",
                "kernel": kernel_name, "kernel_share": dom["ms"] / total_ms,
                "hbm_achieved_gbs": dom["bytes"] / (dom["ms"] * 1e-3) / 1e9,
                "hbm_peak_gbs": peaks["hbm_gbs"]}
    elif dom_name == "contract_tc":
        ach = dom["flops"] / (dom["ms"] * 1e-3) / 1e12
        pk = peaks["bf16_tflops"]
        # the split form runs three products (hi*hi, hi*lo, lo*hi) per algorithmic FLOP; TF32
        # operands run at half the BF16 tensor rate
        op_peak = pk / 2 if args.precision == "split_tf32" else pk
        roof = {"bound": "tensor", "achieved": ach, "peak": pk, "unit": "TFLOP/s", "frac": ach / pk,
                "traffic": traffic, "peak_source": f"bf16_tflops of {peak_src}", "kernel": kernel_name,
                "kernel_share": dom["ms"] / total_ms,
                "tensor_executed_tflops": 3 * ach,
                "tensor_peak_for_operand_type": op_peak,
                "tensor_frac": 3 * ach / op_peak,
                "tensor_note": "executed tensor FLOPs = 3 x algorithmic (three split products); the operand "
                               "type's peak = measured bf16 peak, halved for TF32 operands"}
    else:
        ach = dom["bytes"] / (dom["ms"] * 1e-3) / 1e9
        pk = peaks["hbm_gbs"]
        roof = {"bound": "hbm", "achieved": ach, "peak": pk, "unit": "GB/s", "frac": ach / pk, "traffic": traffic,
                "peak_source": f"hbm_gbs of {peak_src}", "kernel": kernel_name, "kernel_share": dom["ms"] / total_ms}
    # per kernel class over the profiled steps; tc_pack moves operands for the tensor cores and
    # has no algorithmic bytes of its own (its entry counts the bytes it reads and writes)
    roof["kernels"] = {k: {"launches": v["launches"], "ms": round(v["ms"], 3), "share": v["ms"] / total_ms,
                           ("bytes_moved" if k == "tc_pack" else "algorithmic_bytes"): v["bytes"],
                           "algorithmic_flops": v["flops"]}
                       for k, v in sorted(by_kind.items(), key=lambda kv: -kv[1]["ms"])}
    roof["profiled_steps"] = psteps
    roof["profile_note"] = ("kernel times from CUDA events around every launch of an eager run (no graph "
                            "replay, no concurrent branches), so their sum exceeds a replayed step")
    top = sorted(rows, key=lambda r: -r["ms"])[:10]
    roof["top_steps"] = [{"instr": r["instr"], "kernel": r["kernel"], "ms_per_pass": round(r["ms"] / psteps, 3),
                          "gb_s": round(r["bytes"] / (r["ms"] * 1e-3) / 1e9, 1) if r["ms"] else None,
                          "tflop_s": round(r["flops"] / (r["ms"] * 1e-3) / 1e12, 2) if r["ms"] else None}
                         for r in top]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic (seeded random circuit, seeded bitstrings)",
            "config": workload_config(info, args, ex_info) | {"parallelism": f"replicas x{ws} (bitstring shards)"},
            "tflops": tflops, "tflops_note": "executed FLOPs (8 |C| K per contraction) / CUDA-event time of all kernels",
            "executed_flops_per_amplitude": flops_exec / (psteps * amps_per_step),
            "clocks": clocks, "e2e": e2e, "gpu_launches": int(launches1 - launches0), "roofline": roof,
            "wall_s": wall}
    got = d_out.cpu().numpy().view("complex128").reshape(nb, out_size)
    ex.close()
    # ---- the plain ComplexF64 executor on the same programme and bitstrings, and the error ----
    if not args.no_fp64 and args.precision != "fp64":
        n64 = min(args.fp64_bits or nb, nb)
        line["fp64"], ref64 = fp64_arm(q, prog, all_bits[:n64], out_size, local, dev, stream_of=torch, args=args)
        line["split_over_fp64"] = value / line["fp64"]["value"]
        line["err_vs_fp64"] = error_stats(got[:n64], ref64)
    if rank == 0 and ws == 1 and not args.no_gradient and args.precision != "fp64":
        line["gradient"] = gradient_leg(q, args, max(1, min(args.steps, 3)), 2)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(prog, bits, info, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def gradient_leg(q, args, steps: int, warmup: int) -> dict:
    """Forward vs reverse-mode gradient on the parametrised 5x5, 12-layer circuit (840 angles,
    256 bitstrings, L = sum |amplitude|^2): seconds per evaluation through the host API (each
    replayed from CUDA graphs unless --no-graphs), the ratio, and the angle gradient's error
    against the FP64 gradient on the first 8 bitstrings."""
    import numpy as np
    import torch
    circ = q.create_parametrised_circuit(5, 5, 12, seed=args.seed)
    bits = list(q.amplitudes_uniform(25, args.seed, 256))
    # planned like the param_5x5_l12 workload (its pinned plan seed, trials and planner, ranked
    # with the bitstring batch)
    spec = q.workloads.WORKLOADS["param_5x5_l12"]
    plan_opts = dict(seed=args.plan_seed if args.plan_seed is not None else spec["plan_seed"], time=spec["plan_time"],
                     width_cap=q.workloads.WIDTH_CAP, beta=spec["nbits"], planner=args.planner or spec.get("planner", "python"))
    f = q.gradients.ParametrisedCircuitLoss(circ, precision=args.precision, use_graphs=not args.no_graphs,
                                            **plan_opts)
    for _ in range(max(1, warmup)):
        f.executor.amplitudes(bits)
        f.loss_and_grad(bits)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        f.executor.amplitudes(bits)
    fwd = (time.perf_counter() - t0) / steps
    t0 = time.perf_counter()
    for _ in range(steps):
        L, g, _ = f.loss_and_grad(bits)
    grad = (time.perf_counter() - t0) / steps
    sub = bits[:8]
    ref = q.gradients.ParametrisedCircuitLoss(circ, precision="fp64", **plan_opts)
    _, g64, _ = ref.loss_and_grad(sub)
    _, gs, _ = f.loss_and_grad(sub)
    ref.close()
    info = f.executor.info()
    f.close()
    return {"workload": "param_5x5_l12", "params": circ.num_params, "bitstrings": len(bits),
            "precision": args.precision, "plan_steps": info["num_steps"], "planner": plan_opts["planner"],
            "flops_per_amplitude": info["flops_per_amplitude"], "steps": steps, "warmup": max(1, warmup),
            "forward_s": fwd, "gradient_s": grad, "gradient_over_forward": grad / fwd,
            "amplitudes_per_s_forward": len(bits) / fwd, "loss": L,
            "max_abs_err_vs_fp64_8bits": float(np.max(np.abs(gs - g64))),
            "max_rel_err_vs_fp64_8bits": float(np.max(np.abs(gs - g64)) / np.max(np.abs(g64)))}


def run_gradient(args):
    """The gradient leg alone, as its own JSON line (metric: gradient seconds / forward seconds)."""
    import torch
    import __graft_entry__ as entry
    q = entry.load()
    torch.cuda.set_device(0)
    g = gradient_leg(q, args, args.steps, args.warmup)
    line = {"metric": "gradient seconds / forward seconds (reverse-mode adjoint)", "value": g["gradient_over_forward"],
            "unit": "ratio", "higher_is_better": False, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic (seeded angles, bitstrings)",
            "config": {k: g[k] for k in ("workload", "params", "bitstrings", "precision", "plan_steps", "planner",
                                         "flops_per_amplitude")}}
    line.update({k: g[k] for k in ("forward_s", "gradient_s", "amplitudes_per_s_forward", "loss",
                                   "max_abs_err_vs_fp64_8bits", "max_rel_err_vs_fp64_8bits")})
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.gradient:
        run_gradient(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
