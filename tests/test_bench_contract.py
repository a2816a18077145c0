"""bench.py's reference arm on the host cores: the JSON line it prints and its rank behaviour.

The reference arm times the reference's CPU contraction arithmetic restated in FP64 (permute +
OpenBLAS zgemm per ncon, oracle/blas_walk.py) on a bounded sample of the default workload; it
needs no GPU, so its output contract is checked
here: one JSON line with the metric, value, unit, the cpu_baseline description and an e2e block
without host-device traffic.  Under several ranks only rank 0 works and prints.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                           "--warmup", "0", "--cpu-seconds", "2"], capture_output=True, text=True, env=env,
                          cwd=ROOT, timeout=600)


def test_reference_arm_prints_the_contract_line():
    sys.path.insert(0, str(ROOT))
    import bench
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["warmup"] == 0
    assert d["config"]["workload"] == "rqc_7x7_d10_w22"
    # the arm describes itself: FP64 on the host, no GPU options
    assert d["config"]["precision"] == "fp64" and "cuda_graphs" not in d["config"]
    assert d["executed_flops_per_amplitude"] > 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert "zgemm" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert r.returncode == 0, r.stderr[-2000:]
    assert not [x for x in r.stdout.splitlines() if x.startswith("{")]


def test_cpu_baseline_leg_of_the_gpu_arm(q):
    """The `cpu_baseline` object the GPU arm adds to its line (rank 0, one GPU), computed on the
    host alone for a small sliced workload: a complete walk, a positive rate, the BLAS named."""
    sys.path.insert(0, str(ROOT))
    import bench
    prog, bits, info = q.workloads.build_workload("rqc_3x4_d8_s3")
    cb = bench.cpu_baseline(prog, bits, info, 3.0)
    assert cb["kind"] == "port" and cb["unit"] == bench.UNIT and cb["cores"] >= 1
    assert cb["value"] > 0 and cb["gflops"] > 0
    assert "complete" in cb["sample"] and "zgemm" in cb["sample"]
