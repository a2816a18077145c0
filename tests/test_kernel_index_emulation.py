"""Index work of the compact row-form, long-sum and batched small GEMM kernels, emulated on the CPU.

The kernels keep their addressing in `__host__ __device__` phase functions (fill, walk, per-lane
blocks, chunk elements and bases, reduce); `tests/emu/kernel_index_emu.cu` runs those phases for
every lane of every warp (every thread of every block for the batched GEMM) on seeded random bit
layouts -- permuted row, summed, column and batch bits, conjugation, 16-byte pairs, column chunks,
short row counts, result chunks across the grid, K cut into ranges with FP64 partials -- and
compares each result with a direct evaluation of the contraction (within 1e-5 of the largest
result).  The host build uses AddressSanitizer, so an index that leaves an operand, a shared-memory
buffer or table, or the partial buffer fails the test.  Needs nvcc (the harness includes the kernel
sources); no GPU.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "emu" / "kernel_index_emu.cu"


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    return None


@pytest.mark.timeout(900)
def test_row_form_and_long_sum_index_work(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    obj, exe = tmp_path / "emu.o", tmp_path / "emu"
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-relaxed-constexpr",
           "-I", str(ROOT / "include"), "-Xcompiler=-fsanitize=address,-fno-omit-frame-pointer", "-c", str(SRC),
           "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    cuda_lib = Path(nvcc).resolve().parent.parent / "lib64"
    r = subprocess.run(["g++", str(obj), "-o", str(exe), "-fsanitize=address", f"-L{cuda_lib}", "-lcudart"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    env["LD_LIBRARY_PATH"] = f"{cuda_lib}:{env.get('LD_LIBRARY_PATH', '')}"
    r = subprocess.run([str(exe), "7", "300", "60"], capture_output=True, text=True, env=env, timeout=800)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "failed" in r.stdout


JOIN_SRC = ROOT / "tests" / "emu" / "tc_join_emu.cu"


@pytest.mark.timeout(600)
def test_tensor_core_join_index_work(tmp_path):
    """The tensor-core join (tc_join.cu): its planner on seeded random layouts (batch bits on top or
    anywhere, P = A or B, 8-32 free values of Q, K ranges), then per block the delta walk of the
    chunk bases, the segment copies into a slot of the planned size (each byte once, 16-byte
    aligned) and the splitters' slot reads, summed in FP64 against the direct contraction."""
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    obj, exe = tmp_path / "join.o", tmp_path / "join"
    cmd = [nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a", "--expt-relaxed-constexpr",
           "-I", str(ROOT / "include"), "-Xcompiler=-fsanitize=address,-fno-omit-frame-pointer", "-c",
           str(JOIN_SRC), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    cuda_lib = Path(nvcc).resolve().parent.parent / "lib64"
    r = subprocess.run(["g++", str(obj), "-o", str(exe), "-fsanitize=address", f"-L{cuda_lib}", "-lcudart"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=0")
    env["LD_LIBRARY_PATH"] = f"{cuda_lib}:{env.get('LD_LIBRARY_PATH', '')}"
    r = subprocess.run([str(exe), "5", "80"], capture_output=True, text=True, env=env, timeout=500)
    assert r.returncode == 0, (r.stdout[-3000:], r.stderr[-3000:])
    assert "0 failed" in r.stdout
