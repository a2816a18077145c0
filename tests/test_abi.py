"""The C-ABI library: it loads without a GPU, exports every symbol include/qxgpu.h declares,
its structs have the header's layout, and malformed programmes are rejected with an error
code and message before any device work."""
import ctypes as ct
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    text = (ROOT / "include" / "qxgpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(qxg_[a-z_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for f in ("qxg_program_create", "qxg_program_set_data", "qxg_amplitudes", "qxg_amplitudes_device",
              "qxg_program_destroy", "qxg_ncon", "qxg_last_error", "qxg_program_info_get"):
        assert f in names


def test_library_exports_every_declared_symbol(gpu_lib):
    for name in declared_functions():
        assert hasattr(gpu_lib, name), f"{name} declared in include/qxgpu.h but not exported"
    assert gpu_lib.qxg_version().decode().startswith("qxgpu")


def test_struct_layouts(q, tmp_path):
    """ctypes mirrors of the header's structs have the C compiler's sizes and offsets."""
    import shutil
    import subprocess
    from qxtools_gb300 import executor as ex
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = {"qxg_instr": ex.qxg_instr, "qxg_options": ex.qxg_options, "qxg_program_info": ex.qxg_program_info,
              "qxg_qx_sizes": ex.qxg_qx_sizes, "qxg_yml_output": ex.qxg_yml_output,
              "qxg_plan_options": ex.qxg_plan_options, "qxg_plan_stats": ex.qxg_plan_stats}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "qxgpu.h"', "int main(void){"]
    for s, cls in fields.items():
        lines.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f, _ in cls._fields_:
            lines.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    lines.append("return 0;}")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    out = dict(l.split() for l in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for s, cls in fields.items():
        assert int(out[s]) == ct.sizeof(cls), s
        for f, _ in cls._fields_:
            assert int(out[f"{s}.{f}"]) == getattr(cls, f).offset, f"{s}.{f}"


def _create(gpu_lib, q, instrs, labels, data_dims, nqubits=2):
    from qxtools_gb300 import executor as ex
    ins = np.ascontiguousarray(np.array(instrs, dtype=np.int32).reshape(-1, 10))
    arr = (ex.qxg_instr * ins.shape[0]).from_buffer_copy(ins.tobytes())
    lab = np.ascontiguousarray(np.array(labels or [0], dtype=np.int32))
    rank = np.array([len(d) for d in data_dims], dtype=np.int32)
    dims = np.array([x for d in data_dims for x in d] or [0], dtype=np.int64)
    h = ct.c_void_p()
    rc = gpu_lib.qxg_program_create(arr, ins.shape[0], lab.ctypes.data_as(ct.POINTER(ct.c_int32)),
                                    len(labels), rank.ctypes.data_as(ct.POINTER(ct.c_int32)),
                                    dims.ctypes.data_as(ct.POINTER(ct.c_int64)), len(data_dims), nqubits,
                                    None, ct.byref(h))
    return rc, gpu_lib.qxg_last_error().decode()


@pytest.mark.parametrize("case,msg", [
    # ncon label count does not match the operand's rank
    ([[1, 0, 0, 0, 0, 0, 0, 0, 0, 0], [1, 1, 1, 0, 0, 0, 0, 0, 0, 0], [4, 2, 0, 1, 0, 0, 0, 1, 1, 0],
      [5, 0, 2, 0, 0, 0, 0, 0, 0, 0]], "rank"),
    # operand used before definition
    ([[1, 0, 0, 0, 0, 0, 0, 0, 0, 0], [4, 2, 0, 1, 0, 0, 0, 2, 1, 0], [5, 0, 2, 0, 0, 0, 0, 0, 0, 0]],
     "before definition"),
    # no save
    ([[1, 0, 0, 0, 0, 0, 0, 0, 0, 0]], "save"),
    # view of a rank position outside the tensor
    ([[1, 0, 0, 0, 0, 0, 0, 0, 0, 0], [2, 1, 0, 0, 5, 2, 0, 0, 0, 0], [5, 0, 1, 0, 0, 0, 0, 0, 0, 0]],
     "rank position"),
])
def test_malformed_programmes_are_rejected(gpu_lib, q, case, msg):
    rc, err = _create(gpu_lib, q, case, [1, 2, 2], [(2, 2), (2,)])
    assert rc == -1
    assert msg in err


def test_label_dimension_mismatch_rejected(gpu_lib, q):
    # A: (2,2) labels 1,2 ; B: (4,) label 2 -> label 2 is 2 in A and 4 in B
    ins = [[1, 0, 0, 0, 0, 0, 0, 0, 0, 0], [1, 1, 1, 0, 0, 0, 0, 0, 0, 0], [4, 2, 0, 1, 0, 0, 1, 2, 1, 0],
           [5, 0, 2, 0, 0, 0, 0, 0, 0, 0]]
    rc, err = _create(gpu_lib, q, ins, [1, 1, 2, 2], [(2, 2), (4,)])
    assert rc == -1 and "different dimensions" in err


def test_bad_precision_rejected(gpu_lib, q):
    from qxtools_gb300 import executor as ex
    ins = np.array([[1, 0, 0, 0, 0, 0, 0, 0, 0, 0], [5, 0, 0, 0, 0, 0, 0, 0, 0, 0]], dtype=np.int32)
    arr = (ex.qxg_instr * 2).from_buffer_copy(ins.tobytes())
    opts = ex.qxg_options()
    opts.precision = 9
    rank = np.array([1], dtype=np.int32)
    dims = np.array([2], dtype=np.int64)
    h = ct.c_void_p()
    rc = gpu_lib.qxg_program_create(arr, 2, None, 0, rank.ctypes.data_as(ct.POINTER(ct.c_int32)),
                                    dims.ctypes.data_as(ct.POINTER(ct.c_int64)), 1, 0, ct.byref(opts), ct.byref(h))
    assert rc == -1 and "precision" in gpu_lib.qxg_last_error().decode()


def test_executor_fails_loudly_without_library(q, tmp_path):
    with pytest.raises(q.QXGError):
        q.load_library(tmp_path / "missing.so")
