"""qxg_parse_qx, the library's `.qx` parser (no device needed), against the Python path.

For the users-guide programme (golden file) and seeded random-circuit programmes with sliced
bonds and open qubits, the native parse of the `.qx` text must give the same instruction array,
labels, data shapes and bitstring length as Programme.from_commands on the Python parse (data ids
remapped: the native parser numbers data keys in order of first `load`).  Malformed text is
rejected with the line number in the message.
"""
import ctypes as ct
from collections import OrderedDict
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


def _programmes(q):
    import json
    g = json.loads((GOLD / "golden.json").read_text())["users_guide_ghz2"]
    text = (GOLD / "users_guide_ghz2.qx").read_text()
    cmds, _ = q.dsl.parse_qx(text)
    data = OrderedDict((k, np.array([complex(*x) for x in v]).reshape(g["data_dims"][k], order="F"))
                       for k, v in g["data"].items())
    yield "users_guide", text, cmds, data, 2
    for rows, cols, depth, nslice, seed in [(3, 3, 5, 2, 1), (3, 4, 8, 3, 5), (2, 3, 4, 0, 2)]:
        circ = q.create_rqc_circuit(rows, cols, depth, seed=seed)
        tnc = q.convert_to_tnc(circ, decompose=True)
        groups, plan, _ = q.contraction_scheme(tnc, nslice, seed=seed, time=1)
        graph = q.build_compute_graph(tnc, plan, groups)
        text = q.dsl.format_qx(graph, {"circuit": f"rqc {rows}x{cols} d{depth}"})
        nq = max([c.qubit for c in graph.commands if isinstance(c, q.Output)], default=0)
        yield f"rqc{rows}x{cols}d{depth}s{nslice}", text, graph.commands, graph.data, nq


def test_native_parse_matches_python(q, gpu_lib):
    for name, text, cmds, data, nq in _programmes(q):
        ref = q.Programme.from_commands(cmds, data, nq)
        got = q.Programme.from_qx_text(text, data, lib=gpu_lib)
        assert got.nqubits == nq, name
        # data ids: the native parser's key order -> the Python programme's
        remap = {i: ref.data_keys.index(k) for i, k in enumerate(got.data_keys)}
        gi = got.instrs.copy()
        load = gi[:, 0] == 1
        gi[load, 2] = [remap[int(x)] for x in gi[load, 2]]
        assert np.array_equal(gi, ref.instrs), name
        assert np.array_equal(got.labels, ref.labels), name
        for i, k in enumerate(got.data_keys):
            assert np.array_equal(got.data[i], ref.data[ref.data_keys.index(k)]), (name, k)


@pytest.mark.parametrize("text,msg", [
    ("load t1 data_1 2,2\nfrobnicate t2\n", "line 2: unknown command"),
    ("load t1 data_1 2,2\nncon t2 1 t9 1,2 t1 2,1\n", "line 2: tensor t9 used before definition"),
    ("load t1 data_1 2,2\nload t1 data_2 2\n", "line 2: tensor t1 defined twice"),
    ("load t1 data_1 2,2\nload t2 data_1 4\n", "line 2: data key data_1 loaded with two shapes"),
    ("# version: 0.4.0\nload t1 data_1 2,x\n", "line 2: bad dims"),
    ("load t1 data_1 2,2\nview t2 t1 w1 1 2\n", "line 2: bad slice variable"),
    ("load t1 data_1 2,2\nncon t2 1 t1 1,2\n", "line 2: ncon takes"),
    ("# only comments\n\n", "no commands"),
])
def test_native_parse_rejects_malformed_text(gpu_lib, q, text, msg):
    from qxtools_gb300 import executor as ex
    sz = ex.qxg_qx_sizes()
    rc = gpu_lib.qxg_parse_qx(text.encode(), ct.byref(sz), None, None, None, None, None)
    assert rc == -1
    assert msg in gpu_lib.qxg_last_error().decode()


def test_native_parse_checks_capacities(gpu_lib, q):
    from qxtools_gb300 import executor as ex
    text = b"load t1 data_1 2,2\nload t2 data_2 2\nncon t3 1 t1 1,2 t2 2\nsave out t3\n"
    sz = ex.qxg_qx_sizes()
    assert gpu_lib.qxg_parse_qx(text, ct.byref(sz), None, None, None, None, None) == 0
    assert (sz.ninstr, sz.nlabels, sz.ndata, sz.ndims, sz.key_bytes) == (4, 4, 2, 3, 14)
    sz.ninstr = 3                                          # one instruction short
    ins = (ex.qxg_instr * 4)()
    lab = (ct.c_int32 * 4)()
    rank = (ct.c_int32 * 2)()
    dims = (ct.c_int64 * 3)()
    keys = ct.create_string_buffer(14)
    assert gpu_lib.qxg_parse_qx(text, ct.byref(sz), ins, lab, rank, dims, keys) == -1
    assert "smaller" in gpu_lib.qxg_last_error().decode()
