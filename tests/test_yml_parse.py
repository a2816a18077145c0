"""qxg_parse_yml_output, the library's reader of the `.yml` `output:` block (no device needed).

The three output methods of output_params_dict (src/outputs.jl:47-78), written by the Python
mirror of generate_parameter_file, must read back as the same dict through the native reader;
the users-guide List example (docs/src/users_guide.md:22-35), flow sequences, plain scalars and
comments read as YAML does for this subset; malformed text is rejected with the line number.
"""
import ctypes as ct
from collections import OrderedDict

import pytest


def _yml(q, params):
    return q.dsl.format_yml(OrderedDict([("output", params)]))


@pytest.mark.parametrize("method,kw", [
    ("List", dict(seed=7)),
    ("List", dict(bitstrings=["01+-", "1111", "0000"])),
    ("Uniform", dict(seed=3)),
    ("Uniform", dict(seed=None)),
    ("Rejection", dict(seed=11, M=0.25, fix_M=True)),
    ("Rejection", dict()),
])
def test_native_reader_matches_output_params_dict(q, gpu_lib, method, kw):
    p = q.output_params_dict(6, 9, output_method=method, **kw)
    text = _yml(q, p)
    got = q.executor.parse_yml_output(text, lib=gpu_lib)
    assert got == q.dsl.parse_yml(text)["output"]
    assert got["method"] == p["method"]
    assert dict(got["params"]) == dict(p["params"])


def test_users_guide_list_example(q, gpu_lib):
    text = 'output:\n  method: List\n  params:\n    num_samples: 3\n    bitstrings:\n      - "010"\n      - "101"\n      - "111"\n'
    got = q.executor.parse_yml_output(text, lib=gpu_lib)
    assert got["method"] == "List"
    assert got["params"]["bitstrings"] == ["010", "101", "111"]
    assert got["params"]["num_samples"] == 3


def test_yaml_forms_of_the_subset(q, gpu_lib):
    from qxtools_gb300 import executor as ex
    # flow sequence, plain scalars taken as written, comments, a sequence at the key's indentation,
    # another top-level key, CRLF line ends, no num_samples (defaults to the list's length)
    text = ("# parameters\r\nsimulation:\r\n  name: x\r\noutput:\r\n  method: :List\r\n  params:\r\n"
            "    bitstrings: [010, '101', \"1-1\"]\r\n")
    got = q.executor.parse_yml_output(text, lib=gpu_lib)
    assert got["params"]["bitstrings"] == ["010", "101", "1-1"] and got["params"]["num_samples"] == 3
    text = "output:\n  method: List\n  params:\n    bitstrings:\n    - 00\n    - 11\n"
    assert q.executor.parse_yml_output(text, lib=gpu_lib)["params"]["bitstrings"] == ["00", "11"]
    text = "output:\n  params:\n    M: 1.5e-3\n    num_qubits: 5\n    num_samples: 4\n    seed: ~\n  method: Rejection\n"
    o = ex.qxg_yml_output()
    assert gpu_lib.qxg_parse_yml_output(text.encode(), ct.byref(o), None, 0) == 0
    assert (o.method, o.num_qubits, o.num_samples, o.has_seed, o.fix_M, o.M) == (2, 5, 4, 0, 0, 1.5e-3)
    # an empty List gives no bitstrings
    text = "output:\n  method: List\n  params:\n    num_samples: 0\n    bitstrings: []\n"
    assert q.executor.parse_yml_output(text, lib=gpu_lib)["params"]["bitstrings"] == []


@pytest.mark.parametrize("text,msg", [
    ("simulation:\n  a: 1\n", "no output: block"),
    ("output:\n  params:\n    num_samples: 1\n", "has no method"),
    ("output:\n  method: Sobol\n  params:\n    num_samples: 1\n", "line 2: output method Sobol not supported"),
    ("output:\n  method: List\n", "has no params"),
    ("output:\n  method: List\n  params:\n    bitstrings:\n      - \"01\"\n      - \"012\"\n", "line 6: bitstring '012' has"),
    ("output:\n  method: List\n  params:\n    bitstrings:\n      - \"01\"\n      - \"011\"\n", "line 6: bitstring '011' differs in length"),
    ("output:\n  method: Uniform\n  params:\n    num_samples: 4\n", "num_qubits missing"),
    ("output:\n  method: Uniform\n  params:\n    num_qubits: 4\n    num_samples: four\n", "line 5: params.num_samples is not an integer"),
    ("output:\n  method: Rejection\n  params:\n    num_qubits: 4\n    num_samples: 2\n    fix_M: maybe\n", "line 6: params.fix_M is not a boolean"),
    ("output:\n  method: List\n    params: 1\n", "line 3: bad indentation"),
    ("output:\n\tmethod: List\n", "line 2: tab in indentation"),
    ("output:\n  method: List\n  method: Uniform\n", "line 3: key method given twice"),
    ("output:\n  method: List\n  params:\n    bitstrings: [\"01\", \"10\"\n", "line 4: unterminated flow sequence"),
    ("output:\n  method: \"List\n", "line 2: bad quoted scalar"),
])
def test_native_reader_rejects_malformed_text(q, gpu_lib, text, msg):
    from qxtools_gb300 import executor as ex
    o = ex.qxg_yml_output()
    assert gpu_lib.qxg_parse_yml_output(text.encode(), ct.byref(o), None, 0) == -1
    assert msg in gpu_lib.qxg_last_error().decode()


def test_native_reader_checks_capacity(q, gpu_lib):
    from qxtools_gb300 import executor as ex
    text = b'output:\n  method: List\n  params:\n    bitstrings:\n      - "0101"\n      - "1100"\n'
    o = ex.qxg_yml_output()
    assert gpu_lib.qxg_parse_yml_output(text, ct.byref(o), None, 0) == 0
    assert (o.nbitstrings, o.num_qubits) == (2, 4)
    buf = ct.create_string_buffer(8)
    assert gpu_lib.qxg_parse_yml_output(text, ct.byref(o), buf, 7) == -1
    assert "smaller" in gpu_lib.qxg_last_error().decode()
    assert gpu_lib.qxg_parse_yml_output(text, ct.byref(o), buf, 8) == 0
    assert buf.raw == b"01011100"
