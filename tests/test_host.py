"""Host-side mirror of the reference's API, tested the way the reference tests it.

Mirrors test/test_tn_conversion.jl (tensor counts), test/test_contraction_planning.jl (graph and
line-graph sizes, plan lengths, slicing), test/test_compute_graph.jl (TensorCache eps rule, node
count) and test/test_simulation.jl / test_bin.jl (bitstring generators, parameter files), plus the
`.qx` / `.yml` formats.
"""
import json
from collections import Counter
from pathlib import Path

import numpy as np
import pytest

GOLD = Path(__file__).resolve().parent / "golden"


def test_tn_conversion_counts(q):
    circ = q.create_test_circuit()
    tnc = q.convert_to_tnc(circ, no_input=True, no_output=True, decompose=False)
    assert tnc.qubits == 3 and len(tnc) == 3
    assert all(a != b for a, b in zip(tnc.input_indices, tnc.output_indices))
    tnc = q.convert_to_tnc(circ, no_input=True, no_output=True, decompose=True)
    assert len(tnc) == 5
    tnc = q.convert_to_tnc(circ, no_input=False, no_output=True, decompose=False)
    assert len(tnc) == 6
    first = tnc.keys()[0]
    assert np.array_equal(tnc.tn.tensors[first].data, q.gate_matrix(circ.circ_ops[0]))


def test_graph_and_line_graph_sizes(q):
    circ = q.create_test_circuit()
    tnc = q.convert_to_tnc(circ, no_input=True, no_output=True, decompose=False)
    g = q.convert_to_graph(tnc)
    assert g.number_of_nodes() == 3 and g.number_of_edges() == 2
    tnc.add_input()
    tnc.add_output()
    g = q.convert_to_graph(tnc)
    assert g.number_of_nodes() == 9 and g.number_of_edges() == 8
    lg, smap = q.convert_to_line_graph(tnc)
    assert lg.number_of_nodes() == 8 and lg.number_of_edges() == 13
    tnc = q.convert_to_tnc(q.create_test_circuit(), decompose=True)
    lg, smap = q.convert_to_line_graph(tnc, use_hyperedges=True)
    assert lg.number_of_nodes() == 6 and lg.number_of_edges() == 7
    assert Counter(len(v) for v in smap.values()) == {4: 2, 2: 4}


def test_plan_lengths_match_reference_asserts(q):
    asserts = {a["line"]: a["length"] for a in json.loads((GOLD / "golden.json").read_text())["plan_lengths"]["asserts"]}
    circ = q.create_test_circuit()
    tnc = q.convert_to_tnc(circ, no_output=True, decompose=False)
    assert len(q.flow_cutter_contraction_plan(tnc, time=1)) == asserts[55]
    assert len(q.flow_cutter_contraction_plan(tnc, time=0)) == asserts[123]
    assert len(q.min_fill_contraction_plan(tnc)) == asserts[139]
    assert len(q.netcon(tnc)) == asserts[155]
    tnc = q.convert_to_tnc(circ, decompose=False)
    assert len(q.flow_cutter_contraction_plan(tnc, time=1, hypergraph=True)) == asserts[81]
    # one hyperedge of 42 tensors (40 Z gates) -> min-fill fallback inside the order conversion
    c = q.Circuit(1)
    for _ in range(40):
        c.add("z", [1], q.gates.Z)
    tnc = q.convert_to_tnc(c)
    assert len(q.flow_cutter_contraction_plan(tnc, time=1, hypergraph=True)) == asserts[98]
    # elimination order -> plan on the decomposed network (line 184)
    tnc = q.convert_to_tnc(circ, decompose=True)
    lg, smap = q.convert_to_line_graph(tnc)
    _, order = q.min_fill(lg)
    plan = q.order_to_contraction_plan([smap[v] for v in order], q.hyper_network(tnc))
    assert len(plan) == asserts[184]


def test_contraction_scheme_slicing(q):
    circ = q.create_test_circuit()
    tnc = q.convert_to_tnc(circ, decompose=False)
    groups, plan, meta = q.contraction_scheme(tnc, 3, time=1, hypergraph=False)
    assert sum(len(g) for g in groups) >= 3
    assert len(plan) == len(tnc) - 1 - 3
    groups, plan, meta = q.contraction_scheme(tnc, 0, time=1)
    assert len(groups) == 0 and len(plan) == len(tnc) - 1
    assert "Slicing" in meta and "Determination of contraction plan" in meta


def test_tensor_cache_eps_rule(q):
    g = json.loads((GOLD / "golden.json").read_text())["tensor_cache_eps"]
    tc = q.TensorCache()
    rng = np.random.default_rng(0)
    a = rng.random((3, 4, 5))
    sym = tc.push(a)
    assert sym == tc.push(a)
    assert sym != tc.push(rng.random((3, 4, 5)))
    eps = np.finfo(np.float64).eps
    assert sym == tc.push(a + g["same"] * eps)
    assert sym != tc.push(a + g["different"] * eps)
    assert np.array_equal(tc[sym], a)
    assert len(tc) == 3


def test_compute_graph_node_count(q):
    tnc = q.convert_to_tnc(q.create_test_circuit())
    plan = q.min_fill_contraction_plan(tnc)
    cg = q.build_compute_graph(tnc, plan)
    assert len(cg) == len(tnc) + len(plan) + 1


def test_compute_graph_views_and_chains(q):
    circ = q.create_rqc_circuit(2, 3, 4, seed=3)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, _ = q.contraction_scheme(tnc, 2, seed=1, time=1)
    cg = q.build_compute_graph(tnc, plan, groups)
    views = [c for c in cg.commands if isinstance(c, q.View)]
    assert views and all(v.var in ("v1", "v2") for v in views)
    names = {c.name for c in cg.commands if not isinstance(c, q.Save)}
    for v in views:          # a chained view names its source's view
        assert v.src in names
        assert v.name == v.src + "_s"
    defined = set()
    for c in cg.commands:    # post-order: every operand defined before use
        if isinstance(c, q.Ncon):
            assert c.a in defined and c.b in defined
        if isinstance(c, q.View):
            assert c.src in defined
        if not isinstance(c, q.Save):
            defined.add(c.name)
    assert isinstance(cg.commands[-1], q.Save)
    vdim = {v.var: v.dim for v in views}
    assert cg.num_slices == int(np.prod(list(vdim.values())))   # a decomposed bond may be 4-wide


def test_qx_round_trip(q):
    circ = q.create_rqc_circuit(2, 2, 3, seed=1)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, meta = q.contraction_scheme(tnc, 1, seed=1, time=1)
    cg = q.build_compute_graph(tnc, plan, groups)
    text = q.dsl.format_qx(cg, meta)
    cmds, ver = q.dsl.parse_qx(text)
    assert ver == q.dsl.DSL_VERSION
    assert cmds == cg.commands
    text2 = (GOLD / "users_guide_ghz2.qx").read_text()
    cmds2, _ = q.dsl.parse_qx(text2)
    body = [l for l in text2.splitlines() if l and not l.startswith("#")]
    again = [l for l in q.dsl.format_qx(q.ComputeGraph(cmds2, {})).splitlines() if not l.startswith("#")]
    assert again == body
    with pytest.raises(ValueError):
        q.dsl.parse_qx("ncon t1 1 t2\n")


def test_yml_list_round_trip(q, tmp_path):
    params = q.output_params_dict(5, 15, seed=3)
    assert params["method"] == "List" and len(params["params"]["bitstrings"]) == 15
    q.generate_parameter_file(str(tmp_path / "x"), params)
    back = q.dsl.read_yml(str(tmp_path / "x.yml"))
    assert back["output"]["params"]["bitstrings"] == params["params"]["bitstrings"]
    assert back["output"]["params"]["num_samples"] == 15
    rej = q.output_params_dict(5, 20, output_method="Rejection", seed=42)
    q.generate_parameter_file(str(tmp_path / "r"), rej)
    back = q.dsl.read_yml(str(tmp_path / "r.yml"))
    assert back["output"]["method"] == "Rejection" and back["output"]["params"]["num_samples"] == 20
    assert back["output"]["params"]["fix_M"] is False
    doc = 'output:\n  method: List\n  params:\n    num_samples: 3\n    bitstrings:\n      - "010"\n      - "101"\n      - "111"\n'
    assert q.dsl.parse_yml(doc)["output"]["params"]["bitstrings"] == ["010", "101", "111"]


def test_generate_simulation_files(q, tmp_path):
    circ = q.create_rqc_circuit(3, 3, 4, seed=1)
    prefix = str(tmp_path / "rqc_3_3_4")
    q.generate_simulation_files(circ, prefix, 2, seed=1,
                                output_args=q.output_params_dict(9, 15, seed=2))
    for suf in (".qx", ".npz", ".yml"):
        assert Path(prefix + suf).exists()
    assert len(q.dsl.read_yml(prefix + ".yml")["output"]["params"]["bitstrings"]) == 15
    prog = q.simulation.load_programme(prefix + ".qx")
    assert prog.num_slices == 4


def test_amplitude_generators(q):
    a = list(q.amplitudes_all(5))
    assert len(a) == 32 and all(len(x) == 5 for x in a) and a[1] == "00001"
    u = list(q.amplitudes_uniform(5, None, 10))
    assert len(u) == 10 and u == list(q.amplitudes_uniform(5, 0, 10))


def test_programme_encoding(q):
    cmds, _ = q.dsl.parse_qx((GOLD / "users_guide_ghz2.qx").read_text())
    data = {f"data_{i}": np.zeros(d) for i, d in [(1, (2,)), (2, (2, 2)), (3, (2, 2, 2)), (4, (2,))]}
    prog = q.Programme.from_commands(cmds, data, 2)
    ops = [int(r[0]) for r in prog.instrs]
    assert ops.count(1) == 5 and ops.count(2) == 6 and ops.count(3) == 2 and ops.count(4) == 6 and ops[-1] == 5
    v = prog.instrs[ops.index(2)]
    assert (v[3], v[4], v[5]) == (1, 0, 2)      # view t5_s t5 v2 1 2 -> var 1, pos 0, dim 2
    assert prog.num_slices == 4
    with pytest.raises(ValueError):
        q.Programme.from_commands(cmds[1:], data, 2)   # view of an undefined tensor


def test_rqc_generator_family(q):
    c = q.create_rqc_circuit(4, 4, 10, seed=1)
    assert c.num_qubits == 16
    ones = [g for g in c.circ_ops if len(g.qubits) == 1]
    twos = [g for g in c.circ_ops if len(g.qubits) == 2]
    assert len(ones) == 160
    assert {g.name for g in ones} == {"sx", "sy", "sw"}
    last = {}
    for g in ones:      # no repeat on a qubit between consecutive cycles
        assert last.get(g.qubits[0]) != g.name
        last[g.qubits[0]] = g.name
    for g in twos:
        assert np.allclose(g.matrix, q.gates.fsim(np.pi / 2, np.pi / 6))
    for g in c.circ_ops:
        m = g.matrix
        assert np.allclose(m.conj().T @ m, np.eye(m.shape[0]))


def test_chain_rule_to_the_parameters_matches_the_per_gate_sum(q):
    """gradients.chain_rule_tables / apply_chain_rule (one gather + bincount over the flat leaf
    gradient vector) equal the per-gate sum 2 Re sum conj(dL/d conj T) dT/dtheta, with leaves of
    several shapes laid out column-major and parameters shared between gates."""
    rng = np.random.default_rng(5)
    shapes = [(2, 2), (4, 4), (2, 2, 2, 2), (), (2, 4)]
    layout, o = {}, 0
    for i in range(40):
        s = shapes[i % len(shapes)]
        layout[3 * i] = (o, s)
        o += int(np.prod(s)) if s else 1
    gvec = rng.standard_normal(o) + 1j * rng.standard_normal(o)
    terms = []
    for instr, (_, s) in layout.items():
        for _ in range(int(rng.integers(1, 3))):
            dt = rng.standard_normal(s) + 1j * rng.standard_normal(s)
            terms.append((int(rng.integers(0, 25)), instr, dt))
    want = np.zeros(25)
    for pid, instr, dt in terms:
        off, s = layout[instr]
        n = int(np.prod(s)) if s else 1
        leaf = gvec[off:off + n].reshape(s, order="F")
        want[pid] += 2.0 * float(np.real(np.sum(np.conj(leaf) * dt)))
    got = q.gradients.apply_chain_rule(gvec, q.gradients.chain_rule_tables(terms, layout), 25)
    assert got.shape == (25,)
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.max(np.abs(want)))
