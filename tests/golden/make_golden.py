"""Regenerate the golden fixtures from the reference's own documents and tests (read as text).

Run in a checkout where the reference is available:  python tests/golden/make_golden.py [REF_DIR]
(default REF_DIR: /root/reference).  Writes tests/golden/golden.json and
tests/golden/users_guide_ghz2.qx.  Nothing here runs the reference (it is Julia).

Fixtures:
  - users_guide_ghz2.qx: the DSL example of docs/src/users_guide.md (two-qubit GHZ circuit,
    two sliced bonds v1, v2; views, chained views, batched `ncon`, a scalar result).  The page
    gives the programme but not its data; the leaf values are those of the circuit it encodes
    (H on qubit 1, CX control 1 -> target 2, decomposed, inputs |0>):
        data_1 = |0> (both input tensors t4, t5 share it: TensorCache dedup),
        data_2 = H (t1: H[out, in]; index 1 is the sliced output wire, index 2 the input),
        data_3 = CX target half T[out, in, b] = X^b (t2: index 3 is the bond tied to the control),
        data_4 = [1, 1] (t3: the control half, a delta reduced over its tied indices).
    Expected amplitudes <x1 x2|GHZ>: 1/sqrt(2) for 00 and 11, 0 otherwise.
  - ghz3_state: the 8-element state vector [1/sqrt2, 0, ..., 0, 1/sqrt2] asserted in
    test/test_tn_conversion.jl and test/test_contraction_planning.jl (`ref[[1,8]] .= 1/sqrt(2)`).
  - ghz5: `results["0"^n] ≈ results["1"^n] ≈ 1/sqrt(2)` with n = 5, 2^n results
    (test/test_simulation.jl).
  - tensor_cache_eps: 0.1*eps matches, 1.1*eps does not (test/test_compute_graph.jl).
  - plan_lengths: the `length(plan) == k` assertions of test/test_contraction_planning.jl.
"""
from __future__ import annotations

import json
import math
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _find(lines, pattern):
    rx = re.compile(pattern)
    for i, l in enumerate(lines, start=1):
        m = rx.search(l)
        if m:
            return i, m
    raise SystemExit(f"pattern {pattern!r} not found")


def main(ref: Path):
    ug = (ref / "docs/src/users_guide.md").read_text().splitlines()
    start, _ = _find(ug, r"^### Example DSL file")
    i = start
    while not ug[i].startswith("```"):
        i += 1
    j = i + 1
    while not ug[j].startswith("```"):
        j += 1
    dsl = "\n".join(ug[i + 1:j]) + "\n"
    (HERE / "users_guide_ghz2.qx").write_text(dsl)
    r = 1 / math.sqrt(2)
    golden = {
        "users_guide_ghz2": {
            "source": f"docs/src/users_guide.md:{i + 2}-{j}",
            "nqubits": 2,
            "data": {
                "data_1": [[1, 0], [0, 0]],
                "data_2": [[r, 0], [r, 0], [r, 0], [-r, 0]],
                "data_3": [[1, 0], [0, 0], [0, 0], [1, 0], [0, 0], [1, 0], [1, 0], [0, 0]],
                "data_4": [[1, 0], [1, 0]],
            },
            "data_dims": {"data_1": [2], "data_2": [2, 2], "data_3": [2, 2, 2], "data_4": [2]},
            "amplitudes": {"00": [r, 0], "01": [0, 0], "10": [0, 0], "11": [r, 0]},
        }
    }
    tc = (ref / "test/test_tn_conversion.jl").read_text().splitlines()
    ln, _ = _find(tc, r"ref\[\[1,8\]\] \.= 1/sqrt\(2\)")
    golden["ghz3_state"] = {"source": f"test/test_tn_conversion.jl:{ln}",
                            "nonzero_1based": [1, 8], "value": r, "length": 8}
    ts = (ref / "test/test_simulation.jl").read_text().splitlines()
    ln_n, m = _find(ts, r"^\s*n = (\d+)\s*$")
    ln_v, _ = _find(ts, r'results\["0"\^n\] ≈ results\["1"\^n\] ≈ 1/sqrt\(2\)')
    golden["ghz5"] = {"source": f"test/test_simulation.jl:{ln_n},{ln_v}", "n": int(m.group(1)),
                      "value": r, "num_results": 2 ** int(m.group(1))}
    cg = (ref / "test/test_compute_graph.jl").read_text().splitlines()
    ln1, m1 = _find(cg, r"@test sym == push!\(tc, a \.\+ ([0-9.]+)\*eps\(Float64\)\)")
    ln2, m2 = _find(cg, r"@test sym != push!\(tc, a \.\+ ([0-9.]+)\*eps\(Float64\)\)")
    golden["tensor_cache_eps"] = {"source": f"test/test_compute_graph.jl:{ln1},{ln2}",
                                  "same": float(m1.group(1)), "different": float(m2.group(1))}
    cp = (ref / "test/test_contraction_planning.jl").read_text().splitlines()
    lens = []
    for k, l in enumerate(cp, start=1):
        mm = re.search(r"@test length\(plan\) == (\d+)\s*$", l)
        if mm:
            lens.append({"line": k, "length": int(mm.group(1))})
    golden["plan_lengths"] = {"source": "test/test_contraction_planning.jl", "asserts": lens}
    (HERE / "golden.json").write_text(json.dumps(golden, indent=1) + "\n")
    print(f"wrote {HERE / 'golden.json'} and users_guide_ghz2.qx")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path("/root/reference"))
