"""Static check of the Julia binding (qxtools.jl_gb300/julia/QXToolsGPU.jl) against the C ABI.

Neither machine has a Julia toolchain, so the binding cannot run here.  What can drift is
checked from the sources instead:
  * every `struct Qxg...` mirror has the size and field offsets of its C struct, with the
    offsets read from a probe compiled against include/qxgpu.h by gcc;
  * every `ccall((:qxg_..., libqxgpu), Ret, (args...), ...)` has as many arguments as the
    header's prototype, each of the same class (32-bit int, 64-bit int, double, pointer), and
    the same return class.
"""
import re
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
JL = ROOT / "qxtools.jl_gb300" / "julia" / "QXToolsGPU.jl"
HDR = ROOT / "include" / "qxgpu.h"

# Julia struct -> C struct
STRUCTS = {"QxgInstr": "qxg_instr", "QxgOptions": "qxg_options", "QxgQxSizes": "qxg_qx_sizes",
           "QxgYmlOutput": "qxg_yml_output", "QxgPlanOptions": "qxg_plan_options",
           "QxgPlanStats": "qxg_plan_stats"}
JL_SCALAR = {"Int32": 4, "UInt32": 4, "Cint": 4, "Int64": 8, "UInt64": 8, "Float64": 8, "Float32": 4,
             "UInt8": 1, "Int8": 1}


def julia_structs(text):
    """name -> [(field, size, align)] from `struct Name ... end` blocks (fields `a::T; b::T`)."""
    out = {}
    for m in re.finditer(r"^struct (\w+)[^\n]*\n(.*?)^end", text, re.S | re.M):
        fields = []
        for line in m.group(2).splitlines():
            line = line.split("#")[0]
            for f, t in re.findall(r"(\w+)::([\w{}, ]+?)(?:;|$)", line.strip()):
                t = t.strip()
                if t in JL_SCALAR:
                    fields.append((f, JL_SCALAR[t], JL_SCALAR[t]))
                elif t.startswith("Ptr{"):
                    fields.append((f, 8, 8))
                else:
                    tm = re.fullmatch(r"NTuple\{(\d+),\s*(\w+)\}", t)
                    assert tm, f"{m.group(1)}.{f}: unhandled type {t}"
                    k, e = int(tm.group(1)), JL_SCALAR[tm.group(2)]
                    fields.append((f, k * e, e))
        out[m.group(1)] = fields
    return out


def c_layout(fields):
    """C layout rules (natural alignment): -> ([offsets], size)."""
    off, offs, al = 0, [], 1
    for _, size, align in fields:
        off = (off + align - 1) // align * align
        offs.append(off)
        off += size
        al = max(al, align)
    return offs, (off + al - 1) // al * al


def c_struct_fields():
    """C struct -> [field names in order] parsed from the header."""
    text = HDR.read_text()
    out = {}
    for m in re.finditer(r"typedef struct (\w+) \{(.*?)\} \1;", text, re.S):
        body = re.sub(r"/\*.*?\*/", "", m.group(2), flags=re.S)
        names = [re.search(r"(\w+)\s*(\[\d+\])?\s*$", d.strip()).group(1)
                 for d in body.split(";") if d.strip()]
        out[m.group(1)] = names
    return out


@pytest.fixture(scope="module")
def c_offsets(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    fields = c_struct_fields()
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{HDR}"', "int main(void) {"]
    for cs in STRUCTS.values():
        lines.append(f'  printf("{cs} size %zu\\n", sizeof({cs}));')
        for f in fields[cs]:
            lines.append(f'  printf("{cs} {f} %zu\\n", offsetof({cs}, {f}));')
    lines.append('  printf("qxg_program_info num_slices %zu\\n", offsetof(qxg_program_info, num_slices));')
    lines.append('  printf("qxg_program_info output_size %zu\\n", offsetof(qxg_program_info, output_size));')
    lines.append('  printf("qxg_program_info size %zu\\n", sizeof(qxg_program_info));')
    lines.append("  return 0; }")
    d = tmp_path_factory.mktemp("layout")
    (d / "probe.c").write_text("\n".join(lines) + "\n")
    subprocess.run([cc, "-std=c11", "-o", str(d / "probe"), str(d / "probe.c")], check=True)
    res = {}
    for ln in subprocess.run([str(d / "probe")], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = ln.split()
        res[(s, f)] = int(v)
    return res, fields


def test_struct_mirrors_match_the_header(c_offsets):
    res, cfields = c_offsets
    js = julia_structs(JL.read_text())
    for jname, cname in STRUCTS.items():
        assert jname in js, f"{jname} missing from the Julia binding"
        jf = js[jname]
        offs, size = c_layout(jf)
        assert [f for f, _, _ in jf] == cfields[cname], f"{jname}: field order differs from {cname}"
        assert size == res[(cname, "size")], f"{jname}: {size} bytes, {cname} has {res[(cname, 'size')]}"
        for (f, _, _), o in zip(jf, offs):
            assert o == res[(cname, f)], f"{jname}.{f} at {o}, {cname}.{f} at {res[(cname, f)]}"
    # load_qx reads num_slices and output_size from the first 16 bytes of a 128-byte buffer
    assert res[("qxg_program_info", "num_slices")] == 0 and res[("qxg_program_info", "output_size")] == 8
    assert res[("qxg_program_info", "size")] <= 128


def _jl_class(t):
    t = t.strip()
    if t in ("Int32", "Cint", "UInt32"):
        return "i32"
    if t in ("Int64", "UInt64", "Csize_t"):
        return "i64"
    if t == "Float64":
        return "f64"
    if t in ("Cvoid",):
        return "void"
    if t == "Cstring" or t.startswith("Ptr{") or t.startswith("Ref{"):
        return "ptr"
    raise AssertionError(f"unhandled Julia type {t}")


def _c_class(decl):
    decl = decl.strip()
    if "*" in decl:
        return "ptr"
    if re.match(r"(const\s+)?(int32_t|int)\b", decl):
        return "i32"
    if re.match(r"(const\s+)?int64_t\b", decl):
        return "i64"
    if re.match(r"(const\s+)?double\b", decl):
        return "f64"
    if decl == "void":
        return "void"
    raise AssertionError(f"unhandled C declaration {decl}")


def _split_top(s):
    """Split a comma list at depth 0 of {} and ()."""
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch in "{(":
            depth += 1
        elif ch in "})":
            depth -= 1
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
        else:
            cur += ch
    if cur.strip():
        out.append(cur)
    return [x.strip() for x in out if x.strip()]


def _tuple_after(text, i):
    """The balanced (...) starting at or after text[i] -> (inner, end index)."""
    i = text.index("(", i)
    depth = 0
    for j in range(i, len(text)):
        depth += text[j] == "("
        depth -= text[j] == ")"
        if depth == 0:
            return text[i + 1:j], j + 1
    raise AssertionError("unbalanced parentheses")


def header_prototypes():
    text = re.sub(r"/\*.*?\*/", "", HDR.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"^([\w\s\*]+?)\b(qxg_\w+)\s*\(([^)]*)\);", text, re.M):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        params = [] if args.strip() == "void" else [_c_class(a) for a in args.split(",")]
        out[name] = (_c_class(ret), params)
    return out


def julia_ccalls(text):
    """[(name, return class, [argument classes])] for every ccall, resolving `sig` variables."""
    sigs = []     # (position, variable, tuple text): a call uses the nearest earlier definition
    for m in re.finditer(r"^\s*(\w+)\s*=\s*\((Cstring|Ptr|Ref|Int|Float|Cint)", text, re.M):
        inner, _ = _tuple_after(text, m.start(2) - 1)
        sigs.append((m.start(), m.group(1), inner))
    out = []
    for m in re.finditer(r"ccall\(\(:(qxg_\w+),\s*libqxgpu\),\s*(\w+),\s*", text):
        rest = text[m.end():]
        if rest.startswith("("):
            inner, _ = _tuple_after(rest, 0)
        else:
            var = re.match(r"\w+", rest).group(0)
            inner = [t for pos, v, t in sigs if v == var and pos < m.start()][-1]
        out.append((m.group(1), _jl_class(m.group(2)), [_jl_class(t) for t in _split_top(inner)]))
    return out


def test_ccall_signatures_match_the_header():
    protos = header_prototypes()
    calls = julia_ccalls(JL.read_text())
    assert len(calls) >= 10
    for name, ret, args in calls:
        assert name in protos, f"{name} is not declared in include/qxgpu.h"
        cret, cargs = protos[name]
        assert ret == cret, f"{name}: returns {ret} in Julia, {cret} in C"
        assert args == cargs, f"{name}: Julia passes {args}, the header declares {cargs}"


def test_drop_in_methods_have_the_reference_signatures():
    """The binding offers QXTools' own entry points for the path with the reference's argument
    lists: single_amplitude(tnc::TensorNetworkCircuit, plan::Array{NTuple{3, Symbol}, 1},
    amplitude::Union{String, Nothing}=nothing) (src/simulation.jl:86) and run_simulation(circ;
    num_amplitudes, seed) (src/simulation.jl:103-105), each with extra keywords only, and both
    built from QXTools' own build_compute_graph / generate_dsl_files."""
    text = JL.read_text()
    sa = re.search(r"^function single_amplitude\(tnc::QXTools\.TensorNetworkCircuit,\s*plan::Array\{NTuple\{3,\s*"
                   r"Symbol\},\s*1\},\s*amplitude::Union\{String,\s*Nothing\}=nothing;", text, re.M)
    assert sa, "single_amplitude(tnc, plan, amplitude) with the reference's argument types is missing"
    rs = re.search(r"^function run_simulation\(circ;\s*num_amplitudes::Union\{Int64,\s*Nothing\}=nothing,\s*"
                   r"seed::Union\{Int64,\s*Nothing\}=nothing", text, re.M)
    assert rs, "run_simulation(circ; num_amplitudes, seed) is missing"
    assert "QXTools.build_compute_graph(tnc, plan, bond_groups)" in text
    assert "QXTools.generate_dsl_files(cg, prefix; force=true)" in text
    # every exported name is defined
    exported = re.search(r"^export (.*?)\n(?=\S)", text, re.M | re.S).group(1)
    for name in re.findall(r"\w+!?", exported):
        assert re.search(rf"^(function |const |struct |mutable struct ){re.escape(name)}(?![\w!])|^{re.escape(name)}\(",
                         text, re.M), f"{name} is exported but not defined"
