"""`.qx` DSL text and `.yml` parameter files (formats of docs/src/users_guide.md:22-165).

`.qx`: first line `# version: <v>`, further `#` lines are metadata comments, then one command
per line: `load <t> <data_key> <d1,d2,..>`, `view <new> <t> <v_i> <rank pos> <dim>`,
`output <t> <qubit> <dim>`, `ncon <C> <c labels> <A> <a labels> <B> <b labels>` (labels
comma separated, `0` for a scalar), `save <label> <t>`.

`.yml`: the `output:` block written by `generate_parameter_file` (src/simulation.jl:149-155)
from `output_params_dict` (src/outputs.jl:47-78), e.g. method List with `num_samples` and
`bitstrings`.  PyYAML is not available, so a small reader/writer for this subset (nested
mappings, sequences of scalars, ints, floats, booleans, `~`/null and quoted strings) is
implemented here.

Leaf data (`.jld2` in the reference, tensor_cache.jl:90-106) is written as a NumPy `.npz`
archive with the same `data_<k>` keys.
"""
from __future__ import annotations

from collections import OrderedDict

import numpy as np

from .compute_graph import ComputeGraph, Load, Ncon, Output, Save, View

__all__ = ["DSL_VERSION", "write_qx", "format_qx", "parse_qx", "read_qx", "write_data",
           "read_data", "write_yml", "read_yml", "format_yml", "parse_yml"]

DSL_VERSION = "0.4.0"


def _labels(ls) -> str:
    return "0" if len(ls) == 0 else ",".join(str(int(x)) for x in ls)


def _meta_lines(meta, indent=0):
    out = []
    pad = "  " * indent
    for k, v in meta.items():
        if isinstance(v, dict):
            out.append(f"# {pad}{k}:")
            out += _meta_lines(v, indent + 1)
        elif isinstance(v, (list, tuple)):
            out.append(f"# {pad}{k}:")
            out += [f"# {pad}  - {x}" for x in v]
        else:
            out.append(f"# {pad}{k}: {v}")
    return out


def format_qx(graph: ComputeGraph, metadata=None) -> str:
    lines = [f"# version: {DSL_VERSION}"]
    if metadata:
        lines += _meta_lines(metadata)
    for c in graph.commands:
        if isinstance(c, Load):
            lines.append(f"load {c.name} {c.data} {_labels(c.dims) if c.dims else ''}".rstrip())
        elif isinstance(c, View):
            lines.append(f"view {c.name} {c.src} {c.var} {c.pos} {c.dim}")
        elif isinstance(c, Output):
            lines.append(f"output {c.name} {c.qubit} {c.dim}")
        elif isinstance(c, Ncon):
            lines.append(f"ncon {c.name} {_labels(c.c_labels)} {c.a} {_labels(c.a_labels)} "
                         f"{c.b} {_labels(c.b_labels)}")
        elif isinstance(c, Save):
            lines.append(f"save {c.label} {c.name}")
        else:
            raise TypeError(f"unknown command {c!r}")
    return "\n".join(lines) + "\n"


def write_qx(graph: ComputeGraph, path: str, metadata=None):
    with open(path, "w") as f:
        f.write(format_qx(graph, metadata))


def _parse_labels(tok: str) -> tuple:
    if tok == "0":
        return ()
    return tuple(int(x) for x in tok.split(","))


def parse_qx(text: str):
    """Parse `.qx` text -> (commands, version).  Raises ValueError on a malformed line."""
    commands = []
    version = None
    for n, raw in enumerate(text.splitlines(), start=1):
        line = raw.strip()
        if not line:
            continue
        if line.startswith("#"):
            if n == 1 and "version:" in line:
                version = line.split("version:", 1)[1].strip()
            continue
        tok = line.split()
        op = tok[0]
        try:
            if op == "load":
                dims = tuple(int(x) for x in tok[3].split(",")) if len(tok) > 3 else ()
                commands.append(Load(tok[1], tok[2], dims))
            elif op == "view":
                commands.append(View(tok[1], tok[2], tok[3], int(tok[4]), int(tok[5])))
            elif op == "output":
                commands.append(Output(tok[1], int(tok[2]), int(tok[3])))
            elif op == "ncon":
                commands.append(Ncon(tok[1], _parse_labels(tok[2]), tok[3], _parse_labels(tok[4]),
                                     tok[5], _parse_labels(tok[6])))
            elif op == "save":
                commands.append(Save(tok[1], tok[2]))
            else:
                raise ValueError(f"unknown instruction {op!r}")
        except (IndexError, ValueError) as e:
            raise ValueError(f"line {n}: cannot parse {raw!r}: {e}") from None
    return commands, version


def read_qx(path: str):
    with open(path) as f:
        return parse_qx(f.read())


def write_data(data: "OrderedDict[str, np.ndarray]", path: str):
    np.savez(path, **{k: np.asarray(v, dtype=np.complex128) for k, v in data.items()})


def read_data(path: str) -> "OrderedDict[str, np.ndarray]":
    with np.load(path) as z:
        return OrderedDict((k, z[k]) for k in z.files)


# ---------------------------------------------------------------------------------------
# minimal YAML subset
# ---------------------------------------------------------------------------------------
def _scalar_out(v) -> str:
    if v is None:
        return "~"
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (int, np.integer)):
        return str(int(v))
    if isinstance(v, (float, np.floating)):
        return repr(float(v))
    s = str(v)
    return '"' + s.replace("\\", "\\\\").replace('"', '\\"') + '"'


def format_yml(obj, indent=0) -> str:
    pad = "  " * indent
    lines = []
    for k, v in obj.items():
        if isinstance(v, dict):
            lines.append(f"{pad}{k}:")
            lines.append(format_yml(v, indent + 1).rstrip("\n"))
        elif isinstance(v, (list, tuple)):
            lines.append(f"{pad}{k}:")
            lines += [f"{pad}  - {_scalar_out(x)}" for x in v]
        else:
            lines.append(f"{pad}{k}: {_scalar_out(v)}")
    return "\n".join(l for l in lines if l != "") + "\n"


def _scalar_in(s: str):
    s = s.strip()
    if s in ("~", "null", "Null", "NULL", ""):
        return None
    if s in ("true", "True"):
        return True
    if s in ("false", "False"):
        return False
    if len(s) >= 2 and s[0] == s[-1] and s[0] in "\"'":
        body = s[1:-1]
        return body.replace('\\"', '"').replace("\\\\", "\\") if s[0] == '"' else body
    try:
        return int(s)
    except ValueError:
        pass
    try:
        return float(s)
    except ValueError:
        return s


def parse_yml(text: str):
    """Parse the YAML subset written by `format_yml` (and by YAML.write_file for the
    reference's `output:` block)."""
    rows = []
    for raw in text.splitlines():
        if not raw.strip() or raw.strip().startswith("#"):
            continue
        ind = len(raw) - len(raw.lstrip(" "))
        rows.append((ind, raw.strip()))

    def block(i, ind):
        if i < len(rows) and rows[i][1].startswith("- "):
            out = []
            while i < len(rows) and rows[i][0] == ind and rows[i][1].startswith("- "):
                out.append(_scalar_in(rows[i][1][2:]))
                i += 1
            return out, i
        out = OrderedDict()
        while i < len(rows) and rows[i][0] == ind:
            line = rows[i][1]
            if ":" not in line:
                raise ValueError(f"cannot parse YAML line {line!r}")
            k, v = line.split(":", 1)
            k = k.strip()
            i += 1
            if v.strip() == "":
                if i < len(rows) and (rows[i][0] > ind or (rows[i][0] == ind and rows[i][1].startswith("- "))):
                    out[k], i = block(i, rows[i][0])
                else:
                    out[k] = None
            else:
                out[k] = _scalar_in(v)
        return out, i

    obj, _ = block(0, rows[0][0]) if rows else (OrderedDict(), 0)
    return obj


def write_yml(obj, path: str):
    with open(path, "w") as f:
        f.write(format_yml(obj))


def read_yml(path: str):
    with open(path) as f:
        return parse_yml(f.read())
