"""ctypes binding of libqxgpu (include/qxgpu.h) and the programme builder.

`Programme.from_graph(graph)` turns a `.qx` command list (compute_graph.ComputeGraph or parsed
`.qx` text) into the C ABI's arrays: tensor symbols -> dense ids, `data_<k>` keys -> data ids,
`v<i>` -> slice variable i-1, 1-based qubits and rank positions -> 0-based.  `Executor` owns one
`qxg_program` on one GPU.  The library is required: importing works without it, but creating an
Executor raises if libqxgpu.so is missing or no GPU is visible (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes as ct
from collections import OrderedDict
from pathlib import Path

import numpy as np

from .compute_graph import ComputeGraph, Load, Ncon, Output, Save, View

__all__ = ["QXG_OP", "PRECISION", "QXGError", "Programme", "Executor", "load_library",
           "library_path", "ncon_device", "parse_yml_output"]

_HERE = Path(__file__).resolve().parent
_LIB_PATH = _HERE / "_build" / "libqxgpu.so"

QXG_OP = {"load": 1, "view": 2, "output": 3, "ncon": 4, "save": 5}
PRECISION = {"fp64": 0, "split_bf16": 1, "split_tf32": 2, "fp32": 3}
_STATUS = {0: "QXG_OK", -1: "QXG_ERR_INVALID", -2: "QXG_ERR_CUDA", -3: "QXG_ERR_OOM",
           -4: "QXG_ERR_UNSUPPORTED", -5: "QXG_ERR_TIMEOUT", -6: "QXG_ERR_STATE"}


class QXGError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS.get(code, code)}: {msg}")
        self.code = code


class qxg_instr(ct.Structure):
    _fields_ = [(n, ct.c_int32) for n in
                ("op", "dst", "a", "b", "pos", "dim", "nc", "na", "nb", "label_off")]


class qxg_options(ct.Structure):
    _fields_ = [("precision", ct.c_int32), ("device", ct.c_int32), ("workspace_limit", ct.c_int64),
                ("max_bitstring_batch", ct.c_int32), ("max_slice_batch", ct.c_int32),
                ("use_graphs", ct.c_int32), ("tc_tuning", ct.c_int32),
                ("tc_plane_budget_mb", ct.c_int32), ("tc_wait_limit", ct.c_int32), ("tc_stall_test", ct.c_int32),
                ("cuda_core_joins", ct.c_int32), ("reserved", ct.c_int32 * 2)]


class qxg_qx_sizes(ct.Structure):
    _fields_ = [("ninstr", ct.c_int32), ("ndata", ct.c_int32), ("nlabels", ct.c_int64), ("ndims", ct.c_int64),
                ("key_bytes", ct.c_int64), ("nqubits", ct.c_int32), ("reserved", ct.c_int32 * 3)]


class qxg_yml_output(ct.Structure):
    _fields_ = [("method", ct.c_int32), ("num_qubits", ct.c_int32), ("num_samples", ct.c_int64),
                ("nbitstrings", ct.c_int64), ("seed", ct.c_int64), ("M", ct.c_double), ("has_seed", ct.c_int32),
                ("fix_M", ct.c_int32), ("reserved", ct.c_int32 * 4)]


OUTPUT_METHODS = ("List", "Uniform", "Rejection")   # qxg_output_method


class qxg_plan_options(ct.Structure):
    _fields_ = [("trials", ct.c_int32), ("greedy_trials", ct.c_int32), ("seed", ct.c_int64), ("max_log2", ct.c_double),
                ("num_sliced", ct.c_int32), ("max_sliced", ct.c_int32), ("flops_per_s", ct.c_double),
                ("bytes_per_s", ct.c_double), ("tensor_batched", ct.POINTER(ct.c_uint8)), ("batch_log2", ct.c_double),
                ("reserved", ct.c_int32 * 6)]


class qxg_plan_stats(ct.Structure):
    _fields_ = [("log2_flops", ct.c_double), ("log2_flops_total", ct.c_double), ("max_log2", ct.c_double),
                ("time", ct.c_double), ("log2_slices", ct.c_double), ("num_sliced", ct.c_int32),
                ("trees_tried", ct.c_int32), ("reserved", ct.c_int32 * 6)]


class qxg_program_info(ct.Structure):
    _fields_ = [("num_slices", ct.c_int64), ("output_size", ct.c_int64), ("num_qubits", ct.c_int32),
                ("num_steps", ct.c_int32), ("bitstring_batch", ct.c_int32), ("slice_batch", ct.c_int32),
                ("workspace_bytes", ct.c_int64), ("flops_per_amplitude", ct.c_double),
                ("flops_executed_per_pass", ct.c_double), ("bytes_executed_per_pass", ct.c_double),
                ("num_steps_invariant", ct.c_int32), ("num_steps_slice", ct.c_int32),
                ("num_steps_bitstring", ct.c_int32), ("num_steps_tensor_core", ct.c_int32),
                ("num_steps_fused", ct.c_int32), ("num_steps_tuned", ct.c_int32),
                ("reserved", ct.c_int32 * 2)]


class qxg_step_profile(ct.Structure):
    _fields_ = [("instr", ct.c_int32), ("kernel", ct.c_int32), ("launches", ct.c_int64), ("ms", ct.c_double),
                ("flops", ct.c_double), ("bytes", ct.c_double)]


KERNEL_KINDS = {0: "contract_fp64", 1: "contract_fp32", 2: "contract_tc", 3: "view", 4: "output", 5: "reduce",
                6: "tc_pack", 7: "contract_batch"}

_lib = None


def library_path() -> Path:
    return _LIB_PATH


def load_library(path=None):
    """Load libqxgpu.so and declare its signatures (no GPU needed to load)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise QXGError(-6, f"{p} is missing: build it with qxtools.jl_gb300/build.py "
                           "(or __graft_entry__.build())")
    lib = ct.CDLL(str(p))
    P = ct.c_void_p
    lib.qxg_program_create.argtypes = [ct.POINTER(qxg_instr), ct.c_int32, ct.POINTER(ct.c_int32), ct.c_int64,
                                       ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), ct.c_int32, ct.c_int32,
                                       ct.POINTER(qxg_options), ct.POINTER(P)]
    lib.qxg_program_set_data.argtypes = [P, ct.c_int32, ct.POINTER(ct.c_double), ct.c_int64]
    lib.qxg_parse_qx.argtypes = [ct.c_char_p, ct.POINTER(qxg_qx_sizes), ct.POINTER(qxg_instr),
                                 ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), ct.c_char_p]
    lib.qxg_parse_yml_output.argtypes = [ct.c_char_p, ct.POINTER(qxg_yml_output), ct.c_char_p, ct.c_int64]
    lib.qxg_plan_contraction.argtypes = [ct.c_int32, ct.POINTER(ct.c_int64), ct.POINTER(ct.c_int32), ct.c_int32,
                                         ct.POINTER(ct.c_int32), ct.POINTER(ct.c_uint8), ct.POINTER(qxg_plan_options),
                                         ct.POINTER(ct.c_int32), ct.POINTER(ct.c_uint8), ct.POINTER(qxg_plan_stats)]
    lib.qxg_amplitudes.argtypes = [P, ct.c_char_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.POINTER(ct.c_double)]
    lib.qxg_amplitudes_device.argtypes = [P, P, ct.c_int32, ct.c_int64, ct.c_int64, P]
    lib.qxg_program_synchronize.argtypes = [P]
    lib.qxg_program_stream.argtypes = [P]
    lib.qxg_program_stream.restype = P
    lib.qxg_program_info_get.argtypes = [P, ct.POINTER(qxg_program_info)]
    lib.qxg_program_destroy.argtypes = [P]
    lib.qxg_program_destroy.restype = None
    lib.qxg_ncon.argtypes = [ct.c_int32, P, ct.c_int32, ct.POINTER(ct.c_int32), P, ct.c_int32,
                             ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), P, ct.c_int32,
                             ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), P]
    lib.qxg_gradient.argtypes = [P, ct.c_char_p, ct.c_int32, ct.c_int64, ct.c_int64, ct.POINTER(ct.c_double),
                                 ct.POINTER(ct.c_double), ct.POINTER(ct.c_double)]
    lib.qxg_gradient.restype = ct.c_int
    lib.qxg_program_profile.argtypes = [P, ct.c_int32]
    lib.qxg_program_explain.argtypes = [P, ct.c_int32, ct.c_char_p, ct.c_int32]
    lib.qxg_program_tuning_get.argtypes = [P, ct.c_char_p, ct.c_int64]
    lib.qxg_program_tuning_set.argtypes = [P, ct.c_char_p]
    lib.qxg_program_profile_read.argtypes = [P, ct.POINTER(qxg_step_profile), ct.c_int32, ct.POINTER(ct.c_int32),
                                             ct.POINTER(ct.c_int64)]
    lib.qxg_last_error.restype = ct.c_char_p
    lib.qxg_version.restype = ct.c_char_p
    for f in ("qxg_program_create", "qxg_program_set_data", "qxg_amplitudes", "qxg_amplitudes_device",
              "qxg_program_synchronize", "qxg_program_info_get", "qxg_ncon", "qxg_program_profile",
              "qxg_program_profile_read"):
        getattr(lib, f).restype = ct.c_int
    if path is None:
        _lib = lib
    return lib


def _check(lib, rc: int):
    if rc != 0:
        raise QXGError(rc, lib.qxg_last_error().decode())


class Programme:
    """The C ABI's view of a `.qx` programme: instruction array, labels, leaf shapes and data."""

    def __init__(self, instrs: np.ndarray, labels: np.ndarray, data_keys: list, data: list,
                 nqubits: int, tensor_ids: dict):
        self.instrs = instrs            # (n, 10) int32
        self.labels = labels            # int32
        self.data_keys = data_keys
        self.data = data                # complex128 arrays (column-major shape)
        self.nqubits = nqubits
        self.tensor_ids = tensor_ids

    @property
    def data_rank(self) -> np.ndarray:
        return np.array([d.ndim for d in self.data], dtype=np.int32)

    @property
    def data_dims(self) -> np.ndarray:
        return np.array([x for d in self.data for x in d.shape], dtype=np.int64)

    def data_flat(self):
        """(concatenated interleaved doubles, complex offsets per leaf)."""
        offs, parts, o = [], [], 0
        for d in self.data:
            offs.append(o)
            flat = np.asarray(d, dtype=np.complex128).reshape(-1, order="F")
            parts.append(flat)
            o += flat.size
        cat = np.concatenate(parts) if parts else np.zeros(0, np.complex128)
        return np.ascontiguousarray(cat.view(np.float64)), np.array(offs, dtype=np.int64)

    @property
    def num_slices(self) -> int:
        vd = {}
        for r in self.instrs:
            if r[0] == QXG_OP["view"]:
                vd[int(r[3])] = int(r[5])
        n = 1
        for v in vd.values():
            n *= v
        return n

    @classmethod
    def from_commands(cls, commands, data: "OrderedDict[str, np.ndarray]", nqubits: int) -> "Programme":
        ids: dict = {}
        dkeys = list(data.keys())
        dpos = {k: i for i, k in enumerate(dkeys)}
        rows, labels = [], []

        def tid(name, define=False):
            if define:
                if name in ids:
                    raise ValueError(f"tensor {name} defined twice")
                ids[name] = len(ids)
            if name not in ids:
                raise ValueError(f"tensor {name} used before definition")
            return ids[name]

        for c in commands:
            if isinstance(c, Load):
                if c.data not in dpos:
                    raise ValueError(f"no data {c.data}")
                if tuple(np.shape(data[c.data])) != tuple(c.dims):
                    raise ValueError(f"load {c.name}: dims {c.dims} do not match data {np.shape(data[c.data])}")
                rows.append([1, tid(c.name, True), dpos[c.data], 0, 0, 0, 0, 0, 0, 0])
            elif isinstance(c, View):
                if not c.var.startswith("v"):
                    raise ValueError(f"bad slice variable {c.var}")
                src = tid(c.src)
                rows.append([2, tid(c.name, True), src, int(c.var[1:]) - 1, c.pos - 1, c.dim, 0, 0, 0, 0])
            elif isinstance(c, Output):
                rows.append([3, tid(c.name, True), c.qubit - 1, c.dim, 0, 0, 0, 0, 0, 0])
            elif isinstance(c, Ncon):
                a, b = tid(c.a), tid(c.b)
                off = len(labels)
                labels += list(c.c_labels) + list(c.a_labels) + list(c.b_labels)
                rows.append([4, tid(c.name, True), a, b, 0, 0, len(c.c_labels), len(c.a_labels),
                             len(c.b_labels), off])
            elif isinstance(c, Save):
                rows.append([5, 0, tid(c.name), 0, 0, 0, 0, 0, 0, 0])
            else:
                raise TypeError(f"unknown command {c!r}")
        instrs = np.array(rows, dtype=np.int32).reshape(-1, 10)
        return cls(instrs, np.array(labels, dtype=np.int32), dkeys,
                   [np.asarray(data[k], dtype=np.complex128) for k in dkeys], nqubits, ids)

    @classmethod
    def from_qx_text(cls, text: str, data: "OrderedDict[str, np.ndarray]", lib=None) -> "Programme":
        """A programme from `.qx` text through the library's own parser (qxg_parse_qx), with the
        leaf data given by key; the data ids follow the keys' order of first `load`."""
        lib = lib or load_library()
        raw = text.encode()
        sz = qxg_qx_sizes()
        _check(lib, lib.qxg_parse_qx(raw, ct.byref(sz), None, None, None, None, None))
        ins = (qxg_instr * max(sz.ninstr, 1))()
        lab = (ct.c_int32 * max(sz.nlabels, 1))()
        rank = (ct.c_int32 * max(sz.ndata, 1))()
        dims = (ct.c_int64 * max(sz.ndims, 1))()
        keys = ct.create_string_buffer(max(sz.key_bytes, 1))
        _check(lib, lib.qxg_parse_qx(raw, ct.byref(sz), ins, lab, rank, dims, keys))
        names = keys.raw[:sz.key_bytes].split(b"\0")[:sz.ndata]
        dkeys = [n.decode() for n in names]
        instrs = np.frombuffer(bytes(ins), dtype=np.int32)[:10 * sz.ninstr].reshape(-1, 10).copy()
        off, leaves = 0, []
        for i, k in enumerate(dkeys):
            shape = tuple(int(x) for x in dims[off:off + rank[i]])
            off += rank[i]
            if k not in data:
                raise ValueError(f"no data {k}")
            if tuple(np.shape(data[k])) != shape:
                raise ValueError(f"data {k}: shape {np.shape(data[k])}, the .qx loads {shape}")
            leaves.append(np.asarray(data[k], dtype=np.complex128))
        return cls(instrs, np.array(lab[:sz.nlabels], dtype=np.int32), dkeys, leaves, sz.nqubits, {})

    @classmethod
    def from_graph(cls, graph: ComputeGraph) -> "Programme":
        """Bitstrings carry one character per `output` command (qubit numbers 1..k), so a
        programme without outputs (open wires only) takes empty bitstrings."""
        nq = max([c.qubit for c in graph.commands if isinstance(c, Output)], default=0)
        return cls.from_commands(graph.commands, graph.data, nq)


def parse_yml_output(text: str, lib=None) -> "OrderedDict":
    """The `output:` block of `.yml` text through the library's reader (qxg_parse_yml_output),
    as the dict output_params_dict builds (src/outputs.jl:47-78): {"method", "params"} with the
    params each method writes."""
    lib = lib or load_library()
    raw = text.encode()
    o = qxg_yml_output()
    _check(lib, lib.qxg_parse_yml_output(raw, ct.byref(o), None, 0))
    params = OrderedDict()
    method = OUTPUT_METHODS[o.method]
    seed = int(o.seed) if o.has_seed else None
    if method == "List":
        n = o.nbitstrings * o.num_qubits
        buf = ct.create_string_buffer(max(n, 1))
        _check(lib, lib.qxg_parse_yml_output(raw, ct.byref(o), buf, n))
        packed = buf.raw[:n].decode()
        params["num_samples"] = int(o.num_samples)
        params["bitstrings"] = [packed[i * o.num_qubits:(i + 1) * o.num_qubits] for i in range(o.nbitstrings)]
    elif method == "Uniform":
        params["num_qubits"] = int(o.num_qubits)
        params["num_samples"] = int(o.num_samples)
        params["seed"] = seed
    else:
        params["num_qubits"] = int(o.num_qubits)
        params["M"] = float(o.M)
        params["fix_M"] = bool(o.fix_M)
        params["seed"] = seed
        params["num_samples"] = int(o.num_samples)
    return OrderedDict([("method", method), ("params", params)])


def _bitstring_bytes(bitstrings, nqubits: int) -> bytes:
    if isinstance(bitstrings, str):
        bitstrings = [bitstrings]
    out = []
    for b in bitstrings:
        if len(b) != nqubits:
            raise ValueError(f"bitstring {b!r} does not have {nqubits} characters")
        out.append(b)
    return "".join(out).encode("ascii")


class Executor:
    """One compiled programme on one GPU (a `qxg_program` handle)."""

    def __init__(self, programme: Programme, precision: str = "fp64", device: int = 0,
                 workspace_limit: int = 0, max_bitstring_batch: int = 0, max_slice_batch: int = 0,
                 use_graphs: bool = False, tc_tuning="auto", tc_plane_budget_mb: int = 0,
                 tc_wait_limit: int = 0, tc_stall_test: bool = False, cuda_core_joins: bool = False):
        self.lib = load_library()
        self.programme = programme
        self.precision = precision
        opts = qxg_options()
        opts.precision = PRECISION[precision]
        opts.device = device
        opts.workspace_limit = workspace_limit
        opts.max_bitstring_batch = max_bitstring_batch
        opts.max_slice_batch = max_slice_batch
        opts.use_graphs = int(use_graphs)
        opts.tc_plane_budget_mb = int(tc_plane_budget_mb)
        # bounded device waits: polls before giving up (0: the library's 2^20), and the test hook
        # that makes them run out (qxg_options.tc_stall_test)
        opts.tc_wait_limit = int(tc_wait_limit)
        opts.tc_stall_test = int(bool(tc_stall_test))
        # final joins of split-TF32 programmes: the tensor-core join (default) or the CUDA cores'
        # batched small GEMM
        opts.cuda_core_joins = int(bool(cuda_core_joins))
        # "auto": time each tensor-core step's tile variants once and keep the fastest;
        # "fixed" (= 1) or k >= 1: candidate k of every step
        if tc_tuning == "auto":
            opts.tc_tuning = 0
        elif tc_tuning == "fixed":
            opts.tc_tuning = 1
        elif isinstance(tc_tuning, int) and tc_tuning >= 1:
            opts.tc_tuning = tc_tuning
        else:
            raise ValueError("tc_tuning must be 'auto', 'fixed' or a candidate number >= 1")
        ins = np.ascontiguousarray(programme.instrs, dtype=np.int32)
        n = ins.shape[0]
        arr = (qxg_instr * n).from_buffer_copy(ins.tobytes())
        labels = np.ascontiguousarray(programme.labels, dtype=np.int32)
        lab_ptr = labels.ctypes.data_as(ct.POINTER(ct.c_int32)) if labels.size else None
        rank = np.ascontiguousarray(programme.data_rank)
        dims = np.ascontiguousarray(programme.data_dims)
        h = ct.c_void_p()
        _check(self.lib, self.lib.qxg_program_create(
            arr, n, lab_ptr, labels.size, rank.ctypes.data_as(ct.POINTER(ct.c_int32)),
            dims.ctypes.data_as(ct.POINTER(ct.c_int64)) if dims.size else ct.POINTER(ct.c_int64)(),
            len(programme.data), programme.nqubits, ct.byref(opts), ct.byref(h)))
        self._h = h
        for i, d in enumerate(programme.data):
            flat = np.ascontiguousarray(np.asarray(d, dtype=np.complex128).reshape(-1, order="F"))
            _check(self.lib, self.lib.qxg_program_set_data(
                h, i, flat.view(np.float64).ctypes.data_as(ct.POINTER(ct.c_double)), flat.size))

    def close(self):
        if getattr(self, "_h", None):
            self.lib.qxg_program_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def info(self) -> dict:
        inf = qxg_program_info()
        _check(self.lib, self.lib.qxg_program_info_get(self._h, ct.byref(inf)))
        return {f: getattr(inf, f) for f, _ in qxg_program_info._fields_ if f != "reserved"}

    @property
    def num_slices(self) -> int:
        return self.info()["num_slices"]

    def amplitudes(self, bitstrings, slices=None) -> np.ndarray:
        """Saved tensor for each bitstring, summed over slices (host buffers in and out).
        Returns complex128 of shape (n, output_size) (output_size 1: amplitudes)."""
        if isinstance(bitstrings, str):
            bitstrings = [bitstrings]
        bitstrings = list(bitstrings)
        n = len(bitstrings)
        info = self.info()
        s0, s1 = (0, info["num_slices"]) if slices is None else slices
        buf = _bitstring_bytes(bitstrings, self.programme.nqubits)
        out = np.zeros(2 * n * info["output_size"], dtype=np.float64)
        _check(self.lib, self.lib.qxg_amplitudes(self._h, buf, n, s0, s1,
                                                 out.ctypes.data_as(ct.POINTER(ct.c_double))))
        return out.view(np.complex128).reshape(n, info["output_size"])

    def leaf_slices(self) -> dict:
        """instruction index of each `load` -> (offset, shape) of its gradient in the flat vector."""
        if getattr(self, "_leaf_layout", None) is not None:
            return self._leaf_layout
        out, o = {}, 0
        for i, r in enumerate(self.programme.instrs):
            if int(r[0]) == QXG_OP["load"]:
                shape = tuple(self.programme.data[int(r[2])].shape)
                out[i] = (o, shape)
                o += int(np.prod(shape)) if shape else 1
        self._gsize = o
        self._leaf_layout = out
        return out

    def gradient(self, bitstrings, amp_bar=None, slices=None, flat=False):
        """Reverse-mode gradient (qxg_gradient): returns (amplitudes (n, out_size), {instruction
        index of each load: dL/d conj(leaf) as an array of the leaf's shape}).  amp_bar = dL/d
        conj(amplitude) per bitstring, shape (n, out_size); None -> L = sum |amplitude|^2.
        flat=True returns the gradients as the one complex vector that leaf_slices() indexes."""
        if isinstance(bitstrings, str):
            bitstrings = [bitstrings]
        bitstrings = list(bitstrings)
        n = len(bitstrings)
        info = self.info()
        s0, s1 = (0, info["num_slices"]) if slices is None else slices
        lay = self.leaf_slices()
        buf = _bitstring_bytes(bitstrings, self.programme.nqubits)
        out = np.zeros(2 * n * info["output_size"], dtype=np.float64)
        grads = np.zeros(2 * max(self._gsize, 1), dtype=np.float64)
        ab = None
        if amp_bar is not None:
            ab = np.ascontiguousarray(np.asarray(amp_bar, dtype=np.complex128).reshape(n, info["output_size"]))
            ab = ab.view(np.float64).reshape(-1)
        D = ct.POINTER(ct.c_double)
        _check(self.lib, self.lib.qxg_gradient(self._h, buf, n, s0, s1, ab.ctypes.data_as(D) if ab is not None else None,
                                               out.ctypes.data_as(D), grads.ctypes.data_as(D)))
        g = grads.view(np.complex128)
        amps = out.view(np.complex128).reshape(n, info["output_size"])
        if flat:
            return amps, g
        leaf = {i: g[o:o + (int(np.prod(s)) if s else 1)].reshape(s, order="F") for i, (o, s) in lay.items()}
        return amps, leaf

    def amplitudes_device(self, d_bitstrings_ptr: int, n: int, d_out_ptr: int, slices=None):
        """Enqueue on the programme's stream with device-resident inputs/outputs (no sync)."""
        s0, s1 = (0, self.num_slices) if slices is None else slices
        _check(self.lib, self.lib.qxg_amplitudes_device(self._h, ct.c_void_p(d_bitstrings_ptr), n, s0, s1,
                                                        ct.c_void_p(d_out_ptr)))

    def synchronize(self):
        _check(self.lib, self.lib.qxg_program_synchronize(self._h))

    def profile(self, enable: bool = True):
        """Start (clearing earlier records) or stop CUDA-event timing of every launch."""
        _check(self.lib, self.lib.qxg_program_profile(self._h, int(enable)))

    def profile_read(self):
        """-> (list of per-command dicts {instr, kernel, launches, ms, flops, bytes}, total
        kernel launches since creation)."""
        n = ct.c_int32(0)
        launches = ct.c_int64(0)
        _check(self.lib, self.lib.qxg_program_profile_read(self._h, None, 0, ct.byref(n), ct.byref(launches)))
        buf = (qxg_step_profile * max(1, n.value))()
        _check(self.lib, self.lib.qxg_program_profile_read(self._h, buf, n.value, ct.byref(n), ct.byref(launches)))
        rows = [{"instr": b.instr, "kernel": KERNEL_KINDS.get(b.kernel, str(b.kernel)), "launches": b.launches,
                 "ms": b.ms, "flops": b.flops, "bytes": b.bytes} for b in buf[:n.value]]
        return rows, launches.value

    def tuning(self) -> str:
        """The autotuner's decisions as text (qxg_program_tuning_get)."""
        n = self.lib.qxg_program_tuning_get(self._h, None, 0)
        if n < 0:
            _check(self.lib, n)
        buf = ct.create_string_buffer(n + 1)
        self.lib.qxg_program_tuning_get(self._h, buf, n + 1)
        return buf.value.decode()

    def set_tuning(self, text: str):
        """Preload decisions written by tuning(), here or in another process."""
        _check(self.lib, self.lib.qxg_program_tuning_set(self._h, text.encode()))

    def explain(self, instr: int) -> str:
        """One line on how the current plan executes `ncon` command `instr` (qxg_program_explain)."""
        buf = ct.create_string_buffer(4096)
        _check(self.lib, self.lib.qxg_program_explain(self._h, int(instr), buf, len(buf)))
        return buf.value.decode()

    @property
    def stream(self) -> int:
        return self.lib.qxg_program_stream(self._h) or 0


def ncon_device(precision: str, C_ptr: int, c_labels, A_ptr: int, a_labels, a_dims, B_ptr: int, b_labels,
                b_dims, stream: int = 0):
    """One pairwise contraction on device buffers through qxg_ncon."""
    lib = load_library()

    def i32(x):
        a = np.ascontiguousarray(np.asarray(x, dtype=np.int32))
        return a, (a.ctypes.data_as(ct.POINTER(ct.c_int32)) if a.size else None)

    def i64(x):
        a = np.ascontiguousarray(np.asarray(x, dtype=np.int64))
        return a, (a.ctypes.data_as(ct.POINTER(ct.c_int64)) if a.size else None)
    lc, plc = i32(c_labels)
    la, pla = i32(a_labels)
    lb, plb = i32(b_labels)
    ad, pad = i64(a_dims)
    bd, pbd = i64(b_dims)
    _check(lib, lib.qxg_ncon(PRECISION[precision], ct.c_void_p(C_ptr), lc.size, plc, ct.c_void_p(A_ptr), la.size,
                             pla, pad, ct.c_void_p(B_ptr), lb.size, plb, pbd, ct.c_void_p(stream)))
