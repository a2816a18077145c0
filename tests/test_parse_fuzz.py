"""Mutation fuzzing of the library's host-side readers, qxg_parse_qx and qxg_parse_yml_output.

Both read text from files a user hands in, so malformed text must come back as a negative status,
never as a crash or a write past the caller's buffers.  Seeded random edits (deleted, duplicated
and replaced spans, numbers out of range, truncation) are applied to valid `.qx` and `.yml`
texts; each is parsed with the two-call protocol (sizes first, then buffers of exactly those
sizes, with guard bytes after each buffer that must stay untouched).  The loop runs in a child
process so that a crash fails the test instead of ending the test run; a second test runs the
same texts through the readers built with AddressSanitizer and UBSan (tests/emu/parse_driver.cpp).
"""
import shutil
import subprocess
import sys
import textwrap
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
N_MUTANTS = 1500          # mutated texts per valid input

CHILD = textwrap.dedent(r'''
    import ctypes as ct, sys
    import numpy as np
    sys.path.insert(0, sys.argv[1])
    import __graft_entry__ as e
    q = e.load()
    lib = q.load_library()
    ex = q.executor
    GUARD = 64

    def guarded(n, itemsize):
        buf = (ct.c_ubyte * (n * itemsize + GUARD))()
        ct.memset(buf, 0xA5, len(buf))
        return buf

    def intact(buf, used):
        return all(b == 0xA5 for b in bytes(buf)[used:])

    def parse_qx(raw):
        sz = ex.qxg_qx_sizes()
        rc = lib.qxg_parse_qx(raw, ct.byref(sz), None, None, None, None, None)
        if rc != 0:
            assert rc < 0, rc
            return rc
        assert sz.ninstr >= 0 and sz.ndata >= 0 and sz.nlabels >= 0 and sz.ndims >= 0 and sz.key_bytes >= 0
        bufs = [(guarded(sz.ninstr, 40), 40 * sz.ninstr), (guarded(sz.nlabels, 4), 4 * sz.nlabels),
                (guarded(sz.ndata, 4), 4 * sz.ndata), (guarded(sz.ndims, 8), 8 * sz.ndims),
                (guarded(sz.key_bytes, 1), sz.key_bytes)]
        P = [ct.cast(b, t) for (b, _), t in zip(bufs, (ct.POINTER(ex.qxg_instr), ct.POINTER(ct.c_int32),
                                                        ct.POINTER(ct.c_int32), ct.POINTER(ct.c_int64), ct.c_char_p))]
        rc2 = lib.qxg_parse_qx(raw, ct.byref(sz), *P)
        assert rc2 == 0, (rc2, raw[:200])
        for b, used in bufs:
            assert intact(b, used), raw[:200]
        return 0

    def parse_yml(raw):
        o = ex.qxg_yml_output()
        rc = lib.qxg_parse_yml_output(raw, ct.byref(o), None, 0)
        if rc != 0:
            assert rc < 0, rc
            return rc
        n = o.nbitstrings * o.num_qubits
        assert n >= 0
        b = guarded(n, 1)
        rc2 = lib.qxg_parse_yml_output(raw, ct.byref(o), ct.cast(b, ct.c_char_p), n)
        assert rc2 == 0, (rc2, raw[:200])
        assert intact(b, n), raw[:200]
        return 0

    def records(path):
        data = open(path, "rb").read()
        at = 0
        while at < len(data):
            nl = data.index(b"\n", at)
            n = int(data[at:nl])
            yield data[nl + 1:nl + 1 + n]
            at = nl + 1 + n

    ok = bad = 0
    for kind, path in (("qx", sys.argv[2]), ("yml", sys.argv[3])):
        for k, text in enumerate(records(path)):
            rc = (parse_qx if kind == "qx" else parse_yml)(text)
            if k < int(sys.argv[4]):
                assert rc == 0, (kind, k)     # the unmutated inputs come first
            ok += rc == 0
            bad += rc != 0
    print("accepted", ok, "rejected", bad)
''')


TOKENS = [b" ", b"\n", b",", b"0", b"-1", b"9999999999", b"2147483648", b"v", b"#", b"\t", b":",
          b"'", b'"', b"[", b"]", b"ncon", b"view", b"output", b"load", b"save", b"~", b"- "]


def mutate(rng, text: bytes) -> bytes:
    t = bytearray(text)
    for _ in range(int(rng.integers(1, 4))):
        if not t:
            break
        k = int(rng.integers(0, 4))
        i = int(rng.integers(0, len(t)))
        j = min(len(t), i + int(rng.integers(1, 24)))
        if k == 0:
            del t[i:j]
        elif k == 1:
            t[i:i] = t[i:j]
        elif k == 2:
            t[i:j] = TOKENS[int(rng.integers(0, len(TOKENS)))]
        else:
            del t[i:]
    return bytes(t)


@pytest.fixture(scope="module")
def corpus(q, tmp_path_factory):
    """(qx corpus file, yml corpus file, number of unmutated inputs at the head of each)."""
    tmp = tmp_path_factory.mktemp("fuzz")
    circ = q.create_rqc_circuit(2, 3, 4, seed=8)
    tnc = q.convert_to_tnc(circ, decompose=True)
    groups, plan, meta = q.contraction_scheme(tnc, 2, seed=2, time=1)
    q.dsl.write_qx(q.build_compute_graph(tnc, plan, groups), str(tmp / "rqc.qx"), metadata=meta)
    qx = [(ROOT / "tests" / "golden" / "users_guide_ghz2.qx").read_bytes(), (tmp / "rqc.qx").read_bytes()]
    ymls = []
    for k, (method, kw) in enumerate([("List", dict(num_outputs=5, seed=3)),
                                      ("Rejection", dict(num_outputs=7, seed=4)),
                                      ("Uniform", dict(num_outputs=9))]):
        q.generate_parameter_file(str(tmp / f"o{k}"), q.output_params_dict(6, output_method=method, **kw))
        ymls.append((tmp / f"o{k}.yml").read_bytes())
    rng = np.random.default_rng(20261204)
    out = []
    for name, texts in (("qx", qx), ("yml", ymls)):
        recs = list(texts) + [mutate(rng, t) for t in texts for _ in range(N_MUTANTS)]
        p = tmp / f"{name}.corpus"
        p.write_bytes(b"".join(b"%d\n" % len(r) + r for r in recs))
        out.append(p)
    return out[0], out[1], (len(qx), len(ymls))


def test_parsers_survive_mutated_text(gpu_lib, corpus):
    qx, yml, (nqx, nyml) = corpus
    assert nqx == 2 and nyml == 3
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT), str(qx), str(yml), "2"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.returncode, r.stdout[-2000:], r.stderr[-3000:])
    acc, rej = (int(x) for x in r.stdout.split()[1::2])
    assert acc > 0 and rej > 0        # the edits reach both outcomes


@pytest.mark.timeout(600)
def test_parsers_under_address_sanitizer(corpus, tmp_path):
    """The readers built with AddressSanitizer and UBSan over the same corpus: no access past
    the text or the caller's buffers, no undefined behaviour, and the same accept/reject split."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = tmp_path / "parse"
    cuda_inc = next((p for p in ("/usr/local/cuda/include",) if Path(p, "cuda_runtime.h").exists()), None)
    if cuda_inc is None:
        pytest.skip("no CUDA headers")
    cmd = [gxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-sanitize-recover=undefined",
           "-fno-omit-frame-pointer", "-I", str(ROOT / "include"), "-I", cuda_inc,
           "-x", "c++", str(ROOT / "qxtools.jl_gb300" / "csrc" / "qx_parse.cu"),
           "-x", "c++", str(ROOT / "tests" / "emu" / "parse_driver.cpp"), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    qx, yml, _ = corpus
    for kind, path in (("qx", qx), ("yml", yml)):
        r = subprocess.run([str(exe), kind, str(path)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, (kind, r.stdout[-1000:], r.stderr[-4000:])
        acc, rej = (int(x) for x in r.stdout.split()[1::2])
        assert acc > 0 and rej > 0, kind
