"""The C ABI library: loads without a GPU, exports every declared symbol, and
its host-side pieces (SDBF text codec, capacity rule) agree with the oracle
and the reference fixtures.  CPU only -- no kernel is launched here."""
import ctypes as C
import hashlib
import os
import re
import subprocess

import numpy as np

import cases

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    inc = os.path.join(REPO, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            syms |= set(re.findall(r"\b(sdbfg_\w+)\s*\(", src))
    return syms


def test_library_exports_every_declared_symbol(native):
    syms = declared_symbols()
    assert len(syms) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", native._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (sdbfg_\w+)", out))
    missing = syms - exported
    assert not missing, missing
    for s in syms:
        assert hasattr(native, s)


def test_context_create_reports_missing_gpu(native):
    import torch
    if torch.cuda.is_available():
        return
    h = C.c_void_p()
    assert native.sdbfg_ctx_create(0, C.byref(h)) != 0


def test_capacity_rule(native):
    import sdhash_gb300 as g
    lens = [100, 512, 2047, 2048, 1 << 20, (1 << 20) + 511, (1 << 20) + 512]
    assert g.Context.capacity(lens, 0) == sum((n >> 11) + 1 for n in lens if n >= 512)
    B = 16384
    assert g.Context.capacity(lens, B) == sum(n // B + (n % B >= 512) for n in lens if n >= 512)


def test_text_codec_matches_reference_fixtures(native, oracle, golden):
    """sdbfg_to_string / sdbfg_parse on oracle digests reproduce the reference text."""
    import sdhash_gb300 as g
    seen = 0
    for rec in golden["digests"]:
        if rec["status"] != 0:
            continue
        od = oracle.digest(rec["name"], cases.make(rec["spec"]).tobytes(), rec["dd"])
        st = od.st
        filt = np.frombuffer(od.filters(), dtype=np.uint8).copy()
        counts = np.array(od.elem_counts(), dtype=np.uint16) if rec["dd"] else None
        d = g.Digest(rec["name"], st.orig_size, st.bf_count, st.last_count, st.max_elem, st.dd_block_size, filt,
                     counts)
        t = d.to_string()
        assert hashlib.sha256(t.encode()).hexdigest() == rec["sha256"], rec["name"]
        back = g.Digest.from_string(t)
        assert back.to_string() == t
        assert back.name == rec["name"] and back.bf_count == st.bf_count
        seen += 1
    assert seen > 150


def test_parse_rejects_malformed(native):
    import pytest

    import sdhash_gb300 as g
    with pytest.raises(g.SdbfError) as e:
        g.Digest.from_string("sdbf:03:1:a:10")
    assert e.value.code == -1  # shorter than 344 chars (sdbf_class.cc:145)
    with pytest.raises(g.SdbfError) as e:
        g.Digest.from_string("xxxx:" + "A" * 400)
    assert e.value.code == -2  # bad magic (sdbf_class.cc:152-153)
    good = "sdbf:03:1:a:1000:sha1:256:5:7ff:160:1:10:" + "A" * 342 + "==\n"
    assert g.Digest.from_string(good).bf_count == 1
    with pytest.raises(g.SdbfError):
        g.Digest.from_string(good.replace("A" * 342, "A" * 300 + "!" * 42))


def test_cli_segments_follow_reference_rule():
    """sdbf_hash_files_dd's segment sizes (sdhash-src/sdhash_threads.cc:312-340)."""
    from sdhash_gb300.cli import _segments
    M = 1 << 20

    def ref(size, chunk):
        if not (size > chunk and chunk > 0):
            return [size]
        chunks, tail = size // chunk, False
        if size - chunk <= 512:
            chunks = 0
        if size - chunks * chunk <= 512:
            chunks -= 1
            tail = True
        out = []
        for j in range(chunks + 1):
            if j == chunks:
                c = size - chunks * chunk
                if tail:
                    c += size - (chunks + 1) * chunk
            else:
                c = chunk
            out.append(c)
        return out

    for size in (100, 128 * M, 128 * M + 100, 128 * M + 512, 128 * M + 513, 256 * M + 512, 256 * M + 513, 300 * M):
        got = _segments("f", size, 128 * M)
        assert [n for _, _, n in got] == ref(size, 128 * M), size
        assert [o for _, o, _ in got] == [j * 128 * M for j in range(len(got))]
    names = [nm for nm, _, _ in _segments("img", 300 * M, 128 * M)]
    assert names == ["img.0000M", "img.0128M", "img.0256M"]


def test_native_cli_builds_and_answers_without_a_gpu(native):
    """The native command line links against the library; --version and
    --help need no device, and a command that needs one fails cleanly."""
    import subprocess
    from sdhash_gb300 import build
    exe = build.build_cli()
    r = subprocess.run([exe, "--version"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "SDBF v3" in r.stdout
    r = subprocess.run([exe, "--help"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and "--index-search" in r.stdout and "--gen-compare" in r.stdout
    r = subprocess.run([exe, "-s", "4", "x"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 255 and "not offered" in r.stderr
