"""The native command line (sdhash_gb300/sdhash-gb300, sdhash_gb300/cli/
sdhash_main.cpp) against the oracle and the reference's fixtures: digests
(stream, block mode with segments and the zero-filled last segment, the
16 MiB automatic block mode), -g, -c with one and two SDBF files, --fast,
-o, --validate, --index-search and --index."""
import gzip
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def exe(native):
    from sdhash_gb300 import build
    return build.build_cli()


def run(exe, *args, cwd=None):
    r = subprocess.run([exe, *args], capture_output=True, cwd=cwd, timeout=600)
    return r.returncode, r.stdout.decode(), r.stderr.decode()


def _odig(oracle, name, data, dd, orig=None):
    d = oracle.digest(name, data.tobytes(), dd)
    if orig is not None:
        d.st.orig_size = orig
    return d


def test_native_hash_and_compare(exe, tmp_path, oracle):
    files = {"a.bin": synth.mixture_bytes(62, 0, 300_000), "b.bin": synth.mixture_bytes(62, 1, 1_500_000)}
    files["c.bin"] = synth.partner(62, 2, files["b.bin"])
    files["big.bin"] = synth.mixture_bytes(62, 3, 17 << 20)
    files["seg.bin"] = synth.mixture_bytes(62, 4, (2 << 20) + 512)
    for n, d in files.items():
        (tmp_path / n).write_bytes(d.tobytes())
    small = ["a.bin", "b.bin", "c.bin"]
    rc, out, _ = run(exe, *small, "big.bin", cwd=tmp_path)
    want = [_odig(oracle, n, files[n], 0) for n in small] + [_odig(oracle, "big.bin", files["big.bin"], 16384)]
    assert rc == 0 and out == "".join(d.to_string() for d in want)
    rc, out, _ = run(exe, "-g", "-t", "1", *small, cwd=tmp_path)
    assert rc == 0 and out == oracle.compare_all([_odig(oracle, n, files[n], 0) for n in small], 1)
    rc, out, _ = run(exe, "-g", "--fast", "-t", "-1", *small, cwd=tmp_path)
    assert rc == 0 and out == oracle.compare_all([oracle.fast(_odig(oracle, n, files[n], 0)) for n in small], -1)
    # -b 16 -z 1: 1 MiB segments, the last one zero-filled to its length
    rc, out, _ = run(exe, "-b", "16", "-z", "1", "seg.bin", cwd=tmp_path)
    data = files["seg.bin"]
    last = np.zeros((1 << 20) + 1024, dtype=np.uint8)
    last[:(1 << 20) + 512] = data[1 << 20:]
    want = [_odig(oracle, "seg.bin.0000M", data[:1 << 20], 16384),
            _odig(oracle, "seg.bin.0001M", last, 16384, orig=(1 << 20) + 512)]
    assert rc == 0 and out == "".join(d.to_string() for d in want)
    # -c with one file and with two (csv), --fast on the query set
    (tmp_path / "set.sdbf").write_text("".join(_odig(oracle, n, files[n], 0).to_string() for n in small))
    (tmp_path / "q.sdbf").write_text(_odig(oracle, "c.bin", files["c.bin"], 0).to_string())
    ods = [oracle.parse(t) for t in (tmp_path / "set.sdbf").read_text().splitlines(True)]
    oq = [oracle.parse((tmp_path / "q.sdbf").read_text())]
    rc, out, _ = run(exe, "-c", "set.sdbf", "-t", "-1", cwd=tmp_path)
    assert rc == 0 and out == oracle.compare_all(ods, -1)
    rc, out, _ = run(exe, "-c", "--separator", "csv", "q.sdbf", "set.sdbf", cwd=tmp_path)
    assert rc == 0 and out == oracle.compare_to(oq, ods, 1, ",")
    rc, out, _ = run(exe, "-c", "--fast", "set.sdbf", "q.sdbf", "-t", "-1", cwd=tmp_path)
    assert rc == 0 and out == oracle.compare_to([oracle.fast(d) for d in ods], oq, -1)
    # -o and --validate
    rc, _, _ = run(exe, "-o", "out", "a.bin", cwd=tmp_path)
    assert rc == 0 and (tmp_path / "out.sdbf").read_text() == _odig(oracle, "a.bin", files["a.bin"], 0).to_string()
    rc, out, _ = run(exe, "--validate", "set.sdbf", cwd=tmp_path)
    nf = sum(d.bf_count for d in ods)
    assert rc == 0 and out == (f"sdhash: file set.sdbf SDBFs valid, contains 3 hashes.\n"
                               f"contains {nf} bloom filters.\n"
                               f"{sum(len(files[n]) for n in small)} total data size. \n")
    (tmp_path / "bad.sdbf").write_text("sdbf:03:" + "x" * 400 + "\n")
    rc, _, err = run(exe, "-c", "bad.sdbf", cwd=tmp_path)
    assert rc == 255 and "Could not load SDBF file bad.sdbf" in err


def test_native_index_search(exe, tmp_path):
    rec = json.load(open(os.path.join(GOLD, "index", "index_search.json")))
    os.mkdir(tmp_path / "idx")
    for s in ("A", "B"):
        with gzip.open(os.path.join(GOLD, "index", f"{s}.sdbf.idx.gz")) as f:
            (tmp_path / "idx" / f"{s}.sdbf.idx").write_bytes(f.read())
        shutil.copy(os.path.join(GOLD, "index", f"{s}.sdbf"), tmp_path / "idx" / f"{s}.sdbf")
    import importlib.util
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(GOLD, "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    names = []
    for n, d in m.queries():
        (tmp_path / n).write_bytes(d)
        names.append(n)
    rc, out, err = run(exe, "--index-search", "idx", *names, cwd=tmp_path)
    # lines within a block follow the directory order of the index files
    assert rc == 0 and out == "" and sorted(err.splitlines()) == sorted(rec["results"].splitlines())
    rc, _, _ = run(exe, "--index-search", "idx", "-o", "res", *names, cwd=tmp_path)
    assert rc == 0
    assert sorted((tmp_path / "res.idx-result").read_text().splitlines()) == sorted(rec["results"].splitlines())


def test_native_index_build(exe, tmp_path):
    """--index -o out: the group's set file and index as the reference
    builds them (the index file's compressed bytes are this library's)."""
    import ctypes as C
    import hashlib
    import importlib.util
    from sdhash_gb300 import lib
    rec = json.load(open(os.path.join(GOLD, "index", "index_search.json")))["builds"][0]
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(GOLD, "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    items = m.build_inputs()[0]
    for n, d in items:
        (tmp_path / n).write_bytes(d)
    rc, _, err = run(exe, "--index", *[n for n, _ in items], cwd=tmp_path)
    assert rc == 255 and "requires output base filename" in err
    rc, _, _ = run(exe, "--index", "-o", "out", *[n for n, _ in items], cwd=tmp_path)
    assert rc == 0 and (tmp_path / "out0.sdbf").read_text() == rec["sdbf_text"]
    raw = (tmp_path / "out0.sdbf.idx").read_bytes()
    nl = raw.index(b"\n")
    head = raw[:nl].decode().split(":")
    assert head[:5] == rec["header"].split(":")[:5] and head[6] == "out0.sdbf"
    out = np.zeros(64 << 20, dtype=np.uint8)
    L = lib()
    assert L.sdbfg_lz4_decode(raw[nl + 1:], len(raw) - nl - 1, out.ctypes.data, out.size) == int(head[5])
    assert hashlib.sha256(out.tobytes()).hexdigest() == rec["filter_sha256"]
