"""The oracle (plain-C restatement) against FIPS vectors and the reference's
own outputs recorded in tests/golden/golden.json.  CPU only."""
import hashlib
import os
import re

import numpy as np
import pytest

import cases
from sdhash_gb300 import synth

FIPS_SHA1 = [
    (b"abc", "a9993e364706816aba3e25717850c26c9cd0d89d"),
    (b"", "da39a3ee5e6b4b0d3255bfef95601890afd80709"),
    (b"abcdbcdecdefdefgefghfghighijhijkijkljklmklmnlmnomnopnopq", "84983e441c3bd26ebaae4aa1f95129e5e54670f1"),
    (b"abcdefghbcdefghicdefghijdefghijkefghijklfghijklmghijklmnhijklmnoijklmnopjklmnopqklmnopqrlmnopqrsmnopqrstnopqrstu",
     "a49b2446a02c645bf419f995b67091253a04a259"),
]


@pytest.mark.parametrize("msg,digest", FIPS_SHA1)
def test_sha1_fips_vectors(oracle, msg, digest):
    assert oracle.sha1(msg).hex() == digest


def test_sha1_matches_hashlib_on_features(oracle):
    rng = np.random.default_rng(5)
    for n in [64] * 200 + [0, 1, 55, 56, 63, 65, 119, 120, 1000]:
        m = rng.integers(0, 256, n, dtype=np.uint8).tobytes()
        assert oracle.sha1(m) == hashlib.sha1(m).digest()


def test_entropy_table_matches_header(oracle):
    src = open(os.path.join(os.path.dirname(__file__), "..", "sdhash_gb300", "csrc", "sdbf_tables.h")).read()
    body = re.search(r"SDBF_ENTROPY64\[65\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    header = [int(v) for v in re.findall(r"\d+", body)]
    assert header == oracle.entropy_table()


def test_rank_table_shape():
    src = open(os.path.join(os.path.dirname(__file__), "..", "sdhash_gb300", "csrc", "sdbf_tables.h")).read()
    body = re.search(r"SDBF_ENTR64_RANKS\[SDBF_RANK_BINS\]\s*=\s*\{(.*?)\};", src, re.S).group(1)
    ranks = [int(v) for v in re.findall(r"\d+", body)]
    assert len(ranks) == 1001
    assert ranks[:100] == [0] * 100 and ranks[-9:] == [0] * 9
    assert max(ranks) < 1024  # packed in 10 bits on the device


def _digest_text(oracle, name, data, dd):
    d = oracle.digest(name, data.tobytes(), dd)
    return None if d is None else d.to_string()


def test_oracle_small_cases_match_reference(oracle, golden):
    import hashlib as h
    bad = []
    data_cache = {}
    for rec in golden["digests"]:
        key = rec["name"]
        if key not in data_cache:
            data_cache[key] = cases.make(rec["spec"])
        t = _digest_text(oracle, rec["name"], data_cache[key], rec["dd"])
        if rec["status"] != 0:
            if t is not None:
                bad.append((rec["name"], rec["dd"], "expected too-small"))
            continue
        if t is None or h.sha256(t.encode()).hexdigest() != rec["sha256"]:
            bad.append((rec["name"], rec["dd"]))
        elif "text" in rec:
            assert t == rec["text"]
    assert not bad, bad


@pytest.mark.slow
def test_oracle_large_cases_match_reference(oracle, golden):
    import hashlib as h
    for rec in golden["large"]:
        if rec["spec"]["n"] > 33 << 20 and rec["dd"]:
            continue  # keep the CPU suite short; the GPU suite covers all
        t = _digest_text(oracle, rec["name"], cases.make(rec["spec"]), rec["dd"])
        assert h.sha256(t.encode()).hexdigest() == rec["sha256"], (rec["name"], rec["dd"])


def test_oracle_plain_small_compare_all(oracle, golden):
    g = golden["plain_small"]
    names, files = synth.plain_small_set(seed=g["seed"])
    ds = oracle.digest_many([f for f in files], 0, names=names)
    texts = [d.to_string() for d in ds]
    assert [hashlib.sha256(t.encode()).hexdigest() for t in texts] == g["sha256"]
    parsed = [oracle.parse(t) for t in texts]
    assert oracle.compare_all(parsed, 1) == g["compare_all_t1"]


def test_oracle_compare_to_block_vs_stream(oracle, golden):
    g = golden["plain_small"]
    names, files = synth.plain_small_set(seed=g["seed"])
    stream = [oracle.parse(oracle.digest(n, f.tobytes(), 0).to_string()) for n, f in zip(names, files)]
    dd = [oracle.parse(oracle.digest(n + ".dd", f.tobytes(), 16384).to_string()) for n, f in zip(names[:8], files[:8])]
    assert oracle.compare_to(dd, stream, 1) == g["compare_to_dd_vs_stream_t1"]
    assert oracle.compare_all(dd, -1) == g["compare_all_dd_tneg1"]


def test_staged_popcount_cut_semantics(oracle):
    # 8 bits in the first 32 bytes, 100 further bits later: 8*8+48=112 < cut
    # 200 -> the early stage returns 0 although the full count is 108 > cut
    a = bytearray(256)
    b = bytearray(256)
    a[0] = b[0] = 0xFF
    for i in range(40, 40 + 13):
        a[i] = b[i] = 0xFF
    assert oracle.L.orc_match_cut(bytes(a), bytes(b), 200) == 0
    assert oracle.L.orc_match_cut(bytes(a), bytes(b), 100) == 8 + 13 * 8


def test_oracle_fast_mode_matches_reference(oracle, golden):
    """--fast (sdbf::fast folding, CUTOFFS64, 64-byte count) against the
    reference's own --fast results, including its compare_to rule that folds
    only the query set."""
    g = golden["plain_small"]
    names, files = synth.plain_small_set(seed=g["seed"])
    stream = [oracle.parse(oracle.digest(n, f.tobytes(), 0).to_string()) for n, f in zip(names, files)]
    dd = [oracle.parse(oracle.digest(n + ".dd", f.tobytes(), 16384).to_string()) for n, f in zip(names[:8], files[:8])]
    for d in stream:
        oracle.fast(d)
    assert oracle.compare_all(stream, 1) == g["compare_all_fast_t1"]
    assert oracle.compare_to(stream, dd, 1) == g["compare_to_fast_stream_vs_dd_t1"]
    for d in dd:
        oracle.fast(oracle.fast(d))  # folding twice changes nothing
    assert oracle.compare_all(dd, -1) == g["compare_all_dd_fast_tneg1"]


def test_text_load_fixture_lines_are_canonical(oracle):
    """The reference loader's outputs recorded in tests/golden/text_load.json
    (digests re-encoded by to_string) parse and re-encode unchanged in the
    oracle, and the error cases carry the reference's throw values."""
    import json
    with open(os.path.join(os.path.dirname(__file__), "golden", "text_load.json")) as f:
        cases = json.load(f)["cases"]
    ok = [c for c in cases if "lines" in c["expect"]]
    bad = [c for c in cases if "err" in c["expect"]]
    assert len(ok) >= 5 and len(bad) >= 5
    for c in ok:
        for line in c["expect"]["lines"]:
            assert oracle.parse(line).to_string() == line, c["name"]
    assert {c["expect"]["err"] for c in bad} == {-1, -2}
    assert all(c["expect"]["line"] >= 0 for c in bad)
