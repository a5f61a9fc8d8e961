"""Index files on the host: the LZ4 block decoder and the index header
against index files the reference wrote (tests/golden/index/, made by
tests/golden/make_index_golden.py).  No GPU needed."""
import ctypes as C
import gzip
import hashlib
import json
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "index")


def _fixture():
    with open(os.path.join(GOLD, "index_search.json")) as f:
        return json.load(f)


def _decode(native, payload: bytes, out_len: int):
    out = np.zeros(out_len, dtype=np.uint8)
    native.sdbfg_lz4_decode.argtypes = [C.c_char_p, C.c_uint64, C.c_void_p, C.c_uint64]
    native.sdbfg_lz4_decode.restype = C.c_int64
    r = native.sdbfg_lz4_decode(payload, len(payload), out.ctypes.data, out_len)
    return r, out


@pytest.mark.parametrize("stem", ["A", "B"])
def test_lz4_decode_matches_reference_filter(native, stem):
    rec = _fixture()["indexes"][stem]
    raw = gzip.open(os.path.join(GOLD, f"{stem}.sdbf.idx.gz")).read()
    nl = raw.index(b"\n")
    head = raw[:nl].decode()
    assert head == rec["header"]
    f = head.split(":")
    assert f[0] == "sdbf-idx" and int(f[3]) == 5
    size, comp = int(f[1]), int(f[5])
    payload = raw[nl + 1:nl + 1 + comp]
    r, out = _decode(native, payload, size)
    assert r == comp
    assert hashlib.sha256(out.tobytes()).hexdigest() == rec["filter_sha256"]
    assert int(np.unpackbits(out).sum()) == rec["filter_popcount"]


def test_lz4_decode_rejects_malformed(native):
    # literal-only block: token 0x50 + 5 literals
    r, out = _decode(native, b"\x50hello", 5)
    assert r == 6 and out.tobytes() == b"hello"
    # overlapping match: "ab" then offset 2, length 4+4 -> "ababababab"
    r, out = _decode(native, b"\x24ab\x02\x00", 10)
    assert r < 0                       # output not filled by a final literal run
    r, out = _decode(native, b"\x24ab\x02\x00\x10z", 11)
    assert r == 7 and out.tobytes() == b"ababababab" + b"z"
    assert _decode(native, b"\x24ab\x00\x00\x10z", 11)[0] < 0   # offset 0
    assert _decode(native, b"\x24ab\x05\x00\x10z", 11)[0] < 0   # offset before the output start
    assert _decode(native, b"\x50hel", 5)[0] < 0                # truncated literals
    assert _decode(native, b"\x50hello", 4)[0] < 0              # output too small


def test_oracle_index_search_matches_reference(native, oracle):
    """The oracle's restatement of the index search reproduces the
    reference's result text on the fixture's indexes and queries."""
    import importlib.util
    rec = _fixture()
    bits = []
    for s in rec["index_order"]:
        raw = gzip.open(os.path.join(GOLD, f"{s}.sdbf.idx.gz")).read()
        nl = raw.index(b"\n")
        f = raw[:nl].decode().split(":")
        r, out = _decode(native, raw[nl + 1:nl + 1 + int(f[5])], int(f[1]))
        assert r == int(f[5])
        bits.append(out)
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(os.path.dirname(GOLD),
                                                                        "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    qs = m.queries()
    hits = oracle.index_search([d for _, d in qs], rec["dd_block_size"], bits)
    lines = []
    for (n, _), h in zip(qs, hits):
        if h is None:
            continue
        for b in range(h.shape[0]):
            for i, s in enumerate(rec["index_order"]):
                if h[b, i] > 4:
                    lines.append(f"{n} [{b}] |idx/{s}.sdbf|{int(h[b, i])}\n")
    assert "".join(lines) == rec["results"]


def test_lz4_encoder_round_trip(native):
    """The index writer's LZ4 encoder against the decoder, on the reference's
    index filters and on edge inputs (empty, short, runs, random)."""
    native.sdbfg_lz4_encode.argtypes = [C.c_char_p, C.c_uint64, C.c_void_p, C.c_uint64]
    native.sdbfg_lz4_encode.restype = C.c_int64
    rng = np.random.default_rng(3)
    samples = [b"", b"a", b"abcdefghijkl", b"x" * 13, bytes(100000), rng.bytes(70000),
               bytes(rng.integers(0, 3, 50000, dtype=np.uint8))]
    raw = gzip.open(os.path.join(GOLD, "A.sdbf.idx.gz")).read()
    nl = raw.index(b"\n")
    r, bits = _decode(native, raw[nl + 1:], 64 << 20)
    samples.append(bits.tobytes())
    for smp in samples:
        n = native.sdbfg_lz4_encode(smp, len(smp), None, 0)
        enc = np.zeros(max(1, n), dtype=np.uint8)
        assert native.sdbfg_lz4_encode(smp, len(smp), enc.ctypes.data, n) == n
        r, out = _decode(native, enc[:n].tobytes(), len(smp))
        assert r == n and out.tobytes() == smp
    assert n < len(samples[-1]) // 100   # a sparse 64 MiB filter compresses well


def test_reference_reads_written_index(native, tmp_path):
    """An index file written here is read by the reference's own
    bloom_filter(string) to the same filter (needs the reference library
    built from its sources; skipped where it is absent)."""
    import hashlib
    from oracle import REF_SO
    if not os.path.exists(REF_SO):
        pytest.skip("reference library not built here")
    L = C.CDLL(REF_SO)
    L.ref_index_bits.argtypes = [C.c_char_p, C.c_void_p, C.c_ulonglong]
    L.ref_index_bits.restype = C.c_longlong
    rec = _fixture()["indexes"]["B"]
    raw = gzip.open(os.path.join(GOLD, "B.sdbf.idx.gz")).read()
    nl = raw.index(b"\n")
    r, bits = _decode(native, raw[nl + 1:], 64 << 20)
    head = raw[:nl].decode().split(":")
    native.sdbfg_index_write_file.argtypes = [C.c_char_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint32, C.c_char_p]
    path = str(tmp_path / "mine.idx")
    assert native.sdbfg_index_write_file(path.encode(), bits.ctypes.data, bits.size, int(head[2]), 5,
                                         head[6].encode()) == 0
    back = np.zeros(64 << 20, dtype=np.uint8)
    assert L.ref_index_bits(path.encode(), back.ctypes.data, back.size) == 64 << 20
    assert hashlib.sha256(back.tobytes()).hexdigest() == rec["filter_sha256"]


def test_index_groups():
    """--index groups (hash_index_stringlist, sdhash-src/sdhash_threads.cc:
    402-411,446-455): a group closes past 640 MB or at the last file, slot 0
    stays in every later group, and the running size wraps as a C int."""
    from sdhash_gb300.cli import MB, _index_groups
    assert _index_groups([]) == []
    assert _index_groups([10 * MB] * 3) == [[0, 1, 2]]
    assert _index_groups([600 * MB, 50 * MB, 10 * MB, 700 * MB, 1]) == [[0, 1], [0, 2, 3], [0, 4]]
    assert _index_groups([641 * MB, 641 * MB, 641 * MB]) == [[0], [0, 1], [0, 2]]
    # 3 GiB is negative as an int; 3 GiB + 100 MiB + 1 GiB wraps to 100 MiB
    assert _index_groups([3 << 30, 100 * MB, 1 << 30, 5]) == [[0, 1, 2, 3]]
    assert _index_groups([3 << 30, 2 << 30]) == [[0, 1]]


@pytest.mark.parametrize("case", [0, 2], ids=["stream group", "shared-pool stream group"])
def test_oracle_index_build_stream_matches_reference(oracle, case):
    """The oracle's stream-mode index build (files in order, one shared
    index) gives the reference's set text, index filter and element count
    for the fixture groups."""
    import hashlib
    import importlib.util
    import json
    rec = json.load(open(os.path.join(GOLD, "index_search.json")))["builds"][case]
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(os.path.dirname(GOLD), "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    items = m.build_inputs()[case]
    bits = np.zeros(64 << 20, dtype=np.uint8)
    digs, ec = oracle.index_build_stream([d for _, d in items], [n for n, _ in items], bits)
    assert "".join(d.to_string() for d in digs if d is not None) == rec["sdbf_text"]
    assert ec == int(rec["header"].split(":")[2])
    assert hashlib.sha256(bits.tobytes()).hexdigest() == rec["filter_sha256"]
