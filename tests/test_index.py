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
