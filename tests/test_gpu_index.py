"""Index search on the GPU (sdbfg_digest_batch_search, --index-search)
against the reference: its index files and index_results() text for seeded
queries (tests/golden/index/, made by tests/golden/make_index_golden.py)."""
import gzip
import json
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden", "index")


def _fixture():
    with open(os.path.join(GOLD, "index_search.json")) as f:
        return json.load(f)


def _queries():
    # the same seeded inputs as the fixture generator
    import importlib.util
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(os.path.dirname(__file__), "golden",
                                                                        "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.queries()


@pytest.fixture()
def idx_dir(tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    os.mkdir("idx")
    for s in ("A", "B"):
        with gzip.open(os.path.join(GOLD, f"{s}.sdbf.idx.gz")) as f, open(f"idx/{s}.sdbf.idx", "wb") as o:
            o.write(f.read())
        shutil.copy(os.path.join(GOLD, f"{s}.sdbf"), f"idx/{s}.sdbf")
    return tmp_path


def test_search_matches_reference(ctx, idx_dir):
    from sdhash_gb300 import cli
    rec = _fixture()
    indexes = [ctx.load_index(f"idx/{s}.sdbf.idx") for s in rec["index_order"]]
    for s, x in zip(rec["index_order"], indexes):
        assert x.name == f"idx/{s}.sdbf" and x.hash_count == 5 and x.bf_size == 64 << 20
    qs = _queries()
    digs, hits = ctx.digest_search([d for _, d in qs], [n for n, _ in qs], rec["dd_block_size"], indexes)
    import sdhash_gb300 as g
    items = [g.sdbf(_digest=d) for d in digs if d is not None]
    rows = [h for h in hits if h is not None]
    text = cli._index_results(items, rows, [f"idx/{s}.sdbf" for s in rec["index_order"]])
    assert text == rec["results"]
    # the digests themselves are the plain block-mode digests
    plain = ctx.digest_buffers([d for _, d in qs], [n for n, _ in qs], rec["dd_block_size"])
    for a, b in zip(digs, plain):
        assert (a is None) == (b is None)
        if a is not None:
            assert a.to_string() == b.to_string()


def test_cli_index_search(ctx, idx_dir, capsys):
    from sdhash_gb300 import cli
    rec = _fixture()
    for n, d in _queries():
        with open(n, "wb") as f:
            f.write(d)
    names = [n for n, _ in _queries()]
    assert cli.main(["--index-search", "idx", "-o", "res"] + names) == 0
    got = open("res.idx-result").read()
    # lines within a block follow the directory's order of the index files
    assert sorted(got.splitlines()) == sorted(rec["results"].splitlines())
    assert cli.main(["--index-search", "idx"] + names) == 0
    assert sorted(capsys.readouterr().err.splitlines()) == sorted(rec["results"].splitlines())
    assert cli.main(["--index-search", "idx", "-b", "0"] + names) == 0
    assert "only supported in block mode" in capsys.readouterr().err


def test_empty_index_has_no_hits(ctx):
    qs = _queries()
    x = ctx.index_from_bits(np.zeros(1 << 20, dtype=np.uint8))
    full = ctx.index_from_bits(np.full(1 << 10, 0xFF, dtype=np.uint8))
    digs, hits = ctx.digest_search([d for _, d in qs], [n for n, _ in qs], 16384, [x, full])
    for d, h in zip(digs, hits):
        if d is None:
            continue
        assert h.shape == (d.bf_count, 2)
        assert (h[:, 0] == 0).all()
        # every bit set: every sampled feature hits (counted features 0, 4, 8, ...)
        want = (d.elem_counts.astype(np.int64) + 3) // 4
        assert np.array_equal(h[:, 1], want)


def test_hits_match_oracle_dense_indexes(ctx, oracle):
    """Every hit count, for indexes dense enough that most blocks hit, on
    ragged inputs (tails, sub-block inputs, a too-small input)."""
    from sdhash_gb300 import synth
    rng = np.random.default_rng(5)
    bits = [np.packbits(rng.random(8 << 20) < d).astype(np.uint8) for d in (0.5, 0.8, 0.97)]
    sizes = [int(s) for s in synth.log_uniform_sizes(95, 40, 400, 3 << 20)]
    bufs = [synth.mixture_bytes(95, i, s).tobytes() for i, s in enumerate(sizes)]
    idx = [ctx.index_from_bits(b) for b in bits]
    digs, hits = ctx.digest_search(bufs, [f"x{i}" for i in range(len(bufs))], 16384, idx)
    want = oracle.index_search(bufs, 16384, bits)
    for d, h, w in zip(digs, hits, want):
        assert (d is None) == (w is None)
        if d is not None:
            assert np.array_equal(h, w)
    assert sum(int((h > 4).sum()) for h in hits if h is not None) > 100


@pytest.mark.parametrize("case,rounds", [(0, 16), (0, 0), (1, 16), (2, 16), (2, 1), (2, 0)],
                         ids=["stream group", "stream group, sequential commit", "block group",
                              "shared-pool stream group", "shared-pool stream group, one round",
                              "shared-pool stream group, sequential commit"])
def test_index_build_matches_reference(ctx, tmp_path, case, rounds):
    """sdhash --index for one group: the digests (stream mode: features the
    index already holds are dropped), the index bits and its element count
    are the reference's -- from the fixed-point rounds, and from the
    sequential commit when rounds are off or run out; the index file written
    here decodes to the same filter and carries the reference's header fields."""
    import hashlib
    import importlib.util
    rec = _fixture()["builds"][case]
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(os.path.dirname(GOLD), "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    items = m.build_inputs()[case]
    bits = np.zeros(64 << 20, dtype=np.uint8)
    ctx.set_index_rounds(rounds)
    try:
        digs, ec = ctx.digest_index([d for _, d in items], [n for n, _ in items], rec["dd"], bits)
        used = ctx.index_rounds
    finally:
        ctx.set_index_rounds(16)
    if rec["dd"] == 0:
        # commit rounds taken, or 0 when they ran out (or were off) and the
        # sequential commit ran
        assert used <= rounds and (rounds == 0 or rounds == 1 or used >= 1)
    assert "".join(d.to_string() for d in digs) == rec["sdbf_text"]
    assert hashlib.sha256(bits.tobytes()).hexdigest() == rec["filter_sha256"]
    head = rec["header"].split(":")
    assert ec == int(head[2])
    path = str(tmp_path / "x.sdbf.idx")
    ctx.write_index(path, bits, ec, head[6])
    raw = open(path, "rb").read()
    nl = raw.index(b"\n")
    mine = raw[:nl].decode().split(":")
    assert mine[:5] == head[:5] and mine[6] == head[6]
    x = ctx.load_index(path)
    assert (x.bf_size, x.elem_count, x.hash_count, x.bit_mask) == (64 << 20, ec, 5, int(head[4]))
    from sdhash_gb300 import lib
    out = np.zeros(64 << 20, dtype=np.uint8)
    assert lib().sdbfg_lz4_decode(raw[nl + 1:], len(raw) - nl - 1, out.ctypes.data, out.size) == int(mine[5])
    assert np.array_equal(out, bits)


def test_index_build_rounds_match_sequential_large(ctx):
    """A 300 MiB stream-mode group (two launch groups: the first holds at
    most 256 MiB) of files cut from a shared pool: the fixed-point rounds
    give the digests, bits and element count of the sequential commit."""
    from sdhash_gb300 import synth
    pool = synth.mixture_bytes(97, 0, 48 << 20)
    rng = np.random.default_rng(97)
    bufs = []
    for i in range(150):
        n = int(rng.integers(1 << 20, 3 << 20))
        o = int(rng.integers(0, pool.size - n))
        b = pool[o:o + n].copy()
        b[:4096] = synth.random_bytes(97, i + 1, 4096)
        bufs.append(b)
    names = [f"p{i}" for i in range(len(bufs))]
    assert sum(b.size for b in bufs) > 256 << 20
    out = []
    for rounds in (16, 0):
        bits = np.zeros(64 << 20, dtype=np.uint8)
        ctx.set_index_rounds(rounds)
        ctx.profile(True)
        try:
            digs, ec = ctx.digest_index(bufs, names, 0, bits)
            used = ctx.index_rounds
            restarts = ctx.kernel_time("k_stream_commit_round.restarts")[0]
        finally:
            ctx.profile(False)
            ctx.set_index_rounds(16)
        out.append(("".join(d.to_string() for d in digs), bits, ec, used, restarts))
    (t1, b1, e1, u1, r1), (t0, b0, e0, u0, _) = out
    # the rounds ran past the first, and some file restarted from a
    # commit-state checkpoint (a changed predicate 32 or more tiles into it)
    assert u0 == 0 and u1 >= 2 and r1 >= 1, (u1, r1)
    assert t1 == t0 and e1 == e0 and np.array_equal(b1, b0)


def test_cli_index_matches_reference_group(ctx, tmp_path, monkeypatch):
    """sdhash --index -o out <files>: the group's set file and index (bits,
    element count, set name) as the reference builds them."""
    import hashlib
    import importlib.util
    from sdhash_gb300 import cli, lib
    rec = _fixture()["builds"][0]
    spec = importlib.util.spec_from_file_location("mkidx", os.path.join(os.path.dirname(GOLD), "make_index_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    monkeypatch.chdir(tmp_path)
    items = m.build_inputs()[0]
    for n, d in items:
        (tmp_path / n).write_bytes(d)
    assert cli.main(["--index"] + [n for n, _ in items]) == -1      # needs -o
    assert cli.main(["--index", "-o", "out"] + [n for n, _ in items]) == 0
    assert (tmp_path / "out0.sdbf").read_text() == rec["sdbf_text"]
    raw = (tmp_path / "out0.sdbf.idx").read_bytes()
    nl = raw.index(b"\n")
    head = raw[:nl].decode().split(":")
    want = rec["header"].split(":")
    assert head[:5] == want[:5] and head[6] == "out0.sdbf"
    out = np.zeros(64 << 20, dtype=np.uint8)
    assert lib().sdbfg_lz4_decode(raw[nl + 1:], len(raw) - nl - 1, out.ctypes.data, out.size) == int(head[5])
    assert hashlib.sha256(out.tobytes()).hexdigest() == rec["filter_sha256"]


@pytest.mark.parametrize("dd", [0, 16384], ids=["stream", "block"])
def test_index_build_in_two_calls(ctx, oracle, dd):
    """An index built over a group in two calls (the second starting from
    the first call's bits and element count) gives the digests, bits and
    count of one call over the whole group: the second call's features see
    the first call's bits as set before them.  Files below 512 bytes are
    too small and leave the index alone."""
    from sdhash_gb300 import synth
    pool = synth.mixture_bytes(98, 0, 3 << 20)
    rng = np.random.default_rng(98)
    bufs = []
    for i in range(24):
        n = int(rng.integers(20_000, 400_000))
        o = int(rng.integers(0, pool.size - n))
        b = pool[o:o + n].copy()
        b[:2048] = synth.random_bytes(98, i + 1, 2048)
        bufs.append(b)
    bufs[5] = synth.random_bytes(98, 100, 300)    # too small
    bufs[17] = synth.random_bytes(98, 101, 511)   # too small
    names = [f"t{i}" for i in range(len(bufs))]
    whole = np.zeros(64 << 20, dtype=np.uint8)
    d_all, ec_all = ctx.digest_index(bufs, names, dd, whole)
    assert d_all[5] is None and d_all[17] is None
    split = np.zeros(64 << 20, dtype=np.uint8)
    d1, ec1 = ctx.digest_index(bufs[:10], names[:10], dd, split)
    d2, ec2 = ctx.digest_index(bufs[10:], names[10:], dd, split, ec1)
    assert ec2 == ec_all and np.array_equal(split, whole)
    for a, b in zip(d_all, d1 + d2):
        assert (a is None) == (b is None)
        if a is not None:
            assert a.to_string() == b.to_string()
    if dd == 0:
        # the oracle's sequential build agrees
        obits = np.zeros(64 << 20, dtype=np.uint8)
        want, oec = oracle.index_build_stream(bufs, names, obits)
        assert oec == ec_all and np.array_equal(obits, whole)
        for a, w in zip(d_all, want):
            assert (a is None) == (w is None)
            if a is not None:
                assert a.to_string() == w.to_string()
