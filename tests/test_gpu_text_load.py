"""Bulk load of SDBF text on the device (sdbfg_set_load_text) against the
reference's loader: sdbf_set(const char*) over sdbf(const std::string&)
(sdbf/sdbf_set.cc:51-74, sdbf/sdbf_class.cc:144-215).

The golden cases (tests/golden/text_load.json, made by the reference) give,
per text, the loaded digests re-encoded by to_string or the value thrown and
the index of the line that throws.  At full size, a set written out and
loaded back compares exactly like the set it came from."""
import json
import os

import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu

CASES = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "text_load.json")))["cases"]


@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_load_matches_reference_loader(ctx, case):
    import sdhash_gb300 as g
    text = case["text"].encode("latin-1")
    want = case["expect"]
    if "lines" in want:
        ds = ctx.load_text(text)
        assert len(ds) == len(want["lines"])
        assert [ds.digest(i).to_string() for i in range(len(ds))] == want["lines"]
    else:
        with pytest.raises(g.SdbfError) as e:
            ctx.load_text(text)
        assert e.value.code == want["err"] and e.value.line == want["line"]


def test_loaded_set_scores_like_uploaded_set(ctx, oracle):
    """The mixed golden set: scores of the loaded set equal the oracle's on the
    same lines (hamming weights and element counts come from the loader)."""
    case = next(c for c in CASES if c["name"] == "mixed set")
    ds = ctx.load_text(case["text"])
    od = [oracle.parse(t) for t in case["expect"]["lines"]]
    n = len(od)
    got = ctx.compare_all(ds)
    want = oracle.score_all_matrix(od)
    assert np.array_equal(got, want[np.triu_indices(n, 1)])


def test_empty_and_blank_text(ctx):
    assert len(ctx.load_text(b"")) == 0
    assert len(ctx.load_text(b"\n" + CASES[0]["text"].encode())) == 0   # an empty first line ends the file


def test_round_trip_at_size(ctx):
    """Thousands of stream and block digests: text -> device set gives the
    same filters, element counts and scores as the digests uploaded directly."""
    sizes = [int(s) for s in synth.log_uniform_sizes(81, 600, 4 << 10, 2 << 20)]
    bufs = [synth.mixture_bytes(81, i, s).tobytes() for i, s in enumerate(sizes)]
    digs = ctx.digest_buffers(bufs[:400], [f"f{i:04d}" for i in range(400)], 0)
    digs += ctx.digest_buffers(bufs[400:], [f"b{i:04d}" for i in range(400, len(bufs))], 16384)
    digs = [d for d in digs if d is not None]
    text = "".join(d.to_string() for d in digs).encode()
    ds = ctx.load_text(text)
    assert len(ds) == len(digs)
    for i in list(range(0, len(digs), 37)) + [len(digs) - 1]:
        d, got = digs[i], ds.digest(i)
        assert got.name == d.name and got.bf_count == d.bf_count and got.orig_size == d.orig_size
        assert np.array_equal(got.filters, d.filters)
        assert [got.elem_count(k) for k in range(d.bf_count)] == [d.elem_count(k) for k in range(d.bf_count)]
    up = ctx.upload(digs)
    q = ctx.upload(digs[::50])
    assert np.array_equal(ctx.compare_to(q, ds), ctx.compare_to(q, up))
    sub = ctx.load_text("".join(d.to_string() for d in digs[:120]).encode())
    assert np.array_equal(ctx.compare_all(sub), ctx.compare_all(ctx.upload(digs[:120])))


def test_sdbf_set_file_uses_loader(tmp_path, ctx, oracle):
    """sdbf_set(fname): file parsed on the device; compare_all_quiet equals the
    oracle's text, also after fast() folds the items."""
    import sdhash_gb300 as g
    case = next(c for c in CASES if c["name"] == "mixed set")
    p = tmp_path / "set.sdbf"
    p.write_text(case["text"])
    s = g.sdbf_set(str(p))
    assert s.size() == len(case["expect"]["lines"])
    od = [oracle.parse(t) for t in case["expect"]["lines"]]
    assert s.compare_all_quiet(-1) == oracle.compare_all(od, -1)
    assert s.compare_all_quiet(-1, 0, True) == oracle.compare_all([oracle.fast(d) for d in od], -1)
    bad = tmp_path / "bad.sdbf"
    bad.write_text(next(c for c in CASES if c["name"] == "bad magic")["text"])
    with pytest.raises(g.SdbfError) as e:
        g.sdbf_set(str(bad))
    assert e.value.code == -2
