"""GPU digest comparison through the C ABI against the reference's recorded
results and the oracle.  Integer-identical scores."""
import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def plain_set(ctx, golden):
    import sdhash_gb300 as g
    names, files = synth.plain_small_set(seed=golden["plain_small"]["seed"])
    stream = ctx.digest_buffers([f.tobytes() for f in files], names, 0)
    dd = ctx.digest_buffers([f.tobytes() for f in files[:8]], [n + ".dd" for n in names[:8]], 16384)
    return g, names, files, stream, dd


def test_compare_all_plain_small_matches_reference(plain_set, golden):
    g, names, files, stream, dd = plain_set
    s = g.sdbf_set()
    for d in stream:
        s.add(g.sdbf(_digest=d))
    assert s.compare_all_quiet(1) == golden["plain_small"]["compare_all_t1"]


def test_compare_to_block_vs_stream_matches_reference(plain_set, golden):
    g, names, files, stream, dd = plain_set
    q, t = g.sdbf_set(), g.sdbf_set()
    for d in dd:
        q.add(g.sdbf(_digest=d))
    for d in stream:
        t.add(g.sdbf(_digest=d))
    assert q.compare_to_quiet(t, 1) == golden["plain_small"]["compare_to_dd_vs_stream_t1"]
    assert q.compare_all_quiet(-1) == golden["plain_small"]["compare_all_dd_tneg1"]


def test_scores_match_oracle_on_mixed_digests(ctx, oracle):
    """Uneven digests (1..40 filters, stream and block, sparse last filters,
    equal filter counts for the swap tie-break) vs the oracle, all pairs."""
    sizes = [600, 700, 5000, 9000, 20000, 20000, 60000, 120000, 300000, 1 << 20, 2 << 20]
    files = [synth.mixture_bytes(31, i, s) for i, s in enumerate(sizes)]
    files += [synth.random_bytes(32, i, s) for i, s in enumerate(sizes)]
    names = [f"z{i:02d}" if i % 3 else f"a{i:02d}" for i in range(len(files))]
    ds = ctx.digest_buffers([f.tobytes() for f in files], names, 0)
    ds += ctx.digest_buffers([f.tobytes() for f in files[:10]], [n + "b" for n in names[:10]], 4096)
    ods = [oracle.parse(d.to_string()) for d in ds]
    dev = ctx.upload(ds)
    got = ctx.compare_all(dev)
    n = len(ds)
    want = oracle.score_all_matrix(ods)
    k = 0
    for i in range(n):
        for j in range(i + 1, n):
            assert got[k] == want[i, j], (i, j, ds[i].name, ds[j].name)
            k += 1
    cross = ctx.compare_to(dev, dev)
    wantx = oracle.score_cross_matrix(ods, ods)
    assert np.array_equal(cross, wantx)


def test_score_pairs_and_single_compare(ctx, oracle, plain_set):
    g, names, files, stream, dd = plain_set
    a = ctx.upload(stream)
    b = ctx.upload(dd)
    rng = np.random.default_rng(7)
    ia = rng.integers(0, len(stream), 300)
    ib = rng.integers(0, len(dd), 300)
    got = ctx.score_pairs(a, b, ia, ib)
    os_ = [oracle.parse(d.to_string()) for d in stream]
    od = [oracle.parse(d.to_string()) for d in dd]
    for k in range(300):
        assert got[k] == oracle.score(os_[ia[k]], od[ib[k]])


def test_fast_mode_matches_reference(plain_set, golden):
    """--fast on the GPU (fold kernel, CUTOFFS64, 64-byte counts; the
    reference digest's fastmode decides each pair) against the reference."""
    g, names, files, stream, dd = plain_set
    import copy
    s, q = g.sdbf_set(), g.sdbf_set()
    for d in stream:
        s.add(g.sdbf(_digest=copy.deepcopy(d)))
    for d in dd:
        q.add(g.sdbf(_digest=copy.deepcopy(d)))
    gp = golden["plain_small"]
    assert s.compare_all_quiet(1, 0, True) == gp["compare_all_fast_t1"]
    assert s.compare_to_quiet(q, 1, 0, 0, True) == gp["compare_to_fast_stream_vs_dd_t1"]
    assert q.compare_all_quiet(-1, 0, True) == gp["compare_all_dd_fast_tneg1"]


def test_fast_mode_device_fold_both_paths(ctx, oracle, plain_set):
    """Device-side fold of a resident set; batched engine and per-pair path
    agree with the oracle, mixed folded / unfolded pairs included."""
    g, names, files, stream, dd = plain_set
    ds = stream[:20] + dd
    dev = ctx.upload(ds)
    dev.fast(0, 10)           # fold the first ten stream digests only
    dev.fast(20, 4)           # and half the block digests
    ods = [oracle.parse(d.to_string()) for d in ds]
    for k in list(range(10)) + list(range(20, 24)):
        oracle.fast(ods[k])
    want = oracle.score_all_matrix(ods)
    iu = np.triu_indices(len(ds), 1)
    assert np.array_equal(ctx.compare_all(dev), want[iu])
    assert np.array_equal(ctx.score_pairs(dev, dev, iu[0], iu[1]), want[iu])
