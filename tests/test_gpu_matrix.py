"""Batched comparison engine (persistent work units, kernel variants, unit
budgets, split pairs, CUDA-graph replay, autotuner) against the oracle.
Integer-identical scores for every variant and schedule."""
import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def uneven(ctx, oracle):
    """Digests with very uneven filter counts (1..~260), stream and block
    mode, related pairs (partners) so that scores are non-trivial, sparse
    last filters, equal filter counts and equal names for the swap rule's
    tie-breaks."""
    sizes = [int(s) for s in synth.log_uniform_sizes(41, 36, 600, 3 << 20)]
    files = [synth.mixture_bytes(41, i, s) for i, s in enumerate(sizes)]
    files += [synth.partner(41, i, files[i]) for i in range(0, 12)]
    files += [files[3].copy(), files[3].copy()]          # identical digests
    names = [f"u{i:03d}" for i in range(len(files))]
    names[-1] = names[-2]                               # identical names
    ds = ctx.digest_buffers([f.tobytes() for f in files], names, 0)
    ds += ctx.digest_buffers([f.tobytes() for f in files[:10]], [n + ".dd" for n in names[:10]], 4096)
    ds = [d for d in ds if d is not None]
    ods = [oracle.parse(d.to_string()) for d in ds]
    want_all = oracle.score_all_matrix(ods)
    iu = np.triu_indices(len(ds), 1)
    return ds, ods, want_all[iu]


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("unit_work", [1 << 12, 1 << 22])
def test_all_pairs_every_variant_and_budget(ctx, uneven, variant, unit_work):
    ds, ods, want = uneven
    ctx.set_compare_tuning(variant, unit_work, graphs=(variant % 2 == 0))
    try:
        dev = ctx.upload(ds)
        got = ctx.compare_all(dev)
    finally:
        ctx.set_compare_tuning(5, 1 << 22, True)
    assert np.array_equal(got, want)
    assert (want > 0).sum() > 20  # related pairs present


@pytest.mark.parametrize("variant", [3, 5])
def test_cross_with_split_pairs(ctx, oracle, uneven, variant):
    """A unit budget below single-pair sizes row-splits pairs; the maxima go
    through the slot array and the finalize kernel."""
    ds, ods, _ = uneven
    q, t = ds[::3], ds[1::2]
    want = oracle.score_cross_matrix([ods[i] for i in range(0, len(ds), 3)], [ods[i] for i in range(1, len(ds), 2)])
    ctx.set_compare_tuning(variant, 1 << 10, True)
    try:
        got = ctx.compare_to(ctx.upload(q), ctx.upload(t))
    finally:
        ctx.set_compare_tuning(5, 1 << 22, True)
    assert np.array_equal(got, want)


def test_tensor_core_counts_on_dense_and_sparse_filters(ctx, oracle):
    """Counts near the extremes (all-ones, empty and single-bit filters) and
    tiles of every width 1..256 through the tensor-core variant."""
    import sdhash_gb300 as g
    rng = np.random.default_rng(9)
    ds = []
    for i, n in enumerate([1, 2, 15, 16, 17, 31, 33, 100, 255, 256, 257, 300]):
        f = (rng.random((n, 256)) < rng.uniform(0.05, 0.6)).astype(np.uint8) * rng.integers(1, 256, (n, 256),
                                                                                           dtype=np.uint8)
        if i == 3:
            f[0] = 0xFF
        if i == 4:
            f[:] = 0
            f[:, 7] = 1
        counts = rng.integers(0, 193, n).astype(np.uint16)
        ds.append(g.Digest(f"x{i:02d}", 0, n, 0, 192, 16384, f.reshape(-1), counts))
    ods = [oracle.parse(d.to_string()) for d in ds]
    want = oracle.score_all_matrix(ods)
    iu = np.triu_indices(len(ds), 1)
    dev = ctx.upload(ds)
    for v in (0, 5):
        ctx.set_compare_tuning(v, 1 << 22, False)
        try:
            assert np.array_equal(ctx.compare_all(dev), want[iu]), v
        finally:
            ctx.set_compare_tuning(5, 1 << 22, True)


def test_graph_replay_and_device_output(ctx, uneven):
    import torch
    ds, ods, want = uneven
    dev = ctx.upload(ds)
    n = len(ds)
    out = torch.full((n * (n - 1) // 2,), -7, dtype=torch.int32, device="cuda")
    l0 = ctx.launch_count
    ctx.compare_all_device(dev, out.data_ptr())
    ctx.synchronize()
    first = out.cpu().numpy().copy()
    out.fill_(-7)
    ctx.compare_all_device(dev, out.data_ptr())   # replays the captured graph
    ctx.synchronize()
    assert np.array_equal(first, want)
    assert np.array_equal(out.cpu().numpy(), want)
    assert ctx.launch_count - l0 >= 2
    assert ctx.filter_pairs(dev) == sum(a.bf_count * b.bf_count for i, a in enumerate(ds) for b in ds[i + 1:])


def test_autotuner_keeps_results(ctx, uneven):
    ds, ods, want = uneven
    dev = ctx.upload(ds)
    v, w, rate = ctx.autotune_compare(dev, sample_pairs=1 << 20)
    try:
        assert 0 <= v < 6 and w in (1 << 20, 1 << 22, 1 << 24) and rate > 0
        assert ctx.compare_tuning() == (v, w)
        assert np.array_equal(ctx.compare_all(dev), want)
    finally:
        ctx.set_compare_tuning(5, 1 << 22, True)


def test_plain_per_pair_path_agrees(ctx, uneven):
    ds, ods, want = uneven
    dev = ctx.upload(ds)
    iu = np.triu_indices(len(ds), 1)
    got = ctx.score_pairs(dev, dev, iu[0], iu[1])
    assert np.array_equal(got, want)


@pytest.mark.parametrize("threshold", [1, 5, -1])
def test_threshold_matches_in_pair_order(ctx, uneven, threshold):
    ds, ods, want = uneven
    dev = ctx.upload(ds)
    got = ctx.compare_all_matches(dev, threshold)
    iu = np.triu_indices(len(ds), 1)
    keep = want >= threshold
    exp = np.stack([iu[0][keep], iu[1][keep], want[keep]], axis=1).astype(np.int32)
    assert np.array_equal(got, exp)
    q, t = ctx.upload(ds[::2]), ctx.upload(ds[1::3])
    full = ctx.compare_to(q, t)
    qi, ti = np.nonzero(full >= threshold)
    expx = np.stack([qi, ti, full[qi, ti]], axis=1).astype(np.int32)
    assert np.array_equal(ctx.compare_to_matches(q, t, threshold), expx)
