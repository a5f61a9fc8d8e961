"""Serving loop: continuous batching over a resident target set.  Every
query's scores are the same alone and in the mix (integer-identical to a
solo compare_to and to the oracle)."""
import random
import threading
import time

import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def serve_data(ctx, oracle):
    import sdhash_gb300 as g
    tsizes = [int(s) for s in synth.log_uniform_sizes(51, 12, 200 << 10, 6 << 20)]
    tfiles = [synth.mixture_bytes(51, i, s) for i, s in enumerate(tsizes)]
    targets = ctx.digest_buffers([f.tobytes() for f in tfiles], [f"t{i:02d}" for i in range(len(tfiles))], 16384)
    targets += ctx.digest_buffers([f.tobytes() for f in tfiles[:4]], [f"s{i:02d}" for i in range(4)], 0)
    qfiles = []
    rng = np.random.default_rng(52)
    for i in range(48):
        if i % 3 == 0:   # cut from a target: high scores
            f = tfiles[i % len(tfiles)]
            n = int(rng.integers(4096, min(len(f), 1 << 20)))
            o = int(rng.integers(0, len(f) - n + 1))
            qfiles.append(f[o:o + n].copy())
        else:
            qfiles.append(synth.mixture_bytes(53, i, int(rng.integers(4096, 2 << 20))))
    queries = ctx.digest_buffers([f.tobytes() for f in qfiles], [f"q{i:02d}" for i in range(len(qfiles))], 0)
    queries = [q for q in queries if q is not None]
    tset = ctx.upload(targets)
    solo = ctx.compare_to(ctx.upload(queries), tset)
    ot = [oracle.parse(d.to_string()) for d in targets]
    oq = [oracle.parse(d.to_string()) for d in queries]
    assert np.array_equal(solo, oracle.score_cross_matrix(oq, ot))
    return g, targets, queries, tset, solo


def _drain(srv, want, timeout_s=60):
    got = {}
    t_end = time.time() + timeout_s
    while len(got) < want and time.time() < t_end:
        for r, row in srv.poll(64, timeout_ms=50):
            got[int(r.tag)] = (r, row)
    return got


def test_served_results_equal_solo_results(ctx, serve_data):
    g, targets, queries, tset, solo = serve_data
    srv = g.Server(ctx, tset, slots=3, max_batch_queries=6, memory_budget=4 << 20, threshold=1)
    try:
        order = list(range(len(queries))) * 2            # every query twice, different neighbours
        random.Random(7).shuffle(order)

        def feed(part):
            for k in part:
                srv.submit(queries[order[k]], k)
                time.sleep(random.random() * 0.002)

        ths = [threading.Thread(target=feed, args=(range(s, len(order), 2),)) for s in (0, 1)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
        got = _drain(srv, len(order))
        assert len(got) == len(order)
        sizes = set()
        for k, (r, row) in got.items():
            q = order[k]
            assert np.array_equal(row, solo[q]), (k, q)
            assert r.best_score == solo[q].max()
            assert r.matches == int((solo[q] >= 1).sum())
            assert r.submit_ns <= r.start_ns <= r.done_ns
            sizes.add(int(r.batch_queries))
        st = srv.stats()
        assert st["served"] == len(order) and st["pending"] == 0 and st["batches"] >= 2
        # one query alone on an idle server
        srv.submit(queries[5], 10_000)
        (r, row), = _drain(srv, 1).values()
        assert r.batch_queries == 1 and np.array_equal(row, solo[5])
    finally:
        srv.close()


def test_burst_is_batched_and_exact(ctx, serve_data):
    """One slot and a burst of requests: queries arriving while a batch runs
    are admitted together into the next one; every row is still exact."""
    g, targets, queries, tset, solo = serve_data
    srv = g.Server(ctx, tset, slots=1, max_batch_queries=16, memory_budget=4 << 20, threshold=1)
    try:
        order = list(range(len(queries))) * 4
        for k, q in enumerate(order):
            srv.submit(queries[q], k)
        got = _drain(srv, len(order))
        assert len(got) == len(order)
        for k, (r, row) in got.items():
            assert np.array_equal(row, solo[order[k]]), k
        assert max(int(r.batch_queries) for r, _ in got.values()) > 1
    finally:
        srv.close()


def test_server_rejects_oversized_query(ctx, serve_data):
    g, targets, queries, tset, solo = serve_data
    srv = g.Server(ctx, tset, slots=1, max_batch_queries=4, memory_budget=1 << 20)
    try:
        big = g.Digest("big", 0, 5000, 160, 160, 0, np.zeros(5000 * 256, np.uint8), None)
        with pytest.raises(g.EngineError) as e:
            srv.submit(big, 1)
        assert e.value.code == -5  # SDBFG_ERR_CAPACITY
    finally:
        srv.close()
