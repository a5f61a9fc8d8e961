"""GPU digest generation through the C ABI, checked against the reference's
recorded outputs (tests/golden/golden.json) and the oracle.  Bit-exact:
SDBF text byte-identical."""
import hashlib

import numpy as np
import pytest

import cases
from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu


def sha(t: str) -> str:
    return hashlib.sha256(t.encode()).hexdigest()


def _golden_by_mode(golden):
    by = {}
    for rec in golden["digests"]:
        by.setdefault(rec["dd"], []).append(rec)
    return by


@pytest.mark.parametrize("dd", [0, 16384, 4096, 1024, 8192])
def test_small_cases_one_batch(ctx, golden, dd):
    recs = _golden_by_mode(golden)[dd]
    datas = [cases.make(r["spec"]) for r in recs]
    out = ctx.digest_buffers([d.tobytes() for d in datas], [r["name"] for r in recs], dd)
    bad = []
    for r, d in zip(recs, out):
        if r["status"] != 0:
            assert d is None, r["name"]
            continue
        t = d.to_string()
        if sha(t) != r["sha256"]:
            bad.append(r["name"])
    assert not bad, f"dd={dd}: {bad}"


@pytest.mark.parametrize("lead", [0, 3, 17, 48, 128])
def test_short_lead_in_exercises_relink(ctx, golden, lead):
    """Lead-ins from none to the maximum (short ones make speculation fail
    often); the in-tile and cross-tile re-walks keep the digests exact."""
    recs = [r for r in _golden_by_mode(golden)[0] if r["status"] == 0]
    big = [r for r in golden["large"] if r["dd"] == 0 and r["spec"]["n"] <= (8 << 20)]
    datas = [cases.make(r["spec"]) for r in recs + big]
    before = ctx.relinked_tiles
    ctx.set_lead(lead)
    try:
        out = ctx.digest_buffers([d.tobytes() for d in datas], [r["name"] for r in recs + big], 0)
    finally:
        ctx.set_lead(64)  # the default
    bad = [r["name"] for r, d in zip(recs + big, out) if sha(d.to_string()) != r["sha256"]]
    assert not bad, bad
    if lead <= 17:
        assert ctx.relinked_tiles > before  # the cross-tile path actually ran


def test_large_cases(ctx, golden):
    for dd in (0, 16384):
        recs = [r for r in golden["large"] if r["dd"] == dd]
        datas = [cases.make(r["spec"]) for r in recs]
        out = ctx.digest_buffers([d.tobytes() for d in datas], [r["name"] for r in recs], dd)
        for r, d in zip(recs, out):
            t = d.to_string()
            assert t[:96] == r["head"], (r["name"], dd)
            assert sha(t) == r["sha256"], (r["name"], dd)


def test_plain_small_set_digests(ctx, golden):
    g = golden["plain_small"]
    names, files = synth.plain_small_set(seed=g["seed"])
    out = ctx.digest_buffers([f.tobytes() for f in files], names, 0)
    assert [sha(d.to_string()) for d in out] == g["sha256"]
    dd = ctx.digest_buffers([f.tobytes() for f in files[:8]], [n + ".dd" for n in names[:8]], 16384)
    assert [sha(d.to_string()) for d in dd] == g["dd_sha256"]


def test_batch_invariance_and_order(ctx, oracle):
    """A file's digest does not depend on its batch neighbours or position."""
    rng = np.random.default_rng(3)
    sizes = [int(s) for s in synth.log_uniform_sizes(9, 40, 512, 3 << 20)]
    files = [synth.mixture_bytes(9, i, s) for i, s in enumerate(sizes)]
    names = [f"m{i}" for i in range(len(files))]
    together = [d.to_string() for d in ctx.digest_buffers([f.tobytes() for f in files], names, 0)]
    perm = rng.permutation(len(files))
    shuffled = ctx.digest_buffers([files[i].tobytes() for i in perm], [names[i] for i in perm], 0)
    for k, i in enumerate(perm):
        assert shuffled[k].to_string() == together[i]
    for i in (0, 7, 21):
        alone = ctx.digest_buffers([files[i].tobytes()], [names[i]], 0)[0].to_string()
        assert alone == together[i]
        assert alone == oracle.digest(names[i], files[i].tobytes(), 0).to_string()


def test_packed_host_layout_and_device_api(ctx, oracle):
    """digest_packed (one pinned-or-pageable host buffer) and the device-resident
    entry point give the same digests as the oracle."""
    import torch
    sizes = [5000, 70000, 1 << 20, 600, 33 << 10]
    data, offs, lens = synth.fill_many(21, "mixture", sizes)
    host = ctx.digest_packed(data, offs, lens, 0)
    dev = torch.from_numpy(data).cuda()
    cap = ctx.capacity(lens, 0)
    out = torch.zeros(cap * 256, dtype=torch.uint8, device="cuda")
    res = ctx.digest_device(dev.data_ptr(), offs, lens, 0, out.data_ptr(), cap)
    torch.cuda.synchronize()
    outh = out.cpu().numpy()
    for i, (o, n) in enumerate(zip(offs, lens)):
        ref = oracle.digest(f"f{i}", data[int(o):int(o) + int(n)].tobytes(), 0)
        assert host[i].to_string() == ref.to_string()
        r = res[i]
        assert (r.bf_count, r.last_count) == (ref.bf_count, ref.last_count)
        got = outh[r.filter_offset * 256:(r.filter_offset + r.bf_count) * 256].tobytes()
        assert got == ref.filters()


def test_reference_object_api(ctx, oracle):
    import sdhash_gb300 as g
    a = synth.random_bytes(4, 1, 300000)
    b = a.copy()
    b[100000:100100] = 7
    sa, sb = g.sdbf("a", a.tobytes()), g.sdbf("b", b.tobytes())
    oa, ob = oracle.digest("a", a.tobytes(), 0), oracle.digest("b", b.tobytes(), 0)
    assert sa.to_string() == oa.to_string()
    assert sa.compare(sb, 0) == oracle.score(oa, ob)
    with pytest.raises(g.SdbfError) as e:
        g.sdbf("tiny", b"x" * 100)
    assert e.value.code == -3
    back = g.sdbf.from_string(sa.to_string())
    assert back.compare(sb, 0) == sa.compare(sb, 0)


@pytest.mark.parametrize("lead", [0, 5])
def test_short_lead_in_block_mode(ctx, golden, lead):
    """Block mode re-walks mis-speculated segments inside each block."""
    recs = [r for r in _golden_by_mode(golden)[16384] if r["status"] == 0]
    datas = [cases.make(r["spec"]) for r in recs]
    ctx.set_lead(lead)
    try:
        out = ctx.digest_buffers([d.tobytes() for d in datas], [r["name"] for r in recs], 16384)
    finally:
        ctx.set_lead(64)  # the default
    bad = [r["name"] for r, d in zip(recs, out) if sha(d.to_string()) != r["sha256"]]
    assert not bad, bad
