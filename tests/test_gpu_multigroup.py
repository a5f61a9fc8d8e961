"""The digest path at the scale the bulk-generation benchmark runs it.

Smaller tests fit one launch group.  Here about 6 GiB of mixture content
(sixty 64 MiB files of two 32 MiB chunks each, files just over one chunk, a
log-uniform spread of 4 KiB..64 MiB files and a few below the 512-byte
minimum) goes through the C ABI twice:

* host buffers (sdbfg_digest_batch): the pinned input staged on the device
  by a gather kernel per launch group; launch groups of 256 MiB, 512 MiB,
  1 GiB, then 2 GiB, four in flight on their own streams, tile kernels
  chained by events across the streams;
* device-resident input (sdbfg_digest_batch_device): 2 GiB groups.

Every file of both runs is checked against the oracle (filters, bf_count,
last_count; sdbf_core.cc:196-246), and the two runs against each other.
"""
import ctypes as C

import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu

MiB = 1 << 20


def _sizes():
    spread = [int(s) for s in synth.log_uniform_sizes(31, 300, 4096, 64 * MiB)]
    edges = [32 * MiB + 65, 32 * MiB + 1000, 64 * MiB - 1, 64 * MiB - 63, 33 * MiB + 7, 100, 511, 512, 4097]
    sizes = [64 * MiB] * 60 + spread + edges
    rng = np.random.default_rng(5)
    return np.array([sizes[i] for i in rng.permutation(len(sizes))], dtype=np.uint64)


def test_multi_group_batch_matches_oracle(ctx, oracle):
    import torch
    from sdhash_gb300 import DigestResult, _ptr, _u64, lib

    sizes = _sizes()
    offs, total = synth.packed_layout(sizes)
    # host path: groups of 256 MiB, 512 MiB, 1 GiB, then at least two full 2 GiB groups
    assert total > (256 + 512 + 1024) * MiB + 2 * (2 << 30)
    pinned = torch.empty(total, dtype=torch.uint8, pin_memory=True)
    data = pinned.numpy()
    synth.fill_many(41, "mixture", sizes, out=data)
    o64, l64 = _u64(offs), _u64(sizes)
    n = len(sizes)
    cap = ctx.capacity(l64, 0)

    ctx.set_pipeline_depth(4)
    out_host = torch.empty(cap * 256, dtype=torch.uint8, pin_memory=True).numpy()
    res_host = (DigestResult * n)()
    ctx._check(lib().sdbfg_digest_batch(ctx.h, data.ctypes.data, _ptr(o64), _ptr(l64), n, 0, out_host.ctypes.data,
                                        cap, None, res_host))

    dev = torch.from_numpy(data).cuda()
    out_dev = torch.zeros(cap * 256, dtype=torch.uint8, device="cuda")
    res_dev = ctx.digest_device(dev.data_ptr(), offs, sizes, 0, out_dev.data_ptr(), cap)
    torch.cuda.synchronize()
    out_dev_h = out_dev.cpu().numpy()
    del dev, out_dev

    want = oracle.digest_many([data[int(o):int(o) + int(s)] for o, s in zip(offs, sizes)], 0)
    bad = []
    for i in range(n):
        od = want[i]
        for name, r, buf in (("host", res_host[i], out_host), ("device", res_dev[i], out_dev_h)):
            if od is None:
                if r.status == 0:
                    bad.append((i, name, "accepted a file below 512 bytes"))
                continue
            got = buf[r.filter_offset * 256:(r.filter_offset + r.bf_count) * 256].tobytes()
            if r.status != 0 or (r.bf_count, r.last_count) != (od.bf_count, od.last_count) or got != od.filters():
                bad.append((i, name, int(sizes[i])))
    assert not bad, bad[:10]
    # the 64 MiB files carry filters from both of their chunks
    big = [i for i in range(n) if int(sizes[i]) == 64 * MiB]
    assert all(res_host[i].bf_count > 1 for i in big)


def test_pinned_inputs_at_unaligned_offsets(ctx, oracle):
    """Pinned host inputs at offsets that are not multiples of 16 or 4 (the
    staging copy then reads them with narrower loads), as one batch with a
    file of more than one 1 MiB staging piece."""
    import torch
    from sdhash_gb300 import DigestResult, _ptr, _u64, lib

    sizes = [700, 1 << 20, 3 * MiB + 5, 5000, 2 * MiB + 1, 600, 100000]
    offs, pos = [], 0
    for k, n in enumerate(sizes):
        pos += (1, 6, 3, 16, 2, 5, 7)[k]  # gaps that leave odd, even and aligned starts
        offs.append(pos)
        pos += n
    pinned = torch.empty(pos + 64, dtype=torch.uint8, pin_memory=True)
    data = pinned.numpy()
    for k, (o, n) in enumerate(zip(offs, sizes)):
        data[o:o + n] = synth.mixture_bytes(43, k, n)
    o64, l64 = _u64(offs), _u64(sizes)
    cap = ctx.capacity(l64, 0)
    out = torch.empty(cap * 256, dtype=torch.uint8, pin_memory=True).numpy()
    res = (DigestResult * len(sizes))()
    for _ in range(2):  # twice: the staging buffers are reused
        ctx._check(lib().sdbfg_digest_batch(ctx.h, data.ctypes.data, _ptr(o64), _ptr(l64), len(sizes), 0,
                                            out.ctypes.data, cap, None, res))
        for k, (o, n) in enumerate(zip(offs, sizes)):
            od = oracle.digest(f"u{k}", data[o:o + n].tobytes(), 0)
            r = res[k]
            assert (r.bf_count, r.last_count) == (od.bf_count, od.last_count), k
            assert out[r.filter_offset * 256:(r.filter_offset + r.bf_count) * 256].tobytes() == od.filters(), k
