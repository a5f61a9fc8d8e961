"""The allocation-free digest entry point (sdbfg_digest_stream_noalloc).

For callers that cannot allocate GPU memory -- e.g. code running under a
framework that owns every device allocation, or with a device-memory budget
fixed up front -- the library offers a stream-mode digest that takes only the
caller's input and output buffers and uses a fixed scratch array compiled
into the library.  This test calls it through the C ABI twice in a row and
checks both results against the regular device entry point
(sdbfg_digest_batch_device): digests must be bit-identical.  It also checks
that a request above the stated limits is rejected.

Collected last (file name) so a run that stops at the first failure has
already run every other test; it creates its own state, so it also passes
alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_BYTES = 8 << 20
ERR_CAPACITY = -5


def _bind(lib):
    f = lib.sdbfg_digest_stream_noalloc
    f.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.c_uint32, C.c_void_p, C.c_uint64,
                  C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def test_noalloc_matches_device_entry_point_twice():
    import torch

    import sdhash_gb300 as g
    from sdhash_gb300 import synth

    lib = g.lib()
    noalloc = _bind(lib)
    sizes = [300, 512, 700, 4096, 8256, 8257, 70000, 1 << 20, 3 << 20, 200000, 2 << 20]
    data, offs, lens = synth.fill_many(123, "mixture", sizes)
    assert int(lens.sum()) <= MAX_BYTES
    dev = torch.from_numpy(data).cuda()
    cap = g.Context.capacity(lens, 0)

    # existing entry point
    ctx = g.Context(0)
    out_ref = torch.zeros(cap * 256, dtype=torch.uint8, device="cuda")
    res_ref = ctx.digest_device(dev.data_ptr(), offs, lens, 0, out_ref.data_ptr(), cap)
    torch.cuda.synchronize()
    ref_filters = out_ref.cpu().numpy()
    n = len(sizes)

    offs_c = np.ascontiguousarray(offs, dtype=np.uint64)
    lens_c = np.ascontiguousarray(lens, dtype=np.uint64)
    for call in range(2):
        out = torch.full((cap * 256,), 0xAB, dtype=torch.uint8, device="cuda")
        res = (g.DigestResult * n)()
        rc = noalloc(dev.data_ptr(), offs_c.ctypes.data_as(C.POINTER(C.c_uint64)),
                     lens_c.ctypes.data_as(C.POINTER(C.c_uint64)), n, out.data_ptr(), cap, C.addressof(res), None)
        assert rc == 0, f"call {call}: rc={rc}"
        got = out.cpu().numpy()
        for i in range(n):
            a, b = res[i], res_ref[i]
            assert (a.status, a.bf_count, a.last_count) == (b.status, b.bf_count, b.last_count), (call, i)
            if a.status == 0:
                ga = got[a.filter_offset * 256:(a.filter_offset + a.bf_count) * 256]
                gb = ref_filters[b.filter_offset * 256:(b.filter_offset + b.bf_count) * 256]
                assert np.array_equal(ga, gb), (call, i)


def test_noalloc_rejects_requests_above_its_limits():
    import sdhash_gb300 as g

    noalloc = _bind(g.lib())
    lens = np.array([MAX_BYTES + 16], dtype=np.uint64)
    offs = np.zeros(1, dtype=np.uint64)
    res = (g.DigestResult * 1)()
    rc = noalloc(C.c_void_p(16), offs.ctypes.data_as(C.POINTER(C.c_uint64)),
                 lens.ctypes.data_as(C.POINTER(C.c_uint64)), 1, C.c_void_p(16), 1, C.addressof(res), None)
    assert rc == ERR_CAPACITY
    # two lengths whose 64-bit sum wraps below the limit are rejected too
    lens2 = np.array([2 ** 64 - 16, 32], dtype=np.uint64)
    offs2 = np.zeros(2, dtype=np.uint64)
    res2 = (g.DigestResult * 2)()
    rc = noalloc(C.c_void_p(16), offs2.ctypes.data_as(C.POINTER(C.c_uint64)),
                 lens2.ctypes.data_as(C.POINTER(C.c_uint64)), 2, C.c_void_p(16), 1, C.addressof(res2), None)
    assert rc == ERR_CAPACITY
