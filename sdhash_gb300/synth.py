"""Seeded synthetic workloads (wrapper over libsdbf_synth.so, csrc/synth.c).

The reference names no dataset; these generators stand in with the shapes
the benchmark configurations describe:

* ``plain_small_set``  -- 32 uniform-random 1 MiB files, each with a partner
  (30% of its 4 KiB blocks replaced, a 1..63-byte insertion at 90% of the
  length shifting the last 10% of the bytes, truncated back to 1 MiB).
* ``bulk_stream_workload`` -- file sizes log-uniform over [lo, hi], content a
  per-file mixture of random regions, low-entropy runs and order-1 Markov text.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import SYNTH_PATH

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(SYNTH_PATH):
            from .build import build_synth
            build_synth()
        L = C.CDLL(SYNTH_PATH)
        u8p, u64p = C.c_void_p, C.POINTER(C.c_uint64)
        L.synth_fill_random.argtypes = [C.c_uint64, C.c_uint64, u8p, C.c_uint64]
        L.synth_fill_mixture.argtypes = [C.c_uint64, C.c_uint64, u8p, C.c_uint64]
        L.synth_partner.argtypes = [C.c_uint64, C.c_uint64, u8p, u8p, C.c_uint64]
        L.synth_log_uniform_sizes.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64, u64p]
        L.synth_fill_many.argtypes = [C.c_uint64, C.c_int, C.c_uint32, u64p, u64p, u8p, C.c_int]
        _lib = L
    return _lib


def random_bytes(seed: int, stream: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    lib().synth_fill_random(seed, stream, out.ctypes.data, n)
    return out


def mixture_bytes(seed: int, stream: int, n: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    lib().synth_fill_mixture(seed, stream, out.ctypes.data, n)
    return out


def partner(seed: int, stream: int, base: np.ndarray) -> np.ndarray:
    base = np.ascontiguousarray(base, dtype=np.uint8)
    out = np.empty_like(base)
    lib().synth_partner(seed, stream, base.ctypes.data, out.ctypes.data, base.size)
    return out


def log_uniform_sizes(seed: int, count: int, lo: int, hi: int) -> np.ndarray:
    out = np.empty(count, dtype=np.uint64)
    lib().synth_log_uniform_sizes(seed, count, lo, hi, out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out


def plain_small_set(seed: int = 1, pairs: int = 32, size: int = 1 << 20):
    """(names, list of uint8 arrays): base_i, partner_i interleaved."""
    names, files = [], []
    for i in range(pairs):
        b = random_bytes(seed, i, size)
        names += [f"base{i:02d}.bin", f"part{i:02d}.bin"]
        files += [b, partner(seed, i, b)]
    return names, files


def packed_layout(sizes, align: int = 16):
    sizes = np.asarray(sizes, dtype=np.uint64)
    padded = (sizes + np.uint64(align - 1)) // np.uint64(align) * np.uint64(align)
    offs = np.zeros(len(sizes), dtype=np.uint64)
    if len(sizes) > 1:
        offs[1:] = np.cumsum(padded[:-1])
    total = int(padded.sum()) if len(sizes) else 0
    return offs, total


def fill_many(seed: int, kind: str, sizes, out: np.ndarray | None = None, nthreads: int | None = None):
    """Fill len(sizes) files packed 16-byte aligned into one buffer.
    kind: 'random' or 'mixture'.  Returns (data, offsets, sizes)."""
    sizes = np.ascontiguousarray(sizes, dtype=np.uint64)
    offs, total = packed_layout(sizes)
    if out is None:
        out = np.empty(max(16, total), dtype=np.uint8)
    nt = nthreads or min(64, os.cpu_count() or 1)
    lib().synth_fill_many(seed, 0 if kind == "random" else 1, len(sizes), offs.ctypes.data_as(C.POINTER(C.c_uint64)),
                          sizes.ctypes.data_as(C.POINTER(C.c_uint64)), out.ctypes.data, nt)
    return out, offs, sizes


def bulk_stream_workload(seed: int = 2, nfiles: int = 4096, lo: int = 4096, hi: int = 64 << 20, out=None):
    sizes = log_uniform_sizes(seed, nfiles, lo, hi)
    return fill_many(seed, "mixture", sizes, out=out)
