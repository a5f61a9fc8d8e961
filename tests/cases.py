"""Deterministic inputs shared by the golden-fixture generator and the tests.

Each case is (name, generator spec); ``make(spec)`` rebuilds the bytes on any
machine (seeded, libm-free generators in sdhash_gb300/csrc/synth.c).
"""
from __future__ import annotations

import numpy as np

from sdhash_gb300 import synth

MiB = 1 << 20
CHUNK = 32 * MiB


def make(spec: dict) -> np.ndarray:
    kind, n = spec["kind"], int(spec["n"])
    seed, stream = int(spec.get("seed", 1)), int(spec.get("stream", 0))
    if kind == "random":
        return synth.random_bytes(seed, stream, n)
    if kind == "mixture":
        return synth.mixture_bytes(seed, stream, n)
    if kind == "zeros":
        return np.zeros(n, dtype=np.uint8)
    if kind == "period":  # repeating pattern of `period` random bytes
        p = synth.random_bytes(seed, stream, int(spec["period"]))
        return np.resize(p, n)
    if kind == "ramp":  # 0,1,2,...,255,0,1,... (constant entropy rank)
        return (np.arange(n) % int(spec.get("period", 256))).astype(np.uint8)
    if kind == "repeat_block":  # a random block repeated (duplicate features)
        b = synth.random_bytes(seed, stream, int(spec["block"]))
        return np.resize(b, n)
    if kind == "runs_then_random":  # low-entropy prefix, random tail
        a = np.full(int(spec["prefix"]), 0x41, dtype=np.uint8)
        return np.concatenate([a, synth.random_bytes(seed, stream, n - a.size)])
    raise ValueError(kind)


def _r(n, stream=0, seed=11):
    return {"kind": "random", "n": n, "seed": seed, "stream": stream}


def _m(n, stream=0, seed=12):
    return {"kind": "mixture", "n": n, "seed": seed, "stream": stream}


# Edge sizes: minimum input, window boundaries, stream tile boundaries
# (tiles own 8192 window steps; a chunk of n bytes has n-64 steps), dd block
# boundaries, the 32 MiB stream chunk boundary.
SMALL_CASES = [(f"rnd{n}", _r(n, i)) for i, n in enumerate(
    [511, 512, 513, 575, 576, 577, 640, 700, 1000, 2048, 4095, 4096, 4097, 8191, 8192, 8255, 8256, 8257, 8320,
     12000, 16383, 16384, 16385, 16384 + 511, 16384 + 512, 16448, 16449, 24576 + 64, 70000, 100000, 300000])]
SMALL_CASES += [(f"mix{n}", _m(n, i)) for i, n in enumerate([600, 9000, 50000, 200000, 700000])]
SMALL_CASES += [
    ("zeros100k", {"kind": "zeros", "n": 100000}),
    ("period7", {"kind": "period", "n": 140000, "period": 7, "seed": 3}),
    ("period64", {"kind": "period", "n": 150000, "period": 64, "seed": 4}),
    ("period200", {"kind": "period", "n": 150000, "period": 200, "seed": 5}),
    ("ramp256", {"kind": "ramp", "n": 120000, "period": 256}),
    ("ramp97", {"kind": "ramp", "n": 90000, "period": 97}),
    ("rep100k", {"kind": "repeat_block", "n": 1024000, "block": 102400, "seed": 6}),
    ("rep9k", {"kind": "repeat_block", "n": 300000, "block": 9000, "seed": 7}),
    ("runs_rand", {"kind": "runs_then_random", "n": 60000, "prefix": 20000, "seed": 8}),
]

# Larger stream inputs: many tiles, the chunk boundary, big-filter roll-over.
LARGE_CASES = [
    ("rnd4M", _r(4 * MiB, 100)),
    ("mix6M", _m(6 * MiB, 101)),
    ("rnd32M", _r(CHUNK, 102)),
    ("rnd32M+1000", _r(CHUNK + 1000, 103)),
    ("mix32M+65", _m(CHUNK + 65, 104)),
    ("rnd32M+600", _r(CHUNK + 600, 105)),
    ("mix40M", _m(40 * MiB, 106)),
]

DD_SIZES = [16384, 4096, 1024, 8192]
