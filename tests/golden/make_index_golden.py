"""Generate the index-search fixtures (tests/golden/index/) from the REFERENCE
sdhash.

Builds two indexes as sdhash --index does (sdhash-src/sdhash_threads.cc:
376-470; one group each): A from two stream-mode digests (the --index path
of files below 16 MiB), B from one block-mode digest (the path of larger
files).  Each is written as the reference writes it: the set as SDBF text
(idx/A.sdbf) and the index file (idx/A.sdbf.idx, LZ4-compressed 64 MiB
filter), stored here gzip-compressed.  Then runs the reference's index
search (sdhash --index-search idx, sdhash.cc:231-266 and 638-652) on five
seeded query inputs in 16 KiB block mode and records index_results(), and
records the sha256 of each index filter as the reference decompresses it.
Also builds three more indexes from fresh (a stream-mode group whose later
files repeat earlier ones, a block-mode group, and a stream-mode group of
40 files cut from one shared pool) and records the set text, the index
header and the filter's sha256 of each.

Inputs are seeded synthetic mixture content (sdhash_gb300/synth.py), so the
GPU tests regenerate them on any machine.

Needs the reference source tree (only in the build container):
    SDHASH_REFERENCE_SRC=<tree> python tests/golden/make_index_golden.py
"""
from __future__ import annotations

import ctypes as C
import gzip
import hashlib
import json
import os
import shutil
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import Reference, build_reference  # noqa: E402
from sdhash_gb300 import synth  # noqa: E402

OUT = os.path.join(HERE, "index")


def index_inputs():
    """(name, bytes) of the indexed files: group A (stream) and B (block)."""
    a = [(f"a{i}.bin", synth.mixture_bytes(91, i, n).tobytes()) for i, n in enumerate((40_000, 56_000))]
    b = [("b0.bin", synth.mixture_bytes(92, 0, 256 << 10).tobytes())]
    return a, b


def queries():
    """(name, bytes) of the searched inputs."""
    a, b = index_inputs()
    return [("q0.bin", a[1][1][5_000:35_000]),
            ("q1.bin", b[0][1][10_000:110_000]),
            ("q2.bin", synth.random_bytes(93, 0, 50_000).tobytes()),
            ("q3.bin", a[0][1][:20_000] + b[0][1][130_000:170_000]),
            ("q4.bin", synth.random_bytes(93, 1, 700).tobytes())]


def build_inputs():
    """(name, bytes) groups indexed with sdhash --index's two paths: stream
    mode (later files repeat parts of earlier ones, so the index drops their
    features from their digests) and 16 KiB block mode."""
    s0 = synth.mixture_bytes(94, 0, 120_000).tobytes()
    s2 = synth.mixture_bytes(94, 2, 60_000).tobytes()
    stream = [("s0.bin", s0), ("s1.bin", s0[20_000:100_000] + synth.random_bytes(94, 1, 30_000).tobytes()),
              ("s2.bin", s2), ("s3.bin", s0), ("s4.bin", s2[:30_000] + s0[:30_000])]
    b0 = synth.mixture_bytes(95, 0, 300_000).tobytes()
    block = [("b0.bin", b0), ("b1.bin", b0[50_000:250_000] + synth.mixture_bytes(95, 1, 100_000).tobytes())]
    return stream, block, dense_stream()


def dense_stream():
    """A stream-mode group of 40 files cut from one shared 400 KB pool
    (three slices each, plus fresh bytes), so that most features recur in
    several files and each file's digest depends on many earlier ones."""
    import numpy as np
    pool = synth.mixture_bytes(96, 0, 400_000).tobytes()
    rng = np.random.default_rng(96)
    out = []
    for i in range(40):
        parts = []
        for _ in range(3):
            n = int(rng.integers(8_000, 40_000))
            o = int(rng.integers(0, len(pool) - n))
            parts.append(pool[o:o + n])
        parts.append(synth.random_bytes(96, i + 1, int(rng.integers(0, 6_000))).tobytes())
        out.append((f"d{i}.bin", b"".join(parts)))
    return out


def _arr(items):
    names = (C.c_char_p * len(items))(*[n.encode() for n, _ in items])
    bufs = (C.c_char_p * len(items))(*[d for _, d in items])
    lens = (C.c_ulonglong * len(items))(*[len(d) for _, d in items])
    return names, bufs, lens


def main():
    build_reference()
    R = Reference()
    L = R.L
    L.ref_index_build.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_uint, C.c_char_p, C.c_char_p]
    L.ref_index_search.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                   C.c_uint]
    L.ref_index_search.restype = C.c_void_p
    L.ref_index_bits.argtypes = [C.c_char_p, C.c_void_p, C.c_ulonglong]
    L.ref_index_bits.restype = C.c_longlong
    a, b = index_inputs()
    cwd = os.getcwd()
    tmp = tempfile.mkdtemp()
    try:
        os.chdir(tmp)
        os.mkdir("idx")
        for items, dd, stem in ((a, 0, "A"), (b, 16384, "B")):
            names, bufs, lens = _arr(items)
            rc = L.ref_index_build(names, bufs, lens, len(items), dd, f"idx/{stem}.sdbf".encode(),
                                   f"idx/{stem}.sdbf.idx".encode())
            assert rc == 0, rc
        qs = queries()
        names, bufs, lens = _arr(qs)
        order = ["A", "B"]
        idx = (C.c_char_p * 2)(*[f"idx/{s}.sdbf.idx".encode() for s in order])
        sets = (C.c_char_p * 2)(*[f"idx/{s}.sdbf".encode() for s in order])
        text = R._take(L.ref_index_search(idx, sets, 2, names, bufs, lens, len(qs), 16384))
        rec = {"generator": "tests/golden/make_index_golden.py",
               "reference": "sdhash 4.0 --index / --index-search through its library API",
               "index_order": order, "dd_block_size": 16384, "results": text, "indexes": {}}
        os.makedirs(OUT, exist_ok=True)
        for s in order:
            raw = open(f"idx/{s}.sdbf.idx", "rb").read()
            buf = (C.c_ubyte * (64 << 20))()
            size = L.ref_index_bits(f"idx/{s}.sdbf.idx".encode(), buf, 64 << 20)
            assert size == 64 << 20, size
            head = raw[:raw.index(b"\n")].decode()
            rec["indexes"][s] = {"header": head, "filter_sha256": hashlib.sha256(bytes(buf)).hexdigest(),
                                 "filter_popcount": int(sum(bin(x).count("1") for x in bytes(buf) if x))}
            with open(os.path.join(OUT, f"{s}.sdbf.idx.gz"), "wb") as fo:
                with gzip.GzipFile(fileobj=fo, mode="wb", compresslevel=9, mtime=0) as f:
                    f.write(raw)
            shutil.copy(f"idx/{s}.sdbf", os.path.join(OUT, f"{s}.sdbf"))
        # index builds (stream and block groups) from fresh indexes
        rec["builds"] = []
        for items, dd, stem in zip(build_inputs(), (0, 16384, 0), ("S", "K", "D")):
            names, bufs, lens = _arr(items)
            rc = L.ref_index_build(names, bufs, lens, len(items), dd, f"idx/{stem}.sdbf".encode(),
                                   f"idx/{stem}.sdbf.idx".encode())
            assert rc == 0, rc
            raw = open(f"idx/{stem}.sdbf.idx", "rb").read()
            buf = (C.c_ubyte * (64 << 20))()
            assert L.ref_index_bits(f"idx/{stem}.sdbf.idx".encode(), buf, 64 << 20) == 64 << 20
            rec["builds"].append({"stem": stem, "dd": dd, "names": [n for n, _ in items],
                                  "header": raw[:raw.index(b"\n")].decode(),
                                  "filter_sha256": hashlib.sha256(bytes(buf)).hexdigest(),
                                  "sdbf_text": open(f"idx/{stem}.sdbf").read()})
        with open(os.path.join(OUT, "index_search.json"), "w") as f:
            json.dump(rec, f, indent=1)
        print(text)
        for s in order:
            print(s, rec["indexes"][s]["header"], os.path.getsize(os.path.join(OUT, f"{s}.sdbf.idx.gz")))
    finally:
        os.chdir(cwd)
        shutil.rmtree(tmp)


if __name__ == "__main__":
    main()
