"""Generate tests/golden/golden.json from the REFERENCE sdhash.

Runs the unmodified reference library (compiled from its own sources by
oracle/Makefile.ref into oracle/_ref/libsdbf_ref.so) on the deterministic
inputs of tests/cases.py and records what it produces:

* for every case and mode (stream, dd 16/4/1/8 KiB): sha256 of the SDBF text
  line, plus the full line when it is short;
* the plain small set (32 random 1 MiB files + partners): sha256 of every
  digest and the full ``compare_all`` result text at threshold 1;
* a block-mode query/target ``compare_to`` result.

Needs the reference source tree (only in the build container):
    SDHASH_REFERENCE_SRC=<tree> python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

import cases  # noqa: E402
from oracle import Reference, build_reference  # noqa: E402
from sdhash_gb300 import synth  # noqa: E402


def sha(s: str) -> str:
    return hashlib.sha256(s.encode()).hexdigest()


def main():
    build_reference()
    R = Reference()
    out = {"generator": "tests/golden/make_golden.py", "reference": "sdhash 4.0 (sdbf/*, base64/*) + system libcrypto",
           "digests": [], "large": []}
    for name, spec in cases.SMALL_CASES:
        data = cases.make(spec).tobytes()
        for dd in [0] + cases.DD_SIZES:
            t = R.digest(name, data, dd)
            rec = {"name": name, "spec": spec, "dd": dd, "status": 0 if t else -3}
            if t:
                rec["sha256"] = sha(t)
                if len(t) <= 3000:
                    rec["text"] = t
            out["digests"].append(rec)
    for name, spec in cases.LARGE_CASES:
        data = cases.make(spec).tobytes()
        for dd in (0, 16384):
            t = R.digest(name, data, dd)
            out["large"].append({"name": name, "spec": spec, "dd": dd, "sha256": sha(t),
                                 "head": t[:96], "bytes": len(t)})
        print("large", name, flush=True)
    # plain small set: stream digests + all-pairs
    names, files = synth.plain_small_set(seed=1)
    texts = [R.digest(n, f.tobytes(), 0) for n, f in zip(names, files)]
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "set.sdbf")
        with open(p, "w") as f:
            f.write("".join(texts))
        cmp_all = R.compare_all_file(p, 1)
        # block-mode digests of the same files, compared against the stream set
        dd_texts = [R.digest(n + ".dd", f.tobytes(), 16384) for n, f in zip(names[:8], files[:8])]
        q = os.path.join(td, "q.sdbf")
        with open(q, "w") as f:
            f.write("".join(dd_texts))
        cmp_to = R.compare_to_files(q, p, 1)
        cmp_all_neg = R.compare_all_file(q, -1)
    out["plain_small"] = {"seed": 1, "names": names, "sha256": [sha(t) for t in texts],
                          "compare_all_t1": cmp_all, "dd_sha256": [sha(t) for t in dd_texts],
                          "compare_to_dd_vs_stream_t1": cmp_to, "compare_all_dd_tneg1": cmp_all_neg}
    add_fast(R, out)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print("wrote golden.json:", len(out["digests"]), "digests,", len(cmp_all.splitlines()), "compare lines")


def add_fast(R, out):
    """--fast results of the reference on the plain small set: all pairs of
    the stream digests, the stream digests (queries, folded by the reference)
    against the block digests (targets, left unfolded: compare_to folds only
    the query set, sdbf/sdbf_set.cc:321-331), all pairs of the block digests."""
    names, files = synth.plain_small_set(seed=1)
    texts = [R.digest(n, f.tobytes(), 0) for n, f in zip(names, files)]
    dd_texts = [R.digest(n + ".dd", f.tobytes(), 16384) for n, f in zip(names[:8], files[:8])]
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "set.sdbf")
        with open(p, "w") as f:
            f.write("".join(texts))
        q = os.path.join(td, "q.sdbf")
        with open(q, "w") as f:
            f.write("".join(dd_texts))
        out["plain_small"]["compare_all_fast_t1"] = R.compare_all_file(p, 1, fast=True)
        out["plain_small"]["compare_to_fast_stream_vs_dd_t1"] = R.compare_to_files(p, q, 1, fast=True)
        out["plain_small"]["compare_all_dd_fast_tneg1"] = R.compare_all_file(q, -1, fast=True)


if __name__ == "__main__":
    if "--fast-only" in sys.argv:   # add the --fast results to an existing golden.json
        path = os.path.join(HERE, "golden.json")
        with open(path) as f:
            g = json.load(f)
        add_fast(Reference(), g)
        with open(path, "w") as f:
            json.dump(g, f, indent=0, sort_keys=True)
        print("added --fast results to golden.json")
    else:
        main()
