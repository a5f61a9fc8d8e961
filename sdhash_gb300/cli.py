"""Command-line front end with the reference's sdhash options
(sdhash-src/sdhash.cc:100-640), over the GPU engine.

    python -m sdhash_gb300.cli [options] files...

Hashing: files below 16 MiB are digested in stream mode, larger ones in
block mode with 16 KiB blocks and 128 MiB segments (sdhash.cc:487-605;
`-b 0` keeps stream mode, `-b N` puts every file in N KiB block mode);
digests are printed in the reference's order for `-p 1`: the small files,
then the large ones, each in argument order.  `-g` compares all hashed
pairs, `-c` compares the digests of one SDBF file (all pairs) or of two
(every digest of the first against every digest of the second).  Result
lines, separators, thresholds and `--fast` are the reference's.  Not
offered: `-s` (filter sampling seeds rand() from time() in the reference),
`--large`, `--details`.  `--index` builds an index per group of files as
the reference does with one thread; `--index-search DIR` looks every block
up in the directory's index files on the GPU.
"""
from __future__ import annotations

import argparse
import os
import sys

MB = 1 << 20
KB = 1 << 10
VERSION = "sdhash_gb300 (sdhash 4.0 digest format, SDBF v3)"


def _segments(path: str, size: int, seg: int):
    """sdbf_hash_files_dd's segmentation (sdhash-src/sdhash_threads.cc:300-373):
    (name, offset, length) of each segment digest of a file."""
    if not (size > seg and seg > 0):
        return [(path, 0, size)]
    chunks = size // seg
    tail = False
    if size - seg <= 512:
        chunks = 0
    if size - chunks * seg <= 512:
        chunks -= 1
        tail = True
    out = []
    for j in range(chunks + 1):
        name = path if not (j > 0 or chunks > 0) else f"{path}.{j * seg // MB:04d}M"
        if j == chunks:
            csize = size - chunks * seg
            if tail:
                csize = csize + (size - (chunks + 1) * seg)
        else:
            csize = seg
        out.append((name, j * seg, csize))
    return out


def _collect(inputs, deep: bool):
    files = []
    for p in inputs:
        if deep and os.path.isdir(p):
            for root, dirs, names in os.walk(p):
                dirs.sort()  # each directory's files in name order, then its subdirectories in name order
                for n in sorted(names):
                    q = os.path.join(root, n)
                    if os.path.isfile(q):
                        files.append(q)
        if os.path.isfile(p):
            files.append(p)
    return files


def _hash(ctx, files, block_kb: int, seg: int, name_for_stdin=None, stdin_data=None, indexes=None):
    """Digests of the inputs in the reference's set order; with indexes
    (block mode only) also each digest's index-search hits per block."""
    import numpy as np
    import sdhash_gb300 as g
    digs = []
    hits = []

    def seg_digests(data, name, dd):
        # a segment digests csize bytes read from the stream, zero-filled past
        # its end, and records the bytes actually read (sdbf_class.cc:71-88)
        segs = _segments(name, len(data), seg)
        bufs, got = [], []
        for _, o, n in segs:
            b = np.zeros(n, dtype=np.uint8)
            part = np.frombuffer(bytes(data[o:o + n]), dtype=np.uint8) if not isinstance(data, np.ndarray) \
                else data[o:o + n]
            b[:len(part)] = part
            bufs.append(b)
            got.append(len(part))
        names = [nm for nm, _, _ in segs]
        if indexes is not None:
            out, hr = ctx.digest_search(bufs, names, dd, indexes)
        else:
            out, hr = ctx.digest_buffers(bufs, names, dd), [None] * len(bufs)
        res = []
        for d, h, n in zip(out, hr, got):
            if d is not None and n >= 512:
                d.orig_size = n
                res.append(d)
                hits.append(h)
        return res

    def done():
        items = [g.sdbf(_digest=d) for d in digs]
        return (items, hits) if indexes is not None else items

    if stdin_data is not None:
        dd = (block_kb if block_kb > 0 else 16) * KB
        digs += seg_digests(stdin_data, name_for_stdin or "stdin", dd)
        return done()
    small = [f for f in files if os.path.getsize(f) < 16 * MB]
    large = [f for f in files if os.path.getsize(f) >= 16 * MB]
    for group, is_large in ((small, False), (large, True)):
        if not group:
            continue
        if block_kb == 0 or (block_kb < 0 and not is_large):
            # stream mode, the whole file
            bufs = [open(f, "rb").read() for f in group]
            for d in ctx.digest_buffers(bufs, group, 0):
                if d is not None:
                    digs.append(d)
        else:
            dd = (16 if block_kb < 0 else block_kb) * KB
            for f in group:
                digs += seg_digests(np.fromfile(f, dtype=np.uint8), f, dd)
    return done()


INDEX_BYTES = 64 << 20   # bloom_filter(64*MB, 5, 0, 0.01), sdhash_threads.cc:414,460
INDEX_GROUP = 640 * MB   # a group ends once its files exceed this (sdhash_threads.cc:409,455)


def _index_files(ctx, files, output: str, seg: int):
    """hash_index_stringlist (sdhash-src/sdhash_threads.cc:376-470) for one of
    the small / large file lists: files in groups of just over 640 MB, each
    hashed with a fresh 64 MiB index (files below 16 MiB in stream mode, the
    others in 16 KiB block mode with 128 MiB segments), written as
    <output><k>.sdbf and its index <output><k>.sdbf.idx, k counting from 0.
    The reference's file-list array is reproduced as it behaves: after a
    group its count restarts at 1, so each later group also hashes the file
    left in slot 0."""
    import numpy as np
    for count, gi in enumerate(_index_groups([os.path.getsize(f) for f in files])):
        group = [files[i] for i in gi]
        bits = np.zeros(INDEX_BYTES, dtype=np.uint8)
        if os.path.getsize(group[0]) < 16 * MB and all(os.path.getsize(x) < 16 * MB for x in group):
            bufs = [open(x, "rb").read() for x in group]
            digs, ec = ctx.digest_index(bufs, group, 0, bits)
        else:
            names, bufs, got = [], [], []
            for x in group:
                data = np.fromfile(x, dtype=np.uint8)
                for nm, o, n in _segments(x, len(data), seg):
                    b = np.zeros(n, dtype=np.uint8)
                    part = data[o:o + n]
                    b[:len(part)] = part
                    names.append(nm)
                    bufs.append(b)
                    got.append(len(part))
            digs, ec = ctx.digest_index(bufs, names, 16 * KB, bits)
            for d, n in zip(digs, got):
                if d is not None:
                    d.orig_size = n
            digs = [d for d, n in zip(digs, got) if d is not None and n >= 512]
        name = f"{output}{count}.sdbf"
        with open(name, "w") as fh:
            fh.write("".join(d.to_string() for d in digs if d is not None))
        ctx.write_index(name + ".idx", bits, ec, name)
    return 0


def _index_groups(sizes):
    """The groups hash_index_stringlist hashes (sdhash-src/
    sdhash_threads.cc:402-411,446-455), as lists of positions in the file
    list: a group closes once the running size passes 640 MB or at the last
    file.  Its file array keeps the entry in slot 0 after a group (the
    count restarts at 1), and the running size is a C int, which wraps
    modulo 2^32 (a file of 2 GiB or more makes it negative)."""
    groups, slots, filect, total = [], [], 0, 0
    for i, n in enumerate(sizes):
        if filect < len(slots):
            slots[filect] = i
        else:
            slots.append(i)
        total = ((total + n + (1 << 31)) & 0xFFFFFFFF) - (1 << 31)
        if total > INDEX_GROUP or i == len(sizes) - 1:
            groups.append(slots[:filect + 1])
            total, filect = 0, 0
        filect += 1
    return groups


def _load_indexes(ctx, idx_dir: str):
    """The --index-search list (sdhash-src/sdhash.cc:241-266): every regular
    '*.idx' file of the directory in directory order, each with the name of
    the SDBF set stored beside it (idx_dir + "/" + the file name without
    '.idx'; sdbf_set(fname) names a set after the path only when the file
    exists, and throws on a malformed one)."""
    import sdhash_gb300 as g
    out = []
    if not os.path.isdir(idx_dir):
        return out
    with os.scandir(idx_dir) as it:
        for e in it:
            stem, ext = os.path.splitext(e.name)
            if not (e.is_file() and ext == ".idx" and stem):
                continue
            index = ctx.load_index(os.path.join(idx_dir, e.name))
            set_path = idx_dir + "/" + stem
            name = ""
            if os.path.isfile(set_path):
                ctx.load_file(set_path).close()
                name = set_path
            out.append((index, name))
    return out


def _index_results(items, hits, set_names) -> str:
    """sdbf_set::index_results (sdbf/sdbf_set.cc:161-167): per digest in set
    order, per block, per index with more than 4 hits (_FP_THRESHOLD,
    sdbf_defines.h:36): "<digest> [<block>] |<index set>|<hits>" (print_indexes,
    sdbf/sdbf_core.cc:458-472)."""
    lines = []
    for it, h in zip(items, hits):
        for b in range(h.shape[0]):
            for i, nm in enumerate(set_names):
                if h[b, i] > 4:
                    lines.append(f"{it.name()} [{b}] |{nm}|{int(h[b, i])}\n")
    return "".join(lines)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="sdhash", add_help=True)
    ap.add_argument("-r", "--deep", action="store_true", help="generate SDBFs from directories and files")
    ap.add_argument("-f", "--target-list", action="store_true", help="generate SDBFs from list(s) of filenames")
    ap.add_argument("-c", "--compare", action="store_true", help="compare SDBFs in file, or two SDBF files")
    ap.add_argument("-g", "--gen-compare", action="store_true", help="compare all pairs in source data")
    ap.add_argument("-t", "--threshold", type=int, default=1, help="only show results >=threshold")
    ap.add_argument("-b", "--block-size", type=int, default=-1, help="hashes input files in nKB blocks")
    ap.add_argument("-p", "--threads", type=int, default=0, help="accepted; the GPU does not use it")
    ap.add_argument("-s", "--sample-size", type=int, default=0, help="not offered (must be 0)")
    ap.add_argument("-z", "--segment-size", type=int, default=128, help="file segment size in MB")
    ap.add_argument("-o", "--output", default=None, help="send output to files")
    ap.add_argument("--separator", default="pipe", choices=["pipe", "csv", "tab", "tabs"])
    ap.add_argument("--hash-name", default=None, help="set name of hash on stdin")
    ap.add_argument("--fast", action="store_true", help="shrink sdbf filters for speedup")
    ap.add_argument("--validate", action="store_true", help="parse SDBF file to check if it is valid")
    ap.add_argument("--index", action="store_true", help="generate indexes while hashing (needs -o)")
    ap.add_argument("--index-search", default=None, metavar="DIR",
                    help="search directory of reference indexes (block mode)")
    ap.add_argument("--version", action="store_true")
    ap.add_argument("files", nargs="*")
    a = ap.parse_args(argv)
    if a.version:
        print(VERSION)
        return 0
    if a.sample_size:
        print("sdhash: filter sampling (-s) is not offered by this engine", file=sys.stderr)
        return -1
    import sdhash_gb300 as g
    sep = {"pipe": "|", "csv": ",", "tab": "\t", "tabs": "\t"}[a.separator]
    block_kb = a.block_size
    if block_kb > 16:
        block_kb = 16          # sdhash.cc:215-219
    if block_kb < -1:
        block_kb = -1
    out = sys.stdout

    def emit(text: str, suffix: str):
        if a.output:
            with open(a.output + suffix, "w") as f:
                f.write(text)
        else:
            out.write(text)

    if a.compare:
        if len(a.files) not in (1, 2):
            print("sdhash: ERROR: Comparison requires 1 or 2 arguments.", file=sys.stderr)
            return -1
        sets = []
        for p in a.files:
            try:
                s = g.sdbf_set(p)
            except Exception:
                print(f"sdhash: ERROR: Could not load SDBF file {p}. Exiting", file=sys.stderr)
                return -1
            s.set_separator(sep)
            sets.append(s)
        if len(sets) == 1:
            emit(sets[0].compare_all_quiet(a.threshold, 0, a.fast), ".compare")
        else:
            emit(sets[0].compare_to_quiet(sets[1], a.threshold, 0, 0, a.fast), ".compare")
        return 0
    if a.validate:
        for p in a.files:
            if not os.path.isfile(p):
                print(f"sdhash: ERROR file {p} not readable or not found.")
                continue
            try:
                s = g.sdbf_set(p)
            except Exception:
                print(f"sdhash: ERROR: Could not load file of SDBFs, {p} is empty or invalid.", file=sys.stderr)
                continue
            print(f"sdhash: file {p} SDBFs valid, contains {s.size()} hashes.")
            print(f"contains {sum(x.filter_count() for x in s.items)} bloom filters.")
            print(f"{s.input_size()} total data size. ")
        return 0
    if a.index and not a.output:
        print("sdhash:  ERROR: indexing requires output base filename ", file=sys.stderr)
        return -1
    ctx = g.default_context()
    seg = a.segment_size * MB
    if a.index:
        inputs = a.files
        if a.target_list:
            inputs = []
            for lst in a.files:
                with open(lst) as f:
                    inputs += [ln.rstrip("\n") for ln in f if ln.strip()]
        files = _collect(inputs, a.deep)
        # sdhash.cc:556-561: the small list, then the large one, each from k = 0
        _index_files(ctx, [f for f in files if os.path.getsize(f) < 16 * MB], a.output, seg)
        _index_files(ctx, [f for f in files if os.path.getsize(f) >= 16 * MB], a.output, 128 * MB)
        return 0
    indexes = None
    if a.index_search is not None:
        if block_kb == 0:
            print("ERROR: Index searching only supported in block mode", file=sys.stderr)
            return 0
        if block_kb == -1:
            block_kb = 16      # sdhash.cc:245-249
        loaded = _load_indexes(ctx, a.index_search)
        indexes = [x for x, _ in loaded]
        set_names = [nm for _, nm in loaded]
    hits = None
    if a.files == ["-"]:
        data = sys.stdin.buffer.read()
        items = _hash(ctx, [], block_kb, seg, a.hash_name, data, indexes=indexes)
        if indexes is not None:
            items, hits = items
    else:
        inputs = a.files
        if a.target_list:
            inputs = []
            for lst in a.files:
                with open(lst) as f:
                    inputs += [ln.rstrip("\n") for ln in f if ln.strip()]
        files = _collect(inputs, a.deep)
        if not files:
            print(VERSION + "\n\nUsage: sdhash <options> <files>")
            return 0
        items = _hash(ctx, files, block_kb, seg, indexes=indexes)
        if indexes is not None:
            items, hits = items
    s = g.sdbf_set()
    s.set_separator(sep)
    for it in items:
        s.add(it)
    if a.gen_compare:
        emit(s.compare_all_quiet(a.threshold, 0, a.fast), ".compare")
    elif indexes is not None:
        # sdhash.cc:638-652: the hashes are not written; the results go to
        # <output>.idx-result, or to stderr
        text = _index_results(items, hits, set_names)
        if a.output:
            with open(a.output + ".idx-result", "w") as f:
                f.write(text)
        else:
            sys.stderr.write(text)
    else:
        emit(s.to_string(), ".sdbf")
    return 0


if __name__ == "__main__":
    sys.exit(main())
