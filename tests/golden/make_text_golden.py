"""Generate tests/golden/text_load.json from the REFERENCE sdhash.

Each case is a small SDBF text file (digests made by the reference from
seeded synthetic content, then edited where the case says so) and what the
reference's loader does with it: sdbf_set(const char* fname)
(sdbf/sdbf_set.cc:51-74) over sdbf(const std::string&)
(sdbf/sdbf_class.cc:144-215).  The record is either the loaded digests
re-encoded by to_string (one line each) or the value the constructor throws
plus the index of the first line that throws.

Only inputs on which the reference's behaviour is defined are used: no
header field that fails boost::lexical_cast (it throws a non-int), no
block record field shorter than 344 characters (the reference decodes 344
characters from it regardless).

Needs the reference source tree (only in the build container):
    SDHASH_REFERENCE_SRC=<tree> python tests/golden/make_text_golden.py
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import Reference, build_reference  # noqa: E402
from sdhash_gb300 import synth  # noqa: E402


def digests(R):
    """Stream digests with 1..7 filters (every case of the 3-filter groups
    of the base64 payload) and block digests with 1..5 filters."""
    out, have, size, i = [], set(), 3000, 0
    while len(have) < 7 and size < (4 << 20):
        t = R.digest(f"s{i}.bin", synth.mixture_bytes(71, i, size).tobytes(), 0)
        bf = int(t.split(":")[10]) if t else 0
        if 1 <= bf <= 7 and bf not in have:
            have.add(bf)
            out.append(t)
        size, i = int(size * 1.15), i + 1
    for i, size in enumerate([2000, 16384, 40000, 70000]):
        t = R.digest(f"d{i}.bin", synth.mixture_bytes(72, i, size).tobytes(), 16384)
        if t:
            out.append(t)
    return out


def load(R, text: str):
    import ctypes as C
    fd, path = tempfile.mkstemp(suffix=".sdbf")
    with os.fdopen(fd, "wb") as f:
        f.write(text.encode("latin-1"))
    try:
        R.L.ref_load_file.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]
        R.L.ref_load_file.restype = C.c_void_p
        err, bad = C.c_int(0), C.c_int(-1)
        p = R.L.ref_load_file(path.encode(), C.byref(err), C.byref(bad))
        if p:
            return {"lines": R._take(p).splitlines(True)}
        return {"err": err.value, "line": bad.value}
    finally:
        os.unlink(path)


def payload_pos(line: str) -> int:
    """Offset of the first payload character of a stream line (after 12 ':')."""
    k = -1
    for _ in range(12):
        k = line.index(":", k + 1)
    return k + 1


def main():
    build_reference()
    R = Reference()
    ds = digests(R)
    stream = [d for d in ds if d.startswith("sdbf:")]
    block = [d for d in ds if d.startswith("sdbf-dd:")]
    cases = []

    def add(name, text):
        cases.append({"name": name, "text": text, "expect": load(R, text)})

    add("mixed set", "".join(ds))
    add("no final newline", "".join(ds)[:-1])
    add("empty line ends the file", "".join(ds[:3]) + "\n" + "".join(ds[3:]))
    add("crlf line ends", "".join(d[:-1] + "\r\n" for d in ds))
    # block records whose counts are not two lower-case hex digits
    b = block[-1]
    i = b.index(":16384:") + 6          # records start at the ':' after the block size
    head, recs = b[:i], b[i:]
    parts = recs.split(":")             # '', count, base64, count, base64, ...
    parts[1] = (parts[1].lstrip("0") or "0") if parts[1].startswith("0") else "0" + parts[1]
    add("element count not two digits", head + ":".join(parts))
    add("upper-case hex", head + _upper_hex(recs))
    # extra characters after the last record's 344 (the reference decodes 344)
    add("trailing characters in the last record", b[:-1] + "XYZ\n")
    # errors
    s = stream[3]
    p = payload_pos(s) + 100
    add("invalid character in a stream payload", "".join(stream[:2]) + s[:p] + "*" + s[p + 1:] + "".join(block))
    add("pad character inside a stream payload", s[:p] + "=" + s[p + 1:])
    q = i + 4 + 50
    add("invalid character in a block record", stream[0] + b[:q] + "!" + b[q + 1:])
    k = i + 4 + 342                     # padding of record 0: "xx==" -> "xxA="
    add("wrong padding in a block record", stream[0] + b[:k] + "A" + b[k + 1:])
    add("short line", "".join(stream[:2]) + "sdbf:03:1:x:1:sha1\n" + stream[2])
    add("bad magic", stream[0] + "SDBF" + stream[1][4:])
    cut = payload_pos(stream[5]) + 400
    add("truncated stream payload", stream[0] + stream[5][:cut] + "\n" + stream[1])
    out = {"generator": "tests/golden/make_text_golden.py",
           "reference": "sdbf_set(const char*) over sdbf(const std::string&), sdhash 4.0", "cases": cases}
    with open(os.path.join(HERE, "text_load.json"), "w") as f:
        json.dump(out, f, indent=0)
    for c in cases:
        e = c["expect"]
        print(c["name"], "->", ("%d digests" % len(e["lines"])) if "lines" in e else e)


def _upper_hex(records: str) -> str:
    """Upper-cases the element-count fields (not the base64) of block records."""
    parts = records.split(":")
    # parts[0] is empty (records start with ':'); then count, base64, count, ...
    for i in range(1, len(parts), 2):
        parts[i] = parts[i].upper()
    return ":".join(parts)


if __name__ == "__main__":
    main()
