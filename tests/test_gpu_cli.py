"""The sdhash-compatible command line (sdhash_gb300/cli.py) against the
oracle: digests, -g, -c with one and two SDBF files, block mode with
segmentation and the zero-filled last segment, the 16 MiB auto block mode."""
import numpy as np
import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu


def _odig(oracle, name, data, dd, orig=None):
    d = oracle.digest(name, data.tobytes(), dd)
    if orig is not None:
        d.st.orig_size = orig
    return d


def test_cli_hash_compare(tmp_path, capsys, monkeypatch, oracle):
    from sdhash_gb300 import cli
    monkeypatch.chdir(tmp_path)
    files = {"a.bin": synth.mixture_bytes(61, 0, 300_000), "b.bin": synth.mixture_bytes(61, 1, 1_500_000)}
    files["c.bin"] = synth.partner(61, 2, files["b.bin"])
    files["big.bin"] = synth.mixture_bytes(61, 3, 17 << 20)     # >= 16 MiB: block mode by default
    files["seg.bin"] = synth.mixture_bytes(61, 4, (2 << 20) + 512)
    for n, d in files.items():
        (tmp_path / n).write_bytes(d.tobytes())
    small = ["a.bin", "b.bin", "c.bin"]
    # default mode: small files stream, the large one 16 KiB blocks, small first
    assert cli.main(small + ["big.bin"]) == 0
    got = capsys.readouterr().out
    want = [_odig(oracle, n, files[n], 0) for n in small] + [_odig(oracle, "big.bin", files["big.bin"], 16384)]
    assert got == "".join(d.to_string() for d in want)
    # -g: all pairs of the hashed set
    assert cli.main(["-g", "-t", "1"] + small) == 0
    assert capsys.readouterr().out == oracle.compare_all([_odig(oracle, n, files[n], 0) for n in small], 1)
    # -b 16 -z 1: 1 MiB segments; the last one reads 1 MiB + 1024 bytes past 1 MiB
    # (1 MiB + 512 available, zero-filled) as the reference's istream does
    assert cli.main(["-b", "16", "-z", "1", "seg.bin"]) == 0
    got = capsys.readouterr().out
    data = files["seg.bin"]
    last = np.zeros((1 << 20) + 1024, dtype=np.uint8)
    last[:(1 << 20) + 512] = data[1 << 20:]
    want = [_odig(oracle, "seg.bin.0000M", data[:1 << 20], 16384),
            _odig(oracle, "seg.bin.0001M", last, 16384, orig=(1 << 20) + 512)]
    assert got == "".join(d.to_string() for d in want)
    # -c with one file (all pairs) and two files (query x target), csv separator
    (tmp_path / "set.sdbf").write_text("".join(_odig(oracle, n, files[n], 0).to_string() for n in small))
    (tmp_path / "q.sdbf").write_text(_odig(oracle, "c.bin", files["c.bin"], 0).to_string())
    assert cli.main(["-c", "set.sdbf", "-t", "-1"]) == 0
    ods = [oracle.parse(t) for t in (tmp_path / "set.sdbf").read_text().splitlines(True)]
    assert capsys.readouterr().out == oracle.compare_all(ods, -1)
    assert cli.main(["-c", "--separator", "csv", "q.sdbf", "set.sdbf"]) == 0
    oq = [oracle.parse((tmp_path / "q.sdbf").read_text())]
    assert capsys.readouterr().out == oracle.compare_to(oq, ods, 1, ",")
    # -o: results to <base>.sdbf
    assert cli.main(["-o", "out", "a.bin"]) == 0
    assert (tmp_path / "out.sdbf").read_text() == _odig(oracle, "a.bin", files["a.bin"], 0).to_string()
