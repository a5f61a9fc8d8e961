"""A C++ caller of the reference's object API, relinked against the GB300
library, produces the reference's outputs (checked via the oracle)."""
import os
import subprocess

import pytest

from sdhash_gb300 import synth

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_compat_demo(tmp_path, native, oracle):
    exe = tmp_path / "demo"
    src = os.path.join(REPO, "tests", "cpp", "sdbf_api_demo.cc")
    libdir = os.path.join(REPO, "sdhash_gb300")
    subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(libdir, "compat"), src, "-o", str(exe),
                    "-L", libdir, "-lsdbf_gb300", f"-Wl,-rpath,{libdir}"], check=True)
    a = synth.mixture_bytes(41, 0, 900000)
    b = a.copy()
    b[300000:300050] = 1
    fa, fb = tmp_path / "a.bin", tmp_path / "b.bin"
    fa.write_bytes(a.tobytes())
    fb.write_bytes(b.tobytes())
    files = [synth.random_bytes(42, i, 200000 + 1000 * i) for i in range(5)]
    files.append(files[0][:150000].copy())
    lines = [oracle.digest(f"s{i}", f.tobytes(), 0).to_string() for i, f in enumerate(files)]
    setf = tmp_path / "set.sdbf"
    setf.write_text("".join(lines))
    out = subprocess.run([str(exe), str(fa), str(fb), str(setf)], capture_output=True, text=True, check=True).stdout
    oa = oracle.digest(str(fa), a.tobytes(), 0)
    ob = oracle.digest(str(fb), b.tobytes(), 16384)
    expect = oa.to_string() + ob.to_string()
    s = oracle.score(oa, ob)
    expect += f"a vs b {s}\na2 vs b2 {s}\nistream equal 1\n"
    expect += oracle.compare_all([oracle.parse(x) for x in lines], 1)
    folded = [oracle.fast(oracle.parse(x)) for x in lines]
    expect += oracle.compare_all(folded, 1)
    expect += folded[0].to_string()
    expect += "tiny throws -3\n"
    assert out == expect
