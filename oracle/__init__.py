"""Oracle loaders (test infrastructure, never the product).

* ``Oracle``    -- ctypes wrapper over liboracle_sdbf.so, the plain-C
  restatement of sdhash's hot paths (oracle/sdbf_oracle.c).
* ``Reference`` -- ctypes wrapper over oracle/_ref/libsdbf_ref.so, the
  unmodified reference library compiled from its own sources by
  oracle/Makefile.ref (only where the reference sources exist).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg
import this package.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "liboracle_sdbf.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SO = os.path.join(REF_DIR, "libsdbf_ref.so")
REFERENCE_SRC = os.environ.get("SDHASH_REFERENCE_SRC", "")


def build_oracle(quiet: bool = True) -> str:
    """Compile the C restatement (gcc, a second or two)."""
    out = subprocess.run(["make", "-s", "-C", HERE], capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + (out.stdout or "") + (out.stderr or ""))
    return ORACLE_SO


def build_reference(quiet: bool = True, src: str | None = None) -> str | None:
    """Compile the reference from its sources into oracle/_ref (only where the
    reference tree exists; it does not travel to other machines).  The tree
    is `src`, else $SDHASH_REFERENCE_SRC; neither set: nothing is built."""
    src = src or REFERENCE_SRC
    if not src or not os.path.isdir(os.path.join(src, "sdbf")):
        return None
    repo = os.path.dirname(HERE)
    out = subprocess.run(["make", "-s", "-j8", "-f", "oracle/Makefile.ref", f"REF={src}"],
                         cwd=repo, capture_output=quiet, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + (out.stdout or "") + (out.stderr or ""))
    return REF_SO


class _Digest(C.Structure):
    _fields_ = [("name", C.c_char_p), ("orig_size", C.c_uint64), ("bf_count", C.c_uint32),
                ("last_count", C.c_uint32), ("max_elem", C.c_uint32), ("dd_block_size", C.c_uint32),
                ("filters", C.POINTER(C.c_uint8)), ("elem_counts", C.POINTER(C.c_uint16)),
                ("hamming", C.POINTER(C.c_uint16)), ("fastmode", C.c_int32)]


class OracleDigest:
    """An oracle-owned digest; freed with the object."""

    def __init__(self, lib, st: _Digest):
        self._lib = lib
        self.st = st

    def __del__(self):
        try:
            self._lib.orc_digest_free(C.byref(self.st))
        except Exception:
            pass

    @property
    def bf_count(self) -> int:
        return self.st.bf_count

    @property
    def last_count(self) -> int:
        return self.st.last_count

    def filters(self) -> bytes:
        return C.string_at(self.st.filters, 256 * self.st.bf_count)

    def elem_counts(self) -> list[int]:
        if not self.st.elem_counts:
            return []
        return [self.st.elem_counts[i] for i in range(self.st.bf_count)]

    def to_string(self) -> str:
        p = self._lib.orc_to_string(C.byref(self.st))
        s = C.string_at(p).decode()
        _libc.free(p)
        return s


_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]


class Oracle:
    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build_oracle()
        L = C.CDLL(path)
        self.L = L
        u8p, u16p, i32p = C.POINTER(C.c_uint8), C.POINTER(C.c_uint16), C.POINTER(C.c_int32)
        L.orc_sha1.argtypes = [C.c_char_p, C.c_uint64, C.c_char_p]
        L.orc_entropy_table.argtypes = [C.POINTER(C.c_uint64)]
        L.orc_ranks.argtypes = [C.c_char_p, C.c_uint64, u16p]
        L.orc_scores.argtypes = [u16p, C.c_uint64, u16p, i32p]
        L.orc_digest_stream.argtypes = [C.c_char_p, C.c_char_p, C.c_uint64, C.POINTER(_Digest)]
        L.orc_digest_block.argtypes = [C.c_char_p, C.c_char_p, C.c_uint64, C.c_uint32, C.POINTER(_Digest)]
        L.orc_digest_free.argtypes = [C.POINTER(_Digest)]
        L.orc_to_string.argtypes = [C.POINTER(_Digest)]
        L.orc_to_string.restype = C.c_void_p
        L.orc_from_string.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(_Digest)]
        L.orc_score.argtypes = [C.POINTER(_Digest), C.POINTER(_Digest)]
        L.orc_score.restype = C.c_int32
        L.orc_match_cut.argtypes = [C.c_char_p, C.c_char_p, C.c_uint32]
        L.orc_match_cut.restype = C.c_uint32
        L.orc_max_score.argtypes = [C.POINTER(_Digest), C.c_uint32, C.POINTER(_Digest)]
        L.orc_max_score.restype = C.c_double
        L.orc_compare_all.argtypes = [C.POINTER(_Digest), C.c_uint32, C.c_int32, C.c_char]
        L.orc_compare_all.restype = C.c_void_p
        L.orc_compare_to.argtypes = [C.POINTER(_Digest), C.c_uint32, C.POINTER(_Digest), C.c_uint32,
                                     C.c_int32, C.c_char]
        L.orc_compare_to.restype = C.c_void_p
        L.orc_score_all_matrix.argtypes = [C.POINTER(_Digest), C.c_uint32, i32p, C.c_int]
        L.orc_score_cross_matrix.argtypes = [C.POINTER(_Digest), C.c_uint32, C.POINTER(_Digest), C.c_uint32,
                                             i32p, C.c_int]
        L.orc_fast.argtypes = [C.POINTER(_Digest)]
        L.orc_fast.restype = None
        L.orc_score_pairs.argtypes = [C.POINTER(_Digest), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                      C.c_uint64, i32p, C.c_int]
        L.orc_digest_many.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.POINTER(C.c_char_p),
                                      C.c_uint32, C.c_uint32, C.c_int, C.POINTER(_Digest), C.POINTER(C.c_int)]
        L.orc_index_search_many.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.c_uint32, C.c_uint32,
                                            C.POINTER(C.c_void_p), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                            C.c_uint32, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_int)]
        L.orc_index_build_stream.argtypes = [C.POINTER(C.c_void_p), C.POINTER(C.c_uint64), C.POINTER(C.c_char_p),
                                             C.c_uint32, C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64),
                                             C.POINTER(_Digest), C.POINTER(C.c_int)]
        L.orc_b64_encode.argtypes = [C.c_char_p, C.c_size_t, C.c_char_p]
        L.orc_b64_encode.restype = C.c_size_t

    # -- primitives -------------------------------------------------------
    def sha1(self, data: bytes) -> bytes:
        out = C.create_string_buffer(20)
        self.L.orc_sha1(data, len(data), out)
        return out.raw

    def entropy_table(self) -> list[int]:
        t = (C.c_uint64 * 65)()
        self.L.orc_entropy_table(t)
        return list(t)

    def ranks(self, data: bytes):
        import numpy as np
        r = np.zeros(len(data), dtype=np.uint16)
        self.L.orc_ranks(data, len(data), r.ctypes.data_as(C.POINTER(C.c_uint16)))
        return r

    def scores(self, ranks):
        import numpy as np
        ranks = np.ascontiguousarray(ranks, dtype=np.uint16)
        s = np.zeros(len(ranks), dtype=np.uint16)
        h = np.zeros(66, dtype=np.int32)
        self.L.orc_scores(ranks.ctypes.data_as(C.POINTER(C.c_uint16)), len(ranks),
                          s.ctypes.data_as(C.POINTER(C.c_uint16)), h.ctypes.data_as(C.POINTER(C.c_int32)))
        return s, h

    # -- digests ----------------------------------------------------------
    def digest(self, name: str, data: bytes, dd_block_size: int = 0) -> OracleDigest | None:
        st = _Digest()
        if dd_block_size:
            rc = self.L.orc_digest_block(name.encode(), data, len(data), dd_block_size, C.byref(st))
        else:
            rc = self.L.orc_digest_stream(name.encode(), data, len(data), C.byref(st))
        if rc != 0:
            return None
        return OracleDigest(self.L, st)

    def parse(self, line: str) -> OracleDigest:
        st = _Digest()
        b = line.encode()
        rc = self.L.orc_from_string(b, len(b), C.byref(st))
        if rc != 0:
            raise ValueError(f"oracle parse failed ({rc})")
        return OracleDigest(self.L, st)

    def fast(self, d: OracleDigest) -> OracleDigest:
        """sdbf::fast: fold the digest's filters to 64 bytes in place."""
        self.L.orc_fast(C.byref(d.st))
        return d

    def score(self, a: OracleDigest, b: OracleDigest) -> int:
        return self.L.orc_score(C.byref(a.st), C.byref(b.st))

    @staticmethod
    def _array(ds):
        arr = (_Digest * len(ds))()
        for i, d in enumerate(ds):
            arr[i] = d.st
        return arr

    def compare_all(self, ds, threshold: int = 1, sep: str = "|") -> str:
        arr = self._array(ds)
        p = self.L.orc_compare_all(arr, len(ds), threshold, sep.encode())
        s = C.string_at(p).decode()
        _libc.free(p)
        return s

    def compare_to(self, qs, ts, threshold: int = 1, sep: str = "|") -> str:
        qa, ta = self._array(qs), self._array(ts)
        p = self.L.orc_compare_to(qa, len(qs), ta, len(ts), threshold, sep.encode())
        s = C.string_at(p).decode()
        _libc.free(p)
        return s

    def score_all_matrix(self, ds, nthreads: int = 0):
        import numpy as np
        n = len(ds)
        out = np.full((n, n), -2, dtype=np.int32)
        self.L.orc_score_all_matrix(self._array(ds), n, out.ctypes.data_as(C.POINTER(C.c_int32)), nthreads)
        return out

    def score_cross_matrix(self, qs, ts, nthreads: int = 0):
        import numpy as np
        out = np.zeros((len(qs), len(ts)), dtype=np.int32)
        self.L.orc_score_cross_matrix(self._array(qs), len(qs), self._array(ts), len(ts),
                                      out.ctypes.data_as(C.POINTER(C.c_int32)), nthreads)
        return out

    def score_pairs(self, ds, pi, pj, nthreads: int = 0):
        """Scores of pairs (ds[pi[k]], ds[pj[k]]) as sdbf_score(ds[pi], ds[pj]), multithreaded."""
        import numpy as np
        pi = np.ascontiguousarray(pi, dtype=np.uint32)
        pj = np.ascontiguousarray(pj, dtype=np.uint32)
        out = np.zeros(max(1, len(pi)), dtype=np.int32)
        self.L.orc_score_pairs(self._array(ds), pi.ctypes.data_as(C.POINTER(C.c_uint32)),
                               pj.ctypes.data_as(C.POINTER(C.c_uint32)), len(pi),
                               out.ctypes.data_as(C.POINTER(C.c_int32)), nthreads)
        return out[: len(pi)]

    def index_search(self, bufs, dd_block_size: int, index_bits, nthreads: int = 0, hash_count: int = 5):
        """Index search of block-mode hashing (gen_block_hash with an index
        list): per input, a (bf_count, nidx) uint8 array of sampled features
        found in each index (None for inputs below 512 bytes).  index_bits:
        uint8 arrays, power-of-two sizes (mask = 8 * size - 1)."""
        import numpy as np
        n, nidx = len(bufs), len(index_bits)
        ptrs = (C.c_void_p * max(1, n))()
        lens = (C.c_uint64 * max(1, n))()
        keep = []
        for i, b in enumerate(bufs):
            arr = np.ascontiguousarray(np.frombuffer(bytes(b), dtype=np.uint8) if isinstance(b, (bytes, bytearray))
                                       else b, dtype=np.uint8)
            keep.append(arr)
            ptrs[i] = arr.ctypes.data
            lens[i] = arr.size
        bits = (C.c_void_p * max(1, nidx))(*[np.ascontiguousarray(x, dtype=np.uint8).ctypes.data for x in index_bits])
        masks = (C.c_uint32 * max(1, nidx))(*[min(0xFFFFFFFF, 8 * len(x) - 1) for x in index_bits])
        hcs = (C.c_uint32 * max(1, nidx))(*([hash_count] * nidx))
        rows = []
        for i in range(n):
            nb = int(lens[i]) // dd_block_size + (1 if int(lens[i]) % dd_block_size >= 512 else 0)
            rows.append(np.zeros((max(1, nb), max(1, nidx)), dtype=np.uint8))
        hp = (C.c_void_p * max(1, n))(*[r.ctypes.data for r in rows])
        status = (C.c_int * max(1, n))()
        self.L.orc_index_search_many(ptrs, lens, n, dd_block_size, bits, masks, hcs, nidx, nthreads, hp, status)
        out = []
        for i in range(n):
            if status[i] != 0:
                out.append(None)
            else:
                nb = int(lens[i]) // dd_block_size + (1 if int(lens[i]) % dd_block_size >= 512 else 0)
                out.append(rows[i][:nb, :nidx])
        return out

    @staticmethod
    def _buffers(bufs):
        n = len(bufs)
        ptrs = (C.c_void_p * n)()
        lens = (C.c_uint64 * n)()
        keep = []
        for i, b in enumerate(bufs):
            if isinstance(b, (bytes, bytearray)):
                cb = C.c_char_p(bytes(b))
                keep.append(cb)
                ptrs[i] = C.cast(cb, C.c_void_p)
            else:  # numpy array
                ptrs[i] = b.ctypes.data
            lens[i] = len(b)
        return ptrs, lens, keep

    def index_build_stream(self, bufs, names, index_bits, elem_count: int = 0):
        """Stream-mode digests of one sdhash --index group, in order, with
        the shared index index_bits (uint8 numpy array, power-of-two size,
        updated in place).  Returns (digests, elem_count after the group)."""
        import numpy as np
        assert isinstance(index_bits, np.ndarray) and index_bits.dtype == np.uint8 and index_bits.flags.c_contiguous
        n = len(bufs)
        ptrs, lens, keep = self._buffers(bufs)
        cnames = (C.c_char_p * n)(*[x.encode() for x in names])
        outs = (_Digest * n)()
        status = (C.c_int * n)()
        ec = C.c_uint64(elem_count)
        self.L.orc_index_build_stream(ptrs, lens, cnames, n, index_bits.ctypes.data, index_bits.size * 8 - 1,
                                      C.byref(ec), outs, status)
        del keep
        return [OracleDigest(self.L, outs[i]) if status[i] == 0 else None for i in range(n)], int(ec.value)

    def digest_many(self, bufs, dd_block_size: int = 0, nthreads: int = 0, names=None):
        """Digest a list of bytes-like buffers on nthreads threads (file-parallel)."""
        n = len(bufs)
        cnames = None
        if names is not None:
            cnames = (C.c_char_p * n)(*[x.encode() for x in names])
        ptrs, lens, keep = self._buffers(bufs)
        outs = (_Digest * n)()
        status = (C.c_int * n)()
        self.L.orc_digest_many(ptrs, lens, cnames, n, dd_block_size, nthreads, outs, status)
        res = []
        for i in range(n):
            res.append(OracleDigest(self.L, outs[i]) if status[i] == 0 else None)
        return res


class Reference:
    """The unmodified reference library driven through its own C++ API."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.L = L
        L.ref_digest_buffer.argtypes = [C.c_char_p, C.c_char_p, C.c_ulonglong, C.c_uint, C.POINTER(C.c_int)]
        L.ref_digest_buffer.restype = C.c_void_p
        L.ref_compare_text.argtypes = [C.c_char_p, C.c_char_p, C.c_uint]
        L.ref_compare_text.restype = C.c_int
        L.ref_compare_all_file.argtypes = [C.c_char_p, C.c_int]
        L.ref_compare_all_file.restype = C.c_void_p
        L.ref_compare_to_files.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.c_uint]
        L.ref_compare_to_files.restype = C.c_void_p
        L.ref_compare_all_file_fast.argtypes = [C.c_char_p, C.c_int]
        L.ref_compare_all_file_fast.restype = C.c_void_p
        L.ref_compare_to_files_fast.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
        L.ref_compare_to_files_fast.restype = C.c_void_p
        L.ref_free.argtypes = [C.c_void_p]

    def _take(self, p) -> str:
        s = C.string_at(p).decode()
        self.L.ref_free(p)
        return s

    def digest(self, name: str, data: bytes, dd_block_size: int = 0) -> str | None:
        err = C.c_int(0)
        p = self.L.ref_digest_buffer(name.encode(), data, len(data), dd_block_size, C.byref(err))
        if not p:
            return None
        return self._take(p)

    def compare_text(self, a: str, b: str) -> int:
        return self.L.ref_compare_text(a.encode(), b.encode(), 0)

    def compare_all_file(self, path: str, threshold: int = 1, fast: bool = False) -> str:
        if fast:
            return self._take(self.L.ref_compare_all_file_fast(path.encode(), threshold))
        return self._take(self.L.ref_compare_all_file(path.encode(), threshold))

    def compare_to_files(self, q: str, t: str, threshold: int = 1, fast: bool = False) -> str:
        if fast:
            return self._take(self.L.ref_compare_to_files_fast(q.encode(), t.encode(), threshold))
        return self._take(self.L.ref_compare_to_files(q.encode(), t.encode(), threshold, 0))
