"""sdhash_gb300 -- GB300-native SDBF digest generation and comparison.

Python binding over the C ABI of libsdbf_gb300.so (include/sdbf_gb300.h).
The compute runs in hand-written sm_103a CUDA kernels; this module only
marshals arguments.  There is no CPU fallback: if the native library is
missing, every entry point raises.

Two layers:
* ``Context`` -- batched calls (digest many inputs, upload digest sets,
  all-pairs / query-target comparison).
* ``sdbf`` / ``sdbf_set`` -- the reference's object API (sdbf/sdbf_class.h,
  sdbf/sdbf_set.h) with the same method names, argument meaning, result text
  and error behaviour (constructors raise ``SdbfError`` carrying the
  reference's throw codes -1 / -2 / -3).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsdbf_gb300.so")
SYNTH_PATH = os.path.join(HERE, "libsdbf_synth.so")

MIN_FILE_SIZE = 512
STREAM_MAX_ELEM = 160
BLOCK_MAX_ELEM = 192


class SdbfError(Exception):
    """Raised where the reference throws an int (its value is ``code``)."""

    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"sdbf error {code}: {msg}" if msg else f"sdbf error {code}")
        self.code = code


class EngineError(RuntimeError):
    """A C-ABI call returned a status code (``code``: SDBFG_ERR_*)."""

    def __init__(self, code: int, msg: str = ""):
        super().__init__(f"sdbf_gb300 error {code}: {msg}")
        self.code = code


class DigestResult(C.Structure):
    _fields_ = [("bf_count", C.c_uint32), ("last_count", C.c_uint32), ("status", C.c_int32),
                ("reserved", C.c_uint32), ("filter_offset", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_uint32), ("max_batch_queries", C.c_uint32), ("memory_budget", C.c_uint64),
                ("threshold", C.c_int32), ("pad", C.c_uint32), ("max_batch_pairs", C.c_uint64)]


class ServerResult(C.Structure):
    _fields_ = [("tag", C.c_uint64), ("status", C.c_int32), ("best_score", C.c_int32), ("best_target", C.c_uint32),
                ("matches", C.c_uint32), ("batch_queries", C.c_uint32), ("pad", C.c_uint32),
                ("submit_ns", C.c_uint64), ("start_ns", C.c_uint64), ("done_ns", C.c_uint64)]


class DigestDesc(C.Structure):
    _fields_ = [("name", C.c_char_p), ("filters", C.c_void_p), ("elem_counts", C.c_void_p),
                ("bf_count", C.c_uint32), ("last_count", C.c_uint32), ("max_elem", C.c_uint32),
                ("dd_block_size", C.c_uint32), ("orig_size", C.c_uint64)]


_lib = None
_lib_lock = threading.Lock()


def lib() -> C.CDLL:
    """Load libsdbf_gb300.so (raises if it was not built)."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} not built: run `python -m sdhash_gb300.build`")
        L = C.CDLL(LIB_PATH)
        vp, u64p, u32p, i32p = C.c_void_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint32), C.POINTER(C.c_int32)
        L.sdbfg_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.sdbfg_ctx_destroy.argtypes = [vp]
        L.sdbfg_last_error.argtypes = [vp]
        L.sdbfg_last_error.restype = C.c_char_p
        L.sdbfg_ctx_set_stream.argtypes = [vp, vp]
        L.sdbfg_ctx_synchronize.argtypes = [vp]
        L.sdbfg_ctx_launch_count.argtypes = [vp]
        L.sdbfg_ctx_launch_count.restype = C.c_uint64
        L.sdbfg_ctx_set_lead.argtypes = [vp, C.c_uint32]
        L.sdbfg_ctx_set_pipeline_depth.argtypes = [vp, C.c_int]
        L.sdbfg_ctx_pipeline_depth.argtypes = [vp]
        L.sdbfg_ctx_profile.argtypes = [vp, C.c_int]
        L.sdbfg_ctx_kernel_time.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_uint64)]
        L.sdbfg_ctx_relinked_tiles.argtypes = [vp]
        L.sdbfg_ctx_relinked_tiles.restype = C.c_uint64
        L.sdbfg_ctx_set_index_rounds.argtypes = [vp, C.c_uint32]
        L.sdbfg_ctx_index_rounds.argtypes = [vp]
        L.sdbfg_ctx_index_rounds.restype = C.c_uint32
        L.sdbfg_digest_capacity.argtypes = [u64p, C.c_uint32, C.c_uint32]
        L.sdbfg_digest_capacity.restype = C.c_uint64
        L.sdbfg_digest_batch.argtypes = [vp, vp, u64p, u64p, C.c_uint32, C.c_uint32, vp, C.c_uint64, vp,
                                         C.POINTER(DigestResult)]
        L.sdbfg_digest_batch_device.argtypes = [vp, vp, u64p, u64p, C.c_uint32, C.c_uint32, vp, C.c_uint64, vp,
                                                C.POINTER(DigestResult)]
        L.sdbfg_set_upload.argtypes = [vp, C.POINTER(DigestDesc), C.c_uint32, C.POINTER(vp)]
        L.sdbfg_set_free.argtypes = [vp]
        L.sdbfg_set_fast.argtypes = [vp, vp, C.c_uint32, C.c_uint32]
        L.sdbfg_set_size.argtypes = [vp]
        L.sdbfg_index_load_file.argtypes = [vp, C.c_char_p, C.POINTER(vp)]
        L.sdbfg_index_create.argtypes = [vp, vp, C.c_uint64, C.c_uint32, C.c_char_p, C.POINTER(vp)]
        L.sdbfg_index_free.argtypes = [vp]
        L.sdbfg_index_free.restype = None
        L.sdbfg_index_info.argtypes = [vp, u64p, u64p, C.POINTER(C.c_uint32), u64p, C.POINTER(C.c_char_p)]
        L.sdbfg_digest_batch_search.argtypes = [vp, vp, u64p, u64p, C.c_uint32, C.c_uint32, vp, C.c_uint64, vp, vp,
                                                C.POINTER(vp), C.c_uint32, vp]
        L.sdbfg_digest_batch_index.argtypes = [vp, vp, u64p, u64p, C.c_uint32, C.c_uint32, vp, C.c_uint64, vp, vp,
                                               vp, C.c_uint64, u64p]
        L.sdbfg_index_write_file.argtypes = [C.c_char_p, vp, C.c_uint64, C.c_uint64, C.c_uint32, C.c_char_p]
        L.sdbfg_lz4_encode.argtypes = [vp, C.c_uint64, vp, C.c_uint64]
        L.sdbfg_lz4_encode.restype = C.c_int64
        L.sdbfg_lz4_decode.argtypes = [vp, C.c_uint64, vp, C.c_uint64]
        L.sdbfg_lz4_decode.restype = C.c_int64
        L.sdbfg_set_load_text.argtypes = [vp, C.c_char_p, C.c_uint64, C.POINTER(vp), C.POINTER(C.c_int64),
                                          C.POINTER(C.c_int32)]
        L.sdbfg_set_digest_info.argtypes = [vp, C.c_uint32, C.POINTER(DigestDesc)]
        L.sdbfg_set_read_digest.argtypes = [vp, vp, C.c_uint32, vp, vp]
        L.sdbfg_set_size.restype = C.c_uint32
        L.sdbfg_score_pairs.argtypes = [vp, vp, vp, u32p, u32p, C.c_uint64, i32p]
        L.sdbfg_compare_all.argtypes = [vp, vp, i32p]
        L.sdbfg_compare_to.argtypes = [vp, vp, vp, i32p]
        L.sdbfg_compare_all_device.argtypes = [vp, vp, vp]
        L.sdbfg_compare_all_matches.argtypes = [vp, vp, C.c_int32, vp, C.c_uint64, u64p]
        L.sdbfg_compare_to_matches.argtypes = [vp, vp, vp, C.c_int32, vp, C.c_uint64, u64p]
        L.sdbfg_compare_to_device.argtypes = [vp, vp, vp, vp]
        L.sdbfg_compare_filter_pairs.argtypes = [vp, vp, vp]
        L.sdbfg_compare_filter_pairs.restype = C.c_uint64
        L.sdbfg_ctx_set_compare_tuning.argtypes = [vp, C.c_int, C.c_uint64, C.c_int]
        L.sdbfg_ctx_get_compare_tuning.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_uint64)]
        L.sdbfg_compare_autotune.argtypes = [vp, vp, vp, C.c_uint64, C.POINTER(C.c_int), C.POINTER(C.c_uint64),
                                             C.POINTER(C.c_double)]
        L.sdbfg_server_create.argtypes = [vp, vp, C.POINTER(ServerConfig), C.POINTER(vp)]
        L.sdbfg_server_submit.argtypes = [vp, C.POINTER(DigestDesc), C.c_uint64]
        L.sdbfg_server_poll.argtypes = [vp, C.POINTER(ServerResult), i32p, C.c_uint32, C.POINTER(C.c_uint32),
                                        C.c_int]
        L.sdbfg_server_stats.argtypes = [vp, u64p, u64p, u64p, u64p]
        L.sdbfg_server_destroy.argtypes = [vp]
        L.sdbfg_server_destroy.restype = None
        L.sdbfg_to_string.argtypes = [C.POINTER(DigestDesc), C.c_char_p, C.c_uint64]
        L.sdbfg_to_string.restype = C.c_int64
        L.sdbfg_parse.argtypes = [C.c_char_p, C.c_uint64, C.POINTER(DigestDesc), C.c_char_p, C.c_uint64, vp, vp]
        _lib = L
        return L


def _u64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint64)


def _ptr(a: np.ndarray, t=C.c_uint64):
    return a.ctypes.data_as(C.POINTER(t))


class Digest:
    """A similarity digest: the data fields of the reference's sdbf object."""

    __slots__ = ("name", "orig_size", "bf_count", "last_count", "max_elem", "dd_block_size", "filters",
                 "elem_counts", "fastmode")

    def __init__(self, name: str, orig_size: int, bf_count: int, last_count: int, max_elem: int,
                 dd_block_size: int, filters: np.ndarray, elem_counts: np.ndarray | None):
        self.name = name
        self.orig_size = orig_size
        self.bf_count = bf_count
        self.last_count = last_count
        self.max_elem = max_elem
        self.dd_block_size = dd_block_size
        self.filters = np.ascontiguousarray(filters, dtype=np.uint8).reshape(-1)
        self.elem_counts = None if elem_counts is None else np.ascontiguousarray(elem_counts, dtype=np.uint16)
        self.fastmode = False

    def fast(self) -> "Digest":
        """sdbf::fast (sdbf/sdbf_class.cc:425-439): fold each filter into its
        first 64 bytes (bloom_filter::fold(2)); the other bytes are kept."""
        f = self.filters.reshape(-1, 256).view(np.uint64)
        folded = f[:, 0:8] | f[:, 8:16] | f[:, 16:24] | f[:, 24:32]
        f[:, 0:8] = folded
        self.fastmode = True
        return self

    def _desc(self, keep: list) -> DigestDesc:
        name = self.name.encode()
        keep.append(name)
        d = DigestDesc()
        d.name = name
        d.filters = self.filters.ctypes.data
        d.elem_counts = self.elem_counts.ctypes.data if self.elem_counts is not None else None
        d.bf_count = self.bf_count
        d.last_count = self.last_count
        d.max_elem = self.max_elem
        d.dd_block_size = self.dd_block_size
        d.orig_size = self.orig_size
        return d

    def to_string(self) -> str:
        """SDBF v3 text line (sdbf::to_string, sdbf/sdbf_class.cc:293-334)."""
        keep: list = []
        d = self._desc(keep)
        n = lib().sdbfg_to_string(C.byref(d), None, 0)
        if n < 0:
            raise SdbfError(int(n), "to_string")
        buf = C.create_string_buffer(int(n) + 1)
        lib().sdbfg_to_string(C.byref(d), buf, n + 1)
        return buf.raw[:n].decode()

    @staticmethod
    def from_string(line: str) -> "Digest":
        """Parse one SDBF line (sdbf(const std::string&), sdbf_class.cc:144-215)."""
        b = line.encode()
        d = DigestDesc()
        rc = lib().sdbfg_parse(b, len(b), C.byref(d), None, 0, None, None)
        if rc != 0:
            raise SdbfError(-1 if rc == -1 else -2, "parse")
        n = d.bf_count
        filters = np.zeros(n * 256, dtype=np.uint8)
        counts = np.zeros(n, dtype=np.uint16) if d.dd_block_size else None
        name = C.create_string_buffer(len(b) + 1)
        rc = lib().sdbfg_parse(b, len(b), C.byref(d), name, len(b) + 1, filters.ctypes.data,
                               counts.ctypes.data if counts is not None else None)
        if rc != 0:
            raise SdbfError(-2, "parse")
        return Digest(name.value.decode(), d.orig_size, d.bf_count, d.last_count, d.max_elem, d.dd_block_size,
                      filters, counts)

    def elem_count(self, i: int) -> int:
        """get_elem_count (sdbf/sdbf_class.cc:406-415)."""
        if self.elem_counts is not None:
            return int(self.elem_counts[i])
        return self.max_elem if i < self.bf_count - 1 else self.last_count


class Index:
    """An index filter resident on the device (sdbfg_index): the reference's
    bloom_filter as read from an index file (sdbf/bloom_filter.cc:87-118)."""

    def __init__(self, ctx: "Context", handle):
        self.ctx = ctx
        self.h = handle
        size, elem, mask = C.c_uint64(), C.c_uint64(), C.c_uint64()
        hc, name = C.c_uint32(), C.c_char_p()
        lib().sdbfg_index_info(handle, C.byref(size), C.byref(elem), C.byref(hc), C.byref(mask), C.byref(name))
        self.bf_size, self.elem_count, self.hash_count, self.bit_mask = size.value, elem.value, hc.value, mask.value
        self.name = (name.value or b"").decode(errors="surrogateescape")

    def close(self):
        if getattr(self, "h", None):
            lib().sdbfg_index_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceSet:
    """Digests resident in device memory (sdbfg_set).  ``digests`` holds the
    host digests a set was uploaded from, or None for a set loaded from SDBF
    text on the device (``digest(i)`` reads one back)."""

    def __init__(self, ctx: "Context", digests: list[Digest] | None, _handle=None):
        self.ctx = ctx
        self.digests = digests
        if _handle is not None:
            self.h = _handle
            self.n = int(lib().sdbfg_set_size(_handle))
            return
        keep: list = []
        arr = (DigestDesc * max(1, len(digests)))()
        for i, d in enumerate(digests):
            arr[i] = d._desc(keep)
        h = C.c_void_p()
        rc = lib().sdbfg_set_upload(ctx.h, arr, len(digests), C.byref(h))
        ctx._check(rc)
        self.h = h
        self.n = len(digests)

    def __len__(self):
        return self.n

    def _info(self, i: int) -> DigestDesc:
        d = DigestDesc()
        if lib().sdbfg_set_digest_info(self.h, i, C.byref(d)) != 0:
            raise IndexError(i)
        return d

    def name(self, i: int) -> str:
        if self.digests is not None:
            return self.digests[i].name
        return self._info(i).name.decode()

    def names(self) -> list[str]:
        return [self.name(i) for i in range(self.n)]

    def digest(self, i: int) -> Digest:
        """Digest i as held on the device (folded filters after fast())."""
        d = self._info(i)
        filters = np.zeros(d.bf_count * 256, dtype=np.uint8)
        counts = np.zeros(d.bf_count, dtype=np.uint16)
        self.ctx._check(lib().sdbfg_set_read_digest(self.ctx.h, self.h, i, filters.ctypes.data, counts.ctypes.data))
        out = Digest(d.name.decode(), d.orig_size, d.bf_count, d.last_count, d.max_elem, d.dd_block_size, filters,
                     counts if d.dd_block_size else None)
        return out

    def fast(self, first: int = 0, count: int | None = None) -> "DeviceSet":
        """sdbf::fast on digests [first, first+count): fold to 64 bytes on the device."""
        n = self.n - first if count is None else count
        self.ctx._check(lib().sdbfg_set_fast(self.ctx.h, self.h, first, n))
        return self

    def close(self):
        if getattr(self, "h", None):
            lib().sdbfg_set_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One device, one stream, reusable device buffers (sdbfg_ctx)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib().sdbfg_ctx_create(device, C.byref(h))
        if rc != 0:
            raise RuntimeError(f"sdbfg_ctx_create failed ({rc}): no usable CUDA device {device}")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().sdbfg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            raise EngineError(rc, lib().sdbfg_last_error(self.h).decode())

    def set_stream(self, stream_handle: int | None):
        """Launch on this CUDA stream (a torch.cuda.Stream's cuda_stream).  None:
        the context's own stream; 0 (the legacy default stream) is passed as
        cudaStreamLegacy so that it is not mistaken for None."""
        if stream_handle is None:
            h = None
        else:
            h = stream_handle if stream_handle != 0 else 1  # cudaStreamLegacy
        self._check(lib().sdbfg_ctx_set_stream(self.h, h))

    def synchronize(self):
        self._check(lib().sdbfg_ctx_synchronize(self.h))

    def set_lead(self, steps: int):
        """Speculative lead-in of the parallel score walk (exact for any value)."""
        self._check(lib().sdbfg_ctx_set_lead(self.h, steps))

    @property
    def pipeline_depth(self) -> int:
        """Stream-mode launch groups kept in flight."""
        return int(lib().sdbfg_ctx_pipeline_depth(self.h))

    def set_pipeline_depth(self, depth: int):
        """Stream-mode launch groups in flight (1..8); 1 = no overlap."""
        self._check(lib().sdbfg_ctx_set_pipeline_depth(self.h, depth))

    def profile(self, enable: bool = True):
        """Per-kernel CUDA-event timing on the launch stream."""
        self._check(lib().sdbfg_ctx_profile(self.h, 1 if enable else 0))

    def kernel_time(self, name: str) -> tuple[float, int]:
        """(total milliseconds, launches) of one kernel since profiling was enabled."""
        ms, n = C.c_double(), C.c_uint64()
        self._check(lib().sdbfg_ctx_kernel_time(self.h, name.encode(), C.byref(ms), C.byref(n)))
        return ms.value, int(n.value)

    @property
    def launch_count(self) -> int:
        return int(lib().sdbfg_ctx_launch_count(self.h))

    @property
    def relinked_tiles(self) -> int:
        return int(lib().sdbfg_ctx_relinked_tiles(self.h))

    def set_index_rounds(self, max_rounds: int):
        """Stream-mode index build: parallel fixed-point rounds per launch
        group before the sequential commit (0 = sequential only; exact either way)."""
        self._check(lib().sdbfg_ctx_set_index_rounds(self.h, max_rounds))

    @property
    def index_rounds(self) -> int:
        """Rounds the last stream-mode index launch group took (0: sequential commit)."""
        return int(lib().sdbfg_ctx_index_rounds(self.h))

    # ------------------------------------------------------------ digests
    @staticmethod
    def capacity(lens, dd_block_size: int = 0) -> int:
        lens = _u64(lens)
        return int(lib().sdbfg_digest_capacity(_ptr(lens), len(lens), dd_block_size))

    def digest_packed(self, data: np.ndarray, offsets, lens, dd_block_size: int = 0, names=None,
                      out_filters: np.ndarray | None = None):
        """Digest inputs packed in one host buffer (input i = data[offsets[i]:offsets[i]+lens[i]]).
        Returns a list of Digest (None for inputs below 512 bytes)."""
        data = np.ascontiguousarray(data, dtype=np.uint8)
        offsets, lens = _u64(offsets), _u64(lens)
        n = len(lens)
        cap = self.capacity(lens, dd_block_size)
        # a buffer made here is the digests' own storage (each Digest views
        # its slice); a caller's buffer may be reused, so its slices are copied
        own = out_filters is None or out_filters.size < cap * 256
        if own:
            out_filters = np.zeros(max(1, cap) * 256, dtype=np.uint8)
        counts = np.zeros(max(1, cap), dtype=np.uint16)
        res = (DigestResult * max(1, n))()
        rc = lib().sdbfg_digest_batch(self.h, data.ctypes.data, _ptr(offsets), _ptr(lens), n, dd_block_size,
                                      out_filters.ctypes.data, cap, counts.ctypes.data if dd_block_size else None,
                                      res)
        self._check(rc)
        out = []
        for i in range(n):
            r = res[i]
            if r.status != 0:
                out.append(None)
                continue
            o, k = int(r.filter_offset), int(r.bf_count)
            name = names[i] if names is not None else f"f{i}"
            filt = out_filters[o * 256:(o + k) * 256]
            if not own:
                filt = filt.copy()
            if dd_block_size:
                out.append(Digest(name, int(lens[i]), k, 0, BLOCK_MAX_ELEM, dd_block_size, filt,
                                  counts[o:o + k].copy()))
            else:
                out.append(Digest(name, int(lens[i]), k, int(r.last_count), STREAM_MAX_ELEM, 0, filt, None))
        return out

    def load_index(self, path: str) -> Index:
        """bloom_filter(string indexfilename): an index file, resident on the device.
        An unreadable file raises SdbfError(-1), a malformed one SdbfError(-2)."""
        h = C.c_void_p()
        rc = lib().sdbfg_index_load_file(self.h, os.fsencode(path), C.byref(h))
        if rc == -1:
            raise SdbfError(-1, path)
        if rc == -4:
            raise SdbfError(-2, path)
        self._check(rc)
        return Index(self, h)

    def index_from_bits(self, bits: np.ndarray, hash_count: int = 5, name: str = "") -> Index:
        """An index from raw filter bytes (size a power of two >= 64)."""
        bits = np.ascontiguousarray(bits, dtype=np.uint8)
        h = C.c_void_p()
        self._check(lib().sdbfg_index_create(self.h, bits.ctypes.data, bits.size, hash_count, name.encode(),
                                             C.byref(h)))
        return Index(self, h)

    def digest_search(self, buffers, names, dd_block_size: int, indexes: list[Index]):
        """Block-mode digests with the index search of sdhash --index-search
        (sdbf_core.cc:141-191): returns (digests, hits) where hits[k] is a
        (bf_count, len(indexes)) uint8 array for digest k (None where the
        input is too small): sampled features of each block found in each index."""
        lens = np.array([len(b) for b in buffers], dtype=np.uint64)
        offs = np.zeros(len(buffers), dtype=np.uint64)
        tot = 0
        for i, b in enumerate(buffers):
            offs[i] = tot
            tot += (len(b) + 15) & ~15
        data = np.zeros(max(16, tot), dtype=np.uint8)
        for i, b in enumerate(buffers):
            data[int(offs[i]):int(offs[i]) + len(b)] = np.frombuffer(bytes(b), dtype=np.uint8)
        n, nidx = len(lens), len(indexes)
        cap = self.capacity(lens, dd_block_size)
        out_filters = np.zeros(max(1, cap) * 256, dtype=np.uint8)
        counts = np.zeros(max(1, cap), dtype=np.uint16)
        hits = np.zeros(max(1, cap * nidx), dtype=np.uint8)
        res = (DigestResult * max(1, n))()
        arr = (C.c_void_p * max(1, nidx))(*[x.h for x in indexes])
        self._check(lib().sdbfg_digest_batch_search(self.h, data.ctypes.data, _ptr(offs), _ptr(lens), n, dd_block_size,
                                                    out_filters.ctypes.data, cap, counts.ctypes.data, res, arr, nidx,
                                                    hits.ctypes.data))
        digs, hit_rows = [], []
        for i in range(n):
            r = res[i]
            if r.status != 0:
                digs.append(None)
                hit_rows.append(None)
                continue
            o, k = int(r.filter_offset), int(r.bf_count)
            digs.append(Digest(names[i], int(lens[i]), k, 0, BLOCK_MAX_ELEM, dd_block_size,
                               out_filters[o * 256:(o + k) * 256], counts[o:o + k].copy()))
            hit_rows.append(hits[o * nidx:(o + k) * nidx].reshape(k, nidx).copy())
        return digs, hit_rows

    def digest_index(self, buffers, names, dd_block_size: int, index_bits: np.ndarray, elem_count: int = 0):
        """Digests with an index being built (sdhash --index for one group of
        files): stream mode takes the inputs in order and drops features the
        index already holds, block mode inserts every counted feature.
        index_bits (uint8, power-of-two size) is updated in place; returns
        (digests, elem_count after the batch)."""
        lens = np.array([len(b) for b in buffers], dtype=np.uint64)
        offs = np.zeros(len(buffers), dtype=np.uint64)
        tot = 0
        for i, b in enumerate(buffers):
            offs[i] = tot
            tot += (len(b) + 15) & ~15
        data = np.zeros(max(16, tot), dtype=np.uint8)
        for i, b in enumerate(buffers):
            data[int(offs[i]):int(offs[i]) + len(b)] = np.frombuffer(bytes(b), dtype=np.uint8)
        n = len(lens)
        cap = self.capacity(lens, dd_block_size)
        out_filters = np.zeros(max(1, cap) * 256, dtype=np.uint8)
        counts = np.zeros(max(1, cap), dtype=np.uint16)
        res = (DigestResult * max(1, n))()
        assert index_bits.dtype == np.uint8 and index_bits.flags.c_contiguous
        ec = np.array([elem_count], dtype=np.uint64)
        self._check(lib().sdbfg_digest_batch_index(self.h, data.ctypes.data, _ptr(offs), _ptr(lens), n, dd_block_size,
                                                   out_filters.ctypes.data, cap, counts.ctypes.data, res,
                                                   index_bits.ctypes.data, index_bits.size, _ptr(ec)))
        digs = []
        for i in range(n):
            r = res[i]
            if r.status != 0:
                digs.append(None)
                continue
            o, k = int(r.filter_offset), int(r.bf_count)
            f = out_filters[o * 256:(o + k) * 256]
            if dd_block_size:
                digs.append(Digest(names[i], int(lens[i]), k, 0, BLOCK_MAX_ELEM, dd_block_size, f, counts[o:o + k].copy()))
            else:
                digs.append(Digest(names[i], int(lens[i]), k, int(r.last_count), STREAM_MAX_ELEM, 0, f, None))
        return digs, int(ec[0])

    @staticmethod
    def write_index(path: str, bits: np.ndarray, elem_count: int, set_name: str, hash_count: int = 5):
        """bloom_filter::write_out: an index file the reference can read."""
        bits = np.ascontiguousarray(bits, dtype=np.uint8)
        rc = lib().sdbfg_index_write_file(os.fsencode(path), bits.ctypes.data, bits.size, elem_count, hash_count,
                                          set_name.encode())
        if rc != 0:
            raise SdbfError(-2, f"cannot write {path}")

    def digest_buffers(self, buffers, names=None, dd_block_size: int = 0):
        """Digest a list of bytes-like inputs."""
        lens = np.array([len(b) for b in buffers], dtype=np.uint64)
        offs = np.zeros(len(buffers), dtype=np.uint64)
        tot = 0
        for i, b in enumerate(buffers):
            offs[i] = tot
            tot += (len(b) + 15) & ~15
        data = np.zeros(max(16, tot), dtype=np.uint8)
        for i, b in enumerate(buffers):
            data[int(offs[i]):int(offs[i]) + len(b)] = np.frombuffer(bytes(b), dtype=np.uint8)
        return self.digest_packed(data, offs, lens, dd_block_size, names)

    def digest_device(self, dev_data: int, offsets, lens, dd_block_size: int, dev_out_filters: int, out_cap: int,
                      dev_out_counts: int | None = None):
        """Digest inputs already in device memory; returns (bf_count, last_count, status, filter_offset) arrays."""
        offsets, lens = _u64(offsets), _u64(lens)
        n = len(lens)
        res = (DigestResult * max(1, n))()
        rc = lib().sdbfg_digest_batch_device(self.h, dev_data, _ptr(offsets), _ptr(lens), n, dd_block_size,
                                             dev_out_filters, out_cap, dev_out_counts, res)
        self._check(rc)
        return res

    # ---------------------------------------------------------- compare
    def load_text(self, text: bytes | str) -> DeviceSet:
        """A resident set from SDBF v3 text, one digest per line, as
        sdbf_set(const char* fname) loads a file (sdbf/sdbf_set.cc:51-74):
        headers read on the host, base64 payloads decoded on the device.
        A malformed line raises SdbfError with the reference constructor's
        throw value (-1 or -2) and ``line`` = its index."""
        b = text.encode() if isinstance(text, str) else bytes(text)
        h = C.c_void_p()
        bad_line, bad_code = C.c_int64(-1), C.c_int32(0)
        rc = lib().sdbfg_set_load_text(self.h, b, len(b), C.byref(h), C.byref(bad_line), C.byref(bad_code))
        if rc == -4:  # SDBFG_ERR_FORMAT
            e = SdbfError(int(bad_code.value), f"line {bad_line.value}")
            e.line = int(bad_line.value)
            raise e
        self._check(rc)
        return DeviceSet(self, None, _handle=h)

    def load_file(self, path: str) -> DeviceSet:
        """load_text of a file's contents (sdbf_set(const char* fname))."""
        with open(path, "rb") as f:
            return self.load_text(f.read())

    def upload(self, digests: list[Digest]) -> DeviceSet:
        """Resident set; digests folded with Digest.fast() keep their fast mode."""
        ds = DeviceSet(self, digests)
        i, n = 0, len(digests)
        while i < n:
            if digests[i].fastmode:
                j = i
                while j < n and digests[j].fastmode:
                    j += 1
                ds.fast(i, j - i)
                i = j
            else:
                i += 1
        return ds

    def compare_all(self, s: DeviceSet) -> np.ndarray:
        n = len(s)
        out = np.zeros(max(1, n * (n - 1) // 2), dtype=np.int32)
        if n > 1:
            self._check(lib().sdbfg_compare_all(self.h, s.h, _ptr(out, C.c_int32)))
        return out[: n * (n - 1) // 2]

    def compare_to(self, q: DeviceSet, t: DeviceSet) -> np.ndarray:
        out = np.zeros(max(1, len(q) * len(t)), dtype=np.int32)
        if len(q) and len(t):
            self._check(lib().sdbfg_compare_to(self.h, q.h, t.h, _ptr(out, C.c_int32)))
        return out[: len(q) * len(t)].reshape(len(q), len(t))

    def _matches(self, fn, args, threshold):
        cnt = C.c_uint64()
        cap = 1 << 16
        while True:
            out = np.zeros((cap, 3), dtype=np.int32)
            rc = fn(self.h, *args, threshold, out.ctypes.data, cap, C.byref(cnt))
            if rc == -5 and cnt.value > cap:  # SDBFG_ERR_CAPACITY: room for the reported count
                cap = int(cnt.value)
                continue
            self._check(rc)
            return out[: cnt.value].copy()

    def compare_all_matches(self, s: DeviceSet, threshold: int = 1) -> np.ndarray:
        """(i, j, score) rows with score >= threshold, i < j, in pair order."""
        return self._matches(lib().sdbfg_compare_all_matches, (s.h,), threshold)

    def compare_to_matches(self, q: DeviceSet, t: DeviceSet, threshold: int = 1) -> np.ndarray:
        """(query, target, score) rows with score >= threshold, in pair order."""
        return self._matches(lib().sdbfg_compare_to_matches, (q.h, t.h), threshold)

    def compare_all_device(self, s: DeviceSet, dev_scores: int):
        """Queue all-pairs scores of s into a device int32 array (n*(n-1)/2)."""
        self._check(lib().sdbfg_compare_all_device(self.h, s.h, C.c_void_p(dev_scores)))

    def compare_to_device(self, q: DeviceSet, t: DeviceSet, dev_scores: int):
        """Queue query x target scores into a device int32 array (nq*nt)."""
        self._check(lib().sdbfg_compare_to_device(self.h, q.h, t.h, C.c_void_p(dev_scores)))

    def filter_pairs(self, a: DeviceSet, b: DeviceSet | None = None) -> int:
        return int(lib().sdbfg_compare_filter_pairs(self.h, a.h, b.h if b is not None else None))

    def set_compare_tuning(self, variant: int = 0, unit_work: int = 1 << 22, graphs: bool = True):
        self._check(lib().sdbfg_ctx_set_compare_tuning(self.h, variant, unit_work, int(graphs)))

    def compare_tuning(self) -> tuple[int, int]:
        v, w = C.c_int(), C.c_uint64()
        self._check(lib().sdbfg_ctx_get_compare_tuning(self.h, C.byref(v), C.byref(w)))
        return v.value, w.value

    def autotune_compare(self, a: DeviceSet, b: DeviceSet | None = None, sample_pairs: int = 1 << 34):
        """Pick the fastest kernel variant and unit budget; returns (variant, unit_work, pairs/s)."""
        v, w, r = C.c_int(), C.c_uint64(), C.c_double()
        self._check(lib().sdbfg_compare_autotune(self.h, a.h, b.h if b is not None else None, sample_pairs,
                                                 C.byref(v), C.byref(w), C.byref(r)))
        return v.value, w.value, r.value

    def score_pairs(self, a: DeviceSet, b: DeviceSet, ia, ib) -> np.ndarray:
        ia = np.ascontiguousarray(ia, dtype=np.uint32)
        ib = np.ascontiguousarray(ib, dtype=np.uint32)
        out = np.zeros(max(1, len(ia)), dtype=np.int32)
        if len(ia):
            self._check(lib().sdbfg_score_pairs(self.h, a.h, b.h, _ptr(ia, C.c_uint32), _ptr(ib, C.c_uint32),
                                                len(ia), _ptr(out, C.c_int32)))
        return out[: len(ia)]


class Server:
    """Serving loop over a device-resident target set (sdbfg_server): submit
    query digests from any thread, poll finished ones with their score rows."""

    def __init__(self, ctx: "Context", targets: DeviceSet, slots: int = 3, max_batch_queries: int = 256,
                 memory_budget: int = 256 << 20, threshold: int = 1, max_batch_pairs: int = 1 << 31):
        self.ctx, self.targets = ctx, targets
        cfg = ServerConfig(slots, max_batch_queries, memory_budget, threshold, 0, max_batch_pairs)
        h = C.c_void_p()
        ctx._check(lib().sdbfg_server_create(ctx.h, targets.h, C.byref(cfg), C.byref(h)))
        self.h = h
        self.nt = len(targets)

    def submit(self, d: "Digest", tag: int):
        keep: list = []
        desc = d._desc(keep)
        self.ctx._check(lib().sdbfg_server_submit(self.h, C.byref(desc), tag))

    def poll(self, max_results: int = 1024, timeout_ms: int = 0, scores: bool = True):
        """List of (result, score row or None)."""
        res = (ServerResult * max_results)()
        sc = np.zeros(max_results * self.nt if scores else 1, dtype=np.int32)
        n = C.c_uint32()
        self.ctx._check(lib().sdbfg_server_poll(self.h, res, _ptr(sc, C.c_int32) if scores else None, max_results,
                                                C.byref(n), timeout_ms))
        return [(res[k], sc[k * self.nt:(k + 1) * self.nt].copy() if scores else None) for k in range(n.value)]

    def stats(self) -> dict:
        v = [C.c_uint64() for _ in range(4)]
        self.ctx._check(lib().sdbfg_server_stats(self.h, *[C.byref(x) for x in v]))
        return dict(zip(("pending", "served", "batches", "launches"), (x.value for x in v)))

    def close(self):
        if getattr(self, "h", None):
            lib().sdbfg_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------- reference object API
_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(int(os.environ.get("SDBFG_DEVICE", "0")))
    return _default_ctx


class sdbf:  # noqa: N801 -- the reference's class name
    """Mirror of the reference's ``class sdbf`` (sdbf/sdbf_class.h:23-121).

    sdbf(name, data, dd_block_size=0)   -- sdbf(const char*, char*, uint32_t, uint64_t, index_info*)
    sdbf.from_file(path, dd_block_size) -- sdbf(const char *filename, uint32_t dd_block_size)
    sdbf.from_string(line)              -- sdbf(const std::string&)
    """

    def __init__(self, name: str | None = None, data=None, dd_block_size: int = 0, *, _digest: Digest | None = None):
        if _digest is not None:
            self._d = _digest
            return
        if data is None or len(data) < MIN_FILE_SIZE:
            raise SdbfError(-3, "input too small")  # sdbf_class.cc:116-117
        d = default_context().digest_buffers([data], [name], dd_block_size)[0]
        if d is None:
            raise SdbfError(-3, "input too small")
        self._d = d

    @classmethod
    def from_file(cls, path: str, dd_block_size: int = 0) -> "sdbf":
        try:
            with open(path, "rb") as f:
                data = f.read()
        except OSError:
            raise SdbfError(-1, "cannot read file")  # sdbf_class.cc:36-37
        if len(data) < MIN_FILE_SIZE:
            raise SdbfError(-1, "file too small")
        return cls(path, data, dd_block_size)

    @classmethod
    def from_string(cls, line: str) -> "sdbf":
        return cls(_digest=Digest.from_string(line))

    @property
    def digest(self) -> Digest:
        return self._d

    def name(self) -> str:
        return self._d.name

    def size(self) -> int:
        return self._d.bf_count * 256

    def input_size(self) -> int:
        return self._d.orig_size

    def filter_count(self) -> int:
        return self._d.bf_count

    def clone_filter(self, pos: int) -> bytes | None:
        if pos >= self._d.bf_count:
            return None
        return self._d.filters[pos * 256:(pos + 1) * 256].tobytes()

    @staticmethod
    def get_elem_count(s: "sdbf", index: int) -> int:
        return s._d.elem_count(index)

    def fast(self) -> None:
        """sdbf::fast (sdbf/sdbf_class.cc:425-439): destructive fold to 64-byte filters."""
        self._d.fast()

    def compare(self, other: "sdbf", sample: int = 0) -> int:
        """sdbf::compare (sdbf/sdbf_class.cc:266); sample must be 0."""
        if sample:
            raise NotImplementedError("filter sampling (random, unpinned in the reference) is not supported")
        ctx = default_context()
        s = ctx.upload([self._d, other._d])
        return int(ctx.score_pairs(s, s, [0], [1])[0])

    def to_string(self) -> str:
        return self._d.to_string()

    def __str__(self):
        return self.to_string()


def _result_lines(names_a, names_b, pairs, scores, threshold: int, sep: str) -> str:
    # sdbf_set.cc:254-262: "a|b|%03d", -1 unpadded, only scores >= threshold
    out = []
    for (i, j), s in zip(pairs, scores):
        s = int(s)
        if s >= threshold:
            out.append(f"{names_a[i]}{sep}{names_b[j]}{sep}{s:03d}\n" if s != -1
                       else f"{names_a[i]}{sep}{names_b[j]}{sep}{s}\n")
    return "".join(out)


class sdbf_set:  # noqa: N801
    """Mirror of the reference's ``class sdbf_set`` (sdbf/sdbf_set.h:15-96)."""

    def __init__(self, fname: str | None = None):
        self.items: list[sdbf] = []
        self.setname = "default"
        self.sep = "|"
        self._lock = threading.Lock()
        self._resident: DeviceSet | None = None
        self._resident_key = None
        if fname is not None and os.path.isfile(fname):
            # the whole file is parsed on the device (Context.load_file); the
            # resident set is kept for comparisons until the items change
            ds = default_context().load_file(fname)
            self.items = [sdbf(_digest=ds.digest(i)) for i in range(len(ds))]
            self._resident, self._resident_key = ds, self._key()
            self.setname = fname

    def _key(self):
        return tuple((id(s), s.digest.fastmode) for s in self.items)

    def _device_set(self, ctx: "Context") -> "DeviceSet":
        """The items as a resident set: the one loaded from the file while the
        items are unchanged, else a fresh upload."""
        if self._resident is not None and self._resident.ctx is ctx and self._resident_key == self._key():
            return self._resident
        return ctx.upload([s.digest for s in self.items])

    def at(self, pos: int):
        return self.items[pos] if pos < len(self.items) else None

    def add(self, item):
        with self._lock:
            if isinstance(item, sdbf_set):
                self.items.extend(item.items)
            else:
                self.items.append(item)

    def size(self) -> int:
        return len(self.items)

    def input_size(self) -> int:
        return sum(s.input_size() for s in self.items)

    def empty(self) -> int:
        return 1 if not self.items else 0

    def name(self) -> str:
        return self.setname

    def set_name(self, name: str):
        self.setname = name

    def set_separator(self, sep: str):
        self.sep = sep

    def to_string(self) -> str:
        return "".join(s.to_string() for s in self.items)

    def compare_all_quiet(self, threshold: int = 1, thread_count: int = 0, fast: bool = False) -> str:
        """sdbf_set::compare_all_quiet (sdbf/sdbf_set.cc:278-308), in set order."""
        if fast:  # sdbf_set.cc:284-289: every item folded first (destructive)
            for s in self.items:
                s.fast()
        n = len(self.items)
        if n < 2:
            return ""
        ctx = default_context()
        ds = self._device_set(ctx)
        scores = ctx.compare_all(ds)
        pairs = [(i, j) for i in range(n) for j in range(i + 1, n)]
        names = [s.name() for s in self.items]
        return _result_lines(names, names, pairs, scores, threshold, self.sep)

    def compare_all(self, threshold: int = 1, fast: bool = False) -> None:
        print(self.compare_all_quiet(threshold, 0, fast), end="")

    def compare_to_quiet(self, other: "sdbf_set", threshold: int = 1, sample_size: int = 0, thread_count: int = 0,
                         fast: bool = False) -> str:
        """sdbf_set::compare_to_quiet (sdbf/sdbf_set.cc:360-394), in set order."""
        if sample_size:
            raise NotImplementedError("sampling (random, unpinned in the reference) is not supported")
        if fast:
            # sdbf_set.cc:369-378 folds this set's items twice (the first loop
            # runs over other->size() indices of this set: at() throws when the
            # other set is larger) and leaves the other set unfolded
            if len(other.items) > len(self.items):
                raise IndexError("sdbf_set::compare_to with fast: other set larger than this set")
            for s in self.items:
                s.fast()
        if not self.items or not other.items:
            return ""
        ctx = default_context()
        q = self._device_set(ctx)
        t = other._device_set(ctx)
        scores = ctx.compare_to(q, t)
        pairs = [(i, j) for i in range(len(self.items)) for j in range(len(other.items))]
        return _result_lines([s.name() for s in self.items], [s.name() for s in other.items], pairs,
                             scores.reshape(-1), threshold, self.sep)

    def compare_to(self, other: "sdbf_set", threshold: int = 1, sample_size: int = 0, fast: bool = False) -> None:
        print(self.compare_to_quiet(other, threshold, sample_size, 0, fast), end="")
