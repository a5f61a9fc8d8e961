// text_load.cu -- bulk load of SDBF v3 text into a device-resident set.
//
// The reference loads a digest file line by line (sdbf_set(const char*),
// sdbf/sdbf_set.cc:51-74), parsing each line with sdbf(const string&)
// (sdbf/sdbf_class.cc:144-215): header fields, then the base64 payload
// decoded on the host (modp_b64_decode, base64/modp_b64.cc), then the
// hamming weights (compute_hamming, sdbf_class.cc:388-401).  Here the host
// reads only the header of each line and jumps over the payload, whose
// length the header fixes; the whole text goes to the device once and one
// kernel decodes every filter, checks the record layout and the base64
// alphabet, and writes the filters plus their (hamming, element count)
// words straight into the set's arrays.
//
// Payload layouts (sdbf::to_string, sdbf_class.cc:293-334):
//   stream  <base64 of bf_count*256 bytes>       one run; every 1024
//           characters decode to exactly three filters, so a work item is
//           one triple of filters;
//   sdbf-dd {:<elem count, hex>:<base64 of 256 bytes, 344 chars>}
//           a work item is one record.  The writer always emits two hex
//           digits (%02x), so record k sits at payload + 348*k; the kernel
//           checks that layout and flags a line that deviates, and the host
//           re-reads such a line field by field (as the reference's getline
//           loop does) and decodes it in a second launch.
#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ctx_internal.h"

namespace {

constexpr uint32_t kLineIrregular = 1;  // dd record layout is not the 348-char stride
constexpr uint32_t kLineBad = 2;        // invalid base64 or record field

constexpr uint32_t kDdRecord = 348;     // ':' + 2 hex + ':' + 344 base64
constexpr uint32_t kTripleChars = 1024; // base64 of 768 bytes (three filters)

struct TextLine {
    uint64_t payload;   // text offset of the payload (dd: the ':' before record 0)
    uint64_t item0;     // first work item of the line
    uint64_t end;       // text offset of the line end ('\n' or end of text)
    uint32_t first;     // first filter of the digest in the set
    uint32_t nfilters;
    uint32_t elem_full; // stream: max_elem (every filter but the last)
    uint32_t elem_last; // stream: last_count
    uint32_t dd;        // 1: sdbf-dd line
    uint32_t pad;
};

// One record of an irregular dd line, located on the host.
struct TextRecord {
    uint64_t src;       // first of its 344 base64 characters
    uint32_t filter;    // destination filter index
    uint32_t elem;      // parsed element count
    uint32_t line;
    uint32_t pad;
};

constexpr int kLoadWarps = 8;

__device__ __forceinline__ uint32_t b64_value(uint32_t ch) {
    // RFC 4648 alphabet; 64 marks an invalid character
    if (ch - 'A' < 26u) return ch - 'A';
    if (ch - 'a' < 26u) return ch - 'a' + 26;
    if (ch - '0' < 10u) return ch - '0' + 52;
    if (ch == '+') return 62;
    if (ch == '/') return 63;
    return 64;
}

__device__ __forceinline__ int hex_value(uint32_t ch) {
    if (ch - '0' < 10u) return (int)(ch - '0');
    if ((ch | 32u) - 'a' < 6u) return (int)((ch | 32u) - 'a' + 10);
    return -1;
}

// Decodes nbytes (256, 512 or 768) from the base64 at text[src..] into the
// warp's staging area; returns false (warp-uniform) on an invalid character
// or padding.  modp_b64_decode accepts exactly: full groups of alphabet
// characters, then a last group whose trailing '=' count makes the decoded
// length; the unused low bits of the last character are ignored.
__device__ bool decode_run(const uint8_t* __restrict__ text, uint64_t src, uint32_t nbytes, uint8_t* stage) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t ngroups = (nbytes + 2) / 3;
    const uint32_t pads = 3 * ngroups - nbytes;
    bool ok = true;
    for (uint32_t g = lane; g < ngroups; g += 32) {
        const uint8_t* p = text + src + 4ull * g;
        const uint32_t c0 = p[0], c1 = p[1], c2 = p[2], c3 = p[3];
        uint32_t v0 = b64_value(c0), v1 = b64_value(c1), v2 = b64_value(c2), v3 = b64_value(c3);
        if (g + 1 == ngroups && pads) {
            if (c3 != '=') ok = false;
            v3 = 0;
            if (pads == 2) {
                if (c2 != '=') ok = false;
                v2 = 0;
            }
        }
        if ((v0 | v1 | v2 | v3) & 64u) ok = false;
        const uint32_t x = (v0 << 18) | (v1 << 12) | (v2 << 6) | v3;
        const uint32_t o = 3 * g;
        stage[o] = (uint8_t)(x >> 16);
        if (o + 1 < nbytes) stage[o + 1] = (uint8_t)(x >> 8);
        if (o + 2 < nbytes) stage[o + 2] = (uint8_t)x;
    }
    return __all_sync(0xffffffffu, ok);
}

// Copies nf staged filters out and writes meta = (hamming << 16) | elem.
__device__ void store_filters(const uint8_t* stage, uint32_t nf, uint32_t f0, uint32_t e0, uint32_t e1, uint32_t e2,
                              uint8_t* __restrict__ filters, uint32_t* __restrict__ meta) {
    const uint32_t lane = threadIdx.x & 31;
    const uint4* s4 = reinterpret_cast<const uint4*>(stage);
    uint4* d4 = reinterpret_cast<uint4*>(filters + 256ull * f0);
    for (uint32_t base = 0; base < 16 * nf; base += 32) {  // 16 uint4 per filter; half-warps
        const uint32_t u = base + lane;
        uint32_t h = 0;
        if (u < 16 * nf) {
            const uint4 v = s4[u];
            d4[u] = v;
            h = __popc(v.x) + __popc(v.y) + __popc(v.z) + __popc(v.w);
        }
        h += __shfl_xor_sync(0xffffffffu, h, 8);
        h += __shfl_xor_sync(0xffffffffu, h, 4);
        h += __shfl_xor_sync(0xffffffffu, h, 2);
        h += __shfl_xor_sync(0xffffffffu, h, 1);
        if ((lane & 15) == 0 && u < 16 * nf) {
            const uint32_t f = u >> 4;
            const uint32_t e = f == 0 ? e0 : (f == 1 ? e1 : e2);
            meta[f0 + f] = (h << 16) | (e & 0xFFFFu);
        }
    }
}

// Lines mode: one warp per work item (a stream triple or a dd record).
__global__ void __launch_bounds__(kLoadWarps * 32)
k_text_decode(const uint8_t* __restrict__ text, const TextLine* __restrict__ lines, uint32_t nlines, uint64_t nitems,
              uint8_t* __restrict__ filters, uint32_t* __restrict__ meta, uint32_t* __restrict__ line_flags) {
    __shared__ __align__(16) uint8_t stage[kLoadWarps][768 + 16];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint64_t nwarps = (uint64_t)gridDim.x * kLoadWarps;
    for (uint64_t it = (uint64_t)blockIdx.x * kLoadWarps + warp; it < nitems; it += nwarps) {
        // last line whose first item is <= it (every line has >= 1 item)
        uint32_t lo = 0, hi = nlines - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (lines[mid].item0 <= it) lo = mid;
            else hi = mid - 1;
        }
        const TextLine L = lines[lo];
        const uint32_t k = (uint32_t)(it - L.item0);
        uint32_t e0, e1 = 0, e2 = 0;
        uint32_t nf, f0;
        uint64_t src;
        if (L.dd) {
            const uint64_t rec = L.payload + (uint64_t)kDdRecord * k;
            const uint64_t after = rec + kDdRecord;  // ':' of the next record, or the line end
            // every byte read lies inside the line: after <= L.end is checked first
            bool regular = after <= L.end;
            int h1 = -1, h0 = -1;
            if (regular) {
                h1 = hex_value(text[rec + 1]);
                h0 = hex_value(text[rec + 2]);
                regular = text[rec] == ':' && text[rec + 3] == ':' && h1 >= 0 && h0 >= 0 &&
                          (k + 1 < L.nfilters ? (after < L.end && text[after] == ':') : after == L.end);
            }
            if (!regular) {  // warp-uniform: every lane read the same bytes
                if (lane == 0) atomicOr(line_flags + lo, kLineIrregular);
                continue;
            }
            nf = 1;
            f0 = L.first + k;
            src = rec + 4;
            e0 = (uint32_t)(h1 * 16 + h0);
        } else {
            f0 = L.first + 3 * k;
            nf = min(3u, L.nfilters - 3 * k);
            src = L.payload + (uint64_t)kTripleChars * k;
            e0 = (3 * k + 1 < L.nfilters) ? L.elem_full : L.elem_last;
            e1 = (3 * k + 2 < L.nfilters) ? L.elem_full : L.elem_last;
            e2 = (3 * k + 3 < L.nfilters) ? L.elem_full : L.elem_last;
        }
        if (!decode_run(text, src, 256 * nf, stage[warp])) {
            if (lane == 0) atomicOr(line_flags + lo, kLineBad);
            continue;
        }
        __syncwarp();
        store_filters(stage[warp], nf, f0, e0, e1, e2, filters, meta);
        __syncwarp();
    }
}

// Records mode: one warp per record of the irregular dd lines.
__global__ void __launch_bounds__(kLoadWarps * 32)
k_text_decode_records(const uint8_t* __restrict__ text, const TextRecord* __restrict__ recs, uint32_t nrecs,
                      uint8_t* __restrict__ filters, uint32_t* __restrict__ meta, uint32_t* __restrict__ line_flags) {
    __shared__ __align__(16) uint8_t stage[kLoadWarps][768 + 16];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t r = blockIdx.x * kLoadWarps + warp; r < nrecs; r += gridDim.x * kLoadWarps) {
        const TextRecord R = recs[r];
        if (!decode_run(text, R.src, 256, stage[warp])) {
            if (lane == 0) atomicOr(line_flags + R.line, kLineBad);
            continue;
        }
        __syncwarp();
        store_filters(stage[warp], 1, R.filter, R.elem, 0, 0, filters, meta);
        __syncwarp();
    }
}

// ------------------------------------------------------------ host parse

struct Fields {
    const char* p;
    const char* end;
    // Next ':'-separated field (std::getline(ss, s, ':') semantics within one line).
    bool next(const char** f, size_t* n) {
        if (p > end) return false;
        const char* q = static_cast<const char*>(memchr(p, ':', (size_t)(end - p)));
        if (!q) q = end;
        *f = p;
        *n = (size_t)(q - p);
        p = q + 1;
        return true;
    }
    bool number(uint64_t* v) {
        const char* f;
        size_t n;
        if (!next(&f, &n) || n == 0 || n > 20) return false;
        uint64_t x = 0;
        for (size_t i = 0; i < n; i++) {
            if (f[i] < '0' || f[i] > '9') return false;
            x = x * 10 + (uint64_t)(f[i] - '0');
        }
        *v = x;
        return true;
    }
};

struct ParsedLine {
    TextLine line;
    std::string name;
    uint64_t orig_size;
    uint32_t max_elem, last_count, dd_block;
    const char* start;
};

// Parses one line's header.  Returns 0, -1 (line shorter than 344
// characters: sdbf(const string&) throws -1, sdbf_class.cc:145-146) or -2
// (any other format error, the constructor's throw -2).
int parse_header(const char* text, uint64_t ls, uint64_t le, ParsedLine* out) {
    if (le - ls < 344) return -1;
    Fields c{text + ls, text + le};
    const char* f;
    size_t n;
    uint64_t v;
    if (!c.next(&f, &n) || n < 4 || strncmp(f, "sdbf", 4)) return -2;
    const bool dd = (n == 7 && !strncmp(f, "sdbf-dd", 7));
    if (!c.next(&f, &n) || !c.next(&f, &n)) return -2;  // version, name length
    if (!c.next(&f, &n)) return -2;
    out->name.assign(f, n);
    if (!c.number(&v)) return -2;
    out->orig_size = v;
    if (!c.next(&f, &n)) return -2;                // hash name
    if (!c.number(&v) || v != 256) return -2;      // filter size
    if (!c.number(&v) || !c.next(&f, &n)) return -2;  // hash count, mask
    if (!c.number(&v) || v > 0xFFFFu) return -2;
    out->max_elem = (uint32_t)v;
    if (!c.number(&v) || v == 0 || v >= (1ull << 31)) return -2;
    const uint32_t bf = (uint32_t)v;
    TextLine& L = out->line;
    memset(&L, 0, sizeof L);
    L.nfilters = bf;
    L.dd = dd ? 1 : 0;
    L.end = le;
    if (dd) {
        if (!c.number(&v) || v > 0xFFFFFFFFull) return -2;
        out->dd_block = (uint32_t)v;
        out->last_count = 0;
        // c.p is one past the ':' that ends the block size; record 0's ':' is that one
        L.payload = (uint64_t)(c.p - 1 - text);
        if (c.p - 1 >= text + le || c.p[-1] != ':') return -2;
    } else {
        if (!c.number(&v) || v > 0xFFFFu) return -2;
        out->last_count = (uint32_t)v;
        out->dd_block = 0;
        L.payload = (uint64_t)(c.p - text);
        L.elem_full = out->max_elem;
        L.elem_last = out->last_count;
        const uint64_t bytes = (uint64_t)bf * 256;
        const uint64_t need = 4 * ((bytes + 2) / 3);
        // ss.read of the payload: a short line leaves NUL characters, which
        // fail the decode (sdbf_class.cc:199-209); extra characters are ignored
        if (L.payload > le || le - L.payload < need) return -2;
    }
    return 0;
}

// Locates the records of a dd line field by field, as the reference's loop
// does (sdbf_class.cc:176-194): an element count parsed as hex, then a
// field whose first 344 characters are decoded.
int scan_dd_records(const char* text, const TextLine& L, uint32_t line, std::vector<TextRecord>& out) {
    Fields c{text + L.payload + 1, text + L.end};
    for (uint32_t k = 0; k < L.nfilters; k++) {
        const char* f;
        size_t n;
        if (!c.next(&f, &n)) return -2;
        uint64_t e = 0;
        size_t i = 0;
        while (i < n && (f[i] == ' ' || f[i] == '\t')) i++;
        for (; i < n; i++) {  // operator>> with std::hex: leading digits, then stop
            const char ch = f[i];
            int d = (ch >= '0' && ch <= '9') ? ch - '0' : ((ch | 32) >= 'a' && (ch | 32) <= 'f') ? (ch | 32) - 'a' + 10 : -1;
            if (d < 0) break;
            e = e * 16 + (uint64_t)d;
            if (e > 0xFFFFu) return -2;
        }
        if (!c.next(&f, &n) || n < 344) return -2;
        out.push_back(TextRecord{(uint64_t)(f - text), L.first + k, (uint32_t)e, line, 0});
    }
    return 0;
}

}  // namespace

extern "C" int sdbfg_set_load_text(sdbfg_ctx* c, const char* text, uint64_t len, sdbfg_set** out,
                                   int64_t* bad_line, int32_t* bad_code) {
    if (!c || !out || (len && !text)) return SDBFG_ERR_ARG;
    *out = nullptr;
    if (bad_line) *bad_line = -1;
    if (bad_code) *bad_code = 0;
    CUDA_TRY(c, cudaSetDevice(c->device));
    // ---- host: line headers (the payload is jumped over)
    std::vector<ParsedLine> pl;
    uint64_t pos = 0, total = 0, items = 0;
    int64_t hdr_bad = -1;
    int32_t hdr_code = 0;
    while (pos < len) {
        // The line end: where the header says the payload ends when a '\n'
        // (or the end of the text) is there, else the next '\n'.
        uint64_t le;
        ParsedLine p, probe;
        int rc = parse_header(text, pos, len, &probe);
        uint64_t predicted = UINT64_MAX;
        if (rc == 0) {
            const TextLine& L = probe.line;
            predicted = L.dd ? L.payload + (uint64_t)kDdRecord * L.nfilters
                             : L.payload + 4 * (((uint64_t)L.nfilters * 256 + 2) / 3);
        }
        if (predicted <= len && (predicted == len || text[predicted] == '\n') &&
            !memchr(text + pos, '\n', (size_t)(probe.line.payload - pos))) {
            le = predicted;
        } else {
            const char* q = static_cast<const char*>(memchr(text + pos, '\n', (size_t)(len - pos)));
            le = q ? (uint64_t)(q - text) : len;
        }
        if (le == pos) break;  // an empty line ends the file (sdbf_set.cc:58-59)
        rc = parse_header(text, pos, le, &p);
        if (rc != 0) {
            hdr_bad = (int64_t)pl.size();
            hdr_code = rc;
            break;
        }
        if (total + p.line.nfilters >= (1ull << 32)) return fail(c, SDBFG_ERR_ARG, "set too large");
        p.line.first = (uint32_t)total;
        p.line.item0 = items;
        total += p.line.nfilters;
        items += p.line.dd ? p.line.nfilters : (p.line.nfilters + 2) / 3;
        pl.push_back(std::move(p));
        pos = le + 1;
    }
    const uint32_t nl = (uint32_t)pl.size();
    auto* s = new sdbfg_set();
    s->ctx = c;
    s->n = nl;
    s->serial = next_set_serial();
    s->total_filters = total;
    s->names.resize(nl);
    s->fast.assign(nl, 0);
    s->bf_count.resize(nl);
    s->last_elem.resize(nl);
    s->orig_size.resize(nl);
    s->max_elem.resize(nl);
    s->last_count.resize(nl);
    s->dd_block.resize(nl);
    s->first.resize(nl);
    std::vector<TextLine> lines(nl);
    std::vector<CmpDigest> dig(nl);
    for (uint32_t i = 0; i < nl; i++) {
        ParsedLine& p = pl[i];
        lines[i] = p.line;
        s->names[i] = std::move(p.name);
        s->bf_count[i] = p.line.nfilters;
        s->orig_size[i] = p.orig_size;
        s->max_elem[i] = p.max_elem;
        s->last_count[i] = p.last_count;
        s->dd_block[i] = p.dd_block;
        s->first[i] = p.line.first;
        dig[i] = {p.line.first, p.line.nfilters};
    }
    auto cleanup = [&](int code) {
        s->d_filters.release();
        s->d_meta.release();
        s->d_digests.release();
        delete s;
        return code;
    };
    const uint64_t text_used = nl ? lines[nl - 1].end : 0;
    DevBuf d_text, d_lines, d_flags, d_recs;
    auto release_scratch = [&]() {
        d_text.release();
        d_lines.release();
        d_flags.release();
        d_recs.release();
    };
    if (s->d_filters.ensure(std::max<uint64_t>(1, total) * 256) || s->d_meta.ensure(std::max<uint64_t>(1, total) * 4) ||
        s->d_digests.ensure(std::max<uint32_t>(1, nl) * sizeof(CmpDigest)) ||
        d_text.ensure(std::max<uint64_t>(16, text_used + 16)) ||
        d_lines.ensure(std::max<uint32_t>(1, nl) * sizeof(TextLine)) || d_flags.ensure(std::max<uint32_t>(1, nl) * 4)) {
        release_scratch();
        cudaGetLastError();
        return cleanup(fail(c, SDBFG_ERR_NOMEM, "set load: out of device memory"));
    }
    cudaStream_t st = c->stream;
    std::vector<uint32_t> flags(nl, 0);
    int rc = SDBFG_OK;
    do {
        if (!nl) break;
        cudaError_t e = cudaMemcpyAsync(d_text.p, text, text_used, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(d_lines.p, lines.data(), nl * sizeof(TextLine), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_digests.p, dig.data(), nl * sizeof(CmpDigest), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(d_flags.p, 0, nl * 4, st);
        if (e != cudaSuccess) {
            rc = fail(c, SDBFG_ERR_CUDA, "set load: %s", cudaGetErrorString(e));
            break;
        }
        const uint32_t grid = (uint32_t)std::min<uint64_t>((items + kLoadWarps - 1) / kLoadWarps, (uint64_t)c->sms * 16);
        cudaEvent_t ev_;
        timer_begin(c, "k_text_decode", &ev_, st);
        k_text_decode<<<grid, kLoadWarps * 32, 0, st>>>(d_text.as<uint8_t>(), d_lines.as<TextLine>(), nl, items,
                                                        s->d_filters.as<uint8_t>(), s->d_meta.as<uint32_t>(),
                                                        d_flags.as<uint32_t>());
        timer_end(c, "k_text_decode", ev_, st);
        c->launches += 1;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(flags.data(), d_flags.p, nl * 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            rc = fail(c, SDBFG_ERR_CUDA, "set load: %s", cudaGetErrorString(e));
            break;
        }
        // irregular dd lines: locate the records on the host, decode them in a second launch
        std::vector<TextRecord> recs;
        int64_t scan_bad = -1;
        for (uint32_t i = 0; i < nl; i++) {
            if (!(flags[i] & kLineIrregular) || (flags[i] & kLineBad)) continue;
            if (scan_dd_records(text, lines[i], i, recs) != 0) {
                flags[i] |= kLineBad;
                if (scan_bad < 0) scan_bad = i;
            }
        }
        if (!recs.empty()) {
            if (d_recs.ensure(recs.size() * sizeof(TextRecord))) {
                cudaGetLastError();
                rc = fail(c, SDBFG_ERR_NOMEM, "set load: out of device memory");
                break;
            }
            e = cudaMemcpyAsync(d_recs.p, recs.data(), recs.size() * sizeof(TextRecord), cudaMemcpyHostToDevice, st);
            const uint32_t g2 = (uint32_t)std::min<uint64_t>((recs.size() + kLoadWarps - 1) / kLoadWarps, (uint64_t)c->sms * 16);
            if (e == cudaSuccess) {
                timer_begin(c, "k_text_decode_records", &ev_, st);
                k_text_decode_records<<<g2, kLoadWarps * 32, 0, st>>>(d_text.as<uint8_t>(), d_recs.as<TextRecord>(),
                                                                      (uint32_t)recs.size(), s->d_filters.as<uint8_t>(),
                                                                      s->d_meta.as<uint32_t>(), d_flags.as<uint32_t>());
                timer_end(c, "k_text_decode_records", ev_, st);
                c->launches += 1;
                e = cudaGetLastError();
            }
            std::vector<uint32_t> f2(nl);
            if (e == cudaSuccess) e = cudaMemcpyAsync(f2.data(), d_flags.p, nl * 4, cudaMemcpyDeviceToHost, st);
            if (e == cudaSuccess) e = cudaStreamSynchronize(st);
            if (e != cudaSuccess) {
                rc = fail(c, SDBFG_ERR_CUDA, "set load: %s", cudaGetErrorString(e));
                break;
            }
            for (uint32_t i = 0; i < nl; i++) flags[i] |= f2[i] & kLineBad;
        }
    } while (0);
    release_scratch();
    timer_collect(c);
    if (rc != SDBFG_OK) return cleanup(rc);
    // the reference stops at the first line that throws
    int64_t first_bad = -1;
    for (uint32_t i = 0; i < nl; i++)
        if (flags[i] & kLineBad) {
            first_bad = i;
            break;
        }
    if (first_bad >= 0 || hdr_bad >= 0) {
        const bool payload_first = first_bad >= 0 && (hdr_bad < 0 || first_bad < hdr_bad);
        if (bad_line) *bad_line = payload_first ? first_bad : hdr_bad;
        if (bad_code) *bad_code = payload_first ? -2 : hdr_code;
        return cleanup(fail(c, SDBFG_ERR_FORMAT, "line %lld: malformed SDBF (%d)",
                            (long long)(payload_first ? first_bad : hdr_bad), payload_first ? -2 : hdr_code));
    }
    // element count of each digest's last filter (the swap rule's tie-break)
    std::vector<uint32_t> lastmeta(nl);
    for (uint32_t i = 0; i < nl; i++) {
        const cudaError_t e = cudaMemcpyAsync(&lastmeta[i], s->d_meta.as<uint32_t>() + lines[i].first + lines[i].nfilters - 1,
                                              4, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) return cleanup(fail(c, SDBFG_ERR_CUDA, "set load: %s", cudaGetErrorString(e)));
    }
    if (cudaStreamSynchronize(st) != cudaSuccess) return cleanup(fail(c, SDBFG_ERR_CUDA, "set load: synchronize"));
    for (uint32_t i = 0; i < nl; i++) s->last_elem[i] = lastmeta[i] & 0xFFFFu;
    *out = s;
    return SDBFG_OK;
}

extern "C" int sdbfg_set_digest_info(const sdbfg_set* s, uint32_t i, sdbfg_digest_desc* d) {
    if (!s || !d || i >= s->n) return SDBFG_ERR_ARG;
    memset(d, 0, sizeof *d);
    d->name = s->names[i].c_str();
    d->bf_count = s->bf_count[i];
    d->last_count = s->last_count[i];
    d->max_elem = s->max_elem[i];
    d->dd_block_size = s->dd_block[i];
    d->orig_size = s->orig_size[i];
    return SDBFG_OK;
}

extern "C" int sdbfg_set_read_digest(sdbfg_ctx* c, const sdbfg_set* s, uint32_t i, uint8_t* filters,
                                     uint16_t* elem_counts) {
    if (!c || !s || i >= s->n || !filters) return SDBFG_ERR_ARG;
    CUDA_TRY(c, cudaSetDevice(c->device));
    const uint32_t f0 = s->first[i], nf = s->bf_count[i];
    CUDA_TRY(c, cudaMemcpyAsync(filters, s->d_filters.as<uint8_t>() + 256ull * f0, 256ull * nf, cudaMemcpyDeviceToHost,
                                c->stream));
    std::vector<uint32_t> meta;
    if (elem_counts) {
        meta.resize(nf);
        CUDA_TRY(c, cudaMemcpyAsync(meta.data(), s->d_meta.as<uint32_t>() + f0, 4ull * nf, cudaMemcpyDeviceToHost, c->stream));
    }
    CUDA_TRY(c, cudaStreamSynchronize(c->stream));
    for (uint32_t f = 0; elem_counts && f < nf; f++) elem_counts[f] = (uint16_t)(meta[f] & 0xFFFFu);
    return SDBFG_OK;
}
