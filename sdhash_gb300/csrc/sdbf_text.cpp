// sdbf_text.cpp -- SDBF v3 text encoding and parsing (host side of the
// drop-in format).
//
// Format (sdbf/sdbf_class.cc:293-334):
//   stream: sdbf:03:<namelen>:<name>:<size>:sha1:256:5:7ff:<max_elem>:
//           <bf_count>:<last_count>:<base64 of all filters>\n
//   block:  sdbf-dd:03:<namelen>:<name>:<size>:sha1:256:5:7ff:<max_elem>:
//           <bf_count>:<dd_block_size>{:<elem count %02x>:<base64 of filter>}\n
// Base64 is RFC 4648 with '=' padding (the reference's modp_b64).  The
// reference encodes stream filters in 1536-byte groups; 1536 is a multiple of
// 3, so the grouped encoding equals a one-shot encoding of all filters.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/sdbf_gb300.h"

namespace {

const char kB64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

void b64_encode(const uint8_t* in, size_t len, std::string& out) {
    size_t i = 0;
    for (; i + 2 < len; i += 3) {
        const uint32_t v = ((uint32_t)in[i] << 16) | ((uint32_t)in[i + 1] << 8) | in[i + 2];
        out.push_back(kB64[v >> 18]);
        out.push_back(kB64[(v >> 12) & 63]);
        out.push_back(kB64[(v >> 6) & 63]);
        out.push_back(kB64[v & 63]);
    }
    if (i < len) {
        uint32_t v = (uint32_t)in[i] << 16;
        if (i + 1 < len) v |= (uint32_t)in[i + 1] << 8;
        out.push_back(kB64[v >> 18]);
        out.push_back(kB64[(v >> 12) & 63]);
        out.push_back(i + 1 < len ? kB64[(v >> 6) & 63] : '=');
        out.push_back('=');
    }
}

int b64_val(char c) {
    if (c >= 'A' && c <= 'Z') return c - 'A';
    if (c >= 'a' && c <= 'z') return c - 'a' + 26;
    if (c >= '0' && c <= '9') return c - '0' + 52;
    if (c == '+') return 62;
    if (c == '/') return 63;
    return -1;
}

// Decodes exactly len characters (a multiple of 4); returns bytes or -1.
long b64_decode(const char* in, size_t len, uint8_t* out) {
    if (len % 4) return -1;
    size_t o = 0;
    for (size_t i = 0; i < len; i += 4) {
        int v[4], pad = 0;
        for (int k = 0; k < 4; k++) {
            if (in[i + k] == '=' && i + 4 == len && k >= 2) {
                v[k] = 0;
                pad++;
            } else if ((v[k] = b64_val(in[i + k])) < 0) {
                return -1;
            }
        }
        const uint32_t x = ((uint32_t)v[0] << 18) | ((uint32_t)v[1] << 12) | ((uint32_t)v[2] << 6) | (uint32_t)v[3];
        out[o++] = (uint8_t)(x >> 16);
        if (pad < 2) out[o++] = (uint8_t)(x >> 8);
        if (pad < 1) out[o++] = (uint8_t)x;
    }
    return (long)o;
}

struct Cursor {
    const char* p;
    const char* end;
    bool next(const char** f, size_t* n) {
        if (p > end) return false;
        const char* q = p;
        while (q < end && *q != ':') q++;
        *f = p;
        *n = (size_t)(q - p);
        p = q + 1;
        return true;
    }
    bool number(uint64_t* v, int base = 10) {
        const char* f;
        size_t n;
        if (!next(&f, &n) || n == 0 || n > 20) return false;
        char tmp[24];
        memcpy(tmp, f, n);
        tmp[n] = 0;
        char* e = nullptr;
        *v = strtoull(tmp, &e, base);
        return e && *e == 0;
    }
};

}  // namespace

extern "C" int64_t sdbfg_to_string(const sdbfg_digest_desc* d, char* out, uint64_t cap) {
    if (!d || !d->filters || d->bf_count == 0) return SDBFG_ERR_ARG;
    const char* name = d->name ? d->name : "";
    std::string s;
    s.reserve(128 + strlen(name) + (size_t)d->bf_count * 352);
    char head[256];
    if (!d->elem_counts) {
        snprintf(head, sizeof head, "sdbf:03:%d:", (int)strlen(name));
        s += head;
        s += name;
        snprintf(head, sizeof head, ":%llu:sha1:256:5:7ff:%u:%u:%u:", (unsigned long long)d->orig_size, d->max_elem,
                 d->bf_count, d->last_count);
        s += head;
        b64_encode(d->filters, (size_t)d->bf_count * 256, s);
    } else {
        snprintf(head, sizeof head, "sdbf-dd:03:%d:", (int)strlen(name));
        s += head;
        s += name;
        snprintf(head, sizeof head, ":%llu:sha1:256:5:7ff:%u:%u:%u", (unsigned long long)d->orig_size, d->max_elem,
                 d->bf_count, d->dd_block_size);
        s += head;
        for (uint32_t i = 0; i < d->bf_count; i++) {
            snprintf(head, sizeof head, ":%02x:", d->elem_counts[i]);
            s += head;
            b64_encode(d->filters + (size_t)i * 256, 256, s);
        }
    }
    s.push_back('\n');
    if (out && cap) {
        const size_t k = s.size() < cap - 1 ? s.size() : (size_t)(cap - 1);
        memcpy(out, s.data(), k);
        out[k] = 0;
    }
    return (int64_t)s.size();
}

extern "C" int sdbfg_parse(const char* line, uint64_t len, sdbfg_digest_desc* d, char* name_buf, uint64_t name_cap,
                           uint8_t* filters, uint16_t* elem_counts) {
    if (!line || !d) return SDBFG_ERR_ARG;
    while (len && (line[len - 1] == '\n' || line[len - 1] == '\r')) len--;
    if (len < 344) return -1;  // sdbf_class.cc:145-146
    memset(d, 0, sizeof *d);
    Cursor c{line, line + len};
    const char* f;
    size_t n;
    uint64_t v;
    if (!c.next(&f, &n) || n < 4 || strncmp(f, "sdbf", 4)) return SDBFG_ERR_FORMAT;
    const bool dd = (n == 7 && !strncmp(f, "sdbf-dd", 7));
    if (!c.next(&f, &n)) return SDBFG_ERR_FORMAT;  // version
    if (!c.next(&f, &n)) return SDBFG_ERR_FORMAT;  // name length
    if (!c.next(&f, &n)) return SDBFG_ERR_FORMAT;  // name
    if (name_buf && name_cap) {
        const size_t k = n < name_cap - 1 ? n : (size_t)(name_cap - 1);
        memcpy(name_buf, f, k);
        name_buf[k] = 0;
        d->name = name_buf;
    }
    if (!c.number(&v)) return SDBFG_ERR_FORMAT;
    d->orig_size = v;
    if (!c.next(&f, &n)) return SDBFG_ERR_FORMAT;  // sha1
    if (!c.number(&v) || v != 256) return SDBFG_ERR_FORMAT;
    if (!c.number(&v)) return SDBFG_ERR_FORMAT;    // hash count
    if (!c.next(&f, &n)) return SDBFG_ERR_FORMAT;  // mask
    if (!c.number(&v)) return SDBFG_ERR_FORMAT;
    d->max_elem = (uint32_t)v;
    if (!c.number(&v) || v == 0 || v >= (1ull << 31)) return SDBFG_ERR_FORMAT;
    d->bf_count = (uint32_t)v;
    if (dd) {
        if (!c.number(&v)) return SDBFG_ERR_FORMAT;
        d->dd_block_size = (uint32_t)v;
        if (!filters) return SDBFG_OK;  // sizing call
        for (uint32_t i = 0; i < d->bf_count; i++) {
            if (!c.number(&v, 16)) return SDBFG_ERR_FORMAT;
            if (elem_counts) elem_counts[i] = (uint16_t)v;
            if (!c.next(&f, &n) || n != 344) return SDBFG_ERR_FORMAT;
            if (b64_decode(f, 344, filters + (size_t)i * 256) != 256) return SDBFG_ERR_FORMAT;
        }
        d->elem_counts = elem_counts;
    } else {
        if (!c.number(&v)) return SDBFG_ERR_FORMAT;
        d->last_count = (uint32_t)v;
        if (!filters) return SDBFG_OK;
        const size_t bytes = (size_t)d->bf_count * 256;
        const size_t need = 4 * ((bytes + 2) / 3);
        if ((size_t)(c.end - c.p) < need) return SDBFG_ERR_FORMAT;
        if (b64_decode(c.p, need, filters) != (long)bytes) return SDBFG_ERR_FORMAT;
    }
    d->filters = filters;
    return SDBFG_OK;
}
