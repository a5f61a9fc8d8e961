// sdhash_main.cpp -- native command-line front end with the reference's
// sdhash options (sdhash-src/sdhash.cc:100-652), over the C ABI of
// libsdbf_gb300.so.  Same behaviour as sdhash_gb300/cli.py:
//
//   hashing   files below 16 MiB in stream mode, larger ones in 16 KiB block
//             mode in 128 MiB segments (sdhash.cc:487-605; -b 0 keeps
//             stream mode, -b N puts every file in N KiB block mode);
//             digests in the reference's -p 1 order: the small files, then
//             the large ones, each in argument order;
//   -g        all pairs of the hashed set;
//   -c        all pairs of one SDBF file, or every digest of the first file
//             against every digest of the second;
//   --index-search DIR   block-mode hashing looked up in DIR's index files.
//
//   --index   an index per group of files, as the reference builds them
//             with one thread.
//
// Not offered: -s (filter sampling seeds rand() from time() in the
// reference), --large, --details.
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/sdbf_gb300.h"

namespace {

constexpr uint64_t kMB = 1ull << 20;
constexpr uint64_t kKB = 1ull << 10;
constexpr uint32_t kMinFile = 512;
const char* kVersion = "sdhash_gb300 (sdhash 4.0 digest format, SDBF v3)";

struct Options {
    bool deep = false, target_list = false, compare = false, gen_compare = false, fast = false;
    bool validate = false, version = false, help = false;
    int threshold = 1, block_kb = -1, sample = 0, segment_mb = 128;
    std::string output, separator = "pipe", hash_name, index_search;
    bool have_index_search = false, index = false;
    std::vector<std::string> files;
};

[[noreturn]] void die(const std::string& msg) {
    std::cerr << "sdhash: ERROR: " << msg << std::endl;
    std::exit(1);
}

void usage(std::ostream& os) {
    os << kVersion << "\n\nUsage: sdhash <options> <files>\n"
       << "  -r [ --deep ]              generate SDBFs from directories and files\n"
       << "  -f [ --target-list ]       generate SDBFs from list(s) of filenames\n"
       << "  -c [ --compare ]           compare SDBFs in file, or two SDBF files\n"
       << "  -g [ --gen-compare ]       compare all pairs in source data\n"
       << "  -t [ --threshold ] arg     only show results >=threshold (default 1)\n"
       << "  -b [ --block-size ] arg    hashes input files in nKB blocks\n"
       << "  -p [ --threads ] arg       accepted; the GPU does not use it\n"
       << "  -s [ --sample-size ] arg   not offered (must be 0)\n"
       << "  -z [ --segment-size ] arg  file segment size in MB (default 128)\n"
       << "  -o [ --output ] arg        send output to files\n"
       << "  --separator arg            pipe (default), csv, tab\n"
       << "  --hash-name arg            set name of hash on stdin\n"
       << "  --fast                     shrink sdbf filters for speedup\n"
       << "  --validate                 parse SDBF file to check if it is valid\n"
       << "  --index                    generate indexes while hashing (needs -o)\n"
       << "  --index-search arg         search directory of reference indexes\n"
       << "  --version                  show version info\n"
       << "  -h [ --help ]              produce help message\n";
}

int to_int(const std::string& s, const char* what) {
    char* e = nullptr;
    const long v = std::strtol(s.c_str(), &e, 10);
    if (s.empty() || !e || *e) die(std::string("invalid value for ") + what + ": " + s);
    return (int)v;
}

Options parse_args(int argc, char** argv) {
    Options o;
    auto value = [&](int& i, const char* name) -> std::string {
        const std::string a = argv[i];
        const size_t eq = a.find('=');
        if (a.rfind("--", 0) == 0 && eq != std::string::npos) return a.substr(eq + 1);
        if (i + 1 >= argc) die(std::string("option ") + name + " needs a value");
        return argv[++i];
    };
    for (int i = 1; i < argc; i++) {
        const std::string a = argv[i];
        const std::string key = a.substr(0, a.find('='));
        if (a == "-r" || a == "--deep") o.deep = true;
        else if (a == "-f" || a == "--target-list") o.target_list = true;
        else if (a == "-c" || a == "--compare") o.compare = true;
        else if (a == "-g" || a == "--gen-compare") o.gen_compare = true;
        else if (a == "--fast") o.fast = true;
        else if (a == "--validate") o.validate = true;
        else if (a == "--index") o.index = true;
        else if (a == "--version") o.version = true;
        else if (a == "-h" || a == "--help") o.help = true;
        else if (a == "-t" || key == "--threshold") o.threshold = to_int(value(i, "threshold"), "threshold");
        else if (a == "-b" || key == "--block-size") o.block_kb = to_int(value(i, "block-size"), "block-size");
        else if (a == "-p" || key == "--threads") to_int(value(i, "threads"), "threads");
        else if (a == "-s" || key == "--sample-size") o.sample = to_int(value(i, "sample-size"), "sample-size");
        else if (a == "-z" || key == "--segment-size") o.segment_mb = to_int(value(i, "segment-size"), "segment-size");
        else if (a == "-o" || key == "--output") o.output = value(i, "output");
        else if (key == "--separator") o.separator = value(i, "separator");
        else if (key == "--hash-name") o.hash_name = value(i, "hash-name");
        else if (key == "--index-search") {
            o.index_search = value(i, "index-search");
            o.have_index_search = true;
        } else if (a.size() > 1 && a[0] == '-' && a != "-") die("unknown option " + a);
        else o.files.push_back(a);
    }
    return o;
}

bool is_file(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISREG(st.st_mode);
}
bool is_dir(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}
uint64_t file_size(const std::string& p) {
    struct stat st;
    return stat(p.c_str(), &st) == 0 ? (uint64_t)st.st_size : 0;
}

std::vector<uint8_t> read_file(const std::string& p) {
    std::ifstream f(p, std::ios::binary);
    if (!f) die("cannot read " + p);
    return std::vector<uint8_t>((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
}

// Regular files under a directory, each directory's entries in name order.
void walk_dir(const std::string& dir, std::vector<std::string>& out) {
    DIR* d = opendir(dir.c_str());
    if (!d) return;
    std::vector<std::string> names;
    while (struct dirent* e = readdir(d)) {
        const std::string n = e->d_name;
        if (n != "." && n != "..") names.push_back(n);
    }
    closedir(d);
    std::sort(names.begin(), names.end());
    std::vector<std::string> subdirs;
    for (const auto& n : names) {
        const std::string p = dir + "/" + n;
        if (is_file(p)) out.push_back(p);
        else if (is_dir(p)) subdirs.push_back(p);
    }
    for (const auto& s : subdirs) walk_dir(s, out);
}

std::vector<std::string> collect(const std::vector<std::string>& inputs, bool deep) {
    std::vector<std::string> files;
    for (const auto& p : inputs) {
        if (deep && is_dir(p)) walk_dir(p, files);
        if (is_file(p)) files.push_back(p);
    }
    return files;
}

// sdbf_hash_files_dd's segmentation (sdhash-src/sdhash_threads.cc:300-373):
// (name, offset, length) of each segment digest of a file.
struct Segment {
    std::string name;
    uint64_t off, len;
};
std::vector<Segment> segments(const std::string& path, uint64_t size, uint64_t seg) {
    if (!(size > seg && seg > 0)) return {{path, 0, size}};
    int64_t chunks = (int64_t)(size / seg);
    bool tail = false;
    if (size - seg <= 512) chunks = 0;
    if ((int64_t)size - chunks * (int64_t)seg <= 512) {
        chunks -= 1;
        tail = true;
    }
    std::vector<Segment> out;
    for (int64_t j = 0; j <= chunks; j++) {
        std::string name = path;
        if (j > 0 || chunks > 0) {
            char buf[32];
            snprintf(buf, sizeof buf, ".%04lluM", (unsigned long long)(j * seg / kMB));
            name += buf;
        }
        uint64_t csize = seg;
        if (j == chunks) {
            csize = size - chunks * seg;
            if (tail) csize += size - (chunks + 1) * seg;
        }
        out.push_back({name, j * seg, csize});
    }
    return out;
}

// A digest held on the host, as the reference's sdbf object holds it.
struct Digest {
    std::string name;
    std::vector<uint8_t> filters;
    std::vector<uint16_t> elem_counts;  // block digests
    uint32_t bf_count = 0, last_count = 0, max_elem = 0, dd_block = 0;
    uint64_t orig_size = 0;
    std::vector<uint8_t> hits;          // index search: [bf_count][nidx]
    sdbfg_digest_desc desc() const {
        sdbfg_digest_desc d{};
        d.name = name.c_str();
        d.filters = filters.data();
        d.elem_counts = dd_block ? elem_counts.data() : nullptr;
        d.bf_count = bf_count;
        d.last_count = last_count;
        d.max_elem = max_elem;
        d.dd_block_size = dd_block;
        d.orig_size = orig_size;
        return d;
    }
};

struct Input {
    std::string name;
    std::vector<uint8_t> data;  // the bytes digested (a segment zero-filled past the file's end)
    uint64_t read;              // bytes actually read (the digest's input size)
};

void check(sdbfg_ctx* c, int rc, const char* what) {
    if (rc != SDBFG_OK) die(std::string(what) + ": " + sdbfg_last_error(c));
}

// Digests of the inputs (stream mode when dd == 0); with indexes, block
// mode with the index search.  Inputs below 512 bytes give no digest.
void digest_inputs(sdbfg_ctx* c, const std::vector<Input>& in, uint32_t dd, const std::vector<sdbfg_index*>& idx,
                   bool search, std::vector<Digest>& out) {
    if (in.empty()) return;
    const uint32_t n = (uint32_t)in.size();
    std::vector<uint64_t> offs(n), lens(n);
    uint64_t tot = 0;
    for (uint32_t i = 0; i < n; i++) {
        offs[i] = tot;
        lens[i] = in[i].data.size();
        tot += (lens[i] + 15) & ~15ull;
    }
    std::vector<uint8_t> data(std::max<uint64_t>(16, tot), 0);
    for (uint32_t i = 0; i < n; i++) std::copy(in[i].data.begin(), in[i].data.end(), data.begin() + offs[i]);
    const uint64_t cap = sdbfg_digest_capacity(lens.data(), n, dd);
    std::vector<uint8_t> filters(std::max<uint64_t>(1, cap) * 256);
    std::vector<uint16_t> counts(std::max<uint64_t>(1, cap));
    std::vector<sdbfg_digest_result> res(n);
    const uint32_t nidx = (uint32_t)idx.size();
    std::vector<uint8_t> hits;
    if (search) {
        hits.assign(std::max<uint64_t>(1, cap * nidx), 0);
        std::vector<const sdbfg_index*> cidx(idx.begin(), idx.end());
        check(c, sdbfg_digest_batch_search(c, data.data(), offs.data(), lens.data(), n, dd, filters.data(), cap,
                                           counts.data(), res.data(), cidx.data(), nidx, hits.data()),
              "digest");
    } else {
        check(c, sdbfg_digest_batch(c, data.data(), offs.data(), lens.data(), n, dd, filters.data(), cap,
                                    dd ? counts.data() : nullptr, res.data()),
              "digest");
    }
    for (uint32_t i = 0; i < n; i++) {
        if (res[i].status != SDBFG_DIGEST_OK || in[i].read < kMinFile) continue;
        Digest d;
        d.name = in[i].name;
        d.bf_count = res[i].bf_count;
        d.orig_size = in[i].read;
        d.dd_block = dd;
        d.max_elem = dd ? 192 : 160;
        d.last_count = dd ? 0 : res[i].last_count;
        const uint64_t o = res[i].filter_offset;
        d.filters.assign(filters.begin() + o * 256, filters.begin() + (o + d.bf_count) * 256);
        if (dd) d.elem_counts.assign(counts.begin() + o, counts.begin() + o + d.bf_count);
        if (search) d.hits.assign(hits.begin() + o * nidx, hits.begin() + (o + d.bf_count) * nidx);
        out.push_back(std::move(d));
    }
}

// The segment digests of one file's bytes in block mode (-b): each segment
// digests its length read from the stream, zero-filled past the end, and
// records the bytes actually read (sdbf_class.cc:71-88).
void segment_inputs(const std::string& name, const std::vector<uint8_t>& bytes, uint64_t seg,
                    std::vector<Input>& out) {
    for (const Segment& s : segments(name, bytes.size(), seg)) {
        Input in;
        in.name = s.name;
        in.data.assign(s.len, 0);
        const uint64_t avail = s.off < bytes.size() ? std::min<uint64_t>(s.len, bytes.size() - s.off) : 0;
        std::copy(bytes.begin() + s.off, bytes.begin() + s.off + avail, in.data.begin());
        in.read = avail;
        out.push_back(std::move(in));
    }
}

// Inputs are digested in batches of at most this many bytes.
constexpr uint64_t kBatchBytes = 1ull << 30;

void flush(sdbfg_ctx* c, std::vector<Input>& pend, uint64_t& bytes, uint32_t dd, const std::vector<sdbfg_index*>& idx,
           bool search, std::vector<Digest>& out) {
    digest_inputs(c, pend, dd, idx, search, out);
    pend.clear();
    bytes = 0;
}

// Digests of the files in the reference's set order (small files, then the
// large ones, each in argument order) or of stdin.
std::vector<Digest> hash_files(sdbfg_ctx* c, const std::vector<std::string>& files, int block_kb, uint64_t seg,
                               const std::vector<sdbfg_index*>& idx, bool search, const std::vector<uint8_t>* stdin_data,
                               const std::string& stdin_name) {
    std::vector<Digest> out;
    std::vector<Input> pend;
    uint64_t bytes = 0;
    if (stdin_data) {
        const uint32_t dd = (uint32_t)((block_kb > 0 ? block_kb : 16) * kKB);
        segment_inputs(stdin_name, *stdin_data, seg, pend);
        flush(c, pend, bytes, dd, idx, search, out);
        return out;
    }
    std::vector<std::string> small, large;
    for (const auto& f : files) (file_size(f) < 16 * kMB ? small : large).push_back(f);
    for (int pass = 0; pass < 2; pass++) {
        const bool is_large = pass == 1;
        const auto& group = is_large ? large : small;
        if (group.empty()) continue;
        const bool stream = block_kb == 0 || (block_kb < 0 && !is_large);
        const uint32_t dd = stream ? 0u : (uint32_t)((block_kb < 0 ? 16 : block_kb) * kKB);
        for (const auto& f : group) {
            std::vector<uint8_t> b = read_file(f);
            if (stream) {
                Input in{f, std::move(b), 0};
                in.read = in.data.size();
                bytes += in.data.size();
                pend.push_back(std::move(in));
            } else {
                segment_inputs(f, b, seg, pend);
                bytes += b.size();
            }
            if (bytes >= kBatchBytes) flush(c, pend, bytes, dd, idx, search, out);
        }
        flush(c, pend, bytes, dd, idx, search, out);
    }
    return out;
}

std::string to_text(const Digest& d) {
    const sdbfg_digest_desc desc = d.desc();
    const int64_t n = sdbfg_to_string(&desc, nullptr, 0);
    if (n < 0) die("cannot encode digest " + d.name);
    std::string s((size_t)n + 1, '\0');
    sdbfg_to_string(&desc, &s[0], (uint64_t)n + 1);
    s.resize((size_t)n);
    return s;
}

sdbfg_set* upload(sdbfg_ctx* c, const std::vector<Digest>& ds) {
    std::vector<sdbfg_digest_desc> descs;
    for (const auto& d : ds) descs.push_back(d.desc());
    sdbfg_set* s = nullptr;
    check(c, sdbfg_set_upload(c, descs.data(), (uint32_t)descs.size(), &s), "upload");
    return s;
}

std::vector<std::string> set_names(const sdbfg_set* s) {
    std::vector<std::string> names;
    for (uint32_t i = 0; i < sdbfg_set_size(s); i++) {
        sdbfg_digest_desc d{};
        sdbfg_set_digest_info(s, i, &d);
        names.push_back(d.name ? d.name : "");
    }
    return names;
}

// Result rows as sdbf_set::compare_all / compare_to print them
// (sdbf/sdbf_set.cc:254-262): "a|b|%03d", -1 unpadded.
std::string result_lines(const std::vector<sdbfg_match>& m, const std::vector<std::string>& na,
                         const std::vector<std::string>& nb, char sep) {
    std::string out;
    char buf[32];
    for (const auto& r : m) {
        if (r.score == -1) snprintf(buf, sizeof buf, "%d", r.score);
        else snprintf(buf, sizeof buf, "%03d", r.score);
        out += na[r.i];
        out += sep;
        out += nb[r.j];
        out += sep;
        out += buf;
        out += '\n';
    }
    return out;
}

std::vector<sdbfg_match> matches(sdbfg_ctx* c, const sdbfg_set* a, const sdbfg_set* b, int threshold) {
    std::vector<sdbfg_match> m(1 << 16);
    for (;;) {
        uint64_t count = 0;
        const int rc = b ? sdbfg_compare_to_matches(c, a, b, threshold, m.data(), m.size(), &count)
                         : sdbfg_compare_all_matches(c, a, threshold, m.data(), m.size(), &count);
        if (rc == SDBFG_ERR_CAPACITY) {
            m.resize(count);
            continue;
        }
        check(c, rc, "compare");
        m.resize(count);
        return m;
    }
}

// sdbf_set(const char* fname) through the device loader; nullptr (and a
// message) when a line is malformed, as the reference's constructor throws.
sdbfg_set* load_set(sdbfg_ctx* c, const std::string& path) {
    std::vector<uint8_t> text = is_file(path) ? read_file(path) : std::vector<uint8_t>();
    sdbfg_set* s = nullptr;
    int64_t bad = -1;
    int32_t code = 0;
    const int rc = sdbfg_set_load_text(c, reinterpret_cast<const char*>(text.data()), text.size(), &s, &bad, &code);
    if (rc == SDBFG_ERR_FORMAT) return nullptr;
    check(c, rc, "load");
    return s;
}

void emit(const Options& o, const std::string& text, const char* suffix) {
    if (o.output.empty()) {
        std::cout << text;
        return;
    }
    std::ofstream f(o.output + suffix, std::ios::binary);
    if (!f) die("cannot write to file " + o.output + suffix);
    f << text;
}

// The --index-search list (sdhash.cc:241-266): every regular "*.idx" file
// of the directory in directory order, each with the name of the SDBF set
// beside it (idx_dir + "/" + the file name without ".idx"; sdbf_set(fname)
// names a set after the path only when the file exists).
void load_indexes(sdbfg_ctx* c, const std::string& dir, std::vector<sdbfg_index*>& idx,
                  std::vector<std::string>& names) {
    DIR* d = opendir(dir.c_str());
    if (!d) return;
    while (struct dirent* e = readdir(d)) {
        const std::string n = e->d_name;
        const size_t dot = n.rfind('.');
        if (dot == std::string::npos || dot == 0 || n.substr(dot) != ".idx") continue;
        const std::string path = dir + "/" + n;
        if (!is_file(path)) continue;
        sdbfg_index* x = nullptr;
        const int rc = sdbfg_index_load_file(c, path.c_str(), &x);
        if (rc != SDBFG_OK) die("cannot load index " + path + ": " + sdbfg_last_error(c));
        const std::string set_path = dir + "/" + n.substr(0, dot);
        std::string name;
        if (is_file(set_path)) {
            sdbfg_set* s = load_set(c, set_path);
            if (!s) die("could not load SDBF file " + set_path);
            sdbfg_set_free(s);
            name = set_path;
        }
        idx.push_back(x);
        names.push_back(name);
    }
    closedir(d);
}

// sdbf_set::index_results (sdbf/sdbf_set.cc:161-167): per digest, per block,
// per index with more than 4 hits: "<digest> [<block>] |<set>|<hits>".
std::string index_results(const std::vector<Digest>& ds, const std::vector<std::string>& names) {
    std::string out;
    const size_t nidx = names.size();
    for (const auto& d : ds)
        for (uint32_t b = 0; b < d.bf_count; b++)
            for (size_t i = 0; i < nidx; i++) {
                const unsigned h = d.hits[b * nidx + i];
                if (h > 4) out += d.name + " [" + std::to_string(b) + "] |" + names[i] + "|" + std::to_string(h) + "\n";
            }
    return out;
}

// hash_index_stringlist (sdhash-src/sdhash_threads.cc:376-470) for one of
// the small / large file lists: groups of just over 640 MiB, each hashed
// with a fresh 64 MiB index (small files in stream mode, large ones in
// 16 KiB block mode with 128 MiB segments) and written as <out><k>.sdbf
// and <out><k>.sdbf.idx, k from 0.  The reference's file-list array is
// reproduced as it behaves: after a group its count restarts at 1, so every
// later group also hashes the file left in slot 0; its running size is a C
// int, which wraps modulo 2^32 (a file of 2 GiB or more makes it negative).
void index_files(sdbfg_ctx* c, const std::vector<std::string>& files, const std::string& out, bool large) {
    std::vector<std::string> slots;
    size_t filect = 0;
    int32_t total = 0;
    int count = 0;
    for (size_t i = 0; i < files.size(); i++) {
        if (filect < slots.size()) slots[filect] = files[i];
        else slots.push_back(files[i]);
        total = (int32_t)((uint32_t)total + (uint32_t)file_size(files[i]));
        if (total > (int32_t)(640 * kMB) || i + 1 == files.size()) {
            std::vector<Input> in;
            for (size_t k = 0; k <= filect; k++) {
                std::vector<uint8_t> b = read_file(slots[k]);
                if (large) {
                    segment_inputs(slots[k], b, 128 * kMB, in);
                } else {
                    Input x{slots[k], std::move(b), 0};
                    x.read = x.data.size();
                    in.push_back(std::move(x));
                }
            }
            const uint32_t dd = large ? 16 * (uint32_t)kKB : 0u;
            const uint32_t n = (uint32_t)in.size();
            std::vector<uint64_t> offs(n), lens(n);
            uint64_t tot = 0;
            for (uint32_t j = 0; j < n; j++) {
                offs[j] = tot;
                lens[j] = in[j].data.size();
                tot += (lens[j] + 15) & ~15ull;
            }
            std::vector<uint8_t> data(std::max<uint64_t>(16, tot), 0);
            for (uint32_t j = 0; j < n; j++) std::copy(in[j].data.begin(), in[j].data.end(), data.begin() + offs[j]);
            const uint64_t cap = sdbfg_digest_capacity(lens.data(), n, dd);
            std::vector<uint8_t> filters(std::max<uint64_t>(1, cap) * 256), bits(64 * kMB, 0);
            std::vector<uint16_t> counts(std::max<uint64_t>(1, cap));
            std::vector<sdbfg_digest_result> res(n);
            uint64_t elem = 0;
            check(c, sdbfg_digest_batch_index(c, data.data(), offs.data(), lens.data(), n, dd, filters.data(), cap,
                                              counts.data(), res.data(), bits.data(), bits.size(), &elem),
                  "index");
            std::string text;
            for (uint32_t j = 0; j < n; j++) {
                if (res[j].status != SDBFG_DIGEST_OK || in[j].read < kMinFile) continue;
                Digest d;
                d.name = in[j].name;
                d.bf_count = res[j].bf_count;
                d.orig_size = in[j].read;
                d.dd_block = dd;
                d.max_elem = dd ? 192 : 160;
                d.last_count = dd ? 0 : res[j].last_count;
                const uint64_t o = res[j].filter_offset;
                d.filters.assign(filters.begin() + o * 256, filters.begin() + (o + d.bf_count) * 256);
                if (dd) d.elem_counts.assign(counts.begin() + o, counts.begin() + o + d.bf_count);
                text += to_text(d);
            }
            const std::string name = out + std::to_string(count) + ".sdbf";
            std::ofstream f(name, std::ios::binary);
            if (!f) die("cannot write to file " + name);
            f << text;
            f.close();
            if (sdbfg_index_write_file((name + ".idx").c_str(), bits.data(), bits.size(), elem, 5, name.c_str()) !=
                SDBFG_OK)
                die("cannot write to file " + name + ".idx");
            count++;
            total = 0;
            filect = 0;
        }
        filect++;
    }
}

}  // namespace

int main(int argc, char** argv) {
    Options o = parse_args(argc, argv);
    if (o.version) {
        std::cout << kVersion << std::endl;
        return 0;
    }
    if (o.help) {
        usage(std::cout);
        return 0;
    }
    if (o.sample) {
        std::cerr << "sdhash: filter sampling (-s) is not offered by this engine" << std::endl;
        return -1;
    }
    char sep = '|';
    if (o.separator == "csv") sep = ',';
    else if (o.separator == "tab" || o.separator == "tabs") sep = '\t';
    else if (o.separator != "pipe") die("unknown separator " + o.separator);
    int block_kb = o.block_kb;
    if (block_kb > 16) block_kb = 16;  // sdhash.cc:215-219
    if (block_kb < -1) block_kb = -1;
    const char* dev = std::getenv("SDBFG_DEVICE");
    sdbfg_ctx* c = nullptr;
    if (sdbfg_ctx_create(dev ? std::atoi(dev) : 0, &c) != SDBFG_OK) die("no usable CUDA device");

    if (o.compare) {
        if (o.files.size() != 1 && o.files.size() != 2) {
            std::cerr << "sdhash: ERROR: Comparison requires 1 or 2 arguments." << std::endl;
            return -1;
        }
        std::vector<sdbfg_set*> sets;
        for (const auto& p : o.files) {
            sdbfg_set* s = load_set(c, p);
            if (!s) {
                std::cerr << "sdhash: ERROR: Could not load SDBF file " << p << ". Exiting" << std::endl;
                return -1;
            }
            sets.push_back(s);
        }
        if (sets.size() == 1) {
            if (o.fast) check(c, sdbfg_set_fast(c, sets[0], 0, sdbfg_set_size(sets[0])), "fast");
            const auto names = set_names(sets[0]);
            emit(o, result_lines(matches(c, sets[0], nullptr, o.threshold), names, names, sep), ".compare");
        } else {
            if (o.fast) {
                // sdbf_set.cc:369-378 folds this set's items, indexing them by the
                // other set's size (out of range when the other set is larger)
                if (sdbfg_set_size(sets[1]) > sdbfg_set_size(sets[0]))
                    die("--fast compare: the second set has more digests than the first");
                check(c, sdbfg_set_fast(c, sets[0], 0, sdbfg_set_size(sets[0])), "fast");
            }
            emit(o, result_lines(matches(c, sets[0], sets[1], o.threshold), set_names(sets[0]), set_names(sets[1]), sep),
                 ".compare");
        }
        for (auto* s : sets) sdbfg_set_free(s);
        sdbfg_ctx_destroy(c);
        return 0;
    }
    if (o.validate) {
        for (const auto& p : o.files) {
            if (!is_file(p)) {
                std::cout << "sdhash: ERROR file " << p << " not readable or not found." << std::endl;
                continue;
            }
            sdbfg_set* s = load_set(c, p);
            if (!s) {
                std::cerr << "sdhash: ERROR: Could not load file of SDBFs, " << p << " is empty or invalid." << std::endl;
                continue;
            }
            uint64_t filters = 0, bytes = 0;
            for (uint32_t i = 0; i < sdbfg_set_size(s); i++) {
                sdbfg_digest_desc d{};
                sdbfg_set_digest_info(s, i, &d);
                filters += d.bf_count;
                bytes += d.orig_size;
            }
            std::cout << "sdhash: file " << p << " SDBFs valid, contains " << sdbfg_set_size(s) << " hashes." << std::endl;
            std::cout << "contains " << filters << " bloom filters." << std::endl;
            std::cout << bytes << " total data size. " << std::endl;
            sdbfg_set_free(s);
        }
        sdbfg_ctx_destroy(c);
        return 0;
    }
    if (o.index) {
        if (o.output.empty()) {
            std::cerr << "sdhash:  ERROR: indexing requires output base filename " << std::endl;
            return -1;
        }
        std::vector<std::string> inputs = o.files;
        if (o.target_list) {
            inputs.clear();
            for (const auto& lst : o.files) {
                std::ifstream f(lst);
                std::string ln;
                while (std::getline(f, ln))
                    if (ln.find_first_not_of(" \t\r\n") != std::string::npos) inputs.push_back(ln);
            }
        }
        std::vector<std::string> small, large;
        for (const auto& f : collect(inputs, o.deep)) (file_size(f) < 16 * kMB ? small : large).push_back(f);
        index_files(c, small, o.output, false);  // sdhash.cc:556-561: small, then large, each from k = 0
        index_files(c, large, o.output, true);
        sdbfg_ctx_destroy(c);
        return 0;
    }
    std::vector<sdbfg_index*> idx;
    std::vector<std::string> idx_names;
    const bool search = o.have_index_search;
    if (search) {
        if (block_kb == 0) {
            std::cerr << "ERROR: Index searching only supported in block mode" << std::endl;
            return 0;
        }
        if (block_kb == -1) block_kb = 16;  // sdhash.cc:245-249
        load_indexes(c, o.index_search, idx, idx_names);
    }
    const uint64_t seg = (uint64_t)o.segment_mb * kMB;
    std::vector<Digest> ds;
    if (o.files.size() == 1 && o.files[0] == "-") {
        std::vector<uint8_t> in((std::istreambuf_iterator<char>(std::cin)), std::istreambuf_iterator<char>());
        ds = hash_files(c, {}, block_kb, seg, idx, search, &in, o.hash_name.empty() ? "stdin" : o.hash_name);
    } else {
        std::vector<std::string> inputs = o.files;
        if (o.target_list) {
            inputs.clear();
            for (const auto& lst : o.files) {
                std::ifstream f(lst);
                std::string ln;
                while (std::getline(f, ln))
                    if (ln.find_first_not_of(" \t\r\n") != std::string::npos) inputs.push_back(ln);
            }
        }
        const std::vector<std::string> files = collect(inputs, o.deep);
        if (files.empty()) {
            std::cout << kVersion << "\n\nUsage: sdhash <options> <files>" << std::endl;
            return 0;
        }
        ds = hash_files(c, files, block_kb, seg, idx, search, nullptr, "");
    }
    if (o.gen_compare) {
        sdbfg_set* s = upload(c, ds);
        if (o.fast) check(c, sdbfg_set_fast(c, s, 0, sdbfg_set_size(s)), "fast");
        std::vector<std::string> names;
        for (const auto& d : ds) names.push_back(d.name);
        emit(o, result_lines(matches(c, s, nullptr, o.threshold), names, names, sep), ".compare");
        sdbfg_set_free(s);
    } else if (search) {
        // sdhash.cc:638-652: the hashes are not written; the results go to
        // <output>.idx-result, or to stderr
        const std::string text = index_results(ds, idx_names);
        if (!o.output.empty()) {
            std::ofstream f(o.output + ".idx-result", std::ios::binary);
            f << text;
        } else {
            std::cerr << text;
        }
    } else {
        std::string text;
        for (const auto& d : ds) text += to_text(d);
        emit(o, text, ".sdbf");
    }
    for (auto* x : idx) sdbfg_index_free(x);
    sdbfg_ctx_destroy(c);
    return 0;
}
