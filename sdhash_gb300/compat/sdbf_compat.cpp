// sdbf_compat.cpp -- the reference's sdbf / sdbf_set object API over the
// C ABI of the GB300 engine.
//
// Behaviour kept from the reference:
//  * constructors throw int -1 (unreadable / too-small file), -2 (bad SDBF
//    text), -3 (input below 512 bytes) -- sdbf/sdbf_class.cc:36-37,79-82,
//    116-117,145-153,189-209;
//  * `hashname` is borrowed from the caller except when parsed from text
//    (sdbf_class.cc:157-159,365);
//  * the istream constructor digests `msize` bytes (zero-filled past the
//    bytes actually read) and records the bytes read as the input size
//    (sdbf_class.cc:75-88);
//  * sdbf_set does not own its items (sdbf_set.cc:76-85);
//  * result lines "a<sep>b<sep>%03d" (-1 unpadded) for scores >= threshold,
//    pairs in set order (sdbf_set.cc:239-394).
//  * fast() folds the filters in place (first 64 bytes of each, hamming of
//    the folded bytes) and switches the digest to fast-mode scoring
//    (sdbf_class.cc:425-439); compare_all(fast) folds every item,
//    compare_to(fast) only this set's items (sdbf_set.cc:284-289, 321-331).
// Differences: comparisons run on the device in one batched launch per
// call (so compare_all output is in set order rather than OpenMP order), the
// thread_count argument only matters for the reference's CPU loop, and
// filter sampling (sample > 0, seeded from time() in the reference and hence
// not reproducible) is not offered: such calls fall back to the full
// comparison and report it on stderr.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>

#include "../../include/sdbf_gb300.h"
#include "sdbf_class.h"
#include "sdbf_set.h"

namespace {

sdbfg_ctx* thread_ctx() {
    // one engine context per host thread: the reference builds digests from
    // several threads at once (sdhash-src/sdhash_threads.cc:275-295)
    thread_local struct Holder {
        sdbfg_ctx* c = nullptr;
        ~Holder() {
            if (c) sdbfg_ctx_destroy(c);
        }
    } h;
    if (!h.c) {
        const char* dev = getenv("SDBFG_DEVICE");
        if (sdbfg_ctx_create(dev ? atoi(dev) : 0, &h.c) != SDBFG_OK) {
            fprintf(stderr, "sdbf: no usable CUDA device\n");
            throw -1;
        }
    }
    return h.c;
}

sdbfg_digest_desc describe(const sdbf* s, uint32_t bf_count, uint32_t last_count, const uint16_t* elem_counts,
                           uint32_t max_elem, uint32_t dd, uint64_t orig, const char* name, const uint8_t* buf) {
    sdbfg_digest_desc d{};
    d.name = name;
    d.filters = buf;
    d.elem_counts = elem_counts;
    d.bf_count = bf_count;
    d.last_count = last_count;
    d.max_elem = max_elem;
    d.dd_block_size = dd;
    d.orig_size = orig;
    (void)s;
    return d;
}

}  // namespace

sdbf_conf::sdbf_conf(uint32_t thread_cnt_, uint32_t warnings_, uint32_t max_elem_ct, uint32_t max_elem_ct_dd)
    : thread_cnt(thread_cnt_), entr_win_size(64), bf_size(256), pop_win_size(64), block_size(4 * KB),
      max_elem(max_elem_ct), max_elem_dd(max_elem_ct_dd), warnings(warnings_), threshold(16), popcnt(true) {}
sdbf_conf::~sdbf_conf() {}

sdbf_conf* sdbf::config = new sdbf_conf(1, FLAG_OFF, _MAX_ELEM_COUNT, _MAX_ELEM_COUNT_DD);

// ---------------------------------------------------------------- sdbf
void sdbf::create(const char* name) {
    hashname = const_cast<char*>(name);
    bf_size = 256;
    hash_count = 5;
    mask = 0x7FF;
    bf_count = 1;
    last_count = 0;
    elem_counts = nullptr;
    dd_block_size = 0;
    orig_file_size = 0;
    hamming = nullptr;
    buffer = nullptr;
    info = nullptr;
    filenamealloc = false;
    fastmode = false;
    max_elem = config->max_elem;
    big_filters = new std::vector<bloom_filter*>();
}

void sdbf::compute_hamming() {
    hamming = (uint16_t*)calloc(bf_count ? bf_count : 1, sizeof(uint16_t));
    for (uint32_t i = 0; i < bf_count; i++) {
        uint32_t h = 0;
        for (uint32_t b = 0; b < 256; b += 8) {
            uint64_t w;
            memcpy(&w, buffer + (uint64_t)i * 256 + b, 8);
            h += (uint32_t)__builtin_popcountll(w);
        }
        hamming[i] = (uint16_t)h;
    }
}

void sdbf::digest(const uint8_t* data, uint64_t len, uint32_t dd) {
    sdbfg_ctx* c = thread_ctx();
    const uint64_t off = 0;
    const uint64_t cap = sdbfg_digest_capacity(&len, 1, dd);
    std::vector<uint8_t> filt(cap * 256);
    std::vector<uint16_t> counts(dd ? cap : 0);
    sdbfg_digest_result r{};
    int rc = sdbfg_digest_batch(c, data, &off, &len, 1, dd, filt.data(), cap, dd ? counts.data() : nullptr, &r);
    if (rc != SDBFG_OK) {
        fprintf(stderr, "sdbf: digest failed: %s\n", sdbfg_last_error(c));
        throw -1;
    }
    if (r.status != SDBFG_DIGEST_OK) throw -3;
    bf_count = r.bf_count;
    buffer = (uint8_t*)malloc((size_t)bf_count * 256);
    memcpy(buffer, filt.data() + r.filter_offset * 256, (size_t)bf_count * 256);
    if (dd) {
        max_elem = config->max_elem_dd;
        dd_block_size = dd;
        elem_counts = (uint16_t*)malloc(sizeof(uint16_t) * bf_count);
        memcpy(elem_counts, counts.data() + r.filter_offset, sizeof(uint16_t) * bf_count);
    } else {
        max_elem = config->max_elem;
        last_count = r.last_count;
    }
    compute_hamming();
}

sdbf::sdbf(const char* filename, uint32_t dd) {
    std::ifstream f(filename, std::ios::binary);
    if (!f) throw -1;
    std::vector<char> data((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
    if (data.size() < 512) throw -1;  // process_file(..., MIN_FILE_SIZE, ...) fails
    create(filename);
    orig_file_size = data.size();
    digest(reinterpret_cast<const uint8_t*>(data.data()), data.size(), dd);
}

sdbf::sdbf(const char* name, std::istream* ifs, uint32_t dd, uint64_t msize, index_info* inf) {
    std::vector<char> data(msize, 0);
    ifs->read(data.data(), (std::streamsize)msize);
    const uint64_t got = (uint64_t)ifs->gcount();
    if (got < 512) throw -3;
    create(name);
    info = inf;
    orig_file_size = got;
    digest(reinterpret_cast<const uint8_t*>(data.data()), msize, dd);
}

sdbf::sdbf(const char* name, char* str, uint32_t dd, uint64_t length, index_info* inf) {
    if (length < 512) throw -3;
    create(name);
    info = inf;
    orig_file_size = length;
    digest(reinterpret_cast<const uint8_t*>(str), length, dd);
}

sdbf::sdbf(const std::string& str) {
    create(nullptr);
    sdbfg_digest_desc d{};
    int rc = sdbfg_parse(str.data(), str.size(), &d, nullptr, 0, nullptr, nullptr);
    if (rc == -1) throw -1;
    if (rc != SDBFG_OK) throw -2;
    std::vector<char> name(str.size() + 1);
    buffer = (uint8_t*)malloc((size_t)d.bf_count * 256);
    if (d.dd_block_size) elem_counts = (uint16_t*)malloc(sizeof(uint16_t) * d.bf_count);
    rc = sdbfg_parse(str.data(), str.size(), &d, name.data(), name.size(), buffer, elem_counts);
    if (rc != SDBFG_OK) throw -2;
    filenamealloc = true;
    hashname = strdup(name.data());
    orig_file_size = d.orig_size;
    max_elem = d.max_elem;
    bf_count = d.bf_count;
    last_count = d.last_count;
    dd_block_size = d.dd_block_size;
    compute_hamming();
}

sdbf::~sdbf() {
    free(buffer);
    free(hamming);
    free(elem_counts);
    if (filenamealloc) free(hashname);
    if (big_filters) delete big_filters;
}

const char* sdbf::name() { return hashname; }
uint64_t sdbf::size() { return (uint64_t)bf_size * bf_count; }
uint64_t sdbf::input_size() { return orig_file_size; }
uint32_t sdbf::filter_count() { return bf_count; }
std::string sdbf::get_index_results() const { return index_results; }

uint8_t* sdbf::clone_filter(uint32_t position) {
    if (position >= bf_count) return nullptr;
    uint8_t* f = (uint8_t*)malloc(256);
    memcpy(f, buffer + (uint64_t)position * 256, 256);
    return f;
}

int32_t sdbf::get_elem_count(sdbf* mine, uint64_t index) {
    if (!mine->elem_counts) return index < mine->bf_count - 1 ? (int32_t)mine->max_elem : (int32_t)mine->last_count;
    return mine->elem_counts[index];
}

void sdbf::fast() {
    // bloom_filter::fold(2) (bloom_filter.cc:262-288): OR the halves twice;
    // only the folded 64 bytes are copied back over the filter
    for (uint32_t i = 0; i < bf_count; i++) {
        uint64_t w[32];
        memcpy(w, buffer + (uint64_t)i * 256, 256);
        uint32_t h = 0;
        for (int j = 0; j < 8; j++) {
            w[j] |= w[j + 8] | w[j + 16] | w[j + 24];
            h += (uint32_t)__builtin_popcountll(w[j]);
        }
        memcpy(buffer + (uint64_t)i * 256, w, 64);
        hamming[i] = (uint16_t)h;
    }
    fastmode = true;
}

// digests of a freshly uploaded set that were folded on the host keep their
// fast mode on the device (folding again changes nothing)
void sdbf_set::mark_fast(sdbfg_ctx* c, sdbfg_set* set, const std::vector<sdbf*>& items) {
    for (uint32_t i = 0; i < items.size();) {
        if (!items[i]->fastmode) {
            i++;
            continue;
        }
        uint32_t j = i;
        while (j < items.size() && items[j]->fastmode) j++;
        if (sdbfg_set_fast(c, set, i, j - i) != SDBFG_OK) throw -1;
        i = j;
    }
}

int32_t sdbf::compare(sdbf* other, uint32_t sample) {
    if (sample) fprintf(stderr, "sdbf: filter sampling is not offered; comparing all filters\n");
    if (config->warnings) std::cerr << name() << " vs " << other->name() << std::endl;
    sdbfg_ctx* c = thread_ctx();
    sdbfg_digest_desc d[2] = {
        describe(this, bf_count, last_count, elem_counts, max_elem, dd_block_size, orig_file_size, hashname, buffer),
        describe(other, other->bf_count, other->last_count, other->elem_counts, other->max_elem, other->dd_block_size,
                 other->orig_file_size, other->hashname, other->buffer)};
    sdbfg_set* s = nullptr;
    if (sdbfg_set_upload(c, d, 2, &s) != SDBFG_OK) throw -1;
    for (uint32_t k = 0; k < 2; k++)
        if ((k == 0 ? this : other)->fastmode && sdbfg_set_fast(c, s, k, 1) != SDBFG_OK) throw -1;
    const uint32_t ia = 0, ib = 1;
    int32_t score = -1;
    int rc = sdbfg_score_pairs(c, s, s, &ia, &ib, 1, &score);
    sdbfg_set_free(s);
    if (rc != SDBFG_OK) throw -1;
    return score;
}

std::string sdbf::to_string() const {
    sdbfg_digest_desc d = describe(this, bf_count, last_count, elem_counts, max_elem, dd_block_size, orig_file_size,
                                   hashname ? hashname : "", buffer);
    int64_t n = sdbfg_to_string(&d, nullptr, 0);
    if (n < 0) return std::string();
    std::string out((size_t)n + 1, '\0');
    sdbfg_to_string(&d, &out[0], (uint64_t)n + 1);
    out.resize((size_t)n);
    return out;
}

std::ostream& operator<<(std::ostream& os, const sdbf& s) { return os << s.to_string(); }
std::ostream& operator<<(std::ostream& os, const sdbf* s) { return os << s->to_string(); }

// ------------------------------------------------------------ bloom_filter
bloom_filter::bloom_filter(uint8_t* data, uint64_t size, int id, int elem, uint16_t ham)
    : bf((uint8_t*)malloc(size)), bf_size(size), bl_id(id), bf_elem_count((uint64_t)elem), hamming(ham) {
    memcpy(bf, data, size);
}
bloom_filter::~bloom_filter() { free(bf); }
void bloom_filter::set_name(std::string n) { setname = n; }

// ---------------------------------------------------------------- sdbf_set
sdbf_set::sdbf_set() : index(nullptr), bf_vector(new std::vector<bloom_filter*>()), setname("default"), sep('|') {}

sdbf_set::sdbf_set(bloom_filter* idx) : index(idx), bf_vector(new std::vector<bloom_filter*>()), setname("default"),
                                        sep('|') {}

sdbf_set::sdbf_set(const char* fname) : index(nullptr), bf_vector(new std::vector<bloom_filter*>()), sep('|') {
    std::ifstream ifs(fname, std::ios::binary);
    std::string line;
    while (ifs && std::getline(ifs, line)) {
        if (line.empty()) break;
        setname = fname;
        items.push_back(new sdbf(line));
    }
    vector_init();
}

sdbf_set::~sdbf_set() {
    for (bloom_filter* b : *bf_vector) delete b;
    delete bf_vector;
}

sdbf* sdbf_set::at(uint32_t pos) { return pos < items.size() ? items[pos] : nullptr; }

void sdbf_set::add(sdbf* hash) {
    std::lock_guard<std::mutex> g(add_hash_mutex);
    items.push_back(hash);
}

void sdbf_set::add(sdbf_set* other) {
    for (sdbf* s : other->items) items.push_back(s);
}

uint64_t sdbf_set::size() { return items.size(); }
uint64_t sdbf_set::input_size() {
    uint64_t t = 0;
    for (sdbf* s : items) t += s->input_size();
    return t;
}
uint64_t sdbf_set::filter_count() { return bf_vector->size(); }
int sdbf_set::empty() { return items.empty() ? 1 : 0; }
std::string sdbf_set::name() const { return setname; }
void sdbf_set::set_name(std::string n) { setname = n; }
void sdbf_set::set_separator(char s) { sep = s; }
std::string sdbf_set::index_results() const { return std::string(); }

std::string sdbf_set::to_string() const {
    std::string out;
    for (sdbf* s : items) out += s->to_string();
    return out;
}

std::ostream& operator<<(std::ostream& os, const sdbf_set& s) { return os << s.to_string(); }
std::ostream& operator<<(std::ostream& os, const sdbf_set* s) { return os << s->to_string(); }

void sdbf_set::vector_init() {
    for (uint32_t i = 0; i < items.size(); i++)
        for (uint32_t n = 0; n < items[i]->filter_count(); n++) {
            bloom_filter* b = new bloom_filter(items[i]->buffer + (uint64_t)n * 256, 256, (int)i,
                                               sdbf::get_elem_count(items[i], n), items[i]->hamming[n]);
            b->set_name(items[i]->name());
            bf_vector->push_back(b);
        }
}

sdbfg_set* sdbf_set::upload_items(sdbfg_ctx* c, std::vector<sdbf*>& items) {
    std::vector<sdbfg_digest_desc> d;
    d.reserve(items.size());
    for (sdbf* s : items)
        d.push_back(describe(s, s->bf_count, s->last_count, s->elem_counts, s->max_elem, s->dd_block_size,
                             s->orig_file_size, s->hashname, s->buffer));
    sdbfg_set* out = nullptr;
    if (sdbfg_set_upload(c, d.data(), (uint32_t)d.size(), &out) != SDBFG_OK) {
        fprintf(stderr, "sdbf_set: upload failed: %s\n", sdbfg_last_error(c));
        throw -1;
    }
    mark_fast(c, out, items);
    return out;
}

static void put(std::ostream& out, const char* a, const char* b, char sep, int32_t score) {
    out << a << sep << b;
    if (score != -1) out << sep << std::setw(3) << score << std::endl;
    else out << sep << score << std::endl;
}

std::string sdbf_set::compare_all_quiet(int32_t threshold, int32_t, bool fast) {
    if (fast)
        for (sdbf* s : items) s->fast();
    std::stringstream out;
    out.fill('0');
    const uint64_t n = items.size();
    if (n < 2) return out.str();
    sdbfg_ctx* c = thread_ctx();
    sdbfg_set* s = upload_items(c, items);
    std::vector<int32_t> scores(n * (n - 1) / 2);
    int rc = sdbfg_compare_all(c, s, scores.data());
    sdbfg_set_free(s);
    if (rc != SDBFG_OK) throw -1;
    uint64_t k = 0;
    for (uint64_t i = 0; i < n; i++)
        for (uint64_t j = i + 1; j < n; j++, k++)
            if (scores[k] >= threshold) put(out, items[i]->name(), items[j]->name(), sep, scores[k]);
    return out.str();
}

void sdbf_set::compare_all(int32_t threshold, bool fast) { std::cout << compare_all_quiet(threshold, 0, fast); }

std::string sdbf_set::compare_to_quiet(sdbf_set* other, int32_t threshold, uint32_t sample_size, int32_t,
                                       bool fast) {
    if (sample_size) fprintf(stderr, "sdbf_set: filter sampling is not offered; comparing all filters\n");
    if (fast) {
        // sdbf_set.cc:321-331: the first loop runs over other->size() indices
        // of this set (items.at() throws past its end), the second over this
        // set; the other set is not folded
        for (size_t i = 0; i < other->items.size(); i++) items.at(i)->fast();
        for (sdbf* s : items) s->fast();
    }
    std::stringstream out;
    out.fill('0');
    if (items.empty() || other->items.empty()) return out.str();
    sdbfg_ctx* c = thread_ctx();
    sdbfg_set* q = upload_items(c, items);
    sdbfg_set* t = upload_items(c, other->items);
    std::vector<int32_t> scores(items.size() * other->items.size());
    int rc = sdbfg_compare_to(c, q, t, scores.data());
    sdbfg_set_free(q);
    sdbfg_set_free(t);
    if (rc != SDBFG_OK) throw -1;
    uint64_t k = 0;
    for (uint64_t i = 0; i < items.size(); i++)
        for (uint64_t j = 0; j < other->items.size(); j++, k++)
            if (scores[k] >= threshold) put(out, items[i]->name(), other->items[j]->name(), sep, scores[k]);
    return out.str();
}

void sdbf_set::compare_to(sdbf_set* other, int32_t threshold, uint32_t sample_size, bool fast) {
    std::cout << compare_to_quiet(other, threshold, sample_size, 0, fast);
}
