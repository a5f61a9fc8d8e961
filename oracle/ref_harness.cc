// Oracle harness: drives the UNMODIFIED reference sdhash library (compiled
// from its own sources by oracle/Makefile.ref) through its public C++ API,
// the same calls the reference CLI makes:
//   * stream / block digests:  new sdbf(name, istream*, dd_block, size, NULL)
//     as in sdhash-src/sdhash_threads.cc:258 (stream, -p 1) and :358 (block,
//     files below the 128 MiB segment size);
//   * buffer digests:          new sdbf(name, char*, dd_block, len, NULL)
//     (sdbf/sdbf_class.cc:115, used by the stdin path sdhash_threads.cc:220);
//   * all-pairs / query-target: sdbf_set::compare_all_quiet /
//     compare_to_quiet (sdbf/sdbf_set.cc:278, :360) with one thread so the
//     output order is the set order.
// Test infrastructure only: nothing in the product links or calls this.
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <cstring>
#include <cstdlib>
#include <sys/stat.h>

#include "sdbf_class.h"
#include "sdbf_set.h"
#include "index_info.h"
#include "sdbf_defines.h"

extern "C" {

// Digest `len` bytes; returns a malloc'd SDBF text line (with trailing '\n')
// or NULL when the reference constructor throws (status in *err).
char *ref_digest_buffer(const char *name, const unsigned char *buf,
                        unsigned long long len, unsigned dd_block_size,
                        int *err) {
    *err = 0;
    std::vector<char> copy(buf, buf + len);
    try {
        sdbf *s = new sdbf(name, copy.empty() ? (char *)"" : &copy[0],
                           dd_block_size, len, NULL);
        std::string t = s->to_string();
        delete s;
        char *out = (char *)malloc(t.size() + 1);
        memcpy(out, t.c_str(), t.size() + 1);
        return out;
    } catch (int e) {
        *err = e;
        return NULL;
    }
}

// Score two SDBF text lines with sdbf::compare (sdbf_class.cc:266).
int ref_compare_text(const char *a, const char *b, unsigned sample) {
    try {
        sdbf x((std::string(a))), y((std::string(b)));
        return x.compare(&y, sample);
    } catch (int e) {
        return -1000 + e;
    }
}

// compare_all_quiet over a file of SDBF lines; returns malloc'd result text.
char *ref_compare_all_file(const char *fname, int threshold) {
    sdbf_set set(fname);
    std::string r = set.compare_all_quiet(threshold, 1, false);
    for (uint32_t i = 0; i < set.size(); i++) delete set.at(i);
    char *out = (char *)malloc(r.size() + 1);
    memcpy(out, r.c_str(), r.size() + 1);
    return out;
}

// compare_to_quiet(query set, target set); returns malloc'd result text.
char *ref_compare_to_files(const char *qname, const char *tname,
                           int threshold, unsigned sample) {
    sdbf_set q(qname), t(tname);
    std::string r = q.compare_to_quiet(&t, threshold, sample, 1, false);
    for (uint32_t i = 0; i < q.size(); i++) delete q.at(i);
    for (uint32_t i = 0; i < t.size(); i++) delete t.at(i);
    char *out = (char *)malloc(r.size() + 1);
    memcpy(out, r.c_str(), r.size() + 1);
    return out;
}

// The same two calls with the reference's --fast flag (sdbf::fast folds the
// filters before comparing; compare_to folds only the query set's items,
// sdbf/sdbf_set.cc:321-331).
char *ref_compare_all_file_fast(const char *fname, int threshold) {
    sdbf_set set(fname);
    std::string r = set.compare_all_quiet(threshold, 1, true);
    for (uint32_t i = 0; i < set.size(); i++) delete set.at(i);
    char *out = (char *)malloc(r.size() + 1);
    memcpy(out, r.c_str(), r.size() + 1);
    return out;
}

char *ref_compare_to_files_fast(const char *qname, const char *tname, int threshold) {
    sdbf_set q(qname), t(tname);
    std::string r = q.compare_to_quiet(&t, threshold, 0, 1, true);
    for (uint32_t i = 0; i < q.size(); i++) delete q.at(i);
    for (uint32_t i = 0; i < t.size(); i++) delete t.at(i);
    char *out = (char *)malloc(r.size() + 1);
    memcpy(out, r.c_str(), r.size() + 1);
    return out;
}

// Loads a file of SDBF lines with sdbf_set(const char*) (sdbf_set.cc:51-74).
// On success returns the loaded digests re-encoded with to_string, one per
// line (malloc'd).  When a line throws, returns NULL with the thrown value in
// *err and, in *bad_line, the index of the first line that sdbf(const
// std::string&) rejects when the file is read line by line the same way.
char *ref_load_file(const char *fname, int *err, int *bad_line) {
    *err = 0;
    *bad_line = -1;
    try {
        sdbf_set set(fname);
        std::string r;
        for (uint32_t i = 0; i < set.size(); i++) {
            r += set.at(i)->to_string();
            delete set.at(i);
        }
        char *out = (char *)malloc(r.size() + 1);
        memcpy(out, r.c_str(), r.size() + 1);
        return out;
    } catch (int e) {
        *err = e;
    }
    std::ifstream f(fname, std::ifstream::in | std::ios::binary);
    std::string line;
    for (int i = 0; std::getline(f, line) && !line.empty(); i++) {
        try {
            sdbf s(line);
        } catch (int) {
            *bad_line = i;
            break;
        }
    }
    return NULL;
}

// sdhash --index for one group of inputs (sdhash-src/sdhash_threads.cc:
// 376-470): a new 64 MiB index, every input hashed into a set with the index
// attached (stream mode when dd_block_size is 0, as --index does for files
// below 16 MiB; block mode otherwise), the set written as SDBF text to
// sdbf_path and the index, named after sdbf_path, to idx_path.
int ref_index_build(const char **names, const unsigned char **bufs, const unsigned long long *lens, int n,
                    unsigned dd_block_size, const char *sdbf_path, const char *idx_path) {
    bloom_filter *index1 = new bloom_filter(64ull << 20, 5, 0, 0.01);
    index_info *info = (index_info *)calloc(1, sizeof(index_info));
    info->index = index1;
    sdbf_set *set1 = new sdbf_set(index1);
    for (int i = 0; i < n; i++) {
        std::vector<char> copy(bufs[i], bufs[i] + lens[i]);
        try {
            set1->add(new sdbf(names[i], &copy[0], dd_block_size, lens[i], info));
        } catch (int) {
        }
    }
    std::ofstream os(sdbf_path, std::ios::out | std::ios::binary);
    os << set1->to_string();
    os.close();
    set1->index->set_name(sdbf_path);
    const int rc = set1->index->write_out(idx_path);
    for (uint32_t i = 0; i < set1->size(); i++) delete set1->at(i);
    delete set1;
    delete index1;
    free(info);
    return rc;
}

// sdhash --index-search (sdhash-src/sdhash.cc:231-266, 638-652): the index
// files and the sets beside them loaded as the CLI loads them, every input
// hashed in block mode with that index list, and set1->index_results()
// returned (malloc'd).
char *ref_index_search(const char **idx_paths, const char **set_paths, int nidx, const char **names,
                       const unsigned char **bufs, const unsigned long long *lens, int n, unsigned dd_block_size) {
    std::vector<bloom_filter *> indexlist;
    std::vector<sdbf_set *> setlist;
    index_info *info = (index_info *)calloc(1, sizeof(index_info));
    info->indexlist = &indexlist;
    info->setlist = &setlist;
    for (int i = 0; i < nidx; i++) {
        bloom_filter *b = new bloom_filter(std::string(idx_paths[i]));
        indexlist.push_back(b);
        sdbf_set *tmp = new sdbf_set(set_paths[i]);
        setlist.push_back(tmp);
        tmp->index = b;
    }
    sdbf_set *set1 = new sdbf_set();
    for (int i = 0; i < n; i++) {
        std::vector<char> copy(bufs[i], bufs[i] + lens[i]);
        try {
            set1->add(new sdbf(names[i], &copy[0], dd_block_size, lens[i], info));
        } catch (int) {
        }
    }
    std::string r = set1->index_results();
    for (uint32_t i = 0; i < set1->size(); i++) delete set1->at(i);
    delete set1;
    for (size_t k = 0; k < setlist.size(); k++) {
        for (uint32_t m = 0; m < setlist[k]->size(); m++) delete setlist[k]->at(m);
        delete setlist[k];
        delete indexlist[k];
    }
    free(info);
    char *out = (char *)malloc(r.size() + 1);
    memcpy(out, r.c_str(), r.size() + 1);
    return out;
}

// An index file read by bloom_filter(string) (bloom_filter.cc:87-118): copies
// its filter bytes (up to cap) and returns the filter size, or -1 / -2 as the
// constructor throws.
long long ref_index_bits(const char *path, unsigned char *out, unsigned long long cap) {
    try {
        bloom_filter b((std::string(path)));
        memcpy(out, b.bf, b.bf_size < cap ? b.bf_size : cap);
        return (long long)b.bf_size;
    } catch (int e) {
        return e;
    }
}

void ref_free(void *p) { free(p); }

}  // extern "C"

#ifdef ORACLE_REF_MAIN
static int usage() {
    std::cerr << "usage: sdhash_ref digest [-b KB] files... | "
                 "compare_all set.sdbf [threshold] | "
                 "compare_to q.sdbf t.sdbf [threshold]\n";
    return 2;
}

int main(int argc, char **argv) {
    if (argc < 2) return usage();
    std::string cmd = argv[1];
    if (cmd == "digest") {
        int i = 2;
        uint32_t dd = 0;
        if (argc > 3 && std::string(argv[2]) == "-b") {
            dd = (uint32_t)atoi(argv[3]) * 1024;
            i = 4;
        }
        for (; i < argc; i++) {
            struct stat st;
            if (stat(argv[i], &st)) continue;
            std::ifstream is(argv[i], std::ios::binary);
            try {
                sdbf *s = new sdbf(argv[i], &is, dd, st.st_size, NULL);
                std::cout << s;
                delete s;
            } catch (int e) {
                std::cerr << "skip " << argv[i] << " (" << e << ")\n";
            }
        }
        return 0;
    }
    if (cmd == "compare_all" && argc >= 3) {
        char *r = ref_compare_all_file(argv[2], argc > 3 ? atoi(argv[3]) : 1);
        std::cout << r;
        free(r);
        return 0;
    }
    if (cmd == "compare_to" && argc >= 4) {
        char *r = ref_compare_to_files(argv[2], argv[3],
                                       argc > 4 ? atoi(argv[4]) : 1, 0);
        std::cout << r;
        free(r);
        return 0;
    }
    return usage();
}
#endif
