// sdbf_class.h -- drop-in replacement for sdhash's `class sdbf`
// (sdbf/sdbf_class.h:23-121) backed by the GB300 engine (include/sdbf_gb300.h).
//
// Same constructors, methods, public fields and throw codes as the
// reference, so callers such as sdhash-src/sdhash.cc and
// sdhash-src/sdhash_threads.cc compile against it unchanged.  Digests are
// generated by the sm_103a kernels; comparisons run on the device.
#ifndef SDBF_GB300_COMPAT_SDBF_CLASS_H
#define SDBF_GB300_COMPAT_SDBF_CLASS_H

#include <stdint.h>

#include <istream>
#include <ostream>
#include <string>
#include <vector>

#include "sdbf_conf.h"

class bloom_filter;
struct index_info_s;
typedef struct index_info_s index_info;

class sdbf {
    friend std::ostream& operator<<(std::ostream& os, const sdbf& s);
    friend std::ostream& operator<<(std::ostream& os, const sdbf* s);

public:
    /// parse one SDBF text line (sdbf_class.cc:144); throws -1 / -2
    sdbf(const std::string& str);
    /// digest a file (sdbf_class.cc:34); throws -1 when unreadable / < 512 B
    sdbf(const char* filename, uint32_t dd_block_size);
    /// digest msize bytes read from a stream (sdbf_class.cc:71); throws -3
    sdbf(const char* name, std::istream* ifs, uint32_t dd_block_size, uint64_t msize, index_info* info);
    /// digest a buffer (sdbf_class.cc:115); throws -3 below 512 bytes
    sdbf(const char* name, char* str, uint32_t dd_block_size, uint64_t length, index_info* info);
    ~sdbf();

    const char* name();
    uint64_t size();
    uint64_t input_size();
    /// sdbf_score (sdbf_core.cc:330-389); sample must be 0 (see sdbf_compat.cpp)
    int32_t compare(sdbf* other, uint32_t sample);
    std::string to_string() const;
    std::string get_index_results() const;
    uint8_t* clone_filter(uint32_t position);
    uint32_t filter_count();
    void fast();

    static class sdbf_conf* config;
    static int32_t get_elem_count(sdbf* mine, uint64_t index);

public:
    uint8_t* buffer;    // bf_count * 256 bytes
    uint16_t* hamming;  // popcount per filter
    uint32_t max_elem;

private:
    void create(const char* name);
    void digest(const uint8_t* data, uint64_t len, uint32_t dd_block_size);
    void compute_hamming();

    index_info* info;
    std::string index_results;
    char* hashname;
    uint32_t bf_count;
    uint32_t bf_size;
    uint32_t hash_count;
    uint32_t mask;
    uint32_t last_count;
    uint16_t* elem_counts;
    uint32_t dd_block_size;
    uint64_t orig_file_size;
    bool filenamealloc;
    bool fastmode;

public:
    std::vector<class bloom_filter*>* big_filters;
    friend class sdbf_set;
};

#endif
