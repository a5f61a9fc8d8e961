// sdbf_set.h -- drop-in replacement for sdhash's `class sdbf_set`
// (sdbf/sdbf_set.h:15-96) backed by the GB300 engine: pairwise comparison
// runs as one batched device launch per call instead of an OpenMP loop.
#ifndef SDBF_GB300_COMPAT_SDBF_SET_H
#define SDBF_GB300_COMPAT_SDBF_SET_H

#include <stdint.h>

#include <mutex>
#include <ostream>
#include <string>
#include <vector>

#include "sdbf_class.h"

struct sdbfg_ctx;
struct sdbfg_set;

/// Minimal stand-in for the reference's bloom_filter (sdbf/bloom_filter.h):
/// the per-filter copies sdbf_set::vector_init builds (sdbf_set.cc:408-420).
class bloom_filter {
public:
    bloom_filter(uint8_t* data, uint64_t size, int id, int bf_elem_count, uint16_t hamming);
    ~bloom_filter();
    void set_name(std::string name);
    uint8_t* bf;
    uint64_t bf_size;
    int bl_id;
    uint64_t bf_elem_count;
    uint16_t hamming;
    std::string setname;
};

class sdbf_set {
    friend std::ostream& operator<<(std::ostream& os, const sdbf_set& s);
    friend std::ostream& operator<<(std::ostream& os, const sdbf_set* s);

public:
    sdbf_set();
    sdbf_set(bloom_filter* index);
    sdbf_set(const char* fname);
    ~sdbf_set();
    class sdbf* at(uint32_t pos);
    void add(class sdbf* hash);
    void add(sdbf_set* hashset);
    uint64_t size();
    uint64_t input_size();
    uint64_t filter_count();
    void compare_all(int32_t threshold, bool fast);
    std::string compare_all_quiet(int32_t threshold, int32_t thread_count, bool fast);
    void compare_to(sdbf_set* other, int32_t threshold, uint32_t sample_size, bool fast);
    std::string compare_to_quiet(sdbf_set* other, int32_t threshold, uint32_t sample_size, int32_t thread_count,
                                 bool fast);
    std::string to_string() const;
    std::string index_results() const;
    int empty();
    std::string name() const;
    void set_name(std::string name);
    void set_separator(char sep);
    void vector_init();

public:
    class bloom_filter* index;
    std::vector<class bloom_filter*>* bf_vector;

private:
    static struct sdbfg_set* upload_items(struct sdbfg_ctx* c, std::vector<class sdbf*>& items);
    static void mark_fast(struct sdbfg_ctx* c, struct sdbfg_set* set, const std::vector<class sdbf*>& items);
    std::vector<class sdbf*> items;
    std::string setname;
    std::mutex add_hash_mutex;
    char sep;
};

#endif
