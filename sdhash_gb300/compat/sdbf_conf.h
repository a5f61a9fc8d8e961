// sdbf_conf.h -- the reference's configuration object (sdbf/sdbf_conf.h:16-58)
// reduced to what callers set: thread count, warnings and the two
// per-filter element caps.  The digest tables live in the engine.
#ifndef SDBF_GB300_COMPAT_SDBF_CONF_H
#define SDBF_GB300_COMPAT_SDBF_CONF_H

#include <stdint.h>

#define _MAX_ELEM_COUNT 160
#define _MAX_ELEM_COUNT_DD 192
#define FLAG_OFF 0x00
#define FLAG_ON 0x01
#ifndef KB
#define KB 1024
#define MB (KB * KB)
#endif

class sdbf_conf {
public:
    sdbf_conf(uint32_t thread_cnt, uint32_t warnings, uint32_t max_elem_ct, uint32_t max_elem_ct_dd);
    ~sdbf_conf();
    uint32_t thread_cnt;
    uint32_t entr_win_size;
    uint32_t bf_size;
    uint32_t pop_win_size;
    uint32_t block_size;
    uint32_t max_elem;
    uint32_t max_elem_dd;
    uint32_t warnings;
    uint32_t threshold;
    bool popcnt;
};

#endif
