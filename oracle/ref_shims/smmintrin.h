/* Portable stand-in for <smmintrin.h>: the reference only uses the 64-bit
 * popcount intrinsic, which is semantically a plain popcount.  Lets the
 * reference sources compile on aarch64 as well as x86-64. */
#ifndef ORACLE_SHIM_SMMINTRIN_H
#define ORACLE_SHIM_SMMINTRIN_H
#include <stdint.h>
static inline long long _mm_popcnt_u64(unsigned long long x) { return __builtin_popcountll(x); }
#endif
