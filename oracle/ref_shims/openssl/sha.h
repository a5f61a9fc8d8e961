/* Minimal stand-in for <openssl/sha.h> used only to compile the reference
 * sdhash sources into the oracle harness.  The reference calls exactly one
 * OpenSSL routine on the hot path (SHA1 of a 64-byte feature); it is resolved
 * at link time against the system libcrypto. */
#ifndef ORACLE_SHIM_OPENSSL_SHA_H
#define ORACLE_SHIM_OPENSSL_SHA_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
unsigned char *SHA1(const unsigned char *d, size_t n, unsigned char *md);
#ifdef __cplusplus
}
#endif
#endif
