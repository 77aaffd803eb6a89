/* SHA-256 (FIPS 180-4) used by the reference driver's hierarchy digests. */
#ifndef GB_REF_SHA256_H
#define GB_REF_SHA256_H
#include <stddef.h>
#include <stdint.h>

typedef struct
{
   uint32_t      h[8];
   uint64_t      len;
   unsigned char buf[64];
   size_t        fill;
} sha256_ctx;

void sha256_init(sha256_ctx *s);
void sha256_update(sha256_ctx *s, const void *data, size_t n);
void sha256_hex(sha256_ctx *s, char out[65]); /* finishes the digest */

#endif
