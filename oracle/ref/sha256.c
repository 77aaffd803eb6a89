/* SHA-256 (FIPS 180-4, section 6.2) for the reference driver's digests of
 * hierarchy arrays.  Test infrastructure: the digests are compared with
 * hashlib.sha256 of the GPU path's arrays (same bytes: little-endian int32 /
 * float64), so both sides hash identical byte streams. */
#include <stdint.h>
#include <string.h>
#include <stdio.h>

#include "sha256.h"

static const uint32_t K[64] = {
   0x428a2f98u, 0x71374491u, 0xb5c0fbcfu, 0xe9b5dba5u, 0x3956c25bu, 0x59f111f1u, 0x923f82a4u, 0xab1c5ed5u,
   0xd807aa98u, 0x12835b01u, 0x243185beu, 0x550c7dc3u, 0x72be5d74u, 0x80deb1feu, 0x9bdc06a7u, 0xc19bf174u,
   0xe49b69c1u, 0xefbe4786u, 0x0fc19dc6u, 0x240ca1ccu, 0x2de92c6fu, 0x4a7484aau, 0x5cb0a9dcu, 0x76f988dau,
   0x983e5152u, 0xa831c66du, 0xb00327c8u, 0xbf597fc7u, 0xc6e00bf3u, 0xd5a79147u, 0x06ca6351u, 0x14292967u,
   0x27b70a85u, 0x2e1b2138u, 0x4d2c6dfcu, 0x53380d13u, 0x650a7354u, 0x766a0abbu, 0x81c2c92eu, 0x92722c85u,
   0xa2bfe8a1u, 0xa81a664bu, 0xc24b8b70u, 0xc76c51a3u, 0xd192e819u, 0xd6990624u, 0xf40e3585u, 0x106aa070u,
   0x19a4c116u, 0x1e376c08u, 0x2748774cu, 0x34b0bcb5u, 0x391c0cb3u, 0x4ed8aa4au, 0x5b9cca4fu, 0x682e6ff3u,
   0x748f82eeu, 0x78a5636fu, 0x84c87814u, 0x8cc70208u, 0x90befffau, 0xa4506cebu, 0xbef9a3f7u, 0xc67178f2u};

#define ROR(x, n) (((x) >> (n)) | ((x) << (32 - (n))))

static void block(uint32_t h[8], const unsigned char *p)
{
   uint32_t w[64];
   for (int t = 0; t < 16; t++)
   {
      w[t] = ((uint32_t) p[4 * t] << 24) | ((uint32_t) p[4 * t + 1] << 16) | ((uint32_t) p[4 * t + 2] << 8) |
             (uint32_t) p[4 * t + 3];
   }
   for (int t = 16; t < 64; t++)
   {
      uint32_t s0 = ROR(w[t - 15], 7) ^ ROR(w[t - 15], 18) ^ (w[t - 15] >> 3);
      uint32_t s1 = ROR(w[t - 2], 17) ^ ROR(w[t - 2], 19) ^ (w[t - 2] >> 10);
      w[t] = w[t - 16] + s0 + w[t - 7] + s1;
   }
   uint32_t a = h[0], b = h[1], c = h[2], d = h[3], e = h[4], f = h[5], g = h[6], k = h[7];
   for (int t = 0; t < 64; t++)
   {
      uint32_t t1 = k + (ROR(e, 6) ^ ROR(e, 11) ^ ROR(e, 25)) + ((e & f) ^ (~e & g)) + K[t] + w[t];
      uint32_t t2 = (ROR(a, 2) ^ ROR(a, 13) ^ ROR(a, 22)) + ((a & b) ^ (a & c) ^ (b & c));
      k = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
   }
   h[0] += a; h[1] += b; h[2] += c; h[3] += d; h[4] += e; h[5] += f; h[6] += g; h[7] += k;
}

void sha256_init(sha256_ctx *s)
{
   static const uint32_t h0[8] = {0x6a09e667u, 0xbb67ae85u, 0x3c6ef372u, 0xa54ff53au,
                                  0x510e527fu, 0x9b05688cu, 0x1f83d9abu, 0x5be0cd19u};
   memcpy(s->h, h0, sizeof(h0));
   s->len = 0;
   s->fill = 0;
}

void sha256_update(sha256_ctx *s, const void *data, size_t n)
{
   const unsigned char *p = (const unsigned char *) data;
   s->len += n;
   if (s->fill)
   {
      size_t take = 64 - s->fill < n ? 64 - s->fill : n;
      memcpy(s->buf + s->fill, p, take);
      s->fill += take; p += take; n -= take;
      if (s->fill < 64) { return; }
      block(s->h, s->buf);
      s->fill = 0;
   }
   for (; n >= 64; n -= 64, p += 64) { block(s->h, p); }
   memcpy(s->buf, p, n);
   s->fill = n;
}

void sha256_hex(sha256_ctx *s, char out[65])
{
   uint64_t bits = (uint64_t) s->len * 8u;
   unsigned char pad[72];
   size_t np = (s->fill < 56) ? 56 - s->fill : 120 - s->fill;
   memset(pad, 0, sizeof(pad));
   pad[0] = 0x80;
   for (int i = 0; i < 8; i++) { pad[np + i] = (unsigned char)(bits >> (56 - 8 * i)); }
   uint64_t keep = s->len;
   sha256_update(s, pad, np + 8);
   s->len = keep;
   for (int i = 0; i < 8; i++) { snprintf(out + 8 * i, 9, "%08x", s->h[i]); }
   out[64] = 0;
}
