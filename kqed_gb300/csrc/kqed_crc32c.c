/* CRC32C, slicing-by-8, tables built at first use from the polynomial. */
#include "kqed_crc32c.h"

static uint32_t T8[8][256];
static int T8_ready = 0;

static void build_tables(void)
{
  for (uint32_t i = 0; i < 256; i++) {
    uint32_t c = i;
    for (int k = 0; k < 8; k++) c = (c & 1u) ? (c >> 1) ^ 0x82F63B78u : (c >> 1);
    T8[0][i] = c;
  }
  for (uint32_t i = 0; i < 256; i++)
    for (int s = 1; s < 8; s++) T8[s][i] = (T8[s - 1][i] >> 8) ^ T8[0][T8[s - 1][i] & 0xffu];
  T8_ready = 1;
}

uint32_t kqed_crc32c(uint32_t crc, const void *buf, size_t len)
{
  if (!T8_ready) build_tables();
  const unsigned char *p = (const unsigned char *)buf;
  while (len >= 8) {
    uint32_t lo, hi;
    /* table-driven over little-endian words; byte order made explicit so the
       result does not depend on host endianness */
    lo = (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
    hi = (uint32_t)p[4] | ((uint32_t)p[5] << 8) | ((uint32_t)p[6] << 16) | ((uint32_t)p[7] << 24);
    lo ^= crc;
    crc = T8[7][lo & 0xff] ^ T8[6][(lo >> 8) & 0xff] ^ T8[5][(lo >> 16) & 0xff] ^
          T8[4][lo >> 24] ^ T8[3][hi & 0xff] ^ T8[2][(hi >> 8) & 0xff] ^
          T8[1][(hi >> 16) & 0xff] ^ T8[0][hi >> 24];
    p += 8;
    len -= 8;
  }
  while (len--) crc = T8[0][(crc ^ *p++) & 0xffu] ^ (crc >> 8);
  return crc;
}

static inline uint32_t rotl32(uint32_t w, uint32_t r)
{
  return r ? (w << r) | (w >> (32u - r)) : w;
}

void kqed_cksum_accum(uint32_t *a, uint32_t *b, uint32_t rank, const void *buf, size_t len)
{
  const uint32_t w = kqed_crc32c(0, buf, len);
  *a ^= rotl32(w, rank % 29u);
  *b ^= rotl32(w, rank % 31u);
}
