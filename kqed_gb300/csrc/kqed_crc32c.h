/* CRC32C (Castagnoli, reflected polynomial 0x82F63B78, zero initial value, no
 * final xor) and the rank-rotated checksum pair that KQED's table files carry.
 * The pair follows src/UTILS/crc32c.c:160-172 of the reference:
 *   work = crc32c(buf); a ^= rotl(work, rank % 29); b ^= rotl(work, rank % 31)
 */
#ifndef KQED_CRC32C_H
#define KQED_CRC32C_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

uint32_t kqed_crc32c(uint32_t crc, const void *buf, size_t len);
void kqed_cksum_accum(uint32_t *a, uint32_t *b, uint32_t rank, const void *buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif
