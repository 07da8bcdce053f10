/* TEST INFRASTRUCTURE: the oracle's own copy of the random stream shared by the
 * CPU oracle, the reference harness and (independently implemented) the GPU path.
 *
 * Philox-4x32-10 as published by Salmon, Moraes, Dror & Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3" (SC'11): 10 rounds, multipliers 0xD2511F53 and
 * 0xCD9E8D57, Weyl key increments 0x9E3779B9 and 0xBB67AE85.
 *
 * Draw k of stream s under seed q is lane (k mod 4) of
 * philox(counter = {k/4 lo, k/4 hi, s, 0}, key = {q lo, q hi}).
 * The rand() replacement returns (u32 >> 1), mapped 0 -> 1, so its range is
 * [1, RAND_MAX] with RAND_MAX = 2^31 - 1 (glibc's); the reference's rejection of
 * a zero uniform (E:2598 "if ( r1 == 0 ) goto gen2") therefore never fires and
 * every step consumes a fixed number of draws for the noise. */
#ifndef TIS_ORACLE_RNG_H
#define TIS_ORACLE_RNG_H
#include <stdint.h>

static inline void tis_o_philox4x32_10(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c[2];
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c[0] = n0; c[1] = n1; c[2] = n2; c[3] = n3;
        k0 += 0x9E3779B9u; k1 += 0xBB67AE85u;
    }
}

static inline uint32_t tis_o_draw_u32(uint64_t seed, uint32_t stream, uint64_t k)
{
    uint64_t blk = k >> 2;
    uint32_t c[4] = { (uint32_t)blk, (uint32_t)(blk >> 32), stream, 0u };
    tis_o_philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return c[k & 3u];
}

/* rand()-compatible integer in [1, 2^31-1]. */
static inline int tis_o_rand_value(uint64_t seed, uint32_t stream, uint64_t k)
{
    uint32_t v = tis_o_draw_u32(seed, stream, k) >> 1;
    return v ? (int)v : 1;
}

#define TIS_O_RAND_MAX 2147483647.0
#endif
