/*
 * Philox4x32-10 counter-based generator and the keyed draw layout shared by
 * the oracles (the C port in qhg_oracle.c and the reference test build in
 * oracle/ref/).
 *
 * ORACLE / TEST INFRASTRUCTURE ONLY: nothing in the product links this file;
 * the CUDA library carries its own implementation of the same published
 * algorithm (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11).
 *
 * Draw layout (identical in the oracles and the GPU path):
 *   key     = (seed & 0xffffffff, seed >> 32)
 *   counter = (stream block, step, id & 0xffffffff, id >> 32)
 *   draw k of a stream starting at block B is word (k % 4) of the block
 *   B + k / 4.
 * Stream bases (block numbers):
 *   0..63    per-agent action windows, keyed by the agent's ID
 *   64..127  pairing, keyed by the ID of the member of the smaller side
 *   128..    birth (gender, strand picks, crossover, mutation), keyed by
 *            the mother's ID
 */
#ifndef QHG_ORACLE_PHILOX4X32_H
#define QHG_ORACLE_PHILOX4X32_H

#include <stdint.h>

#define QHG_STREAM_ACTIONS 0u
#define QHG_STREAM_PAIR    64u
#define QHG_STREAM_BIRTH   128u

static inline void qhg_oracle_mulhilo32(uint32_t a, uint32_t b, uint32_t *hi, uint32_t *lo) {
    uint64_t p = (uint64_t)a * (uint64_t)b;
    *hi = (uint32_t)(p >> 32);
    *lo = (uint32_t)p;
}

/* one Philox4x32 block with 10 rounds */
static inline void qhg_oracle_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint32_t hi0, lo0, hi1, lo1;
        qhg_oracle_mulhilo32(0xD2511F53u, c0, &hi0, &lo0);
        qhg_oracle_mulhilo32(0xCD9E8D57u, c2, &hi1, &lo1);
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n1 = lo1;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        uint32_t n3 = lo0;
        c0 = n0; c1 = n1; c2 = n2; c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* draw k of the stream (seed, step, id) starting at block `base` */
static inline uint32_t qhg_oracle_draw(uint64_t seed, uint32_t step, int64_t id, uint32_t base, uint32_t k) {
    uint32_t key[2] = { (uint32_t)seed, (uint32_t)(seed >> 32) };
    uint64_t uid = (uint64_t)id;
    uint32_t ctr[4] = { base + k / 4u, step, (uint32_t)uid, (uint32_t)(uid >> 32) };
    uint32_t out[4];
    qhg_oracle_philox4x32_10(ctr, key, out);
    return out[k % 4u];
}

#endif
