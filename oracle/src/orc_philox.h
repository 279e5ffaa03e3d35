/* orc_philox.h -- TEST INFRASTRUCTURE (oracle). Not part of the product.
 *
 * Philox4x32-10 counter-based generator, written from the published
 * description (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
 * as 1, 2, 3", SC'11): two 32x32->64 multiplies per round with multipliers
 * 0xD2511F53 / 0xCD9E8D57, Weyl key bump 0x9E3779B9 / 0xBB67AE85, 10 rounds.
 *
 * The uniform stream used everywhere in this project (oracle, reference
 * harness and the CUDA kernels) is defined by:
 *
 *   key  = (seed & 0xffffffff, seed >> 32)
 *   ctr  = (site, (pass << 16) | block, sweep, chain)
 *   out  = philox4x32_10(ctr, key)
 *   draw 2*block   = ((out0 << 32 | out1) >> 11) * 2^-53
 *   draw 2*block+1 = ((out2 << 32 | out3) >> 11) * 2^-53
 *
 * "site" is the parity-ordered site index of the site being updated, "pass"
 * the 0-based index of the half-sweep inside one update_lattice() call, and
 * draw k is the k-th uniform consumed by that site in that pass.  Global
 * (multicanonical) draws use site = 0xffffffff and block = check number.
 * The 53-bit conversion is the same one the reference's dran() applies to
 * its 64-bit Mersenne output (generic/mersenne.c:147-150), so every uniform
 * lies in [0, 1) exactly as the reference's do.
 */
#ifndef ORC_PHILOX_H
#define ORC_PHILOX_H

#include <stdint.h>

#define ORC_GLOBAL_SITE 0xffffffffu

static inline void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4]) {
  uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
  uint32_t k0 = key_in[0], k1 = key_in[1];
  for (int r = 0; r < 10; r++) {
    if (r > 0) { k0 += 0x9E3779B9u; k1 += 0xBB67AE85u; }
    uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)c0;
    uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

static inline double orc_u53(uint32_t hi, uint32_t lo) {
  uint64_t x = ((uint64_t)hi << 32) | (uint64_t)lo;
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

/* One per-site uniform stream. */
typedef struct {
  uint32_t key[2];
  uint32_t site, pass, sweep, chain;
  uint32_t draw;      /* next draw index */
  uint32_t cached_block;
  double cache[2];
  int have_cache;
} orc_stream;

static inline void orc_stream_init(orc_stream* s, uint64_t seed, uint32_t sweep, uint32_t chain) {
  s->key[0] = (uint32_t)(seed & 0xffffffffu);
  s->key[1] = (uint32_t)(seed >> 32);
  s->site = 0; s->pass = 0; s->sweep = sweep; s->chain = chain;
  s->draw = 0; s->have_cache = 0; s->cached_block = 0;
}

static inline void orc_stream_at(orc_stream* s, uint32_t site, uint32_t pass) {
  s->site = site; s->pass = pass; s->draw = 0; s->have_cache = 0;
}

static inline double orc_stream_uniform(orc_stream* s) {
  uint32_t k = s->draw++;
  uint32_t block = k >> 1;
  if (!s->have_cache || s->cached_block != block) {
    uint32_t ctr[4] = { s->site, (s->pass << 16) | (block & 0xffffu), s->sweep, s->chain };
    uint32_t out[4];
    orc_philox4x32_10(ctr, s->key, out);
    s->cache[0] = orc_u53(out[0], out[1]);
    s->cache[1] = orc_u53(out[2], out[3]);
    s->cached_block = block;
    s->have_cache = 1;
  }
  return s->cache[k & 1u];
}

#endif
