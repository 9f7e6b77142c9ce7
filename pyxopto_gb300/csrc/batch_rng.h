/*
 * batch_rng.h - per-packet multiply-with-carry streams of the batched engine.
 *
 * Every packet (simulation s, packet k) owns a stream whose state is derived
 * from (seed, s, k) with the SplitMix64 finalizer (Steele, Lea and Flood,
 * "Fast splittable pseudorandom number generators", OOPSLA 2014); the
 * multiplier is picked from the safe-prime table.  The tallies therefore do
 * not depend on which thread simulates which packet.  Shared by the device
 * code and the CPU oracle.
 */
#ifndef XOPTO_GB300_BATCH_RNG_H
#define XOPTO_GB300_BATCH_RNG_H
#include <stdint.h>

#if defined(__CUDACC__)
#define BR_FN static __host__ __device__ __forceinline__
#else
#define BR_FN static inline
#endif

BR_FN uint64_t br_splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* MWC state (x, a) of packet k of simulation s.  The carry c = x >> 32 is
   kept below a - 1 and the low word below 2^32 - 1, the validity rules of
   the reference's init_RNG (xopto/src/rng/rng.cpp:77-82). */
BR_FN void br_packet_stream(uint64_t seed, uint32_t sim, uint64_t k, const uint32_t *mult,
                            uint32_t num_mult, uint64_t *x, uint32_t *a) {
    uint64_t h = br_splitmix64(seed ^ br_splitmix64(((uint64_t)sim << 40) ^ k));
    uint64_t h2 = br_splitmix64(h);
    uint32_t m = mult[(uint32_t)(h2 % num_mult)];
    uint32_t c = (uint32_t)(h >> 32) % (m - 1u);
    uint32_t x0 = (uint32_t)h;
    if (x0 == 0xFFFFFFFFu) x0 = 0xFFFFFFFEu;
    if (c == 0u && x0 == 0u) x0 = 1u;
    *x = ((uint64_t)c << 32) | x0;
    *a = m;
}
#endif
