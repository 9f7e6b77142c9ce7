/*
 * rng_host.cpp - seeds of the per-thread multiply-with-carry generators.
 *
 * mcgb_rng_safeprimes: the multipliers a of Marsaglia's MWC generator with
 * base 2^32 must make a*2^32 - 1 and a*2^31 - 1 both prime (a "safe prime"
 * pair).  The reference ships a precomputed table of the first 500,000 such
 * a, scanning down from 4294967118 (xopto/src/rng/find_primes.c:40-93, table
 * xopto/data/primes/safeprimes_base32_500k.npz).  Here the table is computed
 * on demand: a segmented sieve over a removes candidates with a small prime
 * factor (a = 2^-32 or 2^-31 mod r), and the survivors get a deterministic
 * Miller-Rabin test for 64-bit integers (bases 2, 325, 9375, 28178, 450775,
 * 9780504, 1795265022, which are exact for every n < 2^64).
 *
 * mcgb_rng_init: expands a 64-bit initializer into stream seeds exactly as
 * the reference's init_RNG (xopto/src/rng/rng.cpp:64-102): the initializer
 * runs an MWC generator with the first multiplier, and each stream i gets
 * a = table[i+1] and x = (c << 32) | x0 with 0 <= c < a, redrawn until
 * x != 0, c < a - 1 and x0 != 2^32 - 1.
 */
#include <cstdint>
#include <cstring>
#include <cmath>
#include <mutex>
#include <vector>
#include "../../include/xopto_gb300.h"

namespace {

typedef unsigned __int128 u128;

uint64_t mulmod(uint64_t a, uint64_t b, uint64_t m) { return (uint64_t)((u128)a * b % m); }

uint64_t powmod(uint64_t b, uint64_t e, uint64_t m) {
    uint64_t r = 1;
    b %= m;
    while (e) {
        if (e & 1) r = mulmod(r, b, m);
        b = mulmod(b, b, m);
        e >>= 1;
    }
    return r;
}

bool is_prime_u64(uint64_t n) {
    if (n < 2) return false;
    static const uint64_t small[] = {2, 3, 5, 7, 11, 13, 17, 19, 23, 29, 31, 37};
    for (uint64_t p : small) {
        if (n % p == 0) return n == p;
    }
    uint64_t d = n - 1;
    int s = 0;
    while ((d & 1) == 0) { d >>= 1; ++s; }
    static const uint64_t bases[] = {2, 325, 9375, 28178, 450775, 9780504, 1795265022};
    for (uint64_t a : bases) {
        uint64_t x = a % n;
        if (x == 0) continue;
        x = powmod(x, d, n);
        if (x == 1 || x == n - 1) continue;
        bool composite = true;
        for (int i = 1; i < s; ++i) {
            x = mulmod(x, x, n);
            if (x == n - 1) { composite = false; break; }
        }
        if (composite) return false;
    }
    return true;
}

/* modular inverse of v mod r (r prime, v not divisible by r) */
uint64_t inv_mod(uint64_t v, uint64_t r) { return powmod(v % r, r - 2, r); }

struct PrimeTable {
    std::mutex mu;
    std::vector<uint32_t> a;          /* found multipliers, descending   */
    uint64_t next = 4294967118ull;    /* next candidate a to examine     */
    std::vector<uint32_t> sieve_primes, res31, res32;

    void init_sieve() {
        if (!sieve_primes.empty()) return;
        const uint32_t B = 1u << 16;
        std::vector<char> comp(B, 0);
        for (uint32_t i = 2; i < B; ++i) {
            if (comp[i]) continue;
            for (uint64_t j = (uint64_t)i * i; j < B; j += i) comp[j] = 1;
            if (i >= 3) {
                sieve_primes.push_back(i);
                res32.push_back((uint32_t)inv_mod(powmod(2, 32, i), i));
                res31.push_back((uint32_t)inv_mod(powmod(2, 31, i), i));
            }
        }
    }

    /* extends the table to at least n entries */
    bool extend(uint32_t n) {
        init_sieve();
        const uint64_t W = 1u << 20;
        std::vector<char> bad(W);
        while (a.size() < n) {
            if (next < W + 2) return false;
            uint64_t hi = next, lo = next - W + 1;   /* window [lo, hi] */
            std::fill(bad.begin(), bad.end(), 0);
            for (size_t k = 0; k < sieve_primes.size(); ++k) {
                uint64_t r = sieve_primes[k];
                uint64_t rs[2] = {res32[k], res31[k]};
                for (uint64_t t : rs) {
                    /* first a >= lo with a = t (mod r) */
                    uint64_t start = lo + ((t + r - lo % r) % r);
                    for (uint64_t v = start; v <= hi; v += r) {
                        /* do not strike the prime itself (never happens for
                           a*2^32-1 > 2^48) */
                        bad[v - lo] = 1;
                    }
                }
            }
            /* scan the window downwards; a request that is satisfied in the
               middle of the window resumes from the next candidate */
            uint64_t v = hi;
            for (; v >= lo; --v) {
                if (a.size() >= n) break;
                if (bad[v - lo]) continue;
                uint64_t p = (v << 32) - 1;
                if (is_prime_u64(p) && is_prime_u64((p - 1) >> 1)) a.push_back((uint32_t)v);
            }
            next = v;   /* == lo - 1 after a full window */
        }
        return true;
    }
};

PrimeTable g_table;

}  // namespace

extern "C" {

int mcgb_rng_safeprimes(uint32_t *host_a, uint32_t n) {
    if (n && !host_a) return MCGB_E_INVALID;
    std::lock_guard<std::mutex> lock(g_table.mu);
    if (!g_table.extend(n)) return MCGB_E_SIZE;
    std::memcpy(host_a, g_table.a.data(), (size_t)n * sizeof(uint32_t));
    return MCGB_OK;
}

int mcgb_rng_init(uint64_t *x, uint32_t *a, uint32_t n, uint64_t xinit) {
    if (n && (!x || !a)) return MCGB_E_INVALID;
    std::vector<uint32_t> fora((size_t)n + 1);
    int r = mcgb_rng_safeprimes(fora.data(), n + 1);
    if (r) return r;
    uint32_t begin = fora[0];
    if ((xinit == 0ull) | (((uint32_t)(xinit >> 32)) >= (begin - 1)) |
        (((uint32_t)xinit) >= 0xffffffffu))
        return MCGB_E_INVALID;
    for (uint32_t i = 0; i < n; ++i) {
        a[i] = fora[i + 1];
        x[i] = 0;
        while ((x[i] == 0) | (((uint32_t)(x[i] >> 32)) >= (fora[i + 1] - 1)) |
               (((uint32_t)x[i]) >= 0xffffffffu)) {
            xinit = (xinit & 0xffffffffull) * begin + (xinit >> 32);
            x[i] = (uint32_t)std::floor(((double)((uint32_t)xinit) / 4294967296.0) * (double)fora[i + 1]);
            x[i] = x[i] << 32;
            xinit = (xinit & 0xffffffffull) * begin + (xinit >> 32);
            x[i] += (uint32_t)xinit;
        }
    }
    return MCGB_OK;
}

}  // extern "C"
