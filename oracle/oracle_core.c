/*
 * oracle_core.c -- CPU oracle: primitives, bitmaps, invariant checker and
 * sequential replays of the product's allocation algorithms.
 *
 * TEST INFRASTRUCTURE ONLY (see pbm_oracle.h).  Each replay runs one
 * request at a time; a GPU launch of the same algorithm with one thread
 * (or one warp for the collaborative walk) must match it bit for bit.
 */
#include "pbm_oracle.h"
#include <stdlib.h>
#include <string.h>

/* ---------------- primitives ---------------- */

/* source/RNG_LCG.cuh:9-12: x' = (int)((1103515245*(long long)x + 12345) % (1<<31)).
 * The divisor 1<<31 is INT_MIN promoted to long long; C remainder truncates
 * toward zero, so the magnitude is reduced mod 2^31 and the sign follows the
 * dividend. */
int32_t orc_lcg(int32_t x) {
    int64_t v = 1103515245LL * (int64_t)x + 12345LL;
    int64_t r = v % 2147483648LL;
    return (int32_t)r;
}

uint32_t orc_idx_mod(int32_t x, uint32_t n) { return (uint32_t)x % n; }

uint32_t orc_idx_hi(int32_t x, uint32_t n) {
    return (uint32_t)((((uint64_t)((uint32_t)x & 0x7fffffffu)) * (uint64_t)n) >> 31);
}

/* murmur3 32-bit finaliser (Appleby) over a linear combination of the
 * stream seed and the request index. */
int32_t orc_seed(uint32_t S, uint32_t r) {
    uint32_t h = r * 0x9E3779B1u + S * 0x85EBCA77u + 0x165667B1u;
    h ^= h >> 16; h *= 0x85EBCA6Bu;
    h ^= h >> 13; h *= 0xC2B2AE35u;
    h ^= h >> 16;
    return (int32_t)(h & 0x7fffffffu);
}

/* splitmix64 output function (Steele, Lea, Flood 2014) applied to a
 * Weyl-sequence counter. */
uint64_t orc_hash64(uint64_t seed, uint64_t ctr) {
    uint64_t z = seed * 0xD1B54A32D192ED03ull + (ctr + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

uint32_t orc_shl32(uint32_t x, uint32_t n) { return n >= 32u ? 0u : (x << n); }

static inline int popc32(uint32_t x) { return __builtin_popcount(x); }
static inline int popc64(uint64_t x) { return __builtin_popcountll(x); }
static inline int ctz32(uint32_t x) { return __builtin_ctz(x); }
static inline int clz32(uint32_t x) { return __builtin_clz(x); }
static inline int ctz64(uint64_t x) { return __builtin_ctzll(x); }

/* lowest k set bits of m */
static uint64_t low_bits64(uint64_t m, int k) {
    uint64_t out = 0;
    while (k-- > 0 && m) { uint64_t b = m & (~m + 1ull); out |= b; m &= m - 1ull; }
    return out;
}

/* ---------------- bitmaps ---------------- */

size_t orc_words_for(uint64_t n_pages, int word_bits) {
    if (word_bits == 64) return (size_t)(((n_pages + 63u) / 64u) * 2u);
    return (size_t)((n_pages + 31u) / 32u);
}

uint64_t orc_thresh53(double occ) {
    if (occ <= 0.0) return 0;
    if (occ >= 1.0) return 1ull << 53;
    return (uint64_t)(occ * 9007199254740992.0);
}

void orc_set_padding(uint32_t *words, uint64_t n_pages) {
    /* pad to the 64-bit word boundary so both word views agree */
    uint64_t end = ((n_pages + 63u) / 64u) * 64u;
    for (uint64_t p = n_pages; p < end; ++p) words[p >> 5] |= 1u << (p & 31u);
}

void orc_prefill_bernoulli(uint32_t *words, uint64_t n_pages, uint64_t thresh53, uint64_t seed) {
    uint64_t nw = ((n_pages + 63u) / 64u) * 2u;
    memset(words, 0, nw * sizeof(uint32_t));
    for (uint64_t p = 0; p < n_pages; ++p) {
        if ((orc_hash64(seed, p) >> 11) < thresh53) words[p >> 5] |= 1u << (p & 31u);
    }
    orc_set_padding(words, n_pages);
}

uint64_t orc_used_pages(const uint32_t *words, uint64_t n_pages) {
    uint64_t full = n_pages / 32u, c = 0;
    for (uint64_t w = 0; w < full; ++w) c += (uint64_t)popc32(words[w]);
    for (uint64_t p = full * 32u; p < n_pages; ++p) c += (words[p >> 5] >> (p & 31u)) & 1u;
    return c;
}

/* ---------------- invariant checker ---------------- */

void orc_check_alloc(const uint32_t *after, const uint32_t *before, uint64_t n_pages,
                     const int32_t *ids, int64_t n, orc_check_t *out) {
    memset(out, 0, sizeof(*out));
    uint32_t *seen = (uint32_t *)calloc((size_t)((n_pages + 31u) / 32u), sizeof(uint32_t));
    for (int64_t i = 0; i < n; ++i) {
        int32_t id = ids[i];
        if (id == -1) { out->n_failed++; continue; }
        if (id < 0 || (uint64_t)id >= n_pages) { out->n_out_of_range++; continue; }
        out->n_ok++;
        uint32_t w = (uint32_t)id >> 5, b = 1u << ((uint32_t)id & 31u);
        if (seen[w] & b) out->n_duplicates++;
        seen[w] |= b;
        if (!(after[w] & b)) out->n_not_marked++;
        if (before && (before[w] & b)) out->n_prefilled++;
    }
    out->used_after = (int64_t)orc_used_pages(after, n_pages);
    free(seen);
}

/* ---------------- product-mode replays ---------------- */

int32_t orc_walk_page(uint32_t *words, uint32_t n_pages, int32_t seed0,
                      uint32_t max_steps, int32_t *steps) {
    int32_t x = seed0;
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = orc_lcg(x);
        uint32_t p = orc_idx_hi(x, n_pages);
        uint32_t w = p >> 5, b = 1u << (p & 31u);
        if (words[w] & b) continue;     /* probe saw a held page */
        words[w] |= b;                  /* atomic OR; sequentially it sticks */
        if (steps) *steps = (int32_t)s;
        return (int32_t)p;
    }
    if (steps) *steps = (int32_t)s;
    return -1;
}

int32_t orc_walk_word(uint32_t *words, uint32_t n_pages, int word_bits, int32_t seed0,
                      uint32_t max_steps, int32_t *steps) {
    int32_t x = seed0;
    uint32_t s = 0;
    if (word_bits == 64) {
        uint32_t L = (uint32_t)((n_pages + 63u) / 64u);
        uint64_t *w64 = (uint64_t *)words;
        while (s < max_steps) {
            ++s;
            x = orc_lcg(x);
            uint32_t w = orc_idx_hi(x, L);
            uint64_t v = w64[w];
            if (v != ~0ull) {
                int b = ctz64(~v);
                w64[w] = v | (1ull << b);
                if (steps) *steps = (int32_t)s;
                return (int32_t)(w * 64u + (uint32_t)b);
            }
        }
    } else {
        uint32_t L = (uint32_t)((n_pages + 31u) / 32u);
        while (s < max_steps) {
            ++s;
            x = orc_lcg(x);
            uint32_t w = orc_idx_hi(x, L);
            uint32_t v = words[w];
            if (v != ~0u) {
                int b = ctz32(~v);
                words[w] = v | (1u << b);
                if (steps) *steps = (int32_t)s;
                return (int32_t)(w * 32u + (uint32_t)b);
            }
        }
    }
    if (steps) *steps = (int32_t)s;
    return -1;
}

void orc_walk_collab(uint32_t *words, uint32_t n_pages, int word_bits, int lanes,
                     const uint8_t *need_in, int32_t seed0, uint32_t stride,
                     uint32_t max_steps, int32_t *ids, int32_t *steps) {
    const int wb = word_bits == 64 ? 64 : 32;
    const uint32_t L = (uint32_t)((n_pages + (uint64_t)wb - 1u) / (uint64_t)wb);
    uint64_t *w64 = (uint64_t *)words;
    uint32_t need = 0;
    for (int i = 0; i < lanes; ++i) {
        if (need_in[i]) { need |= 1u << i; ids[i] = -1; }
    }
    const uint32_t requested = need;
    int32_t x = seed0;
    uint32_t s = 0;
    while (need && s < max_steps) {
        ++s;
        x = orc_lcg(x);
        uint32_t base = orc_idx_hi(x, L);
        uint32_t widx[32];
        uint64_t fr[32];
        int cnt[32];
        for (int i = 0; i < lanes; ++i) {
            widx[i] = (uint32_t)(((uint64_t)base + (uint64_t)i * stride) % L);
            int dup = 0;
            for (int j = 0; j < i; ++j) if (widx[j] == widx[i]) { dup = 1; break; }
            uint64_t v = dup ? ~0ull : (wb == 64 ? w64[widx[i]] : (uint64_t)words[widx[i]] | 0xFFFFFFFF00000000ull);
            fr[i] = ~v;
            cnt[i] = popc64(fr[i]);
        }
        int n = popc32(need), pre = 0;
        int32_t gained[64 * 32];
        int ng = 0;
        for (int i = 0; i < lanes; ++i) {
            int k = n - pre;
            if (k < 0) k = 0;
            if (k > cnt[i]) k = cnt[i];
            pre += cnt[i];
            uint64_t m = low_bits64(fr[i], k);
            if (!m) continue;
            if (wb == 64) w64[widx[i]] |= m; else words[widx[i]] |= (uint32_t)m;
            while (m) {
                int b = ctz64(m);
                m &= m - 1ull;
                gained[ng++] = (int32_t)(widx[i] * (uint32_t)wb + (uint32_t)b);
            }
        }
        int r = 0;
        for (int j = 0; j < lanes && r < ng; ++j) {
            if (need & (1u << j)) { ids[j] = gained[r++]; need &= ~(1u << j); }
        }
    }
    for (int i = 0; i < lanes; ++i) if (requested & (1u << i)) steps[i] = (int32_t)s;
}

int32_t orc_walk_crw(uint32_t *words, uint32_t n_pages, int32_t *cursor, int32_t seed0,
                     uint32_t max_steps, int32_t *steps) {
    const uint32_t L = (uint32_t)((n_pages + 31u) / 32u);
    int32_t s = 0;
    int32_t last = *cursor;
    if (last >= 0) {
        uint32_t w = (uint32_t)last >> 5;
        if (((uint32_t)last & 31u) == 31u) { w += 1u; if (w == L) w = 0; }
        uint32_t v = words[w];
        if (v != ~0u) {
            ++s;
            int b = ctz32(~v);
            words[w] = v | (1u << b);
            *cursor = (int32_t)(w * 32u + (uint32_t)b);
            if (steps) *steps = s;
            return *cursor;
        }
    }
    int32_t x = seed0;
    for (uint32_t j = 0; j < max_steps; ++j) {
        x = orc_lcg(x);
        uint32_t w = orc_idx_hi(x, L);
        uint32_t v = words[w];
        if (v != ~0u) {
            ++s;
            int b = ctz32(~v);
            words[w] = v | (1u << b);
            *cursor = (int32_t)(w * 32u + (uint32_t)b);
            if (steps) *steps = s;
            return *cursor;
        }
    }
    if (steps) *steps = s;
    return -1;
}

int32_t orc_single_clock(uint32_t *words, uint32_t n_pages, uint64_t *arm,
                         uint32_t max_steps, int32_t *steps) {
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        uint64_t a = (*arm)++;
        uint32_t p = (uint32_t)(a % n_pages);
        uint32_t w = p >> 5, b = 1u << (p & 31u);
        if (words[w] & b) continue;
        words[w] |= b;
        if (steps) *steps = (int32_t)s;
        return (int32_t)p;
    }
    if (steps) *steps = (int32_t)s;
    return -1;
}

uint32_t orc_dist_clock_arm0(uint32_t S, uint32_t slot, uint32_t n_pages) {
    return orc_idx_hi(orc_lcg(orc_seed(S, slot)), n_pages);
}

int32_t orc_dist_clock(uint32_t *words, uint32_t n_pages, uint32_t *arm,
                       uint32_t max_steps, int32_t *steps) {
    uint32_t s = 0, a = *arm;
    while (s < max_steps) {
        ++s;
        uint32_t p = a >= n_pages ? a - n_pages : a;
        a = p + 1u;
        uint32_t w = p >> 5, b = 1u << (p & 31u);
        if (words[w] & b) continue;
        words[w] |= b;
        *arm = a;
        if (steps) *steps = (int32_t)s;
        return (int32_t)p;
    }
    *arm = a;
    if (steps) *steps = (int32_t)s;
    return -1;
}

/* bit s of the result is set iff bits s .. s+n-1 of f are all set */
static uint32_t run_starts(uint32_t f, uint32_t n) {
    uint32_t r = f, len = 1;
    while (len < n) {
        uint32_t sh = len < n - len ? len : n - len;
        r &= r >> sh;
        len += sh;
    }
    return r;
}

int32_t orc_walk_run(uint32_t *words, uint32_t n_pages, uint32_t n, int32_t seed0,
                     uint32_t max_steps, int32_t *steps) {
    const uint32_t L = (uint32_t)((n_pages + 31u) / 32u);
    int32_t x = seed0;
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = orc_lcg(x);
        uint32_t w = orc_idx_hi(x, L);
        uint32_t r = run_starts(~words[w], n);
        if (r) {
            uint32_t st = (uint32_t)ctz32(r);
            uint32_t m = (n >= 32u ? ~0u : ((1u << n) - 1u)) << st;
            words[w] |= m;
            if (steps) *steps = (int32_t)s;
            return (int32_t)(w * 32u + st);
        }
    }
    if (steps) *steps = (int32_t)s;
    return -1;
}

static uint32_t bit_range(uint32_t lo, uint32_t hi) {
    return (hi >= 31u ? ~0u : ((1u << (hi + 1u)) - 1u)) & ~((1u << lo) - 1u);
}

static uint32_t span_mask(uint32_t p0, uint32_t n, uint32_t ww) {
    const uint32_t a = p0 >> 5, b = (p0 + n - 1u) >> 5;
    return bit_range(ww == a ? (p0 & 31u) : 0u, ww == b ? ((p0 + n - 1u) & 31u) : 31u);
}

/* Releases n contiguous pages from page id on; the run may cross words. */
void orc_free_run(uint32_t *words, int32_t id, uint32_t n) {
    const uint32_t p0 = (uint32_t)id;
    for (uint32_t ww = p0 >> 5; ww <= (p0 + n - 1u) >> 5; ++ww) words[ww] &= ~span_mask(p0, n, ww);
}

/* First run of n free pages seen from word w on, scanning at most
 * ceil(n/32) + 1 words and never past the last one (-1 if none). */
static int32_t find_span(const uint32_t *words, uint32_t L, uint32_t w, uint32_t n) {
    const uint32_t nscan = (n + 31u) / 32u + 1u;
    uint32_t run = 0, start = 0;
    for (uint32_t k = 0; k < nscan && w + k < L; ++k) {
        const uint32_t ww = w + k;
        const uint32_t val = words[ww];
        const uint32_t lo = val ? (uint32_t)ctz32(val) : 32u;
        if (run > 0u && run + lo >= n) return (int32_t)start;
        if (n <= 32u) {
            const uint32_t r = run_starts(~val, n);
            if (r) return (int32_t)(ww * 32u + (uint32_t)ctz32(r));
        }
        if (val == 0u) {
            if (run == 0u) start = ww * 32u;
            run += 32u;
        } else {
            const uint32_t hi = (uint32_t)clz32(val);
            run = hi;
            start = ww * 32u + 32u - hi;
        }
    }
    return -1;
}

int32_t orc_walk_span(uint32_t *words, uint32_t n_pages, uint32_t n, int32_t seed0,
                      uint32_t max_steps, int32_t *steps) {
    const uint32_t L = (uint32_t)((n_pages + 31u) / 32u);
    int32_t x = seed0;
    uint32_t s = 0;
    while (s < max_steps) {
        ++s;
        x = orc_lcg(x);
        const int32_t found = find_span(words, L, orc_idx_hi(x, L), n);
        if (found < 0) continue;
        const uint32_t p0 = (uint32_t)found;
        for (uint32_t ww = p0 >> 5; ww <= (p0 + n - 1u) >> 5; ++ww) words[ww] |= span_mask(p0, n, ww);
        if (steps) *steps = (int32_t)s;
        return found;
    }
    if (steps) *steps = (int32_t)s;
    return -1;
}

void orc_free_page(uint32_t *words, int32_t id) {
    words[(uint32_t)id >> 5] &= ~(1u << ((uint32_t)id & 31u));
}

/* ---------------- FIFO free list ---------------- */

void orc_fifo_init(orc_fifo_t *q, int32_t *ring, uint32_t capacity, uint32_t n_free) {
    q->ring = ring;
    q->capacity = capacity;
    for (uint32_t i = 0; i < capacity; ++i) ring[i] = i < n_free ? (int32_t)i : -1;
    q->head = 0;
    q->tail = n_free;
    q->avail = n_free;
}

int32_t orc_fifo_get(orc_fifo_t *q) {
    if (q->avail <= 0) return -1;
    q->avail--;
    uint64_t t = q->head++;
    int32_t id = q->ring[t % q->capacity];
    q->ring[t % q->capacity] = -1;
    return id;
}

void orc_fifo_put(orc_fifo_t *q, int32_t id) {
    uint64_t t = q->tail++;
    q->ring[t % q->capacity] = id;
    q->avail++;
}
