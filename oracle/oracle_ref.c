/*
 * oracle_ref.c -- CPU restatements of the reference's device allocation
 * routines, one warp or one thread at a time, quirks included.
 *
 * TEST INFRASTRUCTURE ONLY (see pbm_oracle.h).  Every function follows the
 * cited reference lines step by step; the golden fixtures produced by
 * running the reference's own code on the GPU (tests/golden/) pin them.
 *
 * Conventions carried over from the reference's types: bitmap words and
 * maps are `int`; `0xffffffff` comparisons are unsigned; shifts by 32 or
 * more follow the PTX rule (result 0), which is what the reference's
 * compiled code does for its `x << n` with n >= 32.
 */
#include "pbm_oracle.h"

#define FULL32 0xffffffffu
#define GUARD_ITERS 10000000L   /* replays stop instead of spinning forever */

static inline int ffs32(uint32_t x) { return x ? __builtin_ctz(x) + 1 : 0; }
static inline int popc32(uint32_t x) { return __builtin_popcount(x); }
static inline int clz32(uint32_t x) { return x ? __builtin_clz(x) : 32; }
static inline uint32_t brev32(uint32_t x) {
    uint32_t r = 0;
    for (int i = 0; i < 32; ++i) r |= ((x >> i) & 1u) << (31 - i);
    return r;
}
/* seed = (tid<<15) + (int16_t)clock(), in 32-bit two's complement */
static inline int32_t ref_seed(int32_t tid, int16_t clk) {
    return (int32_t)(((uint32_t)tid << 15) + (uint32_t)(int32_t)clk);
}

/* source/RandomWalkBasic.cuh:54-74 */
int32_t orc_ref_rwbasic_get(int32_t *map, int32_t n_pages, int32_t tid, int16_t clk,
                            int32_t *steps) {
    int32_t seed = ref_seed(tid, clk);
    seed = orc_lcg(seed);
    uint32_t p = (uint32_t)seed % (uint32_t)n_pages;
    int32_t s = 1;
    for (;;) {
        int32_t old = map[p];
        map[p] = 1;                      /* atomicExch(&map[p], 1) */
        if (old != 1) break;
        seed = orc_lcg(seed);
        p = (uint32_t)seed % (uint32_t)n_pages;
        s++;
        if (s > n_pages / 2) { if (steps) *steps = s; return -2; }  /* reference traps */
    }
    if (steps) *steps = s;
    return (int32_t)p;
}

/* source/RandomWalkBasic_BM.cuh:60-89 */
int32_t orc_ref_rwbm_get(int32_t *words, int32_t n_words, int32_t tid, int16_t clk,
                         int32_t *steps) {
    int32_t seed = ref_seed(tid, clk);
    int32_t s = 0, page = -1;
    long guard = 0;
    while (page == -1) {
        if (++guard > GUARD_ITERS) { page = -2; break; }
        s++;
        seed = orc_lcg(seed);
        uint32_t g = (uint32_t)seed % (uint32_t)n_words;
        while ((uint32_t)words[g] != FULL32) {
            uint32_t v = (uint32_t)words[g];
            int b = ffs32(~v) - 1;
            uint32_t bit = 1u << b;
            uint32_t r = (uint32_t)words[g];
            words[g] = (int32_t)(r | bit);          /* atomicOr */
            if ((r & bit) == 0) {
                /* `groupID<<5 + bitPosition` parses as groupID << (5 + bitPosition) */
                page = (int32_t)orc_shl32(g, 5u + (uint32_t)b);
                break;
            }
        }
    }
    if (steps) *steps = s;
    return page;
}

/* source/CollabRW_BM.cuh:81-94 */
static int ref_fks(uint32_t x, int k) {
    if (popc32(x) < k) return 0;
    int left = 1, right = 32;
    while (left < right) {
        int mid = (left + right) / 2;
        int count = popc32((uint32_t)((1u << mid) - 1u) & x);
        if (count < k) left = mid + 1; else right = mid;
    }
    return left;
}

/* source/CollabRW_BM.cuh:114-160 for one warp (blockDim.x == 32). */
void orc_ref_collab_get(int32_t *words, int32_t n_words, uint32_t active, int32_t block,
                        int16_t clk, int32_t *ids, int32_t *steps) {
    int32_t seed = ref_seed(block, clk);
    int32_t s = 0;
    uint32_t need = active;
    int32_t out[32];
    uint32_t p[32], r[32];
    for (int l = 0; l < 32; ++l) { out[l] = -1; r[l] = 0; p[l] = 0; }
    long guard = 0;
    while (need) {
        if (++guard > GUARD_ITERS) break;
        s++;
        seed = orc_lcg(seed);
        uint32_t has = 0;
        for (int l = 0; l < 32; ++l) {
            if (!(active & (1u << l))) continue;
            p[l] = ((uint32_t)seed + (uint32_t)l) % (uint32_t)n_words;
            uint32_t old = (uint32_t)words[p[l]];
            words[p[l]] = (int32_t)FULL32;          /* atomicExch(..., 0xFFFFFFFF) */
            r[l] = ~old;
            if (r[l]) has |= 1u << l;
        }
        while (need && has) {
            int32_t found[32];
            int src[32];
            for (int l = 0; l < 32; ++l) {
                if (!(active & (1u << l))) continue;
                int sn = popc32(~orc_shl32(FULL32, (uint32_t)l) & need);
                src[l] = ref_fks(has, sn + 1) - 1;
                found[l] = (int32_t)(p[l] * 32u + (uint32_t)(ffs32(r[l]) - 1));
            }
            int np = popc32(need);
            for (int l = 0; l < 32; ++l) {
                if (!(active & (1u << l))) continue;
                if (out[l] == -1 && src[l] != -1) out[l] = found[src[l]];
            }
            for (int l = 0; l < 32; ++l) {
                if (!(active & (1u << l))) continue;
                if (r[l] != 0 && popc32(~orc_shl32(FULL32, (uint32_t)l) & has) < np)
                    r[l] &= ~(1u << (ffs32(r[l]) - 1));
            }
            has = 0; need = 0;
            for (int l = 0; l < 32; ++l) {
                if (!(active & (1u << l))) continue;
                if (r[l]) has |= 1u << l;
                if (out[l] == -1) need |= 1u << l;
            }
        }
        if (need == 0) {
            for (int l = 0; l < 32; ++l) {
                if ((active & (1u << l)) && r[l]) words[p[l]] = (int32_t)~r[l];  /* atomicExch */
            }
        }
    }
    for (int l = 0; l < 32; ++l) {
        if (active & (1u << l)) { ids[l] = out[l]; steps[l] = s; }
    }
}

/* source/CRW_BM.cuh:75-142 */
int32_t orc_ref_crw_get(int32_t *words, int32_t n_words, int32_t *last_group,
                        int8_t *last_bit, int32_t tid, int16_t clk, int32_t *steps) {
    int32_t s = 0;
    {
        int32_t g = last_group[tid];
        int8_t bit = last_bit[tid];
        if (g != -1) {
            if (bit == 31) {
                bit = 0;
                g += 1;
                if (g == n_words - 1) g = 0;
            } else {
                bit++;
            }
            while ((uint32_t)words[g] != FULL32) {
                s++;
                bit = (int8_t)(ffs32(~(uint32_t)words[g]) - 1);
                uint32_t m = 1u << bit;
                uint32_t res = (uint32_t)words[g];
                words[g] = (int32_t)(res | m);
                if ((res & m) == 0) {
                    last_group[tid] = g;
                    last_bit[tid] = bit;
                    if (steps) *steps = s;
                    return g * 32 + bit;
                }
            }
        }
    }
    int32_t seed = ref_seed(tid, clk);
    int32_t page = -1;
    long guard = 0;
    while (page == -1) {
        if (++guard > GUARD_ITERS) { page = -2; break; }
        seed = orc_lcg(seed);
        uint32_t g = (uint32_t)seed % (uint32_t)n_words;
        while ((uint32_t)words[g] != FULL32) {
            s++;
            uint32_t v = (uint32_t)words[g];
            int b = ffs32(~v) - 1;
            uint32_t bit = 1u << b;
            uint32_t r = (uint32_t)words[g];
            words[g] = (int32_t)(r | bit);
            if ((r & bit) == 0) {
                page = (int32_t)orc_shl32(g, 5u + (uint32_t)b);
                last_group[tid] = (int32_t)g;
                last_bit[tid] = (int8_t)b;
                break;
            }
        }
    }
    if (steps) *steps = s;
    return page;
}

/* source/RWMalloc.cuh:159-180 */
int32_t orc_ref_find0range(int32_t *x, int32_t *start) {
    if ((uint32_t)*x == FULL32) return 0;
    uint32_t x_rev = brev32((uint32_t)*x);
    int32_t nl0 = clz32(x_rev);
    if (nl0) {
        *start = 0;
        *x = (int32_t)((uint32_t)*x | ~orc_shl32(FULL32, (uint32_t)nl0));
        return nl0;
    }
    int32_t nl1 = clz32(~x_rev);
    x_rev &= orc_shl32(FULL32, (uint32_t)nl1);
    nl0 = clz32(x_rev);
    *start = nl1;
    int32_t len = nl0 - nl1;
    *x = (int32_t)((uint32_t)*x | ~orc_shl32(FULL32, (uint32_t)len));
    return len;
}

/* source/RWMalloc.cuh:203-248 for one warp. */
void orc_ref_getnpage(int32_t *words, int32_t n_words, int32_t n_pages, uint32_t active,
                      int32_t block, int32_t block_dim, const int32_t *n, int16_t clk,
                      int32_t *ids, int32_t *steps) {
    int leader = ffs32(active) - 1;
    int32_t seed = ref_seed(block * block_dim + leader, clk);
    int32_t out[32], P[32], st[32], len[32];
    for (int l = 0; l < 32; ++l) { out[l] = 0; P[l] = 0; st[l] = 0; len[l] = 0; }
    uint32_t need = 0;
    for (int l = 0; l < 32; ++l) {
        if (!(active & (1u << l))) continue;
        out[l] = n[l] > 0 ? -1 : 0;
        if (out[l] == -1) need |= 1u << l;
    }
    int32_t s = 0;
    long guard = 0;
    while (need) {
        if (++guard > GUARD_ITERS) break;
        s++;
        seed = orc_lcg(seed);
        uint32_t has = 0;
        for (int l = 0; l < 32; ++l) {
            if (!(active & (1u << l))) continue;
            uint32_t p = ((uint32_t)seed + (uint32_t)l) % (uint32_t)n_words;
            P[l] = words[p];
            len[l] = orc_ref_find0range(&P[l], &st[l]);
            if (len[l] > 0) has |= 1u << l;
        }
        while (has && need) {
            for (int t = 0; t < 32; ++t) {
                if (!(has & (1u << t))) continue;
                uint32_t range = ((uint32_t)st[t] << 16) | (uint32_t)len[t];
                int32_t len1 = (int32_t)(range & 0xffffu);
                uint32_t take = 0;
                for (int l = 0; l < 32; ++l) {
                    if (!(active & (1u << l))) continue;
                    if (out[l] == -1 && len1 >= n[l]) take |= 1u << l;
                }
                if (take) {
                    int l = ffs32(take) - 1;
                    int32_t start1 = (int32_t)(range >> 16);
                    uint32_t am = orc_shl32(~orc_shl32(FULL32, (uint32_t)n[l]), (uint32_t)start1);
                    uint32_t p = ((uint32_t)seed + (uint32_t)t) % (uint32_t)n_words;
                    uint32_t res = (uint32_t)words[p];
                    words[p] = (int32_t)(res | am);
                    if ((res & am) == 0) out[l] = (int32_t)(p * 32u + (uint32_t)start1);
                }
            }
            need = 0; has = 0;
            for (int l = 0; l < 32; ++l) {
                if (!(active & (1u << l))) continue;
                if (out[l] == -1) need |= 1u << l;
            }
            for (int l = 0; l < 32; ++l) {
                if (!(active & (1u << l))) continue;
                len[l] = orc_ref_find0range(&P[l], &st[l]);
                if (len[l] > 0) has |= 1u << l;
            }
        }
    }
    for (int l = 0; l < 32; ++l) {
        if (active & (1u << l)) { ids[l] = out[l] % n_pages; steps[l] = s; }
    }
}

/* source/parallelPage.cu:1104-1142 (BITMAP_LENGTH passed as n_words) */
int32_t orc_ref_getxpage_rwbm(int32_t *words, int32_t n_words, int32_t X, int32_t tid,
                              int16_t clk, int32_t *steps) {
    int32_t seed = ref_seed(tid, clk);
    int32_t s = 0, page = -1;
    int found = 0;
    uint32_t xbits = ~orc_shl32(FULL32, (uint32_t)X);
    long guard = 0;
    while (!found) {
        if (++guard > GUARD_ITERS) { page = -2; break; }
        s++;
        seed = orc_lcg(seed);
        uint32_t g = (uint32_t)seed % (uint32_t)n_words;
        while (popc32(~(uint32_t)words[g]) >= X) {
            if (++guard > GUARD_ITERS) break;
            uint32_t v = (uint32_t)words[g];
            int b = ffs32(~v) - 1;
            uint32_t m = orc_shl32(xbits, (uint32_t)b);
            uint32_t r = (uint32_t)words[g];
            words[g] = (int32_t)(r | m);
            if ((r & m) == 0) {
                page = (int32_t)(g * 32u + (uint32_t)b);
                found = 1;
                break;
            } else {
                uint32_t revert = ~(r & m);
                words[g] = (int32_t)((uint32_t)words[g] & revert);
            }
        }
    }
    if (steps) *steps = s;
    return page;
}

/* source/parallelPage.cu:491-509 */
int32_t orc_ref_single_clock(int32_t *map, int32_t n_pages, int32_t *arm, int32_t *steps) {
    int32_t s = 0, p = 0;
    for (;;) {
        s++;
        p = *arm;
        *arm = (int32_t)((uint32_t)*arm + 1u);
        p = p % n_pages;
        if (map[p] == 0) { map[p] = 1; break; }
        if (s > 4 * n_pages) { p = -2; break; }
    }
    if (steps) *steps = s;
    return p;
}

/* source/parallelPage.cu:546-555 */
int32_t orc_ref_dist_clock_arm(int32_t tid, int16_t clk, int32_t n_pages) {
    int32_t seed = ref_seed(tid, clk);
    seed = orc_lcg(seed);
    return seed % n_pages;
}

/* source/parallelPage.cu:571-592 */
int32_t orc_ref_dist_clock(int32_t *map, int32_t n_pages, int32_t *arms, int32_t tid,
                           int32_t *steps) {
    int32_t s = 0, p = 0;
    int found = 0;
    while (!found) {
        s++;
        p = arms[tid] % n_pages;
        if (map[p] == 0) {
            int32_t old = map[p];
            map[p] = 1;
            if (old == 0) found = 1;
        }
        arms[tid] = p + 1;
        if (s > 4 * n_pages) { p = -2; break; }
    }
    if (steps) *steps = s;
    return p;
}
