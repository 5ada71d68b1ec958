/* Test infrastructure only (parity checker) — see fame_oracle.h.
 *
 * A plain-C restatement of FAME's single-end matching path and of its index
 * build.  Every function cites the reference lines it follows.  Arithmetic is
 * kept in the reference's integer widths (uint16 counts and DP cells, uint32
 * positions) because the results depend on their wrap-around.  Where the
 * reference reads outside a buffer (undefined behaviour) this file defines the
 * read as a non-matching value; those places are marked "outside".
 */
#include "fame_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* CONST.h:35-110 */
#define KMERLEN 32u
#define HTAB_MASK ((1ull << 30) - 1)
#define WINLEN 2048u
#define MISCOUNT 2u
#define ADDMIS 4u
#define NERR (MISCOUNT + ADDMIS) /* ShiftAnd<E>, E = 6 */
#define QTHRESH 5u
#define KMERCUTOFF 1500u
#define SKIPMOD 2u
#define CPGDUMMY 0xffffffffu
#define SEEDBITS 0xDEFDFFFDu /* 0b11011110111111011111111111111101, CONST.h:58 */
#define DP_BAND (2 * MISCOUNT + ADDMIS) /* LevenshtDP<uint16_t, 8>, ReadQueue.cpp:3626 */
#define NBHD 62u                          /* hopscotch_map NeighborhoodSize default */
#define MAX_PROBES (12u * NBHD)          /* MAX_PROBES_FOR_EMPTY_BUCKET */
#define MAXW 8                            /* ShiftAnd words: reads up to 511 bp */

/* ---------------------------------------------------------------------- */
/* spaced-seed ntHash (spaced_nthash/nthash.hpp:20-26, 88-121, 480-498)     */
/* ---------------------------------------------------------------------- */
static const uint64_t NT_A = 0x3c8bfbb395c60474ULL;
static const uint64_t NT_G = 0x20323ed082572324ULL;
static const uint64_t NT_T = 0x295549f54be24456ULL;

static inline uint64_t rotl64(uint64_t v, unsigned s) { s &= 63u; return s ? (v << s) | (v >> (64 - s)) : v; }

/* msTab row for a byte: C and T share the T seed (reduced alphabet), the small
 * indices 1,3,4,7 are the complement slots of the table, everything else 0. */
static inline uint64_t nt_val(uint8_t c)
{
    switch (c) {
        case 'A': case 'a': case 4: return NT_A;
        case 'C': case 'c': case 'T': case 't': case 1: case 7: return NT_T;
        case 'G': case 'g': case 3: return NT_G;
        default: return 0;
    }
}

/* NTPS64 over a whole k-mer; the rolling form of the reference gives the same
 * value because XOR of rotated seeds is position-wise. */
static inline uint64_t spaced_hash(const uint8_t* s)
{
    uint64_t h = 0;
    for (unsigned i = 0; i < KMERLEN; ++i)
        if ((SEEDBITS >> (31 - i)) & 1u) h ^= rotl64(nt_val(s[i]), 31 - i);
    return h;
}

/* ---------------------------------------------------------------------- */
/* sparse view of tabIndex                                                   */
/* ---------------------------------------------------------------------- */
static void bucket_of(const orc_index* ix, uint64_t key, uint64_t* start, uint64_t* len)
{
    uint64_t lo = 0, hi = ix->n_bucket;
    while (lo < hi) {
        uint64_t mid = (lo + hi) >> 1;
        if (ix->bucket_key[mid] < key) lo = mid + 1; else hi = mid;
    }
    if (lo < ix->n_bucket && ix->bucket_key[lo] == key) { *start = ix->bucket_start[lo]; *len = ix->bucket_len[lo]; }
    else { *start = 0; *len = 0; }
}

/* ---------------------------------------------------------------------- */
/* tsl::hopscotch_map<uint32_t, uint16_t, identity hash> insertion model      */
/* (hopscotch_hash.h:597-628 ctor, 1169-1186 load factor, 1243-1300 rehash,  */
/*  1410-1460 insert, 1465-1486 neighbourhood test, 1491-1500 probe,         */
/*  1541-1575 swap; hopscotch_growth_policy.h:58-115 power of two)            */
/* ---------------------------------------------------------------------- */
typedef struct {
    uint64_t nbk;      /* bucket_count(): power of two or 0 */
    uint64_t mask;
    uint64_t size;     /* m_buckets.size() = nbk + NBHD - 1, or 0 */
    uint32_t* key;
    uint64_t* info;    /* bit0 occupied, bit1 overflow, bits 2.. neighbours */
    uint64_t nb_elem;
    uint32_t* ovf;
    uint64_t n_ovf, cap_ovf;
    uint64_t max_thr, min_thr;
} hmap;

static uint64_t round_pow2(uint64_t v)
{
    if (v && !(v & (v - 1))) return v;
    if (v == 0) return 1;
    --v;
    for (unsigned i = 1; i < 64; i *= 2) v |= v >> i;
    return v + 1;
}

static void hm_init(hmap* m, uint64_t bucket_count)
{
    memset(m, 0, sizeof(*m));
    if (bucket_count > 0) {
        bucket_count = round_pow2(bucket_count);
        m->mask = bucket_count - 1;
        m->nbk = bucket_count;
        m->size = bucket_count + NBHD - 1;
        m->key = (uint32_t*)calloc(m->size, sizeof(uint32_t));
        m->info = (uint64_t*)calloc(m->size, sizeof(uint64_t));
    }
    m->max_thr = (uint64_t)((float)m->nbk * 0.9f);
    m->min_thr = (uint64_t)((float)m->nbk * 0.1f);
}

static void hm_free(hmap* m) { free(m->key); free(m->info); free(m->ovf); memset(m, 0, sizeof(*m)); }

static uint64_t hm_next_count(const hmap* m) { return (m->mask + 1) * 2; }

static void hm_insert_at(hmap* m, uint64_t ib, uint32_t key);

static void hm_rehash(hmap* m, uint64_t count)
{
    uint64_t need = (uint64_t)ceilf((float)m->nb_elem / 0.9f);
    if (need > count) count = need;
    hmap nm;
    hm_init(&nm, count);
    if (m->n_ovf) {
        nm.ovf = m->ovf; nm.n_ovf = m->n_ovf; nm.cap_ovf = m->cap_ovf;
        m->ovf = NULL; m->n_ovf = m->cap_ovf = 0;
        nm.nb_elem += nm.n_ovf;
        for (uint64_t i = 0; i < nm.n_ovf; ++i) nm.info[nm.ovf[i] & nm.mask] |= 2u;
    }
    for (uint64_t b = 0; b < m->size; ++b)
        if (m->info[b] & 1u) hm_insert_at(&nm, m->key[b] & nm.mask, m->key[b]);
    hm_free(m);
    *m = nm;
}

static uint64_t hm_find_empty(const hmap* m, uint64_t ib)
{
    uint64_t lim = ib + MAX_PROBES < m->size ? ib + MAX_PROBES : m->size;
    for (; ib < lim; ++ib) if (!(m->info[ib] & 1u)) return ib;
    return m->size;
}

static int hm_swap_closer(hmap* m, uint64_t* ie)
{
    const uint64_t start = *ie - NBHD + 1;
    for (uint64_t tc = start; tc < *ie; ++tc) {
        uint64_t bm = m->info[tc] >> 2;
        uint64_t ts = tc;
        while (bm != 0 && ts < *ie) {
            if (bm & 1u) {
                m->key[*ie] = m->key[ts];
                m->info[*ie] |= 1u;
                m->info[ts] &= ~(uint64_t)1u;
                m->info[tc] ^= 1ull << ((*ie - tc) + 2);
                m->info[tc] ^= 1ull << ((ts - tc) + 2);
                *ie = ts;
                return 1;
            }
            ++ts;
            bm >>= 1;
        }
    }
    return 0;
}

static int hm_nbhd_changes(const hmap* m, uint64_t ib)
{
    const uint64_t nmask = hm_next_count(m) - 1;
    for (uint64_t b = ib; b < m->size && (b - ib) < NBHD; ++b) {
        uint32_t k = m->key[b];
        if ((k & m->mask) != (k & nmask)) return 1;
    }
    return 0;
}

static void hm_insert_at(hmap* m, uint64_t ib, uint32_t key)
{
    if (m->nb_elem - m->n_ovf >= m->max_thr) {
        hm_rehash(m, hm_next_count(m));
        ib = key & m->mask;
    }
    uint64_t ie = hm_find_empty(m, ib);
    if (ie < m->size) {
        do {
            if (ie - ib < NBHD) {
                m->key[ie] = key;
                m->info[ie] |= 1u;
                m->info[ib] ^= 1ull << ((ie - ib) + 2);
                m->nb_elem++;
                return;
            }
        } while (hm_swap_closer(m, &ie));
    }
    if (m->nb_elem < m->min_thr || !hm_nbhd_changes(m, ib)) {
        if (m->n_ovf == m->cap_ovf) {
            m->cap_ovf = m->cap_ovf ? 2 * m->cap_ovf : 16;
            m->ovf = (uint32_t*)realloc(m->ovf, m->cap_ovf * sizeof(uint32_t));
        }
        m->ovf[m->n_ovf++] = key;
        m->info[ib] |= 2u;
        m->nb_elem++;
        return;
    }
    hm_rehash(m, hm_next_count(m));
    hm_insert_at(m, key & m->mask, key);
}

/* exact membership + uint16 counts for the keys of one map (a plain open-
 * addressing side table; the hopscotch model above only tracks positions). */
typedef struct { uint64_t cap; uint32_t* k; uint16_t* c; uint8_t* used; } cset;

static void cs_init(cset* s, uint64_t n)
{
    s->cap = 16;
    while (s->cap < 2 * n + 16) s->cap <<= 1;
    s->k = (uint32_t*)malloc(s->cap * sizeof(uint32_t));
    s->c = (uint16_t*)calloc(s->cap, sizeof(uint16_t));
    s->used = (uint8_t*)calloc(s->cap, 1);
}
static void cs_free(cset* s) { free(s->k); free(s->c); free(s->used); }
static uint16_t* cs_find(cset* s, uint32_t key)
{
    uint64_t h = (key * 0x9E3779B97F4A7C15ULL) >> 20;
    for (uint64_t i = h & (s->cap - 1);; i = (i + 1) & (s->cap - 1)) {
        if (!s->used[i]) return NULL;
        if (s->k[i] == key) return &s->c[i];
    }
}
static uint16_t* cs_add(cset* s, uint32_t key)
{
    uint64_t h = (key * 0x9E3779B97F4A7C15ULL) >> 20;
    for (uint64_t i = h & (s->cap - 1);; i = (i + 1) & (s->cap - 1)) {
        if (!s->used[i]) { s->used[i] = 1; s->k[i] = key; s->c[i] = 0; return &s->c[i]; }
        if (s->k[i] == key) return &s->c[i];
    }
}

/* The two per-read maps of getSeedRefs. */
typedef struct { hmap hm[2]; cset cs[2]; } seedmaps; /* [0] = rev, [1] = fwd */

/* getSeedRefs (ReadQueue.cpp:2325-2461). */
static void get_seed_refs(const orc_index* ix, const uint8_t* seq, uint32_t size, seedmaps* sm)
{
    const uint32_t nk = size - KMERLEN + 1;
    uint64_t* keys = (uint64_t*)malloc(nk * sizeof(uint64_t));
    uint32_t bucket_count = 0; /* uint32 accumulator, ReadQueue.cpp:2332 */
    uint64_t total = 0;
    for (uint32_t p = 0; p < nk; ++p) {
        uint64_t st, ln;
        keys[p] = spaced_hash(seq + p) & HTAB_MASK;
        bucket_of(ix, keys[p], &st, &ln);
        bucket_count += (uint32_t)ln;
        total += ln;
    }
    bucket_count = bucket_count / 5;
    for (int s = 0; s < 2; ++s) { hm_init(&sm->hm[s], bucket_count); cs_init(&sm->cs[s], total); }
    const uint32_t maxQPos = size - KMERLEN + 1 - QTHRESH;
    for (uint32_t p = 0; p < nk; ++p) {
        uint64_t st, ln;
        bucket_of(ix, keys[p], &st, &ln);
        uint64_t lastId = 0xffffffffffffffffULL;
        int wasFwd = 0;
        const int may_insert = (p == 0) || (p - 1 < maxQPos);
        for (uint64_t i = st; i < st + ln; ++i) {
            const uint32_t metaId = ix->kmer_meta[i] & 0x7fffffffu;
            const int isFwd = ix->strand[i] != 0;
            if (metaId == lastId && isFwd == wasFwd) continue;
            lastId = metaId;
            wasFwd = isFwd;
            uint16_t* c = cs_find(&sm->cs[isFwd], metaId);
            if (c) { ++*c; continue; }
            if (!may_insert) continue;
            c = cs_add(&sm->cs[isFwd], metaId);
            *c = 1;
            hm_insert_at(&sm->hm[isFwd], metaId & sm->hm[isFwd].mask, metaId);
        }
    }
    free(keys);
}

static void seedmaps_free(seedmaps* sm)
{
    for (int s = 0; s < 2; ++s) { hm_free(&sm->hm[s]); cs_free(&sm->cs[s]); }
}

/* iteration order of a map: occupied buckets in array order, then overflow list */
static uint64_t map_order(const hmap* m, uint32_t* out)
{
    uint64_t n = 0;
    for (uint64_t b = 0; b < m->size; ++b) if (m->info[b] & 1u) out[n++] = m->key[b];
    for (uint64_t i = 0; i < m->n_ovf; ++i) out[n++] = m->ovf[i];
    return n;
}

/* ---------------------------------------------------------------------- */
/* ShiftAnd<6> (ShiftAnd.h:121-432)                                          */
/* ---------------------------------------------------------------------- */
typedef struct {
    int W;
    uint64_t pLen;
    uint64_t masks[4][MAXW];
    uint64_t accepted[MAXW];
    uint64_t act[NERR + 1][MAXW];
} sa_t;

static inline int base_idx(uint8_t c)
{
    switch (c) { case 'A': return 0; case 'C': return 1; case 'G': return 2; case 'T': return 3; }
    return -1;
}

/* loadBitmasks (ShiftAnd.h:345-432): a read T also sets the C mask, so a
 * reference C accepts a read T (bisulfite asymmetry). */
static void sa_load(sa_t* sa, const uint8_t* seq, uint64_t len)
{
    sa->pLen = len;
    sa->W = (int)(len / 64 + 1);
    for (int w = 0; w < sa->W; ++w) sa->accepted[w] = 0;
    sa->accepted[len / 64] = 1ull << (len % 64);
    uint64_t mA = ~0ull, mC = ~0ull, mG = ~0ull, mT = ~0ull;
    for (uint64_t i = len; i > 0;) {
        mA <<= 1; mC <<= 1; mG <<= 1; mT <<= 1;
        switch (seq[i - 1]) {
            case 'A': mA |= 1; break;
            case 'C': mC |= 1; break;
            case 'G': mG |= 1; break;
            case 'T': mT |= 1; mC |= 1; break;
        }
        if (i % 64 == 0) {
            sa->masks[0][i / 64] = mA; sa->masks[1][i / 64] = mC;
            sa->masks[2][i / 64] = mG; sa->masks[3][i / 64] = mT;
            mA = mC = mG = mT = ~0ull;
        }
        --i;
    }
    sa->masks[0][0] = (mA << 1) | 1; sa->masks[1][0] = (mC << 1) | 1;
    sa->masks[2][0] = (mG << 1) | 1; sa->masks[3][0] = (mT << 1) | 1;
}

static void sa_reset(sa_t* sa)
{
    for (int i = 0; i <= (int)NERR; ++i) {
        for (int j = sa->W - 1; j > 0; --j) sa->act[i][j] = 0;
        sa->act[i][0] = (1ull << (i + 1)) - 1;
    }
}

/* queryLetter (ShiftAnd.h:276-318) */
static void sa_letter(sa_t* sa, int b)
{
    const uint64_t* mask = sa->masks[b];
    const int W = sa->W;
    for (int i = NERR; i > 0; --i) {
        for (int j = W - 1; j > 0; --j)
            sa->act[i][j] = (((sa->act[i][j] << 1) | (sa->act[i][j - 1] >> 63)) & mask[j]) | sa->act[i - 1][j] |
                            ((sa->act[i - 1][j] << 1) | (sa->act[i - 1][j - 1] >> 63));
        sa->act[i][0] = (((sa->act[i][0] << 1) | 1) & mask[0]) | sa->act[i - 1][0] | (sa->act[i - 1][0] << 1);
    }
    for (int j = W - 1; j > 0; --j)
        sa->act[0][j] = ((sa->act[0][j] << 1) | (sa->act[0][j - 1] >> 63)) & mask[j];
    sa->act[0][0] = ((sa->act[0][0] << 1) | 1) & mask[0];
    for (int i = 1; i <= (int)NERR; ++i) {
        for (int j = W - 1; j > 0; --j) sa->act[i][j] |= (sa->act[i - 1][j] << 1) | (sa->act[i - 1][j - 1] >> 63);
        sa->act[i][0] |= sa->act[i - 1][0] << 1;
    }
}

static int sa_ismatch(const sa_t* sa, uint8_t* err)
{
    for (int i = 0; i <= (int)NERR; ++i)
        for (int j = 0; j < sa->W; ++j)
            if (sa->act[i][j] & sa->accepted[j]) { *err = (uint8_t)i; return 1; }
    return 0;
}

typedef struct { uint64_t* off; uint8_t* err; uint32_t n, cap; } hits;

static void hits_push(hits* h, uint64_t off, uint8_t e)
{
    if (h->n == h->cap) {
        h->cap = h->cap ? 2 * h->cap : 8;
        h->off = (uint64_t*)realloc(h->off, h->cap * sizeof(uint64_t));
        h->err = (uint8_t*)realloc(h->err, h->cap);
    }
    h->off[h->n] = off; h->err[h->n] = e; h->n++;
}

/* querySeq (ShiftAnd.h:130-182): text[0..n) forward */
static void sa_query_fwd(sa_t* sa, const uint8_t* text, uint64_t n, hits* out)
{
    sa_reset(sa);
    int wasMatch = 0;
    uint8_t prevErrs = MISCOUNT + 1;
    uint64_t numCompLets = 0;
    out->n = 0;
    for (uint64_t t = 0; t < n; ++t) {
        if (text[t] == 'N') { sa_reset(sa); continue; }
        sa_letter(sa, base_idx(text[t]));
        ++numCompLets;
        if (numCompLets < sa->pLen - NERR) continue;
        uint8_t e;
        if (sa_ismatch(sa, &e)) {
            if (wasMatch) {
                if (e <= prevErrs) { out->off[out->n - 1] = t + MISCOUNT; out->err[out->n - 1] = e; prevErrs = e; }
            } else {
                hits_push(out, t + MISCOUNT, e);
                wasMatch = 1;
                prevErrs = e;
            }
        } else {
            wasMatch = 0;
        }
    }
}

/* queryRevSeq (ShiftAnd.h:186-255): genome positions hi down to lo+1, each
 * complemented; the offset is measured from lo (the exclusive end). */
static void sa_query_rev(sa_t* sa, const uint8_t* g, int64_t hi, int64_t lo, hits* out)
{
    sa_reset(sa);
    int wasMatch = 0;
    uint8_t prevErrs = MISCOUNT + 1;
    uint64_t numCompLets = 0;
    out->n = 0;
    for (int64_t t = hi; t != lo; --t) {
        int b;
        switch (g[t]) {
            case 'A': b = 3; break;
            case 'C': b = 2; break;
            case 'G': b = 1; break;
            case 'T': b = 0; break;
            default: sa_reset(sa); continue; /* 'N'; other letters end the reference program */
        }
        sa_letter(sa, b);
        ++numCompLets;
        if (numCompLets < sa->pLen - NERR) continue;
        uint8_t e;
        if (sa_ismatch(sa, &e)) {
            const uint64_t off = (uint64_t)(t - lo) + sa->pLen - 1 + MISCOUNT;
            if (wasMatch) {
                if (e <= prevErrs) { out->off[out->n - 1] = off; out->err[out->n - 1] = e; prevErrs = e; }
            } else {
                hits_push(out, off, e);
                wasMatch = 1;
                prevErrs = e;
            }
        } else {
            wasMatch = 0;
        }
    }
}

/* ---------------------------------------------------------------------- */
/* saQuerySeedSetRef (ReadQueue.cpp:1928-2160)                               */
/* ---------------------------------------------------------------------- */
static inline uint64_t mk_match(uint16_t off, uint8_t err, uint64_t fwd, uint64_t start, uint64_t meta)
{
    return (uint64_t)off | ((uint64_t)err << 16) | (fwd << 24) | (start << 25) | (meta << 32);
}
#define M_OFF(m) ((m) & 0xffffull)
#define M_ERR(m) (((m) >> 16) & 0xffull)
#define M_FWD(m) (((m) >> 24) & 1ull)
#define M_START(m) (((m) >> 25) & 1ull)
#define M_META(m) ((uint32_t)((m) >> 32))

static int sa_query_seed_set(const orc_index* ix, seedmaps* sm, sa_t* sa, uint64_t* mat, hits* h)
{
    uint8_t multi[NERR + 1];
    uint64_t uniq[NERR + 1];
    memset(multi, 0, sizeof(multi));
    memset(uniq, 0, sizeof(uniq));
    for (int dir = 1; dir >= 0; --dir) { /* forward windows first, then reverse */
        hmap* m = &sm->hm[dir];
        uint32_t* order = (uint32_t*)malloc((m->nb_elem + 1) * sizeof(uint32_t));
        uint64_t n = map_order(m, order);
        uint8_t prevChr = 0;
        uint64_t prevOff = 0xffffffffffffffffULL;
        for (uint64_t q = 0; q < n; ++q) {
            const uint32_t w = order[q];
            const uint16_t cnt = *cs_find(&sm->cs[dir], w);
            if (cnt < QTHRESH) continue;
            const uint32_t sp = ix->win_start[w];
            const uint8_t ch = ix->win_chrom[w];
            const uint8_t* g = ix->chrom_seq[ch];
            const int64_t L = (int64_t)ix->chrom_len[ch];
            if (dir) {
                int64_t e = (int64_t)sp + WINLEN + MISCOUNT + ADDMIS - 1;
                if (e > L) e = L;
                sa_query_fwd(sa, g + sp, (uint64_t)(e - (int64_t)sp), h);
            } else {
                int64_t lo = sp > 0 ? (int64_t)sp - 1 : 0;
                int64_t hi = (int64_t)sp + WINLEN + MISCOUNT + ADDMIS - 1;
                if (hi >= L) hi = L - 1;
                sa_query_rev(sa, g, hi, lo, h);
            }
            uint32_t i = 0;
            if (h->n > 0 && h->off[0] + sp == prevOff && ch == prevChr) ++i;
            for (; i < h->n; ++i) {
                const uint8_t e = h->err[i];
                if (multi[e]) {
                    const uint64_t m2 = uniq[e];
                    const int same_dir = dir ? (int)M_FWD(m2) : !M_FWD(m2);
                    if (same_dir && !M_START(m2) &&
                        (uint64_t)ix->win_start[M_META(m2)] + M_OFF(m2) == (uint64_t)sp + h->off[i])
                        continue;
                    if (!e) { free(order); return -1; }
                    multi[e] = 2;
                } else {
                    uniq[e] = mk_match((uint16_t)h->off[i], e, (uint64_t)dir, 0, w);
                    multi[e] = 1;
                }
            }
            if (h->n > 0) { prevChr = ch; prevOff = sp + h->off[h->n - 1]; }
            else { prevChr = 0; prevOff = 0xffffffffffffffffULL; }
        }
        free(order);
    }
    for (int i = 0; i <= (int)NERR; ++i) {
        if (!multi[i]) continue;
        *mat = uniq[i];
        return multi[i] > 1 ? -1 : 1;
    }
    return 0;
}

/* ---------------------------------------------------------------------- */
/* LevenshtDP (LevenshtDP.h:191-544) with BandedMatrix storage               */
/* (BandedMatrix.h:67-75): rows of 2*(band+1)+1 cells, index                 */
/* row*(2b+1) + max(b-row, 0) + (col-row+b) with b = band + 1 -- the first   */
/* rows overlap their successor, which the reference relies on as is.        */
/* ---------------------------------------------------------------------- */
typedef struct {
    long B;       /* band */
    long b;       /* storage band = B + 1 */
    long n;       /* pattern length */
    uint16_t* m;
    long msize;
    const uint8_t* row;
    const uint8_t* col;   /* colPat */
    int64_t col_lo, col_hi; /* valid colPat[k] for col_lo <= k < col_hi (relative) */
} lev_t;

static inline long lev_idx(const lev_t* L, long i, long j)
{
    long off = (L->b - i > 0 ? L->b - i : 0) + (j - i + L->b);
    return i * (2 * L->b + 1) + off;
}
static inline uint16_t lev_get(const lev_t* L, long i, long j)
{
    long k = lev_idx(L, i, j);
    return (k >= 0 && k < L->msize) ? L->m[k] : 0xffff; /* outside */
}
static inline void lev_set(lev_t* L, long i, long j, uint16_t v)
{
    long k = lev_idx(L, i, j);
    if (k >= 0 && k < L->msize) L->m[k] = v;
}
static inline uint8_t lev_ref(const lev_t* L, long k)
{
    return (k >= L->col_lo && k < L->col_hi) ? L->col[k] : 0; /* outside */
}

static uint16_t cmp_char(int comp, uint8_t r, uint8_t g)
{
    switch (comp) {
        case 0: return r == g ? 0 : 1;
        case 1: /* CompiFwd, ReadQueue.h:295-307 */
            if (r == 'T' && g == 'C') return 0;
            return r == g ? 0 : 1;
        case 2: /* CompiRev, ReadQueue.h:309-338 */
            switch (r) {
                case 'T': if (g == 'A' || g == 'G') return 0; break;
                case 'G': if (g == 'C') return 0; break;
                case 'A': if (g == 'T') return 0; break;
                case 'C': if (g == 'G') return 0; break;
            }
            return 1;
        default: /* complement comparator of LevenshtDP_unittest.cpp simpleSeqRev */
            switch (r) {
                case 'A': return g == 'T' ? 0 : 1;
                case 'C': return g == 'G' ? 0 : 1;
                case 'G': return g == 'C' ? 0 : 1;
                case 'T': return g == 'A' ? 0 : 1;
            }
            return 1;
    }
}

static void lev_fill(lev_t* L, int rev, int comp)
{
    const long B = L->B, n = L->n;
    lev_set(L, 0, 0, 0);
    for (long c = 1; c <= B; ++c) lev_set(L, 0, c, (uint16_t)c);
    for (long r = 1; r <= B; ++r) lev_set(L, r, 0, (uint16_t)r);
    for (long c = 0; c < n - B; ++c) lev_set(L, c + B + 1, c, (uint16_t)(65535 - c - B - 1));
    for (long r = 0; r < n; ++r) lev_set(L, r, r + B + 1, (uint16_t)(65535 - r - B - 1));
    for (long r = 1; r <= n; ++r) {
        for (long o = -B; o <= B; ++o) {
            const long j = r + o;
            if (j <= 0) continue;
            const uint8_t rc = rev ? L->row[r - 1] : L->row[n - r];
            const int mm = cmp_char(comp, rc, lev_ref(L, 1 - j));
            int v = lev_get(L, r - 1, j) + 1;
            int v2 = lev_get(L, r, j - 1) + 1;
            int v3 = lev_get(L, r - 1, j - 1) + mm;
            if (v2 < v) v = v2;
            if (v3 < v) v = v3;
            lev_set(L, r, j, (uint16_t)v);
        }
    }
}

static uint16_t lev_dist(const lev_t* L)
{
    uint16_t mn = 0xffff;
    for (long o = -L->B; o <= L->B; ++o) { uint16_t v = lev_get(L, L->n, L->n + o); if (v < mn) mn = v; }
    return mn;
}

/* backtrackDP / backtrackDPRev (LevenshtDP.h:327-544); codes as ERROR_T */
static uint32_t lev_back(const lev_t* L, int rev, int comp, uint8_t* al, uint32_t cap)
{
    const long n = L->n;
    uint16_t mn = 0xffff;
    long col = 0;
    uint32_t k = 0;
    for (long o = -L->B; o <= L->B; ++o) {
        uint16_t v = lev_get(L, n, n + o);
        if (v < mn) { col = n + o; mn = v; }
    }
    for (long row = n; row > 0;) {
        const uint8_t rc = rev ? L->row[row - 1] : L->row[n - row];
        const int mm = cmp_char(comp, rc, lev_ref(L, 1 - col));
        const uint16_t up = lev_get(L, row - 1, col), left = lev_get(L, row, col - 1), dg = lev_get(L, row - 1, col - 1);
        uint8_t code;
        if (up < left) {
            if ((int)up + 1 < (int)dg + mm) { code = 2; --row; }
            else { code = mm ? 1 : 0; --row; --col; }
        } else {
            if ((int)left + 1 < (int)dg + mm) { code = 3; --col; }
            else { code = mm ? 1 : 0; --row; --col; }
        }
        if (k < cap) al[k] = code;
        ++k;
    }
    while (col > 0) { if (k < cap) al[k] = 3; ++k; --col; }
    return k;
}

static void lev_setup(lev_t* L, long band, const uint8_t* row, long n, const uint8_t* col, int64_t lo, int64_t hi)
{
    L->B = band; L->b = band + 1; L->n = n;
    L->msize = (n + 1) * (2 * L->b + 1);
    L->m = (uint16_t*)malloc((size_t)L->msize * sizeof(uint16_t));
    for (long i = 0; i < L->msize; ++i) L->m[i] = 0xffff;
    L->row = row; L->col = col; L->col_lo = lo; L->col_hi = hi;
}

int orc_lev(int band, const uint8_t* row, uint32_t row_len, const uint8_t* col, int64_t col_len,
            int64_t col_end, int rev, int comp, uint8_t* trace, uint32_t cap, uint32_t* dist)
{
    lev_t L;
    lev_setup(&L, band, row, row_len, col + col_end, -col_end, col_len - col_end);
    lev_fill(&L, rev, comp);
    *dist = lev_dist(&L);
    uint32_t k = lev_back(&L, rev, comp, trace, cap);
    free(L.m);
    return (int)k;
}

/* ---------------------------------------------------------------------- */
/* computeMethLvl (ReadQueue.cpp:3278-3947)                                  */
/* ---------------------------------------------------------------------- */
static void meth_inc(uint16_t* meth, uint32_t cpg, int slot) { meth[4 * (uint64_t)cpg + slot]++; }

static void compute_meth(const orc_index* ix, uint64_t mat, uint8_t* seq, uint32_t size, uint16_t* meth)
{
    const int isFwd = (int)M_FWD(mat);
    const uint32_t metaID = M_META(mat);
    const uint16_t offset = (uint16_t)M_OFF(mat);
    const uint8_t errNum = (uint8_t)M_ERR(mat);
    const uint32_t RL = ix->readlen;
    if (ix->win_sind[metaID] == CPGDUMMY) return;
    const uint32_t metaPos = ix->win_start[metaID];
    const uint32_t sind = ix->win_sind[metaID], eind = ix->win_eind[metaID];
    if (errNum == 0) {
        const uint32_t minPos = (uint32_t)(metaPos + offset - (size - 1));
        const uint32_t maxPos = metaPos + offset;
        for (uint32_t id = sind; id <= eind; ++id) {
            const uint32_t pos = ix->cpg_pos[id];
            if (pos + RL - 2 < minPos) continue;
            if (isFwd) { if (pos + RL - 2 > maxPos) break; }
            else { if (pos + RL - 1 > maxPos) break; }
            const uint32_t trueCpGPos = pos - 1 + RL - 1;
            const uint32_t readCpGPos = (uint32_t)(size - (uint32_t)(metaPos + offset - trueCpGPos) - 1);
            if (isFwd) {
                if ((uint32_t)(readCpGPos + MISCOUNT) >= size) continue;
                const uint8_t c = seq[(uint32_t)(readCpGPos + MISCOUNT)];
                if (c == 'T') meth_inc(meth, id, 1);
                else if (c == 'C') meth_inc(meth, id, 0);
            } else {
                if ((uint32_t)(readCpGPos + 1 + MISCOUNT + 2) > size) continue;
                const uint8_t c = seq[size - readCpGPos - 1 - MISCOUNT - 2];
                if (c == 'T') meth_inc(meth, id, 3);
                else if (c == 'C') meth_inc(meth, id, 2);
            }
        }
        return;
    }
    const uint8_t chrom = ix->cpg_chrom[sind];
    const uint8_t* g = ix->chrom_seq[chrom];
    const int64_t base = (int64_t)metaPos + offset;
    lev_t L;
    lev_setup(&L, DP_BAND, seq, size, g + base, -base, (int64_t)ix->chrom_len[chrom] - base);
    const uint32_t minPos = (uint32_t)(metaPos + offset - (size - 1));
    const uint32_t maxPos = metaPos + offset;
    int32_t minIndex = (int32_t)sind, maxIndex = (int32_t)eind;
    for (int32_t id = (int32_t)sind; (uint32_t)id <= eind; ++id) {
        const uint32_t pos = ix->cpg_pos[id];
        if (pos + RL - 2 < minPos) ++minIndex;
        else if (pos + RL - 2 > maxPos) { maxIndex = id - 1; break; }
    }
    const uint32_t alcap = 2 * size + 2 * DP_BAND + 8; /* every backtrack step lowers row or column */
    uint8_t* al = (uint8_t*)malloc(alcap);
    lev_fill(&L, !isFwd, isFwd ? 1 : 2);
    const uint32_t alen = lev_back(&L, !isFwd, isFwd ? 1 : 2, al, alcap);
    uint32_t refSeqPos = metaPos + offset;
    int32_t readSeqPos = (int32_t)size - 1;
    int32_t alignPos = (int32_t)alen - 1;
    if (!isFwd) { /* std::reverse on the caller's string, ReadQueue.cpp:3796 */
        for (uint32_t a = 0, b = size - 1; a < b; ++a, --b) { uint8_t t = seq[a]; seq[a] = seq[b]; seq[b] = t; }
    }
    for (int32_t id = maxIndex; id >= minIndex; --id) {
        const uint32_t cpos = ix->cpg_pos[id] + RL - 2;
        while (cpos < refSeqPos && alignPos >= 0) {
            switch (al[alignPos]) {
                case 0: case 1: --readSeqPos; --refSeqPos; break;
                case 3: --refSeqPos; break;
                case 2: --readSeqPos; break;
            }
            if (readSeqPos < 0) break;
            --alignPos;
        }
        if (readSeqPos < 0) break;
        if (isFwd) {
            const uint8_t c = seq[readSeqPos];
            if (c == 'C') meth_inc(meth, (uint32_t)id, 0);
            else if (c == 'T') meth_inc(meth, (uint32_t)id, 1);
        } else {
            const uint8_t c = seq[readSeqPos + 1];
            if (c == 'C') meth_inc(meth, (uint32_t)id, 2);
            else if (c == 'T') meth_inc(meth, (uint32_t)id, 3);
        }
    }
    free(al);
    free(L.m);
}

/* ---------------------------------------------------------------------- */
/* matchReads (ReadQueue.cpp:404-933)                                        */
/* ---------------------------------------------------------------------- */
typedef struct { uint64_t succ, nonu, unsucc, r1f, r1r; int matchR1Fwd; } stats;

static int query_orient(const orc_index* ix, const uint8_t* seq, uint32_t size, uint64_t* mat, sa_t* sa, hits* h)
{
    seedmaps sm;
    get_seed_refs(ix, seq, size, &sm);
    sa_load(sa, seq, size);
    int r = sa_query_seed_set(ix, &sm, sa, mat, h);
    seedmaps_free(&sm);
    return r;
}

static void match_chunk(const orc_index* ix, const uint8_t* seqs, const uint64_t* offs, uint32_t n,
                        int getStranded, int both, stats* st, uint64_t* mats, uint8_t* invalid, uint16_t* meth)
{
    sa_t sa;
    hits h = {0};
    for (uint32_t r = 0; r < n; ++r) {
        const uint32_t size = (uint32_t)(offs[r + 1] - offs[r]);
        uint8_t* fw = (uint8_t*)calloc(size + 1, 1); /* std::string keeps a NUL at [size] */
        uint8_t* rv = (uint8_t*)calloc(size + 1, 1);
        memcpy(fw, seqs + offs[r], size);
        invalid[r] = 0;
        mats[r] = 0;
        if (size < ix->readlen - 20) { invalid[r] = 1; goto next; }
        {
            int nflag = 0;
            for (uint32_t p = 0, q = size - 1; p < size; ++p, --q) {
                switch (fw[p]) {
                    case 'A': rv[q] = 'T'; break;
                    case 'C': rv[q] = 'G'; break;
                    case 'G': rv[q] = 'C'; break;
                    case 'T': rv[q] = 'A'; break;
                    case 'N': nflag = 1; break;
                    default: break; /* reported and left as '\0' */
                }
            }
            if (nflag) { invalid[r] = 1; goto next; }
            uint64_t mF = 0, mR = 0;
            int sF = 0, sR = 0;
            if (both || getStranded || st->matchR1Fwd) sF = query_orient(ix, fw, size, &mF, &sa, &h);
            if (both || getStranded || !st->matchR1Fwd) sR = query_orient(ix, rv, size, &mR, &sa, &h);
            if (sF == 1 && sR == 1) {
                const uint8_t eF = (uint8_t)M_ERR(mF), eR = (uint8_t)M_ERR(mR);
                if (eF < eR) {
                    if (getStranded) st->r1f++;
                    st->succ++; mats[r] = mF; compute_meth(ix, mF, fw, size, meth);
                } else if (eF > eR) {
                    if (getStranded) st->r1r++;
                    st->succ++; mats[r] = mR; compute_meth(ix, mR, rv, size, meth);
                } else {
                    const uint32_t metaF = M_META(mF), metaR = M_META(mR);
                    const uint64_t offF = M_OFF(mF), offR = M_OFF(mR);
                    const int f1 = (int)M_FWD(mF), f2 = (int)M_FWD(mR);
                    const int s1 = (int)M_START(mF), s2 = (int)M_START(mR);
                    uint32_t p1, p2;
                    if (s1 && s2) { p1 = (uint32_t)offF; p2 = (uint32_t)offR; }
                    else { p1 = (uint32_t)(ix->win_start[metaF] + offF); p2 = (uint32_t)(ix->win_start[metaR] + offR); }
                    if (s1 == s2 && f1 == f2 && p1 == p2) {
                        st->succ++;
                        if (getStranded) st->r1f++;
                        mats[r] = mF; compute_meth(ix, mF, fw, size, meth);
                    } else {
                        st->nonu++; invalid[r] = 1;
                    }
                }
            } else if (sF == 1) {
                if (sR == -1) {
                    if (M_ERR(mF) < M_ERR(mR)) {
                        st->succ++; if (getStranded) st->r1f++;
                        mats[r] = mF; compute_meth(ix, mF, fw, size, meth);
                    } else { st->nonu++; invalid[r] = 1; }
                } else {
                    st->succ++; if (getStranded) st->r1f++;
                    mats[r] = mF; compute_meth(ix, mF, fw, size, meth);
                }
            } else if (sR == 1) {
                if (sF == -1) {
                    if (M_ERR(mR) < M_ERR(mF)) {
                        st->succ++; if (getStranded) st->r1r++;
                        mats[r] = mR; compute_meth(ix, mR, rv, size, meth);
                    } else { st->nonu++; invalid[r] = 1; }
                } else {
                    st->succ++; if (getStranded) st->r1r++;
                    mats[r] = mR; compute_meth(ix, mR, rv, size, meth);
                }
            } else {
                invalid[r] = 1;
                if (sF == -1 || sR == -1) st->nonu++; else st->unsucc++;
            }
        }
    next:
        if (invalid[r]) mats[r] = 0;
        free(fw);
        free(rv);
    }
    free(h.off);
    free(h.err);
}

/* queryRoutine loop structure (main.cpp:363-399) and decideStrand (ReadQueue.cpp:376-400) */
int orc_match_se(const orc_index* ix, const uint8_t* seqs, const uint64_t* offs, uint32_t n,
                 uint32_t chunk, int both_strands, uint64_t* mats, uint8_t* invalid, uint16_t* meth,
                 uint64_t* counters)
{
    stats st;
    memset(&st, 0, sizeof(st));
    st.matchR1Fwd = 1;
    if (chunk == 0) chunk = 300000;
    memset(meth, 0, sizeof(uint16_t) * 4 * ix->n_cpg);
    for (uint32_t c0 = 0, ci = 0; c0 < n; c0 += chunk, ++ci) {
        const uint32_t cn = n - c0 < chunk ? n - c0 : chunk;
        const int stranded = ci == 0 && !both_strands;
        match_chunk(ix, seqs, offs + c0, cn, stranded, both_strands, &st, mats + c0, invalid + c0, meth);
        if (stranded) st.matchR1Fwd = st.r1f > st.r1r;
    }
    counters[0] = st.succ; counters[1] = st.nonu; counters[2] = st.unsucc;
    counters[3] = st.r1f; counters[4] = st.r1r; counters[5] = (uint64_t)st.matchR1Fwd;
    return 0;
}

int orc_seed_order(const orc_index* ix, const uint8_t* seq, uint32_t len, uint32_t cap,
                   uint32_t* out_keys, uint32_t* out_counts, uint64_t* n_out)
{
    seedmaps sm;
    get_seed_refs(ix, seq, len, &sm);
    uint64_t k = 0;
    for (int dir = 1; dir >= 0; --dir) {
        uint32_t* order = (uint32_t*)malloc((sm.hm[dir].nb_elem + 1) * sizeof(uint32_t));
        uint64_t n = map_order(&sm.hm[dir], order);
        for (uint64_t i = 0; i < n; ++i, ++k) {
            if (k < cap) { out_keys[k] = order[i]; out_counts[k] = *cs_find(&sm.cs[dir], order[i]); }
        }
        n_out[dir ? 0 : 1] = n;
        free(order);
    }
    n_out[2] = sm.hm[1].nbk;
    n_out[3] = sm.hm[0].nbk;
    seedmaps_free(&sm);
    return k > cap ? -1 : 0;
}

int orc_shiftand(const uint8_t* pat, uint32_t pat_len, const uint8_t* text, uint32_t text_len, int rev,
                 uint64_t* offs, uint8_t* errs, uint32_t cap)
{
    sa_t sa;
    hits h = {0};
    sa_load(&sa, pat, pat_len);
    if (rev) {
        uint8_t* g = (uint8_t*)malloc(text_len + 1);
        g[0] = 'N';
        memcpy(g + 1, text, text_len);
        sa_query_rev(&sa, g, text_len, 0, &h);
        free(g);
    } else {
        sa_query_fwd(&sa, text, text_len, &h);
    }
    for (uint32_t i = 0; i < h.n && i < cap; ++i) { offs[i] = h.off[i]; errs[i] = h.err[i]; }
    int n = (int)h.n;
    free(h.off);
    free(h.err);
    return n;
}

/* ---------------------------------------------------------------------- */
/* index build                                                                */
/* ---------------------------------------------------------------------- */
struct orc_built {
    uint32_t readlen;
    uint32_t n_chrom;
    uint8_t** seq;
    uint64_t* len;
    uint64_t n_cpg, n_cpgs;
    uint8_t *cpg_chrom, *cpgs_chrom;
    uint32_t *cpg_pos, *cpgs_pos;
    uint64_t n_win;
    uint32_t *win_start, *win_sind, *win_eind;
    uint8_t* win_chrom;
    uint64_t n_kmer;             /* entries after filtering */
    uint32_t* e_key;
    uint32_t* e_meta;            /* getCore: start bit | window id */
    uint32_t* e_off;             /* offset inside the window (KMER::getOffset) */
    uint8_t* e_strand;
    uint32_t* e_tmask;
    uint64_t n_filtered;
    uint64_t* filtered;
};

typedef struct { uint32_t key; uint32_t meta; uint32_t off; uint8_t strand; uint64_t seq; } ent;

static int ent_cmp(const void* a, const void* b)
{
    const ent* x = (const ent*)a; const ent* y = (const ent*)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    /* RefGenome.cpp:711-755 fill by decrementing tabIndex: later insertions first */
    return x->seq > y->seq ? -1 : (x->seq < y->seq ? 1 : 0);
}

static inline uint8_t chrom_at(const orc_built* b, uint32_t c, uint64_t p)
{
    return p < b->len[c] ? b->seq[c][p] : 'N'; /* outside: past the chromosome end */
}

/* reproduceKmerSeq (RefGenome.cpp:2028-2132) */
static uint64_t kmer_seq(const orc_built* b, uint32_t meta, uint32_t off, int fwd)
{
    const uint32_t pos = b->win_start[meta & 0x7fffffffu];
    const uint32_t c = b->win_chrom[meta & 0x7fffffffu];
    const uint64_t s0 = (uint64_t)pos + off;
    uint64_t k = 0;
    if (fwd) {
        for (unsigned i = 0; i < KMERLEN; ++i) {
            k <<= 2;
            if ((SEEDBITS >> (31 - i)) & 1u) {
                uint8_t ch = chrom_at(b, c, s0 + i);
                if (ch == 'C' || ch == 'T') k += 3; else if (ch == 'G') k += 2;
            }
        }
    } else {
        for (unsigned i = KMERLEN; i > 0; --i) {
            k <<= 2;
            if ((SEEDBITS >> (31 - (KMERLEN - i))) & 1u) {
                uint8_t ch = chrom_at(b, c, s0 + i - 1);
                if (ch == 'G' || ch == 'A') k += 3; else if (ch == 'C') k += 2;
            }
        }
    }
    return k;
}

/* reproduceTMask (RefGenome.cpp:2135-2189) */
static uint32_t tmask_of(const orc_built* b, uint32_t meta, uint32_t off, int fwd)
{
    const uint32_t pos = b->win_start[meta & 0x7fffffffu];
    const uint32_t c = b->win_chrom[meta & 0x7fffffffu];
    const uint64_t s0 = (uint64_t)pos + off;
    uint32_t t = 0;
    if (fwd) {
        for (unsigned i = 0; i < KMERLEN; ++i) { t <<= 1; if (chrom_at(b, c, s0 + i) == 'T') t |= 1; }
    } else {
        for (unsigned i = KMERLEN; i > 0; --i) { t <<= 1; if (chrom_at(b, c, s0 + i - 1) == 'A') t |= 1; }
    }
    return t;
}

static int u64_cmp(const void* a, const void* b)
{
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

orc_built* orc_build(uint32_t readlen, uint32_t n_chrom, const uint8_t* const* raw_seq, const uint64_t* raw_len,
                     int noloss)
{
    orc_built* b = (orc_built*)calloc(1, sizeof(orc_built));
    b->readlen = readlen;
    b->n_chrom = n_chrom;
    b->seq = (uint8_t**)calloc(n_chrom, sizeof(uint8_t*));
    b->len = (uint64_t*)calloc(n_chrom, sizeof(uint64_t));
    uint64_t cap_cpg = 1024, cap_cpgs = 16;
    b->cpg_chrom = (uint8_t*)malloc(cap_cpg); b->cpg_pos = (uint32_t*)malloc(cap_cpg * 4);
    b->cpgs_chrom = (uint8_t*)malloc(cap_cpgs); b->cpgs_pos = (uint32_t*)malloc(cap_cpgs * 4);
    /* readLine (RefReader_istr.h:48-113): case folding, other letters -> N, CpG table */
    for (uint32_t c = 0; c < n_chrom; ++c) {
        b->len[c] = raw_len[c];
        b->seq[c] = (uint8_t*)malloc(raw_len[c] + 1);
        int lastC = 0;
        for (uint64_t i = 0; i < raw_len[c]; ++i) {
            uint8_t ch = raw_seq[c][i];
            switch (ch) {
                case 'g': case 'G':
                    if (lastC) {
                        if (i >= readlen - 2) {
                            if (b->n_cpg == cap_cpg) {
                                cap_cpg *= 2;
                                b->cpg_chrom = (uint8_t*)realloc(b->cpg_chrom, cap_cpg);
                                b->cpg_pos = (uint32_t*)realloc(b->cpg_pos, cap_cpg * 4);
                            }
                            b->cpg_chrom[b->n_cpg] = (uint8_t)c;
                            b->cpg_pos[b->n_cpg++] = (uint32_t)i - readlen + 1;
                        } else {
                            if (b->n_cpgs == cap_cpgs) {
                                cap_cpgs *= 2;
                                b->cpgs_chrom = (uint8_t*)realloc(b->cpgs_chrom, cap_cpgs);
                                b->cpgs_pos = (uint32_t*)realloc(b->cpgs_pos, cap_cpgs * 4);
                            }
                            b->cpgs_chrom[b->n_cpgs] = (uint8_t)c;
                            b->cpgs_pos[b->n_cpgs++] = (uint32_t)i - 1;
                        }
                        lastC = 0;
                    }
                    b->seq[c][i] = 'G';
                    break;
                case 'c': case 'C': b->seq[c][i] = 'C'; lastC = 1; break;
                case 'a': case 'A': b->seq[c][i] = 'A'; lastC = 0; break;
                case 't': case 'T': b->seq[c][i] = 'T'; lastC = 0; break;
                default: b->seq[c][i] = 'N'; lastC = 0; break;
            }
        }
    }
    /* generateWindows (RefGenome.cpp:532-567) */
    uint64_t capw = 1024;
    b->win_start = (uint32_t*)malloc(capw * 4); b->win_chrom = (uint8_t*)malloc(capw);
    b->win_sind = (uint32_t*)malloc(capw * 4); b->win_eind = (uint32_t*)malloc(capw * 4);
    uint64_t ci = 0;
    for (uint32_t c = 0; c < n_chrom; ++c) {
        for (uint32_t ws = 0; ws < b->len[c]; ws = ws + WINLEN - readlen) {
            const uint32_t we = ws + WINLEN;
            uint32_t s = CPGDUMMY, e = CPGDUMMY;
            while (ci < b->n_cpg && b->cpg_chrom[ci] == c && b->cpg_pos[ci] <= we) {
                if (s == CPGDUMMY) s = (uint32_t)ci;
                e = (uint32_t)ci;
                ++ci;
            }
            /* reads cpgTable[ci] even when ci == size (outside: stop there) */
            while (ci > 0 && ci < b->n_cpg && b->cpg_chrom[ci] == c && b->cpg_pos[ci] >= we - readlen) --ci;
            if (ci > 0) ++ci;
            if (b->n_win == capw) {
                capw *= 2;
                b->win_start = (uint32_t*)realloc(b->win_start, capw * 4); b->win_chrom = (uint8_t*)realloc(b->win_chrom, capw);
                b->win_sind = (uint32_t*)realloc(b->win_sind, capw * 4); b->win_eind = (uint32_t*)realloc(b->win_eind, capw * 4);
            }
            b->win_start[b->n_win] = ws; b->win_chrom[b->n_win] = (uint8_t)c;
            b->win_sind[b->n_win] = s; b->win_eind[b->n_win] = e;
            b->n_win++;
        }
    }
    /* estimateTablesizes + generateHashes (RefGenome.cpp:570-759, 1787-1989) */
    uint64_t cap_e = 1 << 16, n_e = 0, seqno = 0;
    ent* E = (ent*)malloc(cap_e * sizeof(ent));
    uint8_t* red = (uint8_t*)malloc(WINLEN);
    uint8_t* redr = (uint8_t*)malloc(WINLEN);
    uint32_t* iv = (uint32_t*)malloc(2 * (WINLEN + 2) * sizeof(uint32_t));
    for (uint64_t w = 0; w < b->n_win; ++w) {
        memset(red, 0, WINLEN);
        memset(redr, 0, WINLEN);
        const uint32_t c = b->win_chrom[w];
        const uint8_t* g = b->seq[c];
        const uint64_t sp = b->win_start[w];
        const uint64_t stop = sp + WINLEN < b->len[c] ? sp + WINLEN : b->len[c];
        int lastN = 1;
        uint32_t nStart = 0, niv = 0, j = 0;
        for (uint64_t i = sp; i < stop; ++i, ++j) {
            const uint32_t rp = WINLEN - 1 - j;
            switch (g[i]) {
                case 'N':
                    if (!lastN) { iv[2 * niv] = nStart; iv[2 * niv + 1] = j - 1; ++niv; }
                    lastN = 1;
                    red[j] = 'N';
                    red[rp] = 'N'; /* RefGenome.cpp:646 writes the forward buffer */
                    break;
                case 'C': if (lastN) { nStart = j; lastN = 0; } red[j] = 'T'; redr[rp] = 'G'; break;
                case 'G': if (lastN) { nStart = j; lastN = 0; } red[j] = 'G'; redr[rp] = 'T'; break;
                case 'T': if (lastN) { nStart = j; lastN = 0; } red[j] = 'T'; redr[rp] = 'A'; break;
                case 'A': if (lastN) { nStart = j; lastN = 0; } red[j] = 'A'; redr[rp] = 'T'; break;
                default: break;
            }
        }
        if (!lastN) { iv[2 * niv] = nStart; iv[2 * niv + 1] = j - 1; ++niv; }
        for (uint32_t q = 0; q < niv; ++q) {
            const uint32_t first = iv[2 * q], second = iv[2 * q + 1];
            const uint32_t dist = second - first + 1;
            if (dist < readlen) continue;
            const uint8_t* fs = red + first;
            const uint8_t* rs = redr + (WINLEN - 1 - second);
            for (int strand = 0; strand < 2; ++strand) { /* reverse strand first */
                const uint8_t* s = strand ? fs : rs;
                uint64_t kp = strand ? first : (uint64_t)(WINLEN - first - KMERLEN);
                for (int64_t i = -1; i < (int64_t)(dist - KMERLEN); ++i) {
                    if (i >= 0) kp = strand ? kp + 1 : kp - 1;
                    if (i >= 0 && (i % SKIPMOD)) continue;
                    if (n_e == cap_e) { cap_e *= 2; E = (ent*)realloc(E, cap_e * sizeof(ent)); }
                    E[n_e].key = (uint32_t)(spaced_hash(s + i + 1) & HTAB_MASK);
                    E[n_e].meta = (uint32_t)w;
                    E[n_e].off = (uint32_t)kp;
                    E[n_e].strand = (uint8_t)strand;
                    E[n_e].seq = seqno++;
                    ++n_e;
                }
            }
        }
    }
    free(red); free(redr); free(iv);
    qsort(E, n_e, sizeof(ent), ent_cmp);
    /* filterHashTable (RefGenome.cpp:2267-2352): per-bucket k-mer blacklist */
    uint64_t capf = 16;
    b->filtered = (uint64_t*)malloc(capf * 8);
    uint8_t* keep = (uint8_t*)malloc(n_e + 1);
    memset(keep, 1, n_e + 1);
    for (uint64_t s = 0; s < n_e;) {
        uint64_t t = s;
        while (t < n_e && E[t].key == E[s].key) ++t;
        if (!noloss && t - s >= KMERCUTOFF) {
            uint64_t* ks = (uint64_t*)malloc((t - s) * 8);
            uint64_t* sorted = (uint64_t*)malloc((t - s) * 8);
            for (uint64_t i = s; i < t; ++i) ks[i - s] = sorted[i - s] = kmer_seq(b, E[i].meta, E[i].off, E[i].strand);
            qsort(sorted, t - s, 8, u64_cmp);
            for (uint64_t i = s; i < t; ++i) {
                uint64_t lo = 0, hi = t - s, k = ks[i - s];
                while (lo < hi) { uint64_t mid = (lo + hi) >> 1; if (sorted[mid] < k) lo = mid + 1; else hi = mid; }
                uint64_t cnt = 0;
                while (lo + cnt < t - s && sorted[lo + cnt] == k) ++cnt;
                if (cnt >= KMERCUTOFF) {
                    keep[i] = 0;
                    if (b->n_filtered == capf) { capf *= 2; b->filtered = (uint64_t*)realloc(b->filtered, capf * 8); }
                    b->filtered[b->n_filtered++] = k;
                }
            }
            free(ks); free(sorted);
        }
        s = t;
    }
    if (b->n_filtered) { /* the reference keeps them in an unordered_set */
        qsort(b->filtered, b->n_filtered, 8, u64_cmp);
        uint64_t u = 1;
        for (uint64_t i = 1; i < b->n_filtered; ++i) if (b->filtered[i] != b->filtered[u - 1]) b->filtered[u++] = b->filtered[i];
        b->n_filtered = u;
    }
    /* filterRedundancyInHashTable (RefGenome.cpp:2191-2264): within a run of one
     * window and strand keep only entries whose T mask is new in that run */
    uint32_t* runmask = (uint32_t*)malloc((n_e + 1) * 4);
    for (uint64_t s = 0; s < n_e;) {
        uint64_t t = s;
        while (t < n_e && E[t].key == E[s].key) ++t;
        uint64_t prevMeta = 0xffffffffffffffffULL;
        int prevFwd = 0;
        uint64_t nmask = 0;
        for (uint64_t i = s; i < t; ++i) {
            if (!keep[i]) continue;
            const uint32_t tm = tmask_of(b, E[i].meta, E[i].off, E[i].strand);
            if ((uint64_t)E[i].meta != prevMeta || E[i].strand != prevFwd) {
                nmask = 0;
                runmask[nmask++] = tm;
                prevMeta = E[i].meta;
                prevFwd = E[i].strand;
            } else {
                int seen = 0;
                for (uint64_t q = 0; q < nmask; ++q) if (runmask[q] == tm) { seen = 1; break; }
                if (seen) keep[i] = 0; else runmask[nmask++] = tm;
            }
        }
        s = t;
    }
    free(runmask);
    uint64_t nk = 0;
    for (uint64_t i = 0; i < n_e; ++i) nk += keep[i];
    b->n_kmer = nk;
    b->e_key = (uint32_t*)malloc(nk * 4 + 4); b->e_meta = (uint32_t*)malloc(nk * 4 + 4);
    b->e_off = (uint32_t*)malloc(nk * 4 + 4); b->e_strand = (uint8_t*)malloc(nk + 1);
    b->e_tmask = (uint32_t*)malloc(nk * 4 + 4);
    for (uint64_t i = 0, k = 0; i < n_e; ++i) {
        if (!keep[i]) continue;
        b->e_key[k] = E[i].key; b->e_meta[k] = E[i].meta; b->e_off[k] = E[i].off; b->e_strand[k] = E[i].strand;
        ++k;
    }
    free(keep); free(E);
    /* getTMask at save time (RefGenome.h:62-100, RefGenome.cpp:144-153): the strand
     * is looked up at strandTable[window id], and the reverse loop skips base 0 */
    for (uint64_t k = 0; k < nk; ++k) {
        const uint32_t w = b->e_meta[k] & 0x7fffffffu;
        const uint32_t pos = b->win_start[w];
        const uint32_t c = b->win_chrom[w];
        const uint64_t s0 = (uint64_t)pos + b->e_off[k];
        const int fwd = w < nk ? b->e_strand[w] : 0; /* outside: vector<bool> past its end */
        uint32_t t = 0;
        if (fwd) { for (unsigned i = 0; i < KMERLEN; ++i) { t <<= 1; if (chrom_at(b, c, s0 + i) == 'T') t |= 1; } }
        else { for (unsigned i = KMERLEN - 1; i > 0; --i) { t <<= 1; if (chrom_at(b, c, s0 + i) == 'A') t |= 1; } }
        b->e_tmask[k] = t;
    }
    return b;
}

void orc_built_sizes(const orc_built* b, uint64_t* sizes)
{
    uint64_t nb = 0;
    for (uint64_t i = 0; i < b->n_kmer; ++i) nb += (i == 0 || b->e_key[i] != b->e_key[i - 1]);
    sizes[0] = b->n_cpg; sizes[1] = b->n_cpgs; sizes[2] = nb; sizes[3] = b->n_kmer;
    sizes[4] = b->n_win; sizes[5] = b->n_filtered;
}

void orc_built_copy(const orc_built* b, uint8_t* cpg_chrom, uint32_t* cpg_pos, uint8_t* cpgs_chrom,
                    uint32_t* cpgs_pos, uint32_t* bucket_key, uint64_t* bucket_start, uint32_t* bucket_len,
                    uint32_t* kmer_meta, uint32_t* kmer_tmask, uint8_t* strand, uint32_t* win_start,
                    uint8_t* win_chrom, uint32_t* win_sind, uint32_t* win_eind, uint64_t* filtered,
                    uint8_t* const* chrom_seq_out)
{
    memcpy(cpg_chrom, b->cpg_chrom, b->n_cpg); memcpy(cpg_pos, b->cpg_pos, b->n_cpg * 4);
    memcpy(cpgs_chrom, b->cpgs_chrom, b->n_cpgs); memcpy(cpgs_pos, b->cpgs_pos, b->n_cpgs * 4);
    uint64_t nb = 0;
    for (uint64_t i = 0; i < b->n_kmer; ++i) {
        if (i == 0 || b->e_key[i] != b->e_key[i - 1]) {
            bucket_key[nb] = b->e_key[i]; bucket_start[nb] = i; bucket_len[nb] = 0; ++nb;
        }
        bucket_len[nb - 1]++;
        kmer_meta[i] = b->e_meta[i]; kmer_tmask[i] = b->e_tmask[i]; strand[i] = b->e_strand[i];
    }
    memcpy(win_start, b->win_start, b->n_win * 4); memcpy(win_chrom, b->win_chrom, b->n_win);
    memcpy(win_sind, b->win_sind, b->n_win * 4); memcpy(win_eind, b->win_eind, b->n_win * 4);
    memcpy(filtered, b->filtered, b->n_filtered * 8);
    for (uint32_t c = 0; c < b->n_chrom; ++c) memcpy(chrom_seq_out[c], b->seq[c], b->len[c]);
}

void orc_built_free(orc_built* b)
{
    if (!b) return;
    for (uint32_t c = 0; c < b->n_chrom; ++c) free(b->seq[c]);
    free(b->seq); free(b->len);
    free(b->cpg_chrom); free(b->cpg_pos); free(b->cpgs_chrom); free(b->cpgs_pos);
    free(b->win_start); free(b->win_chrom); free(b->win_sind); free(b->win_eind);
    free(b->e_key); free(b->e_meta); free(b->e_off); free(b->e_strand); free(b->e_tmask);
    free(b->filtered);
    free(b);
}

/* Insertion model on an explicit key sequence (pinned against tsl::hopscotch_map). */
int orc_hopscotch(const uint32_t* keys, uint32_t n, uint32_t bucket_count, uint32_t* order, uint64_t* final_buckets)
{
    hmap m;
    cset cs;
    hm_init(&m, bucket_count);
    cs_init(&cs, n);
    for (uint32_t i = 0; i < n; ++i) {
        if (cs_find(&cs, keys[i])) continue;
        *cs_add(&cs, keys[i]) = 1;
        hm_insert_at(&m, keys[i] & m.mask, keys[i]);
    }
    int k = (int)map_order(&m, order);
    *final_buckets = m.nbk;
    hm_free(&m);
    cs_free(&cs);
    return k;
}

/* One matchReads call with explicit flags (ReadQueue.cpp:404-933); meth accumulates.
 * counters: [succ, nonunique, unsucc, r1Fwd, r1Rev] of this call. */
int orc_match_chunk(const orc_index* ix, const uint8_t* seqs, const uint64_t* offs, uint32_t n, int get_stranded,
                    int both_strands, int match_r1_fwd, uint64_t* mats, uint8_t* invalid, uint16_t* meth,
                    uint64_t* counters)
{
    stats st;
    memset(&st, 0, sizeof(st));
    st.matchR1Fwd = match_r1_fwd;
    match_chunk(ix, seqs, offs, n, get_stranded, both_strands, &st, mats, invalid, meth);
    counters[0] = st.succ; counters[1] = st.nonu; counters[2] = st.unsucc;
    counters[3] = st.r1f; counters[4] = st.r1r;
    return 0;
}

/* ====================================================================== */
/* paired-end path (ReadQueue.cpp:935-1655, 2167-2323, 2468-3164, 3255-3275, */
/* 4538-4776)                                                               */
/* ====================================================================== */
#define KMERDIST 10 /* CONST.h:104 */

/* value of a paired map entry: tuple<uint8 count1, uint8 count2, bool f2, bool f3> */
#define PC1(v) ((v) & 0xffu)
#define PC2(v) (((v) >> 8) & 0xffu)
#define PF2 (1u << 16)
#define PF3 (1u << 17)

typedef struct { uint64_t cap; uint32_t* k; uint32_t* v; uint8_t* used; } vmap;

static void vm_init(vmap* s, uint64_t n)
{
    s->cap = 16;
    while (s->cap < 2 * n + 16) s->cap <<= 1;
    s->k = (uint32_t*)malloc(s->cap * sizeof(uint32_t));
    s->v = (uint32_t*)calloc(s->cap, sizeof(uint32_t));
    s->used = (uint8_t*)calloc(s->cap, 1);
}
static void vm_free(vmap* s) { free(s->k); free(s->v); free(s->used); }
static uint32_t* vm_find(vmap* s, uint32_t key)
{
    uint64_t h = (key * 0x9E3779B97F4A7C15ULL) >> 20;
    for (uint64_t i = h & (s->cap - 1);; i = (i + 1) & (s->cap - 1)) {
        if (!s->used[i]) return NULL;
        if (s->k[i] == key) return &s->v[i];
    }
}
static uint32_t* vm_add(vmap* s, uint32_t key)
{
    uint64_t h = (key * 0x9E3779B97F4A7C15ULL) >> 20;
    for (uint64_t i = h & (s->cap - 1);; i = (i + 1) & (s->cap - 1)) {
        if (!s->used[i]) { s->used[i] = 1; s->k[i] = key; s->v[i] = 0; return &s->v[i]; }
        if (s->k[i] == key) return &s->v[i];
    }
}

/* one tsl::hopscotch_map<uint32_t, tuple<...>>: positions + values */
typedef struct { hmap hm; vmap vm; } pmap;

static void pm_init(pmap* p, uint64_t bucket_count, uint64_t expect) { hm_init(&p->hm, bucket_count); vm_init(&p->vm, expect); }
static void pm_free(pmap* p) { hm_free(&p->hm); vm_free(&p->vm); }
static uint32_t* pm_find(pmap* p, uint32_t key) { return vm_find(&p->vm, key); }
static uint32_t* pm_at(pmap* p, uint32_t key) /* operator[] */
{
    uint32_t* v = vm_find(&p->vm, key);
    if (v) return v;
    v = vm_add(&p->vm, key);
    hm_insert_at(&p->hm, key & p->hm.mask, key);
    return vm_find(&p->vm, key);
}
static uint64_t pm_size(const pmap* p) { return p->hm.nb_elem; }

/* libstdc++ std::sort (introsort: median-of-three unguarded partition, heap
 * sort below the depth limit, final insertion sort with a 16-element
 * threshold) for the paired candidate lists; comp(a, b) = count(a) > count(b)
 * (CompiMetaFirst / CompiMetaSecond, ReadQueue.h:340-353). */
typedef struct { uint32_t key; uint32_t v; } pent;
static int pcomp(const pent* a, const pent* b, int second)
{
    return second ? PC2(a->v) > PC2(b->v) : PC1(a->v) > PC1(b->v);
}
static void pswap(pent* a, pent* b) { pent t = *a; *a = *b; *b = t; }
static void ps_insertion(pent* f, pent* l, int sec)
{
    if (f == l) return;
    for (pent* i = f + 1; i != l; ++i) {
        pent val = *i;
        if (pcomp(&val, f, sec)) {
            memmove(f + 1, f, (size_t)(i - f) * sizeof(pent));
            *f = val;
        } else {
            pent* last = i;
            pent* next = i - 1;
            while (pcomp(&val, next, sec)) { *last = *next; last = next; --next; }
            *last = val;
        }
    }
}
static void ps_unguarded_insertion(pent* f, pent* l, int sec)
{
    for (pent* i = f; i != l; ++i) {
        pent val = *i;
        pent* last = i;
        pent* next = i - 1;
        while (pcomp(&val, next, sec)) { *last = *next; last = next; --next; }
        *last = val;
    }
}
static void ps_push_heap(pent* f, long hole, long top, pent val, int sec)
{
    long parent = (hole - 1) / 2;
    while (hole > top && pcomp(f + parent, &val, sec)) {
        f[hole] = f[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    f[hole] = val;
}
static void ps_adjust_heap(pent* f, long hole, long len, pent val, int sec)
{
    const long top = hole;
    long child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (pcomp(f + child, f + (child - 1), sec)) child--;
        f[hole] = f[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        f[hole] = f[child - 1];
        hole = child - 1;
    }
    ps_push_heap(f, hole, top, val, sec);
}
static void ps_make_heap(pent* f, pent* l, int sec)
{
    const long len = l - f;
    if (len < 2) return;
    long parent = (len - 2) / 2;
    while (1) {
        pent val = f[parent];
        ps_adjust_heap(f, parent, len, val, sec);
        if (parent == 0) return;
        parent--;
    }
}
static void ps_pop_heap(pent* f, pent* l, pent* result, int sec)
{
    pent val = *result;
    *result = *f;
    ps_adjust_heap(f, 0, l - f, val, sec);
}
static void ps_partial_sort(pent* f, pent* m, pent* l, int sec)
{
    ps_make_heap(f, m, sec);
    for (pent* i = m; i < l; ++i)
        if (pcomp(i, f, sec)) ps_pop_heap(f, m, i, sec);
    while (m - f > 1) { --m; ps_pop_heap(f, m, m, sec); }
}
static void ps_move_median_first(pent* r, pent* a, pent* b, pent* c, int sec)
{
    if (pcomp(a, b, sec)) {
        if (pcomp(b, c, sec)) pswap(r, b);
        else if (pcomp(a, c, sec)) pswap(r, c);
        else pswap(r, a);
    } else if (pcomp(a, c, sec)) pswap(r, a);
    else if (pcomp(b, c, sec)) pswap(r, c);
    else pswap(r, b);
}
static pent* ps_unguarded_partition(pent* f, pent* l, pent* pivot, int sec)
{
    while (1) {
        while (pcomp(f, pivot, sec)) ++f;
        --l;
        while (pcomp(pivot, l, sec)) --l;
        if (!(f < l)) return f;
        pswap(f, l);
        ++f;
    }
}
static void ps_introsort(pent* f, pent* l, long depth, int sec)
{
    while (l - f > 16) {
        if (depth == 0) { ps_partial_sort(f, l, l, sec); return; }
        --depth;
        pent* mid = f + (l - f) / 2;
        ps_move_median_first(f, f + 1, mid, l - 1, sec);
        pent* cut = ps_unguarded_partition(f + 1, l, f, sec);
        ps_introsort(cut, l, depth, sec);
        l = cut;
    }
}
static void std_sort_desc(pent* f, long n, int sec)
{
    if (n <= 1) return;
    long lg = 0;
    while ((1l << (lg + 1)) <= n) ++lg;
    ps_introsort(f, f + n, 2 * lg, sec);
    if (n > 16) {
        ps_insertion(f, f + 16, sec);
        ps_unguarded_insertion(f + 16, f + n, sec);
    } else {
        ps_insertion(f, f + n, sec);
    }
}

int orc_sort_desc(const uint32_t* keys, const uint8_t* counts, uint32_t n, uint32_t* out)
{
    pent* v = (pent*)malloc((n + 1) * sizeof(pent));
    for (uint32_t i = 0; i < n; ++i) { v[i].key = keys[i]; v[i].v = counts[i]; }
    std_sort_desc(v, n, 0);
    for (uint32_t i = 0; i < n; ++i) out[i] = v[i].key;
    free(v);
    return 0;
}

static int filtered_has(const orc_pe_extra* px, uint64_t k)
{
    uint64_t lo = 0, hi = px->n_filtered;
    while (lo < hi) { uint64_t mid = (lo + hi) >> 1; if (px->filtered[mid] < k) lo = mid + 1; else hi = mid; }
    return lo < px->n_filtered && px->filtered[lo] == k;
}

static inline uint32_t kseq_code(uint8_t c) { return (c == 'C' || c == 'T') ? 3u : (c == 'G' ? 2u : 0u); }

/* getSeedRefsFirstRead (ReadQueue.cpp:2468-2794) */
static void pe_first_read(const orc_index* ix, const orc_pe_extra* px, const uint8_t* seq, uint32_t size, pmap* pm)
{
    const uint32_t nk = size - KMERLEN + 1;
    uint32_t bucket_count = 0;
    uint64_t total = 0;
    uint64_t* keys = (uint64_t*)malloc(nk * sizeof(uint64_t));
    for (uint32_t p = 0; p < nk; ++p) {
        uint64_t st, ln;
        keys[p] = spaced_hash(seq + p) & HTAB_MASK;
        bucket_of(ix, keys[p], &st, &ln);
        bucket_count += (uint32_t)ln;
        total += ln;
    }
    bucket_count /= 5;
    pmap tmp[2];
    for (int s = 0; s < 2; ++s) pm_init(&tmp[s], bucket_count, total);
    uint32_t cMask = 0, kSeq = 0;
    for (uint32_t i = 0; i < KMERLEN; ++i) {
        cMask = (cMask << 1) | (seq[i] == 'C');
        kSeq = (kSeq << 2) + kseq_code(seq[i]);
    }
    const uint32_t maxQPos = size - KMERLEN + 1 - QTHRESH;
    for (uint32_t p = 0; p < nk; ++p) {
        if (p > 0) {
            const uint32_t cIdx = p - 1;
            kSeq = (kSeq << 2) + kseq_code(seq[KMERLEN + cIdx]);
            cMask = (cMask << 1) | (seq[KMERLEN + cIdx] == 'C');
            if (filtered_has(px, kSeq)) continue;
        }
        uint64_t st, ln;
        bucket_of(ix, keys[p], &st, &ln);
        uint64_t lastId = 0xffffffffffffffffULL;
        int wasFwd = 0, wasStart = 0;
        for (uint64_t i = st; i < st + ln; ++i) {
            const uint32_t meta = ix->kmer_meta[i];
            const uint32_t metaId = meta & 0x7fffffffu;
            if (cMask & SEEDBITS & px->kmer_tmask[i]) continue;
            const int isFwd = ix->strand[i] != 0;
            const int isStart = (int)(meta >> 31);
            if (metaId == lastId && isFwd == wasFwd && isStart == wasStart) continue;
            lastId = metaId; wasFwd = isFwd; wasStart = isStart;
            if (p == 0 || p - 1 < maxQPos) {
                uint32_t* v = pm_at(&tmp[isFwd], metaId);
                *v = (*v & ~0xffu) | ((PC1(*v) + 1) & 0xffu);
            } else {
                uint32_t* v = pm_find(&tmp[isFwd], metaId);
                if (v) *v = (*v & ~0xffu) | ((PC1(*v) + 1) & 0xffu);
            }
        }
    }
    free(keys);
    /* keep count1 >= qThreshold in new maps of 20 buckets, in the old order */
    for (int s = 0; s < 2; ++s) {
        pm_init(&pm[s], 20, 64);
        uint32_t* order = (uint32_t*)malloc((tmp[s].hm.nb_elem + 1) * sizeof(uint32_t));
        uint64_t n = map_order(&tmp[s].hm, order);
        for (uint64_t q = 0; q < n; ++q) {
            const uint32_t v = *pm_find(&tmp[s], order[q]);
            if (PC1(v) >= QTHRESH) *pm_at(&pm[s], order[q]) = PC1(v);
        }
        free(order);
        pm_free(&tmp[s]);
    }
}

/* getSeedRefsSecondRead (ReadQueue.cpp:2801-3164); returns hasCpG */
static int pe_second_read(const orc_index* ix, const orc_pe_extra* px, const uint8_t* seq, uint32_t size, pmap* pm)
{
    const int ctx = (int)((double)px->maxpdist / WINLEN) + 1;
    const uint32_t nk = size - KMERLEN + 1;
    uint32_t cMask = 0, kSeq = 0;
    for (uint32_t i = 0; i < KMERLEN; ++i) {
        cMask = (cMask << 1) | (seq[i] == 'C');
        kSeq = (kSeq << 2) + kseq_code(seq[i]);
    }
    const uint32_t maxQPos = size - KMERLEN + 1 - QTHRESH;
    for (uint32_t p = 0; p < nk; ++p) {
        if (p > 0) {
            const uint32_t cIdx = p - 1;
            kSeq = (kSeq << 2) + kseq_code(seq[KMERLEN + cIdx]);
            cMask = (cMask << 1) | (seq[KMERLEN + cIdx] == 'C');
            if (filtered_has(px, kSeq)) continue;
        }
        uint64_t st, ln;
        bucket_of(ix, spaced_hash(seq + p) & HTAB_MASK, &st, &ln);
        uint64_t lastId = 0xffffffffffffffffULL;
        int wasFwd = 0;
        for (uint64_t i = st; i < st + ln; ++i) {
            const uint32_t metaId = ix->kmer_meta[i] & 0x7fffffffu;
            if (cMask & SEEDBITS & px->kmer_tmask[i]) continue;
            const int isFwd = ix->strand[i] != 0;
            if (metaId == lastId && isFwd == wasFwd) continue;
            lastId = metaId; wasFwd = isFwd;
            if (p == 0 || p - 1 < maxQPos) {
                for (int c = -ctx; c <= ctx; ++c) {
                    if (pm_find(&pm[isFwd], metaId + (uint32_t)c)) {
                        uint32_t* v = pm_at(&pm[isFwd], metaId);
                        *v = (*v & ~0xff00u) | (((PC2(*v) + 1) & 0xffu) << 8);
                        break;
                    }
                }
            } else {
                uint32_t* v = pm_find(&pm[isFwd], metaId);
                if (v) *v = (*v & ~0xff00u) | (((PC2(*v) + 1) & 0xffu) << 8);
            }
        }
    }
    for (int dir = 1; dir >= 0; --dir) {
        uint32_t* order = (uint32_t*)malloc((pm[dir].hm.nb_elem + 1) * sizeof(uint32_t));
        uint64_t n = map_order(&pm[dir].hm, order);
        for (uint64_t q = 0; q < n; ++q) {
            uint32_t* v = pm_find(&pm[dir], order[q]);
            if (PC2(*v) >= QTHRESH) {
                *v |= PF2;
                for (int c = 1; c <= ctx; ++c) {
                    uint32_t* w = pm_find(&pm[dir], order[q] + (uint32_t)c);
                    if (w) *w |= PF2;
                    w = pm_find(&pm[dir], order[q] - (uint32_t)c);
                    if (w) *w |= PF2;
                }
            }
        }
        free(order);
    }
    for (int dir = 1; dir >= 0; --dir) {
        uint32_t* order = (uint32_t*)malloc((pm[dir].hm.nb_elem + 1) * sizeof(uint32_t));
        uint64_t n = map_order(&pm[dir].hm, order);
        for (uint64_t q = 0; q < n; ++q) {
            if ((*pm_find(&pm[dir], order[q]) & PF2) && ix->win_sind[order[q]] != CPGDUMMY) { free(order); return 1; }
        }
        free(order);
    }
    return 0;
}

typedef struct { uint64_t* m; uint32_t n, cap; } mvec;
static void mv_push(mvec* v, uint64_t x)
{
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 8; v->m = (uint64_t*)realloc(v->m, v->cap * 8); }
    v->m[v->n++] = x;
}

/* matchFwdFirst / matchRevFirst / matchFwdSecond / matchRevSecond (ReadQueue.cpp:4538-4776) */
static int pe_match_one(const orc_index* ix, const orc_pe_extra* px, pent* meta, int dir, int second, uint8_t* prevChr,
                        uint64_t* prevOff, mvec* mats, int32_t* bmCount, sa_t* sa, hits* h, pmap* pm)
{
    const int ctx = (int)((double)px->maxpdist / WINLEN) + 1;
    const int32_t cnt = (int32_t)(second ? PC2(meta->v) : PC1(meta->v));
    const int32_t thr = *bmCount - KMERDIST > (int32_t)QTHRESH ? *bmCount - KMERDIST : (int32_t)QTHRESH;
    if (cnt < thr) return 0;
    if (!(meta->v & (second ? PF3 : PF2))) return 1;
    const uint32_t w = meta->key;
    const uint32_t sp = ix->win_start[w];
    const uint8_t ch = ix->win_chrom[w];
    const uint8_t* g = ix->chrom_seq[ch];
    const int64_t L = (int64_t)ix->chrom_len[ch];
    if (dir) {
        int64_t e = (int64_t)sp + WINLEN + MISCOUNT + ADDMIS - 1;
        if (e > L) e = L;
        sa_query_fwd(sa, g + sp, (uint64_t)(e - (int64_t)sp), h);
    } else {
        /* matchRevSecond leaves the start unguarded (startPos - 1 for window 0, ReadQueue.cpp:4736) */
        int64_t lo = second ? (int64_t)sp - 1 : (sp > 0 ? (int64_t)sp - 1 : 0);
        int64_t hi = (int64_t)sp + WINLEN + MISCOUNT + ADDMIS - 1;
        if (hi >= L) hi = L - 1;
        sa_query_rev(sa, g, hi, lo, h);
    }
    uint32_t i = 0;
    if (h->n > 0 && h->off[0] + sp == *prevOff && ch == *prevChr) ++i;
    for (; i < h->n; ++i) mv_push(mats, mk_match((uint16_t)h->off[i], h->err[i], (uint64_t)dir, 0, w));
    if (h->n > 0) {
        if (cnt > *bmCount) *bmCount = cnt;
        if (!second) {
            *pm_find(&pm[dir], w) |= PF3;
            for (int c = 1; c <= ctx; ++c) {
                uint32_t* x = pm_find(&pm[dir], w + (uint32_t)c);
                if (x) *x |= PF3;
                x = pm_find(&pm[dir], w - (uint32_t)c);
                if (x) *x |= PF3;
            }
        }
        *prevChr = ch;
        *prevOff = sp + h->off[h->n - 1];
    } else {
        *prevChr = 0;
        *prevOff = 0xffffffffffffffffULL;
    }
    return 1;
}

/* saQuerySeedSetRefFirst / Second (ReadQueue.cpp:2167-2323) */
static void pe_query(const orc_index* ix, const orc_pe_extra* px, pmap* pm, int second, sa_t* sa, hits* h, mvec* mats)
{
    pent* lists[2];
    uint64_t nl[2];
    for (int dir = 0; dir < 2; ++dir) {
        uint32_t* order = (uint32_t*)malloc((pm[dir].hm.nb_elem + 1) * sizeof(uint32_t));
        nl[dir] = map_order(&pm[dir].hm, order);
        lists[dir] = (pent*)malloc((nl[dir] + 1) * sizeof(pent));
        for (uint64_t q = 0; q < nl[dir]; ++q) { lists[dir][q].key = order[q]; lists[dir][q].v = *pm_find(&pm[dir], order[q]); }
        free(order);
        std_sort_desc(lists[dir], (long)nl[dir], second);
    }
    int32_t bmCount = 0;
    uint8_t prevChr = 0;
    uint64_t prevOff = 0xffffffffffffffffULL;
    int order2[2];
    int nwalk = 0;
    if (nl[1] > 0) {
        if (nl[0] > 0) {
            /* both walks compare count1 of the heads (ReadQueue.cpp:2185, 2265) */
            if (PC1(lists[1][0].v) > PC1(lists[0][0].v)) { order2[0] = 1; order2[1] = 0; }
            else { order2[0] = 0; order2[1] = 1; }
            nwalk = 2;
        } else { order2[0] = 1; nwalk = 1; }
    } else if (nl[0] > 0) { order2[0] = 0; nwalk = 1; }
    for (int wk = 0; wk < nwalk; ++wk) {
        const int dir = order2[wk];
        if (wk == 1) { prevChr = 0; prevOff = 0xffffffffffffffffULL; }
        for (uint64_t q = 0; q < nl[dir]; ++q)
            if (!pe_match_one(ix, px, &lists[dir][q], dir, second, &prevChr, &prevOff, mats, &bmCount, sa, h, pm)) break;
    }
    free(lists[0]);
    free(lists[1]);
}

static int pe_extract(const orc_index* ix, const orc_pe_extra* px, uint64_t m1, uint64_t m2)
{
    if (ix->win_chrom[M_META(m1)] != ix->win_chrom[M_META(m2)]) return -1;
    const uint32_t p1 = (uint32_t)(ix->win_start[M_META(m1)] + M_OFF(m1));
    const uint32_t p2 = (uint32_t)(ix->win_start[M_META(m2)] + M_OFF(m2));
    const uint32_t d = p2 > p1 ? p2 - p1 : p1 - p2;
    if (d <= px->maxpdist + ix->readlen) return (int)(M_ERR(m1) + M_ERR(m2));
    return -1;
}

typedef struct { uint64_t succ, nonu, unsucc, paired, tooShort, r1f, r1r; int matchR1Fwd; } pstats;

static int rc_read(const uint8_t* s, uint32_t n, uint8_t* out)
{
    int bad = 0;
    for (uint32_t p = 0, q = n - 1; p < n; ++p, --q) {
        switch (s[p]) {
            case 'A': out[q] = 'T'; break;
            case 'C': out[q] = 'G'; break;
            case 'G': out[q] = 'C'; break;
            case 'T': out[q] = 'A'; break;
            default: bad = 1; break; /* N and other letters invalidate a mate */
        }
    }
    return bad;
}

static void pe_chunk(const orc_index* ix, const orc_pe_extra* px, const uint8_t* s1, const uint64_t* o1, const uint8_t* s2,
                     const uint64_t* o2, uint32_t n, int getStranded, int both, pstats* st, uint64_t* mats1,
                     uint64_t* mats2, uint8_t* inv1, uint8_t* inv2, uint16_t* meth)
{
    sa_t sa;
    hits h = {0};
    const float minlen = ceilf((float)ix->readlen * 0.75f);
    for (uint32_t r = 0; r < n; ++r) {
        const uint32_t n1 = (uint32_t)(o1[r + 1] - o1[r]), n2 = (uint32_t)(o2[r + 1] - o2[r]);
        uint8_t* f1 = (uint8_t*)calloc(n1 + 1, 1);
        uint8_t* f2 = (uint8_t*)calloc(n2 + 1, 1);
        uint8_t* r1 = (uint8_t*)calloc(n1 + 1, 1);
        uint8_t* r2 = (uint8_t*)calloc(n2 + 1, 1);
        memcpy(f1, s1 + o1[r], n1);
        memcpy(f2, s2 + o2[r], n2);
        int bad1 = (float)n1 < minlen, bad2 = (float)n2 < minlen;
        mats1[r] = mats2[r] = 0;
        if (bad1 || bad2) st->tooShort++;
        if (n1 && rc_read(f1, n1, r1)) bad1 = 1;
        if (n2 && rc_read(f2, n2, r2)) bad2 = 1;
        inv1[r] = (uint8_t)bad1;
        inv2[r] = (uint8_t)bad2;
        if (bad1 || bad2) { st->tooShort += 2; goto next; }
        {
            mvec m1F = {0}, m2R = {0}, m1R = {0}, m2F = {0};
            for (int o = 0; o < 2; ++o) {
                const int run = o == 0 ? (both || getStranded || st->matchR1Fwd) : (both || getStranded || !st->matchR1Fwd);
                if (!run) continue;
                uint8_t* first = o == 0 ? f1 : r1;
                uint8_t* sec = o == 0 ? r2 : f2;
                mvec* ma = o == 0 ? &m1F : &m1R;
                mvec* mb = o == 0 ? &m2R : &m2F;
                pmap pm[2];
                pe_first_read(ix, px, first, n1, pm);
                if (pm_size(&pm[1]) || pm_size(&pm[0])) {
                    if (pe_second_read(ix, px, sec, n2, pm)) {
                        sa_load(&sa, first, n1);
                        pe_query(ix, px, pm, 0, &sa, &h, ma);
                        if (ma->n) {
                            sa_load(&sa, sec, n2);
                            pe_query(ix, px, pm, 1, &sa, &h, mb);
                        }
                    }
                }
                pm_free(&pm[0]);
                pm_free(&pm[1]);
            }
            if ((m1F.n == 0 && m1R.n == 0) || (m2F.n == 0 && m2R.n == 0)) {
                inv1[r] = inv2[r] = 1;
                st->unsucc += 2;
            } else {
                const int WORST = 2 * (MISCOUNT + ADDMIS) + 1;
                int best = WORST, nonUnique = 0, orig = 1;
                uint64_t b1 = 0, b2 = 0;
                if (both || getStranded || st->matchR1Fwd)
                    for (uint32_t a = 0; a < m1F.n; ++a)
                        for (uint32_t b = 0; b < m2R.n; ++b) {
                            const int e = pe_extract(ix, px, m1F.m[a], m2R.m[b]);
                            if (e < 0) continue;
                            if (e == best) nonUnique = 1;
                            else if (e < best) { best = e; b1 = m1F.m[a]; b2 = m2R.m[b]; nonUnique = 0; }
                        }
                if (both || getStranded || !st->matchR1Fwd)
                    for (uint32_t a = 0; a < m1R.n; ++a)
                        for (uint32_t b = 0; b < m2F.n; ++b) {
                            const int e = pe_extract(ix, px, m1R.m[a], m2F.m[b]);
                            if (e < 0) continue;
                            if (e == best) nonUnique = 1;
                            else if (e < best) { best = e; b1 = m1R.m[a]; b2 = m2F.m[b]; orig = 0; nonUnique = 0; }
                        }
                if (best == WORST) { inv1[r] = inv2[r] = 1; st->unsucc += 2; }
                else if (nonUnique) { st->nonu += 2; inv1[r] = inv2[r] = 1; }
                else {
                    mats1[r] = b1;
                    mats2[r] = b2;
                    if (orig) {
                        if (getStranded) st->r1f++;
                        compute_meth(ix, b1, f1, n1, meth);
                        compute_meth(ix, b2, r2, n2, meth);
                    } else {
                        if (getStranded) st->r1r++;
                        compute_meth(ix, b1, r1, n1, meth);
                        compute_meth(ix, b2, f2, n2, meth);
                    }
                    const int d1 = ix->win_sind[M_META(b1)] == CPGDUMMY, d2 = ix->win_sind[M_META(b2)] == CPGDUMMY;
                    if (d1 && d2) st->tooShort += 2;
                    else if (d1 || d2) { st->tooShort++; st->succ++; }
                    else { st->paired++; st->succ += 2; }
                }
            }
            free(m1F.m); free(m2R.m); free(m1R.m); free(m2F.m);
        }
    next:
        if (inv1[r]) mats1[r] = 0;
        if (inv2[r]) mats2[r] = 0;
        free(f1); free(f2); free(r1); free(r2);
    }
    free(h.off);
    free(h.err);
}

/* queryRoutinePaired loop (main.cpp:400-441) */
int orc_match_pe(const orc_index* ix, const orc_pe_extra* px, const uint8_t* s1, const uint64_t* o1, const uint8_t* s2,
                 const uint64_t* o2, uint32_t n, uint32_t chunk, int both_strands, uint64_t* mats1, uint64_t* mats2,
                 uint8_t* inv1, uint8_t* inv2, uint16_t* meth, uint64_t* counters)
{
    pstats st;
    memset(&st, 0, sizeof(st));
    st.matchR1Fwd = 1;
    if (chunk == 0) chunk = 300000;
    memset(meth, 0, sizeof(uint16_t) * 4 * ix->n_cpg);
    for (uint32_t c0 = 0, ci = 0; c0 < n; c0 += chunk, ++ci) {
        const uint32_t cn = n - c0 < chunk ? n - c0 : chunk;
        const int stranded = ci == 0 && !both_strands;
        pe_chunk(ix, px, s1, o1 + c0, s2, o2 + c0, cn, stranded, both_strands, &st, mats1 + c0, mats2 + c0, inv1 + c0,
                 inv2 + c0, meth);
        if (stranded) st.matchR1Fwd = st.r1f > st.r1r;
    }
    counters[0] = st.succ; counters[1] = st.nonu; counters[2] = st.unsucc; counters[3] = st.paired;
    counters[4] = st.tooShort; counters[5] = st.r1f; counters[6] = st.r1r; counters[7] = (uint64_t)st.matchR1Fwd;
    return 0;
}
