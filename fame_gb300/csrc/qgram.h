// Exact q-gram pre-filter of the Shift-And window scans (host and device).
//
// Any alignment of a read with <= NERR edits leaves one of NERR + 1 disjoint
// read pieces without an edit, so the first q bases of that piece occur in the
// window text, equal in the reduced alphabet A / G / C=T that the bisulfite
// match implies (a read T matches a reference C, ShiftAnd.h:399-402).  For
// each such occurrence this pass emits the span of scan positions where the
// alignment can end: [x - 1 + m - start_k - NERR, x - 1 + m - start_k + NERR],
// x being the scan position of the occurrence's first base.
//
// The pass walks the packed genome in genome order, 16 bases per word, for
// both scan directions: a reverse window scans the complemented text from its
// last base down, so its scan-order q-gram key, read in genome order, has its
// first scan symbol in the low bits — the same bit order as the packed words.
// A forward window's scan-order key is compared after reversing its symbol
// order.  Bases outside the window are treated like N bases (no q-gram covers
// them), which is also what the full scan does: its q-gram count restarts at
// the window start and after every N.
#pragma once
#include <stdint.h>

#include "fame_const.h"

#if defined(__CUDACC__)
#define FAME_HD __host__ __device__ __forceinline__
#else
#define FAME_HD inline
#endif

namespace fame {

constexpr int QG_PIECES = (int)NERR + 1;

template <class T>
FAME_HD T qg_load(const T* p)
{
#if defined(__CUDA_ARCH__)
    return __ldg(p);
#else
    return *p;
#endif
}

// Reduced symbols (A0 G1 C/T2) of 16 packed bases (A0 C1 G2 T3, base i at bits
// 2i), of the bases themselves (fwd) or of their complements (reverse scans).
FAME_HD uint32_t qg_reduce(uint32_t w, int fwd)
{
    const uint32_t L = w & 0x55555555u, H = (w >> 1) & 0x55555555u;
    return fwd ? ((L << 1) | (H & ~L)) : (((~L & 0x55555555u) << 1) | (L & ~H));
}

FAME_HD uint32_t qg_symrev(uint32_t key, uint32_t q)
{
    uint32_t r = 0;
    for (uint32_t i = 0; i < q; ++i) r |= ((key >> (2 * i)) & 3u) << (2 * (q - 1 - i));
    return r;
}

// Spans for one window whose text is the packed-genome range [G0, G1)
// (forward: scan position u = genome G0 + u; reverse: u = genome G1 - 1 - u).
// pkey[k]: scan-order key of piece k (first symbol most significant), valid
// where bit k of pvalid is set; pstart[k]: the piece's first read position.
// Writes at most CAP spans and returns their number, or -1 when there are more.
template <int CAP>
FAME_HD int qgram_spans(const uint32_t* gpack, const uint32_t* gnmask, uint64_t G0, uint64_t G1, int fwd, uint32_t m,
                        uint32_t q, const uint32_t* pkey, uint32_t pvalid, const uint32_t* pstart, int32_t* ilo,
                        int32_t* ihi)
{
    if (G1 <= G0 || q == 0 || q > 16 || !(pvalid & ((1u << QG_PIECES) - 1))) return 0;
    pvalid &= (1u << QG_PIECES) - 1;
    const int32_t len = (int32_t)(G1 - G0);
    const uint32_t qmask = q >= 16 ? 0xffffffffu : ((1u << (2 * q)) - 1);
    // compare keys in genome order; an invalid piece repeats the key of the
    // first valid one (the hit path skips it)
#if defined(__CUDA_ARCH__)
    const int kv = __ffs(pvalid) - 1;
#else
    const int kv = __builtin_ctz(pvalid);
#endif
    const uint32_t kfill = fwd ? qg_symrev(pkey[kv], q) : pkey[kv];
    uint32_t ckey[QG_PIECES];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
    for (int k = 0; k < QG_PIECES; ++k)
        ckey[k] = ((pvalid >> k) & 1u) ? (fwd ? qg_symrev(pkey[k], q) : pkey[k]) : kfill;
    const uint32_t nq = (1u << q) - 1;
    const uint64_t w0 = G0 >> 4, w1 = (G1 - 1) >> 4;
    uint64_t catS = 0;           // reduced symbols: previous word in bits 0..31, current in 32..63
    uint32_t catN = 0xffffffffu; // excluded bases (N or outside the window), one bit per base, same layout
    int n = 0;
    for (uint64_t wi = w0; wi <= w1; ++wi) {
        uint32_t nb = (qg_load(gnmask + (wi >> 1)) >> (16 * (uint32_t)(wi & 1))) & 0xffffu;
        if (wi == w0) nb |= (1u << (G0 & 15)) - 1;
        if (wi == w1) nb |= (0xffffu << (((G1 - 1) & 15) + 1)) & 0xffffu;
        catS = (catS >> 32) | ((uint64_t)qg_reduce(qg_load(gpack + wi), fwd) << 32);
        catN = (catN >> 16) | (nb << 16);
        // q-gram ending at base i of this word starts at bit 17 + i - q
        const uint64_t sS = catS >> (2 * (17 - q));
        const uint32_t sN = catN >> (17 - q);
        // positions whose key equals a piece key (branch-free; hits are rare)
        uint32_t hm = 0;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int i = 0; i < 16; ++i) {
            const uint32_t key = (uint32_t)(sS >> (2 * i)) & qmask;
            bool eq = false;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
            for (int k = 0; k < QG_PIECES; ++k) eq |= key == ckey[k];
            hm |= (eq ? 1u : 0u) << i;
        }
        if (!hm) continue;
        for (int i = 0; i < 16; ++i) {
            if (!((hm >> i) & 1u) || ((sN >> i) & nq)) continue;
            const uint32_t key = (uint32_t)(sS >> (2 * i)) & qmask;
            const int64_t A = (int64_t)(16 * wi + (uint64_t)i) - (int64_t)q + 1;   // genome start of the q-gram
            const int32_t x = fwd ? (int32_t)(A - (int64_t)G0) : (int32_t)((int64_t)G1 - A - (int64_t)q);
            for (int k = 0; k < QG_PIECES; ++k) {
                if (!((pvalid >> k) & 1u) || key != ckey[k]) continue;
                const int32_t end0 = x - 1 + (int32_t)(m - pstart[k]);
                int32_t a = end0 - (int32_t)NERR, b = end0 + (int32_t)NERR;
                if (b < 0 || a > len - 1) continue;
                if (a < 0) a = 0;
                if (b > len - 1) b = len - 1;
                if (n >= CAP) return -1;
                ilo[n] = a;
                ihi[n] = b;
                ++n;
            }
        }
    }
    return n;
}

}  // namespace fame
