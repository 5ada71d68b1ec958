// Bit-parallel scan that answers, at every text position, what the 7-layer
// ShiftAnd<6> automaton (ShiftAnd.h:121-432) answers there: the smallest
// k <= NERR such that the whole read aligns with <= k edits to a text
// substring ending at this position, or "no match".  Host and device.
//
// ShiftAnd's layer k after text letter t is the set {j : D[j][t] <= k} of the
// edit-distance table D (pattern prefix j, text up to t, free start in the
// text, D[j][0] = j after a reset), so its smallest accepting layer is
// D[m][t] whenever that is <= NERR.  This keeps the column of D as Myers'
// vertical-delta bit-vectors (G. Myers, "A fast bit-vector algorithm for
// approximate string matching based on dynamic programming", J. ACM 46(3),
// 1999): Pv / Mv hold the rows whose delta D[j] - D[j-1] is +1 / -1, one
// step per text letter costs a handful of word operations and one carry
// chain, and D[m][t] is tracked as a running score.
//
// Layout: 32 * NW rows, the read in the top m of them (row d + p = read
// position p, d = 32 * NW - m), so the score row is always the top bit.  The
// d rows below accept every letter and start at D = 0, so D stays 0 there
// and the row under the read acts as the free-start row 0.  Matching is the
// asymmetric bisulfite rule of loadBitmasks (ShiftAnd.h:345-432): a read T
// accepts a text C as well as a text T; a read N accepts nothing.
#pragma once
#include <stdint.h>

#include "fame_const.h"

#if defined(__CUDACC__)
#define FAME_HD __host__ __device__ __forceinline__
#else
#define FAME_HD inline
#endif

namespace fame {

// s = a + b over NW 32-bit words (word 0 least significant).
template <int NW>
FAME_HD void es_add(uint32_t* s, const uint32_t* a, const uint32_t* b)
{
#if defined(__CUDA_ARCH__)
    // one asm statement per width so the carry flag never leaves it
    if constexpr (NW == 2) {
        asm("add.cc.u32 %0, %2, %4;\n\taddc.u32 %1, %3, %5;"
            : "=r"(s[0]), "=r"(s[1]) : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
    } else if constexpr (NW == 4) {
        asm("add.cc.u32 %0, %4, %8;\n\taddc.cc.u32 %1, %5, %9;\n\taddc.cc.u32 %2, %6, %10;\n\taddc.u32 %3, %7, %11;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
    } else if constexpr (NW == 6) {
        asm("add.cc.u32 %0, %6, %12;\n\taddc.cc.u32 %1, %7, %13;\n\taddc.cc.u32 %2, %8, %14;\n\t"
            "addc.cc.u32 %3, %9, %15;\n\taddc.cc.u32 %4, %10, %16;\n\taddc.u32 %5, %11, %17;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]),
              "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]));
    } else {
        static_assert(NW == 8, "EditScan widths are 2, 4, 6 or 8 words");
        asm("add.cc.u32 %0, %8, %16;\n\taddc.cc.u32 %1, %9, %17;\n\taddc.cc.u32 %2, %10, %18;\n\t"
            "addc.cc.u32 %3, %11, %19;\n\taddc.cc.u32 %4, %12, %20;\n\taddc.cc.u32 %5, %13, %21;\n\t"
            "addc.cc.u32 %6, %14, %22;\n\taddc.u32 %7, %15, %23;"
            : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7])
            : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]),
              "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
    }
#else
    uint64_t c = 0;
    for (int j = 0; j < NW; ++j) {
        c += (uint64_t)a[j] + b[j];
        s[j] = (uint32_t)c;
        c >>= 32;
    }
#endif
}

// (hi:lo) << 1, upper word
FAME_HD uint32_t es_shl1(uint32_t lo, uint32_t hi)
{
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, 1);
#else
    return (hi << 1) | (lo >> 31);
#endif
}

// W: 64-bit pattern words of the ShiftAnd layout (read length / 64 + 1); the
// scan uses 2 * W words of 32 bits, enough for reads of up to 64 * W - 1 bases.
template <int W>
struct EditScan {
    static constexpr int NW = 2 * W;
    uint32_t peq[4][NW];   // rows accepting text letter A, C, G, T
    uint32_t pv[NW], mv[NW];
    int score;             // D[m][t]
    uint32_t plen;

    // Read position p is raw[p] (orient 0) or the complement of raw[len-1-p].
    FAME_HD void load(const char* raw, uint32_t len, int orient)
    {
        plen = len;
        const int d = 32 * NW - (int)len;
        // word j holds rows 32j .. 32j + 31, built from its top row down
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = 0; j < NW; ++j) {
            uint32_t tA = 0, tC = 0, tG = 0, tT = 0;
            for (int row = 32 * j + 31; row >= 32 * j; --row) {
                tA <<= 1; tC <<= 1; tG <<= 1; tT <<= 1;
                if (row >= d) {
                    const uint32_t p = (uint32_t)(row - d);
                    uint8_t c = (uint8_t)(orient ? raw[len - 1 - p] : raw[p]);
                    if (orient) c = c == 'A' ? 'T' : c == 'C' ? 'G' : c == 'G' ? 'C' : c == 'T' ? 'A' : c;
                    tA |= c == 'A' ? 1u : 0u;
                    tC |= (c == 'C' || c == 'T') ? 1u : 0u;
                    tG |= c == 'G' ? 1u : 0u;
                    tT |= c == 'T' ? 1u : 0u;
                } else {
                    tA |= 1; tC |= 1; tG |= 1; tT |= 1;
                }
            }
            peq[0][j] = tA; peq[1][j] = tC; peq[2][j] = tG; peq[3][j] = tT;
        }
    }

    // The rows of load() from bit masks already built (row 32j + l of word j).
    FAME_HD void set(const uint32_t* m4, uint32_t len)
    {
        plen = len;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = 0; j < NW; ++j) {
            peq[0][j] = m4[j]; peq[1][j] = m4[NW + j]; peq[2][j] = m4[2 * NW + j]; peq[3][j] = m4[3 * NW + j];
        }
    }

    FAME_HD void reset()
    {
        const int d = 32 * NW - (int)plen;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = 0; j < NW; ++j) {
            const int lo = 32 * j - d;   // rows of word j below the read: -lo of them when lo < 0
            pv[j] = lo >= 0 ? 0xffffffffu : (lo <= -32 ? 0u : 0xffffffffu << (uint32_t)(-lo));
            mv[j] = 0;
        }
        score = (int)plen;
    }

    // One text letter, 0..3 = A C G T.
    FAME_HD void letter(int b)
    {
        uint32_t eq[NW], t[NW], s[NW], ph[NW], mh[NW];
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = 0; j < NW; ++j) {
            const uint32_t x = (b & 1) ? peq[1][j] : peq[0][j];
            const uint32_t y = (b & 1) ? peq[3][j] : peq[2][j];
            eq[j] = (b & 2) ? y : x;
            t[j] = eq[j] & pv[j];
        }
        es_add<NW>(s, t, pv);
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = 0; j < NW; ++j) {
            const uint32_t xh = (s[j] ^ pv[j]) | eq[j];
            ph[j] = mv[j] | ~(xh | pv[j]);
            mh[j] = pv[j] & xh;
        }
        score += (int)(ph[NW - 1] >> 31) - (int)(mh[NW - 1] >> 31);
        // horizontal deltas move up one row; row 0's is 0 (free start in the text)
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = NW - 1; j > 0; --j) {
            ph[j] = es_shl1(ph[j - 1], ph[j]);
            mh[j] = es_shl1(mh[j - 1], mh[j]);
        }
        ph[0] <<= 1;
        mh[0] <<= 1;
#if defined(__CUDA_ARCH__)
#pragma unroll
#endif
        for (int j = 0; j < NW; ++j) {
            const uint32_t xv = eq[j] | mv[j];
            pv[j] = mh[j] | ~(xv | ph[j]);
            mv[j] = ph[j] & xv;
        }
    }

    // isMatch (ShiftAnd.h:323-341): the smallest accepting layer, or -1
    FAME_HD int match() const { return score <= (int)NERR ? score : -1; }
};

}  // namespace fame
