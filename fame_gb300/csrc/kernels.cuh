// Matching kernels after seeding: Shift-And window scans, candidate
// selection with the exact-match CpG calls, and the banded DP CpG calls.
#pragma once
#include <type_traits>

#include "editscan.h"
#include "qgram.h"
#include "seed.cuh"

namespace fame {

// Full scan of one candidate window (querySeq / queryRevSeq, ShiftAnd.h:130-255,
// on the text spans of saQuerySeedSetRef, ReadQueue.cpp:1953-1962, 2048-2058).
// emit(offset, errors) is called once per run of consecutive accepting bases,
// with the last position holding the run's smallest error count.
// unguarded: the reverse scan starts at startPos - 1 even for a window at
// position 0 (matchRevSecond, ReadQueue.cpp:4736), i.e. it includes base 0.
template <int W, class Emit>
__device__ __forceinline__ void scan_window_full(const DevIndex& ix, EditScan<W>& sa, uint32_t wid, int fwd, Emit emit,
                                 bool unguarded = false)
{
    const uint4 wi = ix.win[wid];
    const uint32_t sp = wi.x, ch = wi.y;
    const int64_t L = (int64_t)ix.chrom_len[ch];
    const uint64_t g0 = ix.chrom_off[ch];
    sa.reset();
    bool was = false;
    uint32_t cur_off = 0;
    int cur_err = 0;
    uint32_t ncl = 0;
    const uint32_t gate = sa.plen - NERR;
    if (fwd) {
        int64_t e = (int64_t)sp + WIN_TEXT;
        if (e > L) e = L;
        uint64_t g = g0 + sp;
        uint32_t wpack = __ldg(ix.gpack + (g >> 4)), wn = __ldg(ix.gnmask + (g >> 5));
        for (int64_t t = sp; t < e; ++t, ++g) {
            if ((g & 15) == 0) wpack = __ldg(ix.gpack + (g >> 4));
            if ((g & 31) == 0) wn = __ldg(ix.gnmask + (g >> 5));
            if ((wn >> (g & 31)) & 1u) { sa.reset(); continue; }
            sa.letter((int)((wpack >> (2 * (g & 15))) & 3u));
            if (++ncl < gate) continue;
            const int er = sa.match();
            const uint32_t off = (uint32_t)(t - sp) + MISCOUNT;
            if (er >= 0) {
                if (was) { if (er <= cur_err) { cur_off = off; cur_err = er; } }
                else { was = true; cur_off = off; cur_err = er; }
            } else if (was) {
                emit(cur_off, cur_err);
                was = false;
            }
        }
    } else {
        const int64_t lo = (sp > 0 || unguarded) ? (int64_t)sp - 1 : 0;
        int64_t hi = (int64_t)sp + WIN_TEXT;
        if (hi >= L) hi = L - 1;
        uint64_t g = g0 + (uint64_t)hi;
        uint32_t wpack = __ldg(ix.gpack + (g >> 4)), wn = __ldg(ix.gnmask + (g >> 5));
        for (int64_t t = hi; t != lo; --t, --g) {
            if ((g & 15) == 15) wpack = __ldg(ix.gpack + (g >> 4));
            if ((g & 31) == 31) wn = __ldg(ix.gnmask + (g >> 5));
            if ((wn >> (g & 31)) & 1u) { sa.reset(); continue; }
            sa.letter(3 - (int)((wpack >> (2 * (g & 15))) & 3u));
            if (++ncl < gate) continue;
            const int er = sa.match();
            const uint32_t off = (uint32_t)(t - lo) + sa.plen - 1 + MISCOUNT;
            if (er >= 0) {
                if (was) { if (er <= cur_err) { cur_off = off; cur_err = er; } }
                else { was = true; cur_off = off; cur_err = er; }
            } else if (was) {
                emit(cur_off, cur_err);
                was = false;
            }
        }
    }
    if (was) emit(cur_off, cur_err);
}


// Text of a window in scan order: forward windows run over [sp, e), reverse
// windows from hi down to lo + 1 with every base complemented.
struct ScanText {
    const DevIndex* ix;
    uint64_t g0;      // packed-genome index of scan position 0
    int dir;          // +1 forward, -1 reverse
    uint32_t len;     // scan positions
    uint32_t off_a;   // reported offset = off_a + dir_sign * u (see off())
    int fwd;
    __device__ __forceinline__ uint32_t off(uint32_t u) const { return fwd ? u + MISCOUNT : off_a - u; }
    // genome range [G0, G1) of the text
    __device__ __forceinline__ uint64_t G0() const { return fwd ? g0 : g0 + 1 - len; }
};

// The text querySeq / queryRevSeq scan for window wid (saQuerySeedSetRef,
// ReadQueue.cpp:1953-1962, 2048-2058) for a read of m bases.
__device__ __forceinline__ ScanText window_text(const DevIndex& ix, uint32_t wid, int fwd, bool unguarded,
                                                uint32_t m)
{
    const uint4 wi = ix.win[wid];
    const uint32_t sp = wi.x, ch = wi.y;
    const int64_t L = (int64_t)ix.chrom_len[ch];
    const uint64_t gch = ix.chrom_off[ch];
    ScanText tx;
    tx.ix = &ix;
    tx.fwd = fwd;
    if (fwd) {
        int64_t e = (int64_t)sp + WIN_TEXT;
        if (e > L) e = L;
        tx.g0 = gch + sp;
        tx.dir = 1;
        tx.len = (uint32_t)(e - (int64_t)sp);
        tx.off_a = 0;
    } else {
        const int64_t lo = (sp > 0 || unguarded) ? (int64_t)sp - 1 : 0;
        int64_t hi = (int64_t)sp + WIN_TEXT;
        if (hi >= L) hi = L - 1;
        tx.g0 = gch + (uint64_t)hi;
        tx.dir = -1;
        tx.len = (uint32_t)(hi - lo);
        tx.off_a = (uint32_t)(hi - lo) + m - 1 + MISCOUNT;
    }
    return tx;
}

// The automaton over nm merged spans (ascending, disjoint; span(i) returns
// lo | hi << 16 in scan positions).  Each span is entered at least m + 7
// positions early (the state at a position depends on the last m + 6 bases
// only, and a reset state never accepts where the full scan would not) or
// continued from the previous span, and extended until its run of accepting
// positions ends.  N bases reset the automaton exactly as in the full scan.
template <int W, class Span, class Emit>
__device__ __forceinline__ void run_spans(EditScan<W>& sa, const ScanText& tx, int nm, Span span, Emit emit)
{
    const DevIndex& ix = *tx.ix;
    const uint32_t m = sa.plen;
    const uint32_t gate = m - NERR;
    bool was = false;
    uint32_t cur_off = 0;
    int cur_err = 0;
    uint32_t ncl = 0;
    int64_t cursor = -1;
    uint64_t cw = ~0ull, cwn = ~0ull;   // genome words held in wpack / wn
    uint32_t wpack = 0, wn = 0;
    sa.reset();
    for (int i = 0; i < nm; ++i) {
        const uint32_t sv = span(i);
        const int64_t lo = (int64_t)(sv & 0xffffu), hi = (int64_t)(sv >> 16);
        int64_t start = lo - (int64_t)(m + NERR + 1);
        if (start < 0) start = 0;
        if (start <= cursor + 1) {
            start = cursor + 1;
        } else {
            sa.reset();
            ncl = 0;
        }
        int64_t u = start;
        for (; u < (int64_t)tx.len && (u <= hi || was); ++u) {
            const uint64_t g = tx.dir > 0 ? tx.g0 + (uint64_t)u : tx.g0 - (uint64_t)u;
            if ((g >> 4) != cw) { cw = g >> 4; wpack = __ldg(ix.gpack + cw); }
            if ((g >> 5) != cwn) { cwn = g >> 5; wn = __ldg(ix.gnmask + cwn); }
            if ((wn >> (g & 31)) & 1u) { sa.reset(); continue; }
            const int b = (int)((wpack >> (2 * (g & 15))) & 3u);
            sa.letter(tx.fwd ? b : 3 - b);
            if (++ncl < gate) continue;
            const int er = sa.match();
            if (er >= 0) {
                const uint32_t off = tx.off((uint32_t)u);
                if (was) { if (er <= cur_err) { cur_off = off; cur_err = er; } }
                else { was = true; cur_off = off; cur_err = er; }
            } else if (was) {
                emit(cur_off, cur_err);
                was = false;
            }
        }
        cursor = u - 1;
        if (u >= (int64_t)tx.len) break;
    }
    if (was) emit(cur_off, cur_err);
}

// Scan of one candidate window by one thread, with the same hits as
// scan_window_full.
//
// Any alignment of the read with <= 6 edits leaves one of 7 disjoint read
// pieces without an edit, so that piece's first q bases occur in the text
// (equal in the reduced alphabet A / G / C=T, which the asymmetric match
// implies).  A cheap pass finds those q-gram occurrences and turns each into
// the span of scan positions where the alignment can end; the automaton then
// runs only over the merged spans (run_spans).  Too many spans (repetitive
// windows) fall back to the full scan.
template <int W, class Emit>
__device__ void scan_window(const DevIndex& ix, EditScan<W>& sa, uint32_t wid, int fwd, Emit emit,
                            const uint32_t* pkey, uint32_t pvalid, uint32_t q, const uint32_t* pstart,
                            bool unguarded = false)
{
    constexpr int CAP = 32;
    const ScanText tx = window_text(ix, wid, fwd, unguarded, sa.plen);
    const uint32_t m = sa.plen;
    // ---- q-gram pass
    int32_t ilo[CAP], ihi[CAP];
    const uint64_t G0 = tx.G0(), G1 = G0 + tx.len;
    const int nint = qgram_spans<CAP>(ix.gpack, ix.gnmask, G0, G1, fwd, m, q, pkey, pvalid, pstart, ilo, ihi);
    if (nint < 0) { scan_window_full<W>(ix, sa, wid, fwd, emit, unguarded); return; }
    if (nint == 0) return;
    // sort spans by start and merge overlapping ones
    for (int i = 1; i < nint; ++i) {
        const int32_t a = ilo[i], b = ihi[i];
        int j = i - 1;
        while (j >= 0 && ilo[j] > a) { ilo[j + 1] = ilo[j]; ihi[j + 1] = ihi[j]; --j; }
        ilo[j + 1] = a;
        ihi[j + 1] = b;
    }
    int nm = 0;
    for (int i = 0; i < nint; ++i) {
        if (nm > 0 && ilo[i] <= ihi[nm - 1] + 1) { if (ihi[i] > ihi[nm - 1]) ihi[nm - 1] = ihi[i]; }
        else { ilo[nm] = ilo[i]; ihi[nm] = ihi[i]; ++nm; }
    }
    run_spans<W>(sa, tx, nm, [&](int i) { return (uint32_t)ilo[i] | ((uint32_t)ihi[i] << 16); }, emit);
}

// The q-gram pass of one candidate window run by a whole warp (every lane
// calls it with the same arguments): lane k < 7 builds piece k's key, lanes
// own consecutive packed words of the text (coalesced loads, each word's
// predecessor by shuffle), hits append raw spans to a per-warp list, and the
// list is sorted and merged with warp scans.  Writes the merged spans
// (lo | hi << 16, ascending) to pool[0..) and returns their number, or -1 when
// the window has more than 32 raw spans or more than pool_cap merged ones
// (the caller then scans the whole window).  Same spans as qgram_spans plus
// scan_window's merge.
//
// Key test: when some bit offset s gives the distinct piece keys distinct
// 5-bit fields (key >> s) & 31, the keys sit in a 32-slot table at their
// fields (tab; tabp[slot] = the pieces with that key) and a text position is
// tested with one table read and one compare; otherwise with 7 compares.  The
// N and window-edge masks are only built for a word with a key hit.
__device__ int qgram_spans_warp(const DevIndex& ix, const char* raw, uint32_t m, int orient, const ScanText& tx,
                                uint32_t* pool, int pool_cap, int32_t* rlo, int32_t* rhi, uint32_t* rn,
                                uint32_t* tab, uint32_t* tabp, uint32_t lane)
{
    constexpr uint32_t FULL = 0xffffffffu;
    const uint32_t q = min(16u, m / 7);
    if (q == 0 || tx.len == 0) return 0;
    const int fwd = tx.fwd;
    // ---- piece keys (scan order, first symbol most significant), compared in genome order
    uint32_t key = 0;
    bool ok = lane < (uint32_t)QG_PIECES;
    if (ok) {
        const uint32_t st = (lane * m) / 7;
        for (uint32_t i = 0; i < q; ++i) {
            const uint32_t p = st + i;
            const uint8_t c = orient ? rc_byte((uint8_t)raw[m - 1 - p]) : (uint8_t)raw[p];
            uint32_t sym;
            switch (c) {
                case 'A': sym = 0; break;
                case 'G': sym = 1; break;
                case 'C': case 'T': sym = 2; break;
                default: sym = 3; ok = false; break;
            }
            key = (key << 2) | sym;
        }
        if (fwd) key = qg_symrev(key, q);
    }
    const uint32_t pvalid = __ballot_sync(FULL, ok) & ((1u << QG_PIECES) - 1);
    if (!pvalid) return 0;
    const uint32_t kfill = __shfl_sync(FULL, key, __ffs(pvalid) - 1);
    if (!ok) key = kfill;
    uint32_t ckey[QG_PIECES];
#pragma unroll
    for (int k = 0; k < QG_PIECES; ++k) ckey[k] = __shfl_sync(FULL, key, k);
    const uint32_t qmask = q >= 16 ? 0xffffffffu : ((1u << (2 * q)) - 1);
    const uint32_t nq = (1u << q) - 1;
    // ---- the key table: lane s tests bit offset s (s >= 2: the lookup below
    // takes the slot's byte offset straight from the text bits)
    bool good = lane >= 2 && lane + 5 <= 2 * q;
#pragma unroll
    for (int a = 0; a < QG_PIECES; ++a)
#pragma unroll
        for (int b = a + 1; b < QG_PIECES; ++b)
            if (((ckey[a] >> lane) & 31u) == ((ckey[b] >> lane) & 31u) && ckey[a] != ckey[b]) good = false;
    const uint32_t gm = __ballot_sync(FULL, good);
    const int ts = gm ? __ffs(gm) - 1 : -1;
    __syncwarp();   // every lane is done with the previous window's table and list
    if (ts >= 0) {
        tab[lane] = 0xffffffffu;   // no text key: reduced symbols are 0..2
        tabp[lane] = 0;
        __syncwarp();
        if (lane < (uint32_t)QG_PIECES) {
            tab[(key >> ts) & 31u] = key;
            if ((pvalid >> lane) & 1u) atomicOr(tabp + ((key >> ts) & 31u), 1u << lane);
        }
    }
    const uint32_t tb = (uint32_t)__cvta_generic_to_shared(tab);
    const uint64_t G0 = tx.G0(), G1 = G0 + tx.len;
    const int32_t len = (int32_t)tx.len;
    const uint64_t w0 = G0 >> 4, w1 = (G1 - 1) >> 4;
    const uint32_t nw = (uint32_t)(w1 - w0 + 1);
    if (lane == 0) *rn = 0;
    __syncwarp();
    // excluded bases (N or outside the window) of packed word w, one bit per base
    auto nbits = [&](uint64_t w) -> uint32_t {
        if (w < w0 || w > w1) return 0xffffu;
        uint32_t bb = (__ldg(ix.gnmask + (w >> 1)) >> (16 * (uint32_t)(w & 1))) & 0xffffu;
        if (w == w0) bb |= (1u << (G0 & 15)) - 1;
        if (w == w1) bb |= (0xffffu << (((G1 - 1) & 15) + 1)) & 0xffffu;
        return bb;
    };
    uint32_t carryS = 0;   // reduced symbols of the word before this iteration's first
    for (uint32_t base = 0; base < nw; base += 32) {
        const uint64_t wi = w0 + base + lane;
        const bool act = base + lane < nw;
        const uint32_t cur = act ? qg_reduce(__ldg(ix.gpack + wi), fwd) : 0u;
        uint32_t prevS = __shfl_up_sync(FULL, cur, 1);
        if (lane == 0) prevS = carryS;
        carryS = __shfl_sync(FULL, cur, 31);
        // q-gram ending at base i of this word starts at bit 17 + i - q
        const uint64_t sS = (((uint64_t)cur << 32) | prevS) >> (2 * (17 - q));
        bool anyh = false;
        if (ts >= 0) {
            // bits 2..6 of (sS >> (ts - 2 + 2i)) are position i's key field; the
            // table sits at a 128-byte boundary, so field * 4 | tb is its slot
            const uint64_t sF = sS >> (ts - 2);
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const uint32_t k2 = (uint32_t)(sS >> (2 * i)) & qmask;
                const uint32_t off = ((uint32_t)(sF >> (2 * i)) & 0x7cu) | tb;
                uint32_t t;
                asm volatile("ld.shared.u32 %0, [%1];" : "=r"(t) : "r"(off));
                anyh |= t == k2;
            }
        } else {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
                const uint32_t k2 = (uint32_t)(sS >> (2 * i)) & qmask;
#pragma unroll
                for (int k = 0; k < QG_PIECES; ++k) anyh |= k2 == ckey[k];
            }
        }
        anyh = anyh && act;
        if (__ballot_sync(FULL, anyh) == 0) continue;
        // ---- a word with a key hit: exclusion masks, then the spans of its hits
        const uint32_t nb = act ? nbits(wi) : 0xffffu;
        uint32_t prevN = __shfl_up_sync(FULL, nb, 1);
        if (lane == 0) prevN = wi == w0 ? 0xffffu : nbits(wi - 1);
        const uint32_t sN = (prevN | (nb << 16)) >> (17 - q);
        if (!anyh) continue;
        for (int i = 0; i < 16; ++i) {
            if ((sN >> i) & nq) continue;
            const uint32_t k2 = (uint32_t)(sS >> (2 * i)) & qmask;
            uint32_t pieces = 0;
            if (ts >= 0) {
                const uint32_t f = (k2 >> ts) & 31u;
                if (tab[f] == k2) pieces = tabp[f];
            } else {
#pragma unroll
                for (int k = 0; k < QG_PIECES; ++k)
                    if (k2 == ckey[k]) pieces |= 1u << k;
                pieces &= pvalid;
            }
            if (!pieces) continue;
            const int64_t A = (int64_t)(16 * wi + (uint64_t)i) - (int64_t)q + 1;   // genome start of the q-gram
            const int32_t x = fwd ? (int32_t)(A - (int64_t)G0) : (int32_t)((int64_t)G1 - A - (int64_t)q);
            while (pieces) {
                const uint32_t k = (uint32_t)(__ffs(pieces) - 1);
                pieces &= pieces - 1;
                const int32_t end0 = x - 1 + (int32_t)(m - (k * m) / 7);
                int32_t a = end0 - (int32_t)NERR, b = end0 + (int32_t)NERR;
                if (b < 0 || a > len - 1) continue;
                if (a < 0) a = 0;
                if (b > len - 1) b = len - 1;
                const uint32_t slot = atomicAdd(rn, 1u);
                if (slot < 32) { rlo[slot] = a; rhi[slot] = b; }
            }
        }
    }
    __syncwarp();
    const uint32_t n = *rn;
    if (n > 32) return -1;
    if (n == 0) return 0;
    // ---- sort by start (rank of each raw span), then merge with a prefix maximum of the ends
    int32_t lo = lane < n ? rlo[lane] : 0x7fffffff, hi = lane < n ? rhi[lane] : 0;
    uint32_t rank = 0;
    for (uint32_t j = 0; j < n; ++j) {
        const int32_t lj = __shfl_sync(FULL, lo, j);
        rank += (lj < lo || (lj == lo && j < lane)) ? 1u : 0u;
    }
    __syncwarp();
    if (lane < n) { rlo[rank] = lo; rhi[rank] = hi; }
    __syncwarp();
    lo = lane < n ? rlo[lane] : 0x7fffffff;
    hi = lane < n ? rhi[lane] : 0;
    int32_t incl = hi;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int32_t t = __shfl_up_sync(FULL, incl, d);
        if (lane >= (uint32_t)d && t > incl) incl = t;
    }
    const int32_t excl = __shfl_up_sync(FULL, incl, 1);
    const bool start = lane < n && (lane == 0 || lo > excl + 1);
    const uint32_t sb = __ballot_sync(FULL, start);
    const int nm = __popc(sb);
    if (nm > pool_cap) return -1;
    const int gid = __popc(sb & (0xffffffffu >> (31 - lane))) - 1;
    const bool last = lane < n && (lane == n - 1 || ((sb >> (lane + 1)) & 1u));
    uint16_t* ph = (uint16_t*)pool;
    if (start) ph[2 * gid] = (uint16_t)lo;
    if (last) ph[2 * gid + 1] = (uint16_t)incl;
    __syncwarp();
    return nm;
}

// Reduced-alphabet keys of the first q bases of the 7 read pieces.
struct PieceKeys {
    uint32_t key[7];
    uint32_t start[7];
    uint32_t valid;
    uint32_t q;
    __device__ __forceinline__ void load(const char* raw, uint32_t len, int orient)
    {
        q = min(16u, len / 7);
        valid = 0;
        for (int k = 0; k < 7; ++k) {
            start[k] = (uint32_t)((k * len) / 7);
            uint32_t kk = 0;
            bool ok = true;
            for (uint32_t i = 0; i < q; ++i) {
                const uint32_t p = start[k] + i;
                const uint8_t c = orient ? rc_byte((uint8_t)raw[len - 1 - p]) : (uint8_t)raw[p];
                uint32_t sym;
                switch (c) {
                    case 'A': sym = 0; break;
                    case 'G': sym = 1; break;
                    case 'C': case 'T': sym = 2; break;
                    default: sym = 3; ok = false; break;
                }
                kk = (kk << 2) | sym;
            }
            key[k] = kk;
            if (ok) valid |= 1u << k;
        }
    }
};

// Window scans of the candidates whose read length needs W pattern words (one
// launch per W, so the register file is sized for that W only).  Blocks of
// SA_WARPS warps (launched with 32 * SA_WARPS threads); a warp takes 32
// consecutive candidates, runs the q-gram pass of each with all its lanes
// (qgram_spans_warp, spans into a per-warp pool), then each lane runs the
// automaton over the spans of one candidate.  hits / hit_n as scan_window.
constexpr int SA_WARPS = 4;
constexpr int SA_POOL = 256;   // merged spans per warp for its 32 candidates
struct __align__(128) SaWarp {
    uint32_t tab[32];          // key table of the window being filtered (128-byte aligned)
    uint32_t tabp[32];
    uint32_t pool[SA_POOL];
    int32_t rlo[32], rhi[32];
    uint32_t rn;
    int16_t nsp[32];           // merged spans of each candidate, -1: scan the whole window
    uint16_t off[32];          // first pool entry of each candidate
};
static_assert(sizeof(SaWarp) % 128 == 0, "key tables of the warps must stay 128-byte aligned");

template <int W>
__global__ void __launch_bounds__(32 * SA_WARPS) k_shiftand(DevIndex ix, ChunkBufs cb, uint32_t ncand)
{
    constexpr uint32_t FULL = 0xffffffffu;
    if (ncand == FROM_DEVICE) {
        if (cand_overflow(cb) || !((cb.ctr[CTR_WMASK] >> W) & 1ull)) return;
        ncand = (uint32_t)cb.ctr[CTR_CAND];
    }
    __shared__ SaWarp smem[SA_WARPS];
    const uint32_t lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    SaWarp& S = smem[wib];
    const uint64_t nwarps = (uint64_t)gridDim.x * SA_WARPS;
    for (uint64_t c0 = cb.cand_first + ((uint64_t)blockIdx.x * SA_WARPS + wib) * 32; c0 < ncand; c0 += nwarps * 32) {
        const uint32_t c = (uint32_t)c0 + lane;
        bool mine = c < ncand;
        uint32_t o = 0, len = 0, e = 0;
        uint64_t off0 = 0;
        bool ung = false;
        if (mine) {
            const uint32_t task = cb.cand_task[c];
            mine = task != CAND_HOLE;
        }
        if (mine) {
            const uint32_t task = cb.cand_task[c];
            const uint32_t r = task >> 1;
            o = task & 1;
            off0 = cb.offs[r];
            len = (uint32_t)(cb.offs[r + 1] - off0);
            e = cb.cand[c];
            ung = cb.cand_flags && (cb.cand_flags[c] & 1u);
            mine = (int)(len / 64 + 1) == W;
        }
        // ---- q-gram pass of each candidate, whole warp
        uint32_t todo = __ballot_sync(FULL, mine);
        int used = 0;
        while (todo) {
            const int i = __ffs(todo) - 1;
            todo &= todo - 1;
            const uint32_t mi = __shfl_sync(FULL, len, i), oi = __shfl_sync(FULL, o, i), ei = __shfl_sync(FULL, e, i);
            const bool ui = __shfl_sync(FULL, ung ? 1u : 0u, i) != 0;
            const uint64_t offi = ((uint64_t)__shfl_sync(FULL, (uint32_t)(off0 >> 32), i) << 32) |
                                  __shfl_sync(FULL, (uint32_t)off0, i);
            const ScanText tx = window_text(ix, ei & 0x7fffffffu, (int)(ei >> 31), ui, mi);
            const int nm = qgram_spans_warp(ix, cb.seqs + offi, mi, (int)oi, tx, S.pool + used, SA_POOL - used,
                                            S.rlo, S.rhi, &S.rn, S.tab, S.tabp, lane);
            if (lane == 0) {
                S.nsp[i] = (int16_t)nm;
                S.off[i] = (uint16_t)used;
            }
            if (nm > 0) used += nm;
        }
        __syncwarp();
        // ---- automaton, one candidate per lane
        if (mine) {
            EditScan<W> sa;
            sa.load(cb.seqs + off0, len, (int)o);
            const int nm = S.nsp[lane];
            uint32_t n = 0;
            uint32_t* out = cb.hits + (uint64_t)c * HIT_CAP;
            auto emit = [&](uint32_t off, int err) {
                if (n < HIT_CAP) out[n] = (off << 8) | (uint32_t)err;
                ++n;
            };
            if (nm < 0) {
                scan_window_full<W>(ix, sa, e & 0x7fffffffu, (int)(e >> 31), emit, ung);
            } else if (nm > 0) {
                const ScanText tx = window_text(ix, e & 0x7fffffffu, (int)(e >> 31), ung, len);
                const uint32_t* sp = S.pool + S.off[lane];
                run_spans<W>(sa, tx, nm, [&](int k) { return sp[k]; }, emit);
            }
            cb.hit_n[c] = n;
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// selection: saQuerySeedSetRef's uniqueness walk (ReadQueue.cpp:1928-2160) and
// matchReads' orientation choice (ReadQueue.cpp:629-923)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint64_t mk_match(uint32_t off, uint32_t err, uint64_t fwd, uint64_t meta)
{
    return (uint64_t)(off & 0xffffu) | ((uint64_t)(err & 0xffu) << 16) | (fwd << 24) | (meta << 32);
}

struct Uniq {
    uint8_t multi[NERR + 1];
    uint64_t uniq[NERR + 1];
    uint32_t prevChr;
    uint64_t prevOff;
    bool abort;  // a second zero-error hit: return -1
};

// One hit of candidate window w (dir = forward window); idx = hit index in the window.
__device__ __forceinline__ void uniq_hit(const DevIndex& ix, Uniq& u, uint32_t w, uint32_t sp, int dir, uint32_t off,
                                         uint32_t err)
{
    if (u.multi[err]) {
        const uint64_t m2 = u.uniq[err];
        const bool m2fwd = (m2 >> 24) & 1ull, m2start = (m2 >> 25) & 1ull;
        const bool same_dir = dir ? m2fwd : !m2fwd;
        if (same_dir && !m2start &&
            (uint64_t)ix.win[(uint32_t)(m2 >> 32)].x + (m2 & 0xffffull) == (uint64_t)sp + off)
            return;
        if (err == 0) { u.abort = true; return; }
        u.multi[err] = 2;
    } else {
        u.uniq[err] = mk_match(off, err, (uint64_t)dir, w);
        u.multi[err] = 1;
    }
}

template <int W>
__device__ __noinline__ void rescan_into(const DevIndex& ix, const ChunkBufs& cb, uint32_t task, uint32_t w, int dir, Uniq& u,
                            uint32_t sp, uint32_t ch, uint32_t& nh, uint32_t& last)
{
    const uint32_t r = task >> 1, o = task & 1;
    const uint64_t off0 = cb.offs[r];
    const uint32_t len = (uint32_t)(cb.offs[r + 1] - off0);
    EditScan<W> sa;
    sa.load(cb.seqs + off0, len, (int)o);
    scan_window_full<W>(ix, sa, w, dir, [&](uint32_t off, int err) {
        if (u.abort) return;
        if (!(nh == 0 && (uint64_t)off + sp == u.prevOff && ch == u.prevChr)) uniq_hit(ix, u, w, sp, dir, off, (uint32_t)err);
        last = off;
        ++nh;
    });
}

// returns 1 / 0 / -1 like saQuerySeedSetRef; *mat as the reference leaves it
__device__ int select_task(const DevIndex& ix, const ChunkBufs& cb, uint32_t task, uint64_t* mat)
{
    const uint4 tc = cb.task_cand[task];
    const uint32_t base = tc.x, nf = tc.y, nt = tc.y + tc.z;
    Uniq u;
#pragma unroll
    for (int i = 0; i <= (int)NERR; ++i) { u.multi[i] = 0; u.uniq[i] = 0; }
    u.abort = false;
    const uint32_t r = task >> 1;
    const uint32_t len = (uint32_t)(cb.offs[r + 1] - cb.offs[r]);
    for (uint32_t k = 0; k < nt; ++k) {
        if (k == 0 || k == nf) { u.prevChr = 0; u.prevOff = 0xffffffffffffffffull; }
        const uint32_t c = base + k;
        const uint32_t e = cb.cand[c];
        const uint32_t w = e & 0x7fffffffu;
        const int dir = (int)(e >> 31);
        const uint4 wi = ix.win[w];
        const uint32_t sp = wi.x, ch = wi.y;
        const uint32_t n = cb.hit_n[c];
        uint32_t last = 0, nh = 0;
        if (n <= HIT_CAP) {
            const uint32_t* h = cb.hits + (uint64_t)c * HIT_CAP;
            for (uint32_t i = 0; i < n && !u.abort; ++i) {
                const uint32_t off = h[i] >> 8, err = h[i] & 0xffu;
                if (!(i == 0 && (uint64_t)off + sp == u.prevOff && ch == u.prevChr)) uniq_hit(ix, u, w, sp, dir, off, err);
                last = off;
            }
            nh = n;
        } else {
            switch (len / 64 + 1) {
                case 1: rescan_into<1>(ix, cb, task, w, dir, u, sp, ch, nh, last); break;
                case 2: rescan_into<2>(ix, cb, task, w, dir, u, sp, ch, nh, last); break;
                case 3: rescan_into<3>(ix, cb, task, w, dir, u, sp, ch, nh, last); break;
                default: rescan_into<4>(ix, cb, task, w, dir, u, sp, ch, nh, last); break;
            }
        }
        if (u.abort) return -1;
        if (nh > 0) { u.prevChr = ch; u.prevOff = (uint64_t)sp + last; }
        else { u.prevChr = 0; u.prevOff = 0xffffffffffffffffull; }
    }
    for (int i = 0; i <= (int)NERR; ++i) {
        if (!u.multi[i]) continue;
        *mat = u.uniq[i];
        return u.multi[i] > 1 ? -1 : 1;
    }
    return 0;
}

__device__ __forceinline__ uint8_t oriented_char(const char* raw, uint32_t len, int orient, uint32_t i)
{
    return orient ? rc_byte((uint8_t)raw[len - 1 - i]) : (uint8_t)raw[i];
}

// computeMethLvl for a hit without errors (ReadQueue.cpp:3293-3484)
__device__ void meth_exact(const DevIndex& ix, const ChunkBufs& cb, uint32_t r, int orient, uint64_t mat)
{
    const uint32_t meta = (uint32_t)(mat >> 32);
    const int isFwd = (int)((mat >> 24) & 1ull);
    const uint16_t offset = (uint16_t)(mat & 0xffffull);
    const uint4 wi = ix.win[meta];
    const uint32_t metaPos = wi.x, sind = wi.z, eind = wi.w;
    const uint64_t off0 = cb.offs[r];
    const uint32_t size = (uint32_t)(cb.offs[r + 1] - off0);
    const char* raw = cb.seqs + off0;
    const uint32_t RL = ix.readlen;
    const uint32_t minPos = (uint32_t)(metaPos + offset - (size - 1));
    const uint32_t maxPos = metaPos + offset;
    for (uint32_t id = sind; id <= eind; ++id) {
        const uint32_t pos = ix.cpg_pos[id];
        if (pos + RL - 2 < minPos) continue;
        if (isFwd) { if (pos + RL - 2 > maxPos) break; }
        else { if (pos + RL - 1 > maxPos) break; }
        const uint32_t trueCpGPos = pos - 1 + RL - 1;
        const uint32_t readCpGPos = (uint32_t)(size - (uint32_t)(metaPos + offset - trueCpGPos) - 1);
        if (isFwd) {
            if ((uint32_t)(readCpGPos + MISCOUNT) >= size) continue;
            const uint8_t c = oriented_char(raw, size, orient, (uint32_t)(readCpGPos + MISCOUNT));
            if (c == 'T') atomicAdd(cb.meth + 4ull * id + 1, 1u);
            else if (c == 'C') atomicAdd(cb.meth + 4ull * id + 0, 1u);
        } else {
            if ((uint32_t)(readCpGPos + 1 + MISCOUNT + 2) > size) continue;
            const uint8_t c = oriented_char(raw, size, orient, size - readCpGPos - 1 - MISCOUNT - 2);
            if (c == 'T') atomicAdd(cb.meth + 4ull * id + 3, 1u);
            else if (c == 'C') atomicAdd(cb.meth + 4ull * id + 2, 1u);
        }
    }
}

__global__ void k_select(DevIndex ix, ChunkBufs cb)
{
    if (cand_overflow(cb)) return;
    __shared__ unsigned long long sc[8];
    if (threadIdx.x < 8) sc[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r < cb.n) {
        const uint8_t f = cb.rflags[r];
        uint64_t mat = 0;
        bool ok = false;
        int orient = 0;
        if (f & 1u) atomicAdd(&sc[0], 1ull);
        else if (f & 2u) atomicAdd(&sc[1], 1ull);
        if (!(f & 7u)) {
            const bool runF = cb.orient_mask & 1u, runR = (cb.orient_mask >> 1) & 1u;
            uint64_t mF = 0, mR = 0;
            int sF = 0, sR = 0;
            if (runF) sF = select_task(ix, cb, 2 * r, &mF);
            if (runR) sR = select_task(ix, cb, 2 * r + 1, &mR);
            const uint32_t eF = (uint32_t)((mF >> 16) & 0xff), eR = (uint32_t)((mR >> 16) & 0xff);
            int vote = 0;  // 1 fwd, 2 rev
            if (sF == 1 && sR == 1) {
                if (eF < eR) { ok = true; mat = mF; orient = 0; vote = 1; }
                else if (eF > eR) { ok = true; mat = mR; orient = 1; vote = 2; }
                else {
                    const uint32_t p1 = ix.win[(uint32_t)(mF >> 32)].x + (uint32_t)(mF & 0xffff);
                    const uint32_t p2 = ix.win[(uint32_t)(mR >> 32)].x + (uint32_t)(mR & 0xffff);
                    if (((mF >> 24) & 1) == ((mR >> 24) & 1) && p1 == p2) { ok = true; mat = mF; orient = 0; vote = 1; }
                    else atomicAdd(&sc[3], 1ull);
                }
            } else if (sF == 1) {
                if (sR == -1 && !(eF < eR)) atomicAdd(&sc[3], 1ull);
                else { ok = true; mat = mF; orient = 0; vote = 1; }
            } else if (sR == 1) {
                if (sF == -1 && !(eR < eF)) atomicAdd(&sc[3], 1ull);
                else { ok = true; mat = mR; orient = 1; vote = 2; }
            } else {
                if (sF == -1 || sR == -1) atomicAdd(&sc[3], 1ull);
                else atomicAdd(&sc[4], 1ull);
            }
            if (ok) {
                atomicAdd(&sc[2], 1ull);
                if (cb.stranded) atomicAdd(&sc[vote == 1 ? 5 : 6], 1ull);
            }
        }
        cb.mats[r] = ok ? mat : 0;
        cb.invalid[r] = ok ? 0 : 1;
        if (ok) {
            const uint32_t meta = (uint32_t)(mat >> 32);
            if (ix.win[meta].z != CPGDUMMY) {
                if (((mat >> 16) & 0xff) == 0) meth_exact(ix, cb, r, orient, mat);
                else {
                    const uint32_t slot = (uint32_t)atomicAdd(cb.ctr + CTR_DP, 1ull);
                    cb.dp_list[slot] = r;
                    cb.dp_mat[slot] = mat;
                    cb.dp_orient[slot] = (uint8_t)orient;
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const int map[7] = {CTR_INV_LEN, CTR_INV_N, CTR_SUCC, CTR_NONU, CTR_UNSUCC, CTR_R1F, CTR_R1R};
        for (int i = 0; i < 7; ++i) if (sc[i]) atomicAdd(cb.ctr + map[i], sc[i]);
    }
}

// ---------------------------------------------------------------------------
// banded DP (LevenshtDP<uint16_t, 8>, LevenshtDP.h:191-544) over the storage
// layout of BandedMatrix<uint16_t, 9> (BandedMatrix.h:67-75), then the CpG walk
// of computeMethLvl (ReadQueue.cpp:3620-3944).  The matrix of each thread
// lives in global scratch interleaved across threads (cell-major) so that a
// warp's accesses to one cell coalesce.
// ---------------------------------------------------------------------------
struct DpScratch {
    uint16_t* cells;    // [cell][slot]
    uint8_t* align;     // [step][slot]
    uint32_t nslots;
    uint32_t cell_cap;  // cells per slot
    uint32_t align_cap; // alignment steps per slot
};

constexpr long DPB = DP_BAND;      // band
constexpr long DPS = DP_BAND + 1;  // storage band
constexpr long DPW = 2 * DPS + 1;  // cells per stored row

__device__ __forceinline__ long dp_idx(long i, long j)
{
    return i * DPW + (DPS - i > 0 ? DPS - i : 0) + (j - i + DPS);
}

__device__ __forceinline__ uint16_t cmp_fwd(uint8_t r, uint8_t g)  // CompiFwd, ReadQueue.h:295-307
{
    if (r == 'T' && g == 'C') return 0;
    return r == g ? 0 : 1;
}
__device__ __forceinline__ uint16_t cmp_rev(uint8_t r, uint8_t g)  // CompiRev, ReadQueue.h:309-338
{
    switch (r) {
        case 'T': if (g == 'A' || g == 'G') return 0; break;
        case 'G': if (g == 'C') return 0; break;
        case 'A': if (g == 'T') return 0; break;
        case 'C': if (g == 'G') return 0; break;
    }
    return 1;
}

struct DpView {
    uint16_t* c;
    uint32_t stride;
    long msize;
    __device__ __forceinline__ uint16_t get(long i, long j) const
    {
        const long k = dp_idx(i, j);
        return (k >= 0 && k < msize) ? c[(uint64_t)k * stride] : (uint16_t)0xffff;
    }
    __device__ __forceinline__ void set(long i, long j, uint16_t v) const
    {
        const long k = dp_idx(i, j);
        if (k >= 0 && k < msize) c[(uint64_t)k * stride] = v;
    }
};

__device__ void meth_dp(const DevIndex& ix, const ChunkBufs& cb, const DpScratch& ds, uint32_t slot, uint32_t r,
                        int orient, uint64_t mat)
{
    const uint32_t meta = (uint32_t)(mat >> 32);
    const int isFwd = (int)((mat >> 24) & 1ull);
    const uint16_t offset = (uint16_t)(mat & 0xffffull);
    const uint4 wi = ix.win[meta];
    const uint32_t metaPos = wi.x, sind = wi.z, eind = wi.w;
    const uint64_t off0 = cb.offs[r];
    const uint32_t size = (uint32_t)(cb.offs[r + 1] - off0);
    const char* raw = cb.seqs + off0;
    const uint32_t RL = ix.readlen;
    const uint32_t chrom = ix.cpg_chrom[sind];
    const int64_t base = (int64_t)metaPos + offset;
    const long n = (long)size;
    DpView dv{ds.cells + slot, ds.nslots, (n + 1) * DPW};
    if ((uint64_t)dv.msize > ds.cell_cap) { atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull); return; }
    for (long k = 0; k < dv.msize; ++k) dv.c[(uint64_t)k * ds.nslots] = 0xffff;
    // runDPFill / runDPFillRev (LevenshtDP.h:205-323)
    dv.set(0, 0, 0);
    for (long c = 1; c <= DPB; ++c) dv.set(0, c, (uint16_t)c);
    for (long rr = 1; rr <= DPB; ++rr) dv.set(rr, 0, (uint16_t)rr);
    for (long c = 0; c < n - DPB; ++c) dv.set(c + DPB + 1, c, (uint16_t)(65535 - c - DPB - 1));
    for (long rr = 0; rr < n; ++rr) dv.set(rr, rr + DPB + 1, (uint16_t)(65535 - rr - DPB - 1));
    for (long row = 1; row <= n; ++row) {
        const uint8_t rc = oriented_char(raw, size, orient, isFwd ? (uint32_t)(n - row) : (uint32_t)(row - 1));
        for (long o = -DPB; o <= DPB; ++o) {
            const long j = row + o;
            if (j <= 0) continue;
            const uint8_t g = base_char(gbase(ix, chrom, base + 1 - j));
            const int mm = isFwd ? cmp_fwd(rc, g) : cmp_rev(rc, g);
            int v = dv.get(row - 1, j) + 1;
            const int v2 = dv.get(row, j - 1) + 1;
            const int v3 = dv.get(row - 1, j - 1) + mm;
            if (v2 < v) v = v2;
            if (v3 < v) v = v3;
            dv.set(row, j, (uint16_t)v);
        }
    }
    // backtrackDP / backtrackDPRev (LevenshtDP.h:327-544)
    uint8_t* al = ds.align + slot;
    uint32_t alen = 0;
    {
        uint16_t mn = 0xffff;
        long col = 0;
        for (long o = -DPB; o <= DPB; ++o) {
            const uint16_t v = dv.get(n, n + o);
            if (v < mn) { col = n + o; mn = v; }
        }
        for (long row = n; row > 0;) {
            const uint8_t rc = oriented_char(raw, size, orient, isFwd ? (uint32_t)(n - row) : (uint32_t)(row - 1));
            const uint8_t g = base_char(gbase(ix, chrom, base + 1 - col));
            const int mm = isFwd ? cmp_fwd(rc, g) : cmp_rev(rc, g);
            const uint16_t up = dv.get(row - 1, col), left = dv.get(row, col - 1), dg = dv.get(row - 1, col - 1);
            uint8_t code;
            if (up < left) {
                if ((int)up + 1 < (int)dg + mm) { code = 2; --row; }
                else { code = mm ? 1 : 0; --row; --col; }
            } else {
                if ((int)left + 1 < (int)dg + mm) { code = 3; --col; }
                else { code = mm ? 1 : 0; --row; --col; }
            }
            if (alen >= ds.align_cap) { atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull); return; }
            al[(uint64_t)alen * ds.nslots] = code;
            ++alen;
        }
        while (col > 0) {
            if (alen >= ds.align_cap) { atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull); return; }
            al[(uint64_t)alen * ds.nslots] = 3;
            ++alen;
            --col;
        }
    }
    // CpG range and walk (ReadQueue.cpp:3631-3944)
    const uint32_t minPos = (uint32_t)(metaPos + offset - (size - 1));
    const uint32_t maxPos = metaPos + offset;
    int32_t minIndex = (int32_t)sind, maxIndex = (int32_t)eind;
    for (int32_t id = (int32_t)sind; (uint32_t)id <= eind; ++id) {
        const uint32_t pos = ix.cpg_pos[id];
        if (pos + RL - 2 < minPos) ++minIndex;
        else if (pos + RL - 2 > maxPos) { maxIndex = id - 1; break; }
    }
    uint32_t refSeqPos = metaPos + offset;
    int32_t readSeqPos = (int32_t)size - 1;
    int32_t alignPos = (int32_t)alen - 1;
    for (int32_t id = maxIndex; id >= minIndex; --id) {
        const uint32_t cpos = ix.cpg_pos[id] + RL - 2;
        while (cpos < refSeqPos && alignPos >= 0) {
            switch (al[(uint64_t)alignPos * ds.nslots]) {
                case 0: case 1: --readSeqPos; --refSeqPos; break;
                case 3: --refSeqPos; break;
                default: --readSeqPos; break;
            }
            if (readSeqPos < 0) break;
            --alignPos;
        }
        if (readSeqPos < 0) break;
        if (isFwd) {
            const uint8_t c = oriented_char(raw, size, orient, (uint32_t)readSeqPos);
            if (c == 'C') atomicAdd(cb.meth + 4ull * id + 0, 1u);
            else if (c == 'T') atomicAdd(cb.meth + 4ull * id + 1, 1u);
        } else {
            // the sequence was reversed in place (ReadQueue.cpp:3796); index size reads '\0'
            const uint32_t k = (uint32_t)readSeqPos + 1;
            const uint8_t c = k < size ? oriented_char(raw, size, orient, size - 1 - k) : 0;
            if (c == 'C') atomicAdd(cb.meth + 4ull * id + 2, 1u);
            else if (c == 'T') atomicAdd(cb.meth + 4ull * id + 3, 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// read checks (ReadQueue.cpp:428-490)
// ---------------------------------------------------------------------------
// True when one of the bytes [a, a + len) of the read buffer is 'N'.  Reads
// the 8-byte aligned words (by address) that hold those bytes, so no load
// leaves a word that holds a byte of the range; bytes outside the range are
// made non-zero, then a zero-byte test on the word XOR "NNNNNNNN".
__device__ __forceinline__ bool has_n(const char* seqs, uint64_t a, uint32_t len)
{
    if (len == 0) return false;
    const uintptr_t p = (uintptr_t)(seqs + a), e = p + len;
    for (uintptr_t w = p & ~(uintptr_t)7; w < e; w += 8) {
        uint64_t x = *(const uint64_t*)w ^ 0x4E4E4E4E4E4E4E4Eull;
        if (w < p) x |= (1ull << (8 * (p - w))) - 1;
        if (w + 8 > e) x |= ~0ull << (8 * (e - w));
        if ((x - 0x0101010101010101ull) & ~x & 0x8080808080808080ull) return true;
    }
    return false;
}

__global__ void k_prep(ChunkBufs cb, uint32_t readlen)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t wbit = 0;
    if (r < cb.n) {
        const uint64_t o0 = cb.offs[r];
        const uint32_t len = (uint32_t)(cb.offs[r + 1] - o0);
        uint8_t f = 0;
        if (len < readlen - 20) f = 1;
        else {
            if (has_n(cb.seqs, o0, len)) f = 2;
            if (!f && len > FAME_MAX_READ_LEN) { f = 4; atomicAdd(cb.ctr + CTR_TOO_LONG, 1ull); }
            if (!f) wbit = 1u << min(4u, len / 64 + 1);
        }
        cb.rflags[r] = f;
        cb.task_cand[2 * r] = make_uint4(0, 0, 0, 0);
        cb.task_cand[2 * r + 1] = make_uint4(0, 0, 0, 0);
    }
    // one atomic per warp for the automaton widths present
    wbit = __reduce_or_sync(0xffffffffu, wbit);
    if ((threadIdx.x & 31) == 0 && wbit) atomicOr(cb.ctr + CTR_WMASK, (unsigned long long)wbit);
}

// Light tier: up to 128 gathered entries (the common read of an index with
// fewer entries than buckets), many warps per SM.
constexpr uint32_t L_OPS = 128, L_DT = 256, L_OVF = 32;
using LightR = SeedLayoutR<L_OPS, L_DT, L_OVF>;

// tasks: all (read, orientation) pairs of the chunk in orientation-major order
__global__ void __launch_bounds__(128) k_seed(DevIndex ix, ChunkBufs cb, uint32_t ntask)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const uint32_t wib = threadIdx.x >> 5;
    uint8_t* const base = smem + wib * LightR::BYTES;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const int norient = __popc(cb.orient_mask);
    const uint32_t first_o = (cb.orient_mask & 1u) ? 0 : 1;
    CandRes res;
    for (uint32_t t = blockIdx.x * (blockDim.x >> 5) + wib; t < ntask; t += nwarps) {
        const uint32_t r = norient == 2 ? (t >> 1) : t;
        const uint32_t o = norient == 2 ? (t & 1) : first_o;
        if (cb.rflags[r]) continue;
        const uint32_t task = 2 * r + o;
        const int heavy = seed_task_rec<LightR, L_OPS, L_DT, L_OVF>(ix, cb, base, task, cb.ctr + CTR_GATHER_BYTES, res);
        if (heavy && (threadIdx.x & 31) == 0) {
            const uint32_t h = (uint32_t)atomicAdd(cb.ctr + CTR_HEAVY, 1ull);
            cb.heavy[h] = task;
        }
        __syncwarp();
    }
    cand_res_finish(cb, res);
}

// Middle seeding tiers, for genome-scale indexes (about three entries per
// bucket: a read gathers hundreds of entries, over the light tier's caps).
// One warp per task with its whole working set in shared memory
// (SeedLayoutR), tasks taken one at a time per warp from a work queue
// (counter ctr_q, zero at launch): a task's cost follows its read's bucket
// sizes, so fixed strides would leave warps idle behind a few long tasks.
// The tasks of `list` (its length in counter ctr_in); a task over the caps
// goes to `spill` (counter ctr_spill) for the next tier.  Launched with WPB
// warps per block and WPB * SeedLayoutR<OPS, DT, MID_OVF>::BYTES of dynamic
// shared memory.
constexpr uint32_t MID_OVF = 256;
template <uint32_t OPS, uint32_t DT, int WPB>
__global__ void __launch_bounds__(32 * WPB, 4) k_seed_mid(DevIndex ix, ChunkBufs cb, const uint32_t* list, int ctr_in,
                                                       int ctr_q, uint32_t* spill, int ctr_spill)
{
    extern __shared__ __align__(16) uint8_t smem[];
    using L = SeedLayoutR<OPS, DT, MID_OVF>;
    const uint32_t wib = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint8_t* const base = smem + wib * L::BYTES;
    const uint32_t ntask = (uint32_t)cb.ctr[ctr_in];
    CandRes res;
    while (true) {
        uint32_t i = 0;
        if (lane == 0) i = (uint32_t)atomicAdd(cb.ctr + ctr_q, 1ull);
        i = __shfl_sync(0xffffffffu, i, 0);
        if (i >= ntask) break;
        const uint32_t task = list[i];
        const int over = seed_task_rec<L, OPS, DT, MID_OVF>(ix, cb, base, task, cb.ctr + CTR_GATHER_BYTES, res);
        if (over && lane == 0) spill[(uint32_t)atomicAdd(cb.ctr + ctr_spill, 1ull)] = task;
        __syncwarp();
    }
    cand_res_finish(cb, res);
}

// the two middle tiers: reads gathering up to 511 entries, then up to 1023
constexpr uint32_t MID_S_OPS = 511, MID_S_DT = 1024, MID_L_OPS = 1023, MID_L_DT = 2048;
constexpr int MID_S_WPB = 4, MID_L_WPB = 2;
using MidS = SeedLayoutR<MID_S_OPS, MID_S_DT, MID_OVF>;
using MidL = SeedLayoutR<MID_L_OPS, MID_L_DT, MID_OVF>;

// One warp replays tsl::hopscotch_map insertions of keys[0..n) (distinct,
// bit 31 clear) into a map made with bucket_count buckets, as the seeding
// tiers do, and writes the iteration order; out = {keys written, final
// bucket count, 1 when a cap was exceeded}.  scratch holds the replayed
// buckets, the stack and the overflow list (cap words each).  A test hook
// for the device replay.
__global__ void k_map_order_probe(const uint32_t* keys, uint32_t n, uint32_t bucket_count, uint32_t* scratch,
                                  uint32_t cap, uint32_t* order, uint32_t* out)
{
    const uint32_t lane = threadIdx.x & 31;
    if (threadIdx.x >= 32) return;
    SeedMem s{};
    s.ins = (uint32_t*)keys;
    s.slot = scratch;
    s.stk = scratch + cap;
    s.ovf = scratch + 2 * cap;
    s.slot_cap = cap; s.stk_cap = cap; s.ovf_cap = cap;
    MapSim m;
    sim_init(m, bucket_count);
    m.nb = 0; m.novf = 0; m.sp = 0;
    bool fail = m.size > s.slot_cap;
    if (!fail) {
        for (uint32_t b = lane; b < m.size; b += 32) s.slot[b] = EMPTY_KEY;
        __syncwarp();
        for (uint32_t b0 = 0; b0 < n && !fail; b0 += 32) {
            const unsigned todo = __ballot_sync(0xffffffffu, b0 + lane < n);
            fail = !sim_insert_batch_w(m, s, b0, todo);
        }
    }
    uint32_t no = 0;
    if (!fail) {
        for (uint32_t b0 = 0; b0 < m.size + m.novf; b0 += 32) {
            const uint32_t b = b0 + lane;
            uint32_t x = EMPTY_KEY;
            if (b < m.size) x = s.slot[b];
            else if (b < m.size + m.novf) x = s.ovf[b - m.size];
            const unsigned bm = __ballot_sync(0xffffffffu, x != EMPTY_KEY);
            if (x != EMPTY_KEY) order[no + __popc(bm & ((1u << lane) - 1))] = keys[x];
            no += __popc(bm);
        }
    }
    if (lane == 0) {
        out[0] = no;
        out[1] = m.B;
        out[2] = fail ? 1u : 0u;
    }
}

// Every valid task of the chunk straight to the middle tier's list (indexes
// whose buckets are too large for the shared-memory caps of k_seed: there the
// light attempt would only repeat its bucket reads).
__global__ void k_seed_route(ChunkBufs cb, uint32_t ntask)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const int norient = __popc(cb.orient_mask);
    const uint32_t first_o = (cb.orient_mask & 1u) ? 0 : 1;
    bool take = false;
    uint32_t task = 0;
    if (t < ntask) {
        const uint32_t r = norient == 2 ? (t >> 1) : t;
        const uint32_t o = norient == 2 ? (t & 1) : first_o;
        take = cb.rflags[r] == 0;
        task = 2 * r + o;
    }
    const unsigned bm = __ballot_sync(0xffffffffu, take);
    const uint32_t lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0 && bm) base = (uint32_t)atomicAdd(cb.ctr + CTR_HEAVY, (unsigned long long)__popc(bm));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (take) cb.heavy[base + __popc(bm & ((1u << lane) - 1))] = task;
}

// Heavy path: one warp per task with its working memory in global scratch.
struct HeavyScratch {
    uint8_t* base;
    uint64_t bytes_per_warp;
    uint32_t nwarps;
    uint32_t ops_cap, dt_cap, slot_cap;
};

__device__ __forceinline__ SeedMem heavy_mem(const HeavyScratch& hs, uint32_t w)
{
    uint8_t* b = hs.base + (uint64_t)w * hs.bytes_per_warp;
    SeedMem s;
    const uint64_t oc = hs.ops_cap, dc = hs.dt_cap, sc = hs.slot_cap;
    uint64_t o = 0;
    auto take = [&](uint64_t bytes) { uint8_t* p = b + o; o += (bytes + 15) / 16 * 16; return p; };
    s.seq = take(256);
    s.kst = (uint32_t*)take(256 * 4);
    s.kpre = (uint32_t*)take(260 * 4);
    s.ops = (uint32_t*)take(oc * 4);
    s.opk = take(oc);
    s.dt_key = (uint32_t*)take(dc * 4);
    s.dt_first = (uint32_t*)take(dc * 4);
    s.dt_cnt = (uint32_t*)take(dc * 4);
    s.ins = (uint32_t*)take(oc * 4);
    s.ins_cnt = (uint32_t*)take(oc * 4);
    s.slot = (uint32_t*)take(sc * 4);
    s.stk = (uint32_t*)take(oc * 4);
    s.ovf = (uint32_t*)take(oc * 4);
    s.stage = (uint32_t*)take(oc * 4);
    s.pre = (uint64_t*)s.ops;   // ops, opk and the count table: far more than 8 * 256 bytes
    s.ops_cap = hs.ops_cap; s.dt_cap = hs.dt_cap; s.slot_cap = hs.slot_cap; s.stk_cap = hs.ops_cap; s.ovf_cap = hs.ops_cap;
    return s;
}

__host__ __device__ inline uint64_t heavy_bytes_per_warp(uint64_t ops_cap, uint64_t dt_cap, uint64_t slot_cap)
{
    auto al = [](uint64_t x) { return (x + 15) / 16 * 16; };
    return al(256) + al(256 * 4) + al(260 * 4) + al(ops_cap * 4) + al(ops_cap) + 3 * al(dt_cap * 4) +
           2 * al(ops_cap * 4) + al(slot_cap * 4) + 3 * al(ops_cap * 4);
}

// Seeding tiers with working memory in global scratch, one warp per task:
// the tasks of `list` (its length ntask, or the counter ctr_in when ntask is
// FROM_DEVICE).  A task over this tier's caps goes to `spill` (counter
// ctr_spill) for the next tier; without a next tier it is a capacity error.
// The middle tier has many warps and caps for genome-scale bucket sizes; the
// large-capacity tier has few warps sized by the largest bucket.
__global__ void k_seed_tier(DevIndex ix, ChunkBufs cb, HeavyScratch hs, uint32_t ntask, const uint32_t* list,
                            int ctr_in, uint32_t* spill, int ctr_spill)
{
    const uint32_t w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (w >= hs.nwarps) return;
    if (ntask == FROM_DEVICE) ntask = (uint32_t)cb.ctr[ctr_in];
    const SeedMem s = heavy_mem(hs, w);
    CandRes res;
    for (uint32_t i = w; i < ntask; i += hs.nwarps) {
        const uint32_t task = list[i];
        const int bad = seed_task(ix, cb, s, task, cb.ctr + CTR_GATHER_BYTES, res);
        if (bad && (threadIdx.x & 31) == 0) {
            if (spill) {
                const uint32_t h = (uint32_t)atomicAdd(cb.ctr + ctr_spill, 1ull);
                spill[h] = task;
            } else {
                atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull);
                cb.task_cand[task] = make_uint4(0, 0, 0, 0);
            }
        }
        __syncwarp();
    }
    cand_res_finish(cb, res);
}

// The bucket records of buckets 0 .. n - 1 from the offset table (n + 1
// offsets) and the entries (DevIndex::rec).
__global__ void k_build_rec(const uint32_t* tab, const uint32_t* entry, uint64_t n, uint4* rec)
{
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b0 = tab[k], sz = tab[k + 1] - b0;
        uint32_t e[REC_INLINE];
#pragma unroll
        for (uint32_t j = 0; j < REC_INLINE; ++j) e[j] = j < sz ? entry[b0 + j] : 0u;
        rec[2 * k] = make_uint4(b0, sz, e[0], e[1]);
        rec[2 * k + 1] = make_uint4(e[2], e[3], e[4], e[5]);
    }
}

// The uint16 tallies the reference keeps (its counters wrap at 2^16) from the
// device's uint32 ones, packed for the copy to the host.
__global__ void k_pack_tallies(const uint32_t* meth, uint64_t n4, uint16_t* out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n4; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = (uint16_t)(meth[i] & 0xffffu);
}

// The hashed record layout (DevIndex::rec, small genomes) of buckets
// 0 .. n - 1; rec (mask + 1 slots) starts with every word 0xffffffff.
__global__ void k_build_rec_hashed(const uint32_t* tab, const uint32_t* entry, uint64_t n, uint4* rec, uint32_t mask)
{
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t b0 = tab[k], sz = tab[k + 1] - b0;
        if (sz == 0) continue;
        uint32_t e[5];
#pragma unroll
        for (uint32_t j = 0; j < 5; ++j) e[j] = j < sz ? entry[b0 + j] : 0u;
        // the table has at least twice as many slots as non-empty buckets
        uint32_t h = rec_slot((uint32_t)k, mask);
        for (uint32_t i = 0; i <= mask && atomicCAS(&rec[2ull * h + 1].w, EMPTY_REC_KEY, (uint32_t)k) != EMPTY_REC_KEY; ++i)
            h = (h + 1) & mask;
        rec[2ull * h] = make_uint4(b0, sz, e[0], e[1]);
        rec[2ull * h + 1].x = e[2];
        rec[2ull * h + 1].y = e[3];
        rec[2ull * h + 1].z = e[4];
    }
}

// Non-empty buckets of the index.
__global__ void k_count_nonempty(const uint32_t* tab, uint64_t n, unsigned long long* out)
{
    uint32_t c = 0;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        c += tab[k + 1] > tab[k] ? 1u : 0u;
    for (int d = 16; d > 0; d >>= 1) c += __shfl_xor_sync(0xffffffffu, c, d);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(out, (unsigned long long)c);
}

// Largest bucket of the index (sizes the heavy path).
__global__ void k_max_bucket(const uint32_t* tab, uint64_t n, unsigned int* out)
{
    uint32_t mx = 0;
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n; k += (uint64_t)gridDim.x * blockDim.x)
        mx = max(mx, tab[k + 1] - tab[k]);
    for (int d = 16; d > 0; d >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, d));
    if ((threadIdx.x & 31) == 0) atomicMax(out, mx);
}

}  // namespace fame

namespace fame {

// ---------------------------------------------------------------------------
// Banded DP for the CpG calls of erroneous hits, three reads per warp.
//
// LevenshtDP<uint16_t, 8> (LevenshtDP.h:205-544) fills a 17-cell band per row
// from three neighbours and then backtracks from the smallest cell of the last
// row.  Every cell inside the band is written once and its three inputs are
// final when it is computed, and a computed cell never exceeds n + 8 while the
// band's border cells hold at least 65518, so the backtrack never leaves the
// band: its choice at a cell is a function of that cell's own inputs.  The fill
// therefore records the choice per cell (two bits, as two warp ballots per
// anti-diagonal) instead of the matrix, and keeps the values in registers:
// cells are computed along anti-diagonals
// t = 2 * row + offset, lane k of a 9-lane group holding offset 2k - 8 (even t)
// or 2k - 7 (odd t), so the up and left inputs are neighbour lanes' values of
// step t - 1 (shuffles) and the diagonal input is the lane's own value of step
// t - 2.  Border values follow the reference's initialisation, including its
// storage overlap: cell (9, 0) reads 65518, the value the right border writes
// over it.  Column-0 cells of rows 1..8 always backtrack as insertions.
// ---------------------------------------------------------------------------
constexpr uint32_t DP3_GROUPS = 3;                                     // reads per warp
constexpr uint32_t DP3_MAXN = FAME_MAX_READ_LEN;
constexpr uint32_t DP3_STEPS = 2 * DP3_MAXN + DP_BAND + 2;            // anti-diagonals, rounded up to even
constexpr uint32_t DP3_WORDS = (DP3_STEPS + 15) / 16;                 // 16 two-bit choices per word and lane
constexpr uint32_t DP3_REF = 288;                                      // reference bases, j in [-2, n + 10]
constexpr uint32_t DP3_ALIGN = 2 * DP3_MAXN + 4 * DP_BAND + 10;       // alignment trace
// row-n values, read masks, reference bits, trace; + 16 so that the groups'
// arrays start in different banks
constexpr uint32_t DP3_GROUP_BYTES = 48 + 256 + DP3_REF + DP3_ALIGN + 8 + 16;
constexpr uint32_t DP3_CODE_BYTES = DP3_WORDS * 32 * 4;
constexpr uint32_t DPW_BYTES = DP3_CODE_BYTES + DP3_GROUPS * DP3_GROUP_BYTES;   // per warp
constexpr int DPW_REF0 = 2;
static_assert(DP3_GROUP_BYTES % 16 == 0 && DP3_CODE_BYTES % 16 == 0, "16-byte aligned shared-memory regions");
static_assert(DP3_MAXN + DP_BAND + 2 + DPW_REF0 < DP3_REF, "reference bases fit");

// Reference bases as one bit each (A 1, C 2, G 4, T 8, N 16; 0 outside the
// chromosome) and read characters as the set of reference bases they match
// under CompiFwd / CompiRev (ReadQueue.h:295-338): a cell is a mismatch when
// the two share no bit.
__device__ __forceinline__ uint8_t ref_bit(int b) { return b < 5 ? (uint8_t)(1u << b) : (uint8_t)0; }
__device__ __forceinline__ uint8_t read_mask(uint8_t r, int isFwd)
{
    if (isFwd) return r == 'A' ? 1 : r == 'C' ? 2 : r == 'G' ? 4 : r == 'T' ? (8 | 2) : r == 'N' ? 16 : 0;
    return r == 'T' ? (1 | 4) : r == 'G' ? 2 : r == 'A' ? 8 : r == 'C' ? 4 : 0;
}

__global__ void k_dp_warp(DevIndex ix, ChunkBufs cb)
{
    if (cand_overflow(cb)) return;
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const int grp = lane / 9;                   // 3 groups of 9 lanes, lanes 27..31 idle
    const int k = lane - 9 * grp;
    const bool in_grp = grp < (int)DP3_GROUPS;
    uint8_t* warp_p = smem + (threadIdx.x >> 5) * DPW_BYTES;
    uint32_t* codes = (uint32_t*)warp_p;        // [step / 16][lane]: 2-bit choices, step t % 16 at bits 2 (t % 16)
    uint8_t* gbase_p = warp_p + DP3_CODE_BYTES + (in_grp ? grp : 0) * DP3_GROUP_BYTES;
    uint16_t* rown = (uint16_t*)gbase_p;        // row n, offsets -8..8
    uint8_t* rowm = gbase_p + 48;               // read row masks
    uint8_t* refb = rowm + 256;                 // reference column bits
    uint8_t* al = refb + DP3_REF;
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t ndp = (uint32_t)cb.ctr[CTR_DP];
    const uint32_t RL = ix.readlen;
    for (uint32_t it0 = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * DP3_GROUPS; it0 < ndp;
         it0 += nwarps * DP3_GROUPS) {
        const uint32_t it = it0 + (in_grp ? grp : 0);
        const bool have = in_grp && it < ndp;
        uint32_t r = 0, size = 0, metaPos = 0, sind = 0, eind = 0, chrom = 0;
        uint64_t mat = 0, off0 = 0;
        int orient = 0, isFwd = 0;
        uint16_t offset = 0;
        if (have) {
            r = cb.dp_list[it];
            mat = cb.dp_mat[it];
            orient = cb.dp_orient[it];
            const uint32_t meta = (uint32_t)(mat >> 32);
            isFwd = (int)((mat >> 24) & 1ull);
            offset = (uint16_t)(mat & 0xffffull);
            const uint4 wi = ix.win[meta];
            metaPos = wi.x; sind = wi.z; eind = wi.w;
            off0 = cb.offs[r];
            size = (uint32_t)(cb.offs[r + 1] - off0);
            chrom = ix.cpg_chrom[sind];
        }
        const char* raw = cb.seqs + off0;
        const int n = (int)size;
        const int64_t gb0 = (int64_t)metaPos + offset;
        // the read's CpG range [minIndex, maxIndex] of the window (the loop of
        // ReadQueue.cpp:3651-3664 over its CpGs, which are in position order):
        // counts over the window's CpGs, split over the group's lanes
        uint32_t nlt = 0, nle = 0;
        if (have) {
            const uint32_t minPos = (uint32_t)(metaPos + offset - (size - 1)), maxPos = metaPos + offset;
            for (uint32_t id = sind + (uint32_t)k; id <= eind; id += 9) {
                const uint32_t cp = __ldg(ix.cpg_pos + id) + RL - 2;
                nlt += cp < minPos ? 1u : 0u;
                nle += cp <= maxPos ? 1u : 0u;
            }
        }
        uint32_t cnt_lt = 0, cnt_le = 0;
#pragma unroll
        for (int kk = 0; kk < 9; ++kk) {
            cnt_lt += __shfl_sync(0xffffffffu, nlt, 9 * (in_grp ? grp : 0) + kk);
            cnt_le += __shfl_sync(0xffffffffu, nle, 9 * (in_grp ? grp : 0) + kk);
        }
        if (have) {
            // row i (1..n) compares rowm[i - 1]; reference columns j in [-2, n + 10]
            for (int q = k; q < n; q += 9)
                rowm[q] = read_mask(oriented_char(raw, size, orient, isFwd ? (uint32_t)(n - 1 - q) : (uint32_t)q), isFwd);
            for (int j = k - DPW_REF0; j <= n + (int)DPB + 2; j += 9)
                refb[j + DPW_REF0] = ref_bit(gbase(ix, chrom, gb0 + 1 - j));
        }
        __syncwarp();
        // fill: steps t = 0 .. 2 * nmax + 9 over the group's anti-diagonals, two
        // per iteration (even: lane k holds offset 2k - 8, odd: 2k - 7)
        int nmax = n;
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) nmax = max(nmax, __shfl_xor_sync(0xffffffffu, nmax, d));
        const int o_even = 2 * k - 8, o_odd = 2 * k - 7;
        const bool act_even = have, act_odd = have && k < 8;
        int cur1 = 0xffff, cur2 = 0xffff;   // own values of steps t - 1 and t - 2
        uint32_t acc = 0;
        const int t_end = 2 * nmax + (int)DPB;
        // one anti-diagonal step; from step 10 on every cell is interior (row >= 1,
        // column >= 1) and the first-row / first-column cases drop out
        auto step = [&](const int tt, const int par, auto interior) {
            const int o = par ? o_odd : o_even;
            // up input (row - 1, o + 1) and left input (row, o - 1) are step t - 1
            // values: the own lane's and a neighbour's
            const int nb = par ? __shfl_down_sync(0xffffffffu, cur1, 1) : __shfl_up_sync(0xffffffffu, cur1, 1);
            const int v_up = par ? nb : cur1;
            const int v_lf = par ? cur1 : nb;
            const int row = (tt - o) >> 1;
            const int j = row + o;
            int val = 0xffff;
            uint32_t code = 0;
            const bool act = par ? act_odd : act_even;
            if (decltype(interior)::value ? (act && row <= n) : (act && row >= 0 && row <= n)) {
                if (!decltype(interior)::value && row == 0) {
                    if (o >= 0) val = o;                                     // first row: 0..8
                } else if (!decltype(interior)::value && j == 0) {
                    val = row;                                               // first column, rows 1..8
                } else if (decltype(interior)::value || j > 0) {
                    const int up = (o == (int)DPB) ? 65535 - (row - 1) - (int)DPB - 1 : v_up;
                    const int lf = (o == -(int)DPB) ? (row == (int)DPB + 1 ? 65535 - 2 * (int)DPB - 1 : 65535 - row)
                                                    : v_lf;
                    const int mm = (rowm[row - 1] & refb[j + DPW_REF0]) ? 0 : 1;
                    const int dg = cur2 + mm;
                    int v = min(up + 1, lf + 1);
                    v = min(v, dg);
                    val = v & 0xffff;
                    code = up < lf ? (up + 1 < dg ? 2u : (uint32_t)mm) : (lf + 1 < dg ? 3u : (uint32_t)mm);
                    if (row == n) rown[o + DPB] = (uint16_t)val;
                }
            }
            acc = __funnelshift_r(acc, code, 2);
            if ((tt & 15) == 15) codes[(tt >> 4) * 32 + lane] = acc;
            cur2 = cur1;
            cur1 = val;
        };
        static_assert(DPB + 2 <= 10, "every cell is interior from step DPB + 2 on");
        int t = 0;
        for (; t < 10 && t <= t_end; t += 2) {
            step(t, 0, std::false_type{});
            step(t + 1, 1, std::false_type{});
        }
        for (; t <= t_end; t += 2) {
            step(t, 0, std::true_type{});
            step(t + 1, 1, std::true_type{});
        }
        {
            const int last = t_end + 1;                  // the last step written into acc
            const int rem = (last & 15) + 1;             // steps in its word
            if (rem < 16) codes[(last >> 4) * 32 + lane] = acc >> (2 * (16 - rem));
        }
        __syncwarp();
        if (have && k == 0) {
            // backtrackDP / backtrackDPRev over the recorded choices
            uint32_t alen = 0;
            bool bad = false;
            uint16_t mn = 0xffff;
            long col = 0;
            for (long oo = -DPB; oo <= DPB; ++oo) {
                const uint16_t v = rown[oo + DPB];
                if (v < mn) { col = n + oo; mn = v; }
            }
            for (long row = n; row > 0;) {
                uint8_t code;
                if (col == 0 && row <= DPB) code = 2;
                else {
                    const long oo = col - row;
                    if (oo < -DPB || oo > DPB || col < 1) { bad = true; break; }
                    const long tt = 2 * row + oo;
                    const int ln = 9 * grp + (int)((oo + DPB - (tt & 1)) >> 1);
                    code = (uint8_t)((codes[(tt >> 4) * 32 + ln] >> (2 * (tt & 15))) & 3u);
                }
                if (alen >= DP3_ALIGN) { bad = true; break; }
                al[alen++] = code;
                if (code == 2) --row;
                else if (code == 3) --col;
                else { --row; --col; }
            }
            while (!bad && col > 0) {
                if (alen >= DP3_ALIGN) { bad = true; break; }
                al[alen++] = 3;
                --col;
            }
            if (bad) {
                atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull);
            } else {
                const int32_t minIndex = (int32_t)(sind + cnt_lt), maxIndex = (int32_t)(sind + cnt_le) - 1;
                uint32_t refSeqPos = metaPos + offset;
                int32_t readSeqPos = (int32_t)size - 1;
                int32_t alignPos = (int32_t)alen - 1;
                for (int32_t id = maxIndex; id >= minIndex; --id) {
                    const uint32_t cpos = ix.cpg_pos[id] + RL - 2;
                    while (cpos < refSeqPos && alignPos >= 0) {
                        switch (al[alignPos]) {
                            case 0: case 1: --readSeqPos; --refSeqPos; break;
                            case 3: --refSeqPos; break;
                            default: --readSeqPos; break;
                        }
                        if (readSeqPos < 0) break;
                        --alignPos;
                    }
                    if (readSeqPos < 0) break;
                    if (isFwd) {
                        const uint8_t c = oriented_char(raw, size, orient, (uint32_t)readSeqPos);
                        if (c == 'C') atomicAdd(cb.meth + 4ull * id + 0, 1u);
                        else if (c == 'T') atomicAdd(cb.meth + 4ull * id + 1, 1u);
                    } else {
                        const uint32_t kk = (uint32_t)readSeqPos + 1;
                        const uint8_t c = kk < size ? oriented_char(raw, size, orient, size - 1 - kk) : 0;
                        if (c == 'C') atomicAdd(cb.meth + 4ull * id + 2, 1u);
                        else if (c == 'T') atomicAdd(cb.meth + 4ull * id + 3, 1u);
                    }
                }
            }
        }
        __syncwarp();
    }
}

}  // namespace fame
