// Paired-end matching: one warp per read pair.
//
// Follows matchPairedReads (ReadQueue.cpp:940-1658) per pair and orientation:
//   getSeedRefsFirstRead  (ReadQueue.cpp:2468-2794)   first mate's window counts
//   getSeedRefsSecondRead (ReadQueue.cpp:2801-3164)   mate counts near those windows
//   saQuerySeedSetRefFirst / Second (ReadQueue.cpp:2167-2323) with
//   matchFwd/RevFirst/Second (ReadQueue.cpp:4538-4776)  sorted, pruned walks
//   extractPairedMatch (ReadQueue.cpp:3255-3275) and the pair choice (1300-1638)
//
// The maps of the reference (tsl::hopscotch_map<uint32_t, tuple<u8 count1,
// u8 count2, bool f2, bool f3>>, one per window strand) are kept as a value
// table for lookups plus the sequence of insertions; the iteration order,
// which decides the order of the candidate lists before their (unstable)
// std::sort, is reproduced by replaying those insertions (seed.cuh).  The
// first mate's map is rebuilt after counting into a map of 20 buckets holding
// the windows with count1 >= QTHRESH in the old map's order, and the second
// mate inserts new windows into that map, so the final order is the replay of
// [kept keys in the first map's order] ++ [keys the second mate inserted].
//
// Lanes hash and look up the k-mers; lane 0 applies the map operations in the
// reference's order, replays, sorts and walks.  Pairs whose working set
// exceeds the shared-memory caps are handed to a launch with global scratch.
#pragma once
#include "kernels.cuh"
#include "seedhash.h"

namespace fame {

constexpr uint32_t KMERDIST = 10;  // CONST.h:104

// paired-path tables
struct PeIndex {
    const uint32_t* tmask;     // per k-mer entry (kmerTableSmall.tmask)
    const uint64_t* filtered;  // filteredKmers, sorted
    uint64_t n_filtered;
    uint32_t ctx;              // contextWLen = floor(MAXPDIST / WINLEN) + 1
    uint32_t maxdist;          // MAXPDIST + READLEN
};

// value of a map entry
constexpr uint32_t PV_PRESENT = 1u << 31;
constexpr uint32_t PV_F2 = 1u << 16;
constexpr uint32_t PV_F3 = 1u << 17;
__device__ __forceinline__ uint32_t pv_c1(uint32_t v) { return v & 0xffu; }
__device__ __forceinline__ uint32_t pv_c2(uint32_t v) { return (v >> 8) & 0xffu; }

constexpr uint32_t PE_KMAX = FAME_MAX_READ_LEN - KMERLEN + 1;   // k-mers of the longest read
constexpr uint64_t PE_KMER_AREA = 8 * 256 + 96;                  // pe_kmers' per-read arrays
constexpr uint32_t PE_SEED_WARPS = 2;                            // warps per block of k_pe_seed

// Capacities of one warp's working memory.
struct PeCaps {
    uint32_t icap;      // keys per map and phase
    uint32_t vcap;      // value-table slots per strand (power of two, >= 4 * icap)
    uint32_t slot_cap;  // replayed bucket array
    uint32_t ovf_cap;
    uint32_t hcap;      // hits per mate and orientation
    uint32_t ecap;      // bucket entries of one mate staged in working memory (0: read in place)
    uint32_t kmax;      // k-mers of the longest mate (per-k-mer arrays)
};

struct PeMem {
    uint8_t* rd[2];       // oriented first and second mate
    uint32_t* kst;        // per k-mer: bucket start
    uint32_t* kln;        //            bucket size
    uint32_t* kcm;        //            C mask
    uint8_t* kfl;         //            in filteredKmers
    uint32_t* vk[2];      // value tables per window strand (0 reverse, 1 forward)
    uint32_t* vv[2];
    uint32_t* ins1[2];    // first-mate insertions
    uint32_t* ins2[2];    // second-mate insertions
    uint32_t* seq;        // one replay's insertion sequence
    uint32_t* ord[2];     // final iteration order
    uint32_t* slot;
    uint32_t* stk;
    uint32_t* ovf;
    uint2* list[2];       // (key, value) candidate lists
    uint64_t* hits[4];    // m1F, m2R, m1R, m2F
    uint32_t* kpre;       // per k-mer: first staged entry (exclusive prefix of bucket sizes)
    uint32_t* ge;         // staged entries (window | forward << 31) and their T masks
    uint32_t* gt;
    uint8_t* gk;          // k-mer of each staged entry
    uint8_t* sv;          // staged entry survives the T-mask filter and the dedup
    uint16_t* occ[2];     // value-table slots holding a key, in insertion order (occn[dir] of them):
    uint32_t* occn;       // the sweeps visit these, and the next pair clears only these
    uint32_t area;        // bytes of regions 11 .. 16 (dead while the maps are built)
    PeCaps c;
};

__host__ __device__ inline uint64_t pe_align16(uint64_t x) { return (x + 15) & ~15ull; }

// Byte layout of PeMem for the given caps (PE_LAYOUT_N region offsets into
// off); returns the total.
constexpr int PE_LAYOUT_N = 31;
__host__ __device__ inline uint64_t pe_layout(PeCaps c, uint64_t* off)
{
    uint64_t o = 0;
    int i = 0;
    auto put = [&](uint64_t bytes) { off[i++] = o; o = pe_align16(o + bytes); };
    put(8ull * c.hcap * 4);                 // 0 hits
    put(8ull * c.icap * 2);                 // 1 list[0]
    put(8ull * c.icap * 2);                 // 2 list[1]
    put(4ull * c.vcap);                     // 3 vk[0]
    put(4ull * c.vcap);                     // 4 vk[1]
    put(4ull * c.vcap);                     // 5 vv[0]
    put(4ull * c.vcap);                     // 6 vv[1]
    put(4ull * c.icap);                     // 7 ins1[0]
    put(4ull * c.icap);                     // 8 ins1[1]
    put(4ull * c.icap);                     // 9 ins2[0]
    put(4ull * c.icap);                     // 10 ins2[1]
    put(4ull * c.icap * 2);                 // 11 seq
    put(4ull * c.icap * 2);                 // 12 ord[0]
    put(4ull * c.icap * 2);                 // 13 ord[1]
    put(4ull * c.slot_cap);                 // 14 slot
    put(4ull * c.icap * 2);                 // 15 stk
    put(4ull * c.ovf_cap);                  // 16 ovf
    put(4ull * c.kmax);                     // 17 kst
    put(4ull * c.kmax);                     // 18 kln
    put(4ull * c.kmax);                     // 19 kcm
    put(c.kmax);                            // 20 kfl
    put(256);                               // 21 rd[0]
    put(256);                               // 22 rd[1]
    put(4ull * (c.kmax + 1));               // 23 kpre
    put(4ull * c.ecap);                     // 24 ge
    put(4ull * c.ecap);                     // 25 gt
    put(c.ecap);                            // 26 gk
    put(c.ecap);                            // 27 sv
    put(2ull * c.vcap);                     // 28 occ[0]
    put(2ull * c.vcap);                     // 29 occ[1]
    put(16);                                // 30 occn
    return o;
}

__device__ inline PeMem pe_mem(uint8_t* base, PeCaps c)
{
    uint64_t off[PE_LAYOUT_N];
    pe_layout(c, off);
    PeMem s;
    s.c = c;
    uint64_t* h = (uint64_t*)(base + off[0]);
    for (int k = 0; k < 4; ++k) s.hits[k] = h + (uint64_t)k * c.hcap;
    s.list[0] = (uint2*)(base + off[1]);
    s.list[1] = (uint2*)(base + off[2]);
    s.vk[0] = (uint32_t*)(base + off[3]);
    s.vk[1] = (uint32_t*)(base + off[4]);
    s.vv[0] = (uint32_t*)(base + off[5]);
    s.vv[1] = (uint32_t*)(base + off[6]);
    s.ins1[0] = (uint32_t*)(base + off[7]);
    s.ins1[1] = (uint32_t*)(base + off[8]);
    s.ins2[0] = (uint32_t*)(base + off[9]);
    s.ins2[1] = (uint32_t*)(base + off[10]);
    s.seq = (uint32_t*)(base + off[11]);
    s.ord[0] = (uint32_t*)(base + off[12]);
    s.ord[1] = (uint32_t*)(base + off[13]);
    s.slot = (uint32_t*)(base + off[14]);
    s.stk = (uint32_t*)(base + off[15]);
    s.ovf = (uint32_t*)(base + off[16]);
    s.kst = (uint32_t*)(base + off[17]);
    s.kln = (uint32_t*)(base + off[18]);
    s.kcm = (uint32_t*)(base + off[19]);
    s.kfl = base + off[20];
    s.rd[0] = base + off[21];
    s.rd[1] = base + off[22];
    s.kpre = (uint32_t*)(base + off[23]);
    s.ge = (uint32_t*)(base + off[24]);
    s.gt = (uint32_t*)(base + off[25]);
    s.gk = base + off[26];
    s.sv = base + off[27];
    s.occ[0] = (uint16_t*)(base + off[28]);
    s.occ[1] = (uint16_t*)(base + off[29]);
    s.occn = (uint32_t*)(base + off[30]);
    s.area = (uint32_t)(off[17] - off[11]);
    return s;
}

// Empty value tables and slot lists (all lanes; once per warp and launch:
// from then on each pair clears the slots it occupied when the next starts).
__device__ inline void pe_tables_reset(const PeMem& s)
{
    const int lane = threadIdx.x & 31;
    for (uint32_t i = lane; i < s.c.vcap; i += 32) {
        s.vk[0][i] = EMPTY_KEY;
        s.vk[1][i] = EMPTY_KEY;
        s.vv[0][i] = 0;
        s.vv[1][i] = 0;
    }
    if (lane == 0) {
        s.occn[0] = 0;
        s.occn[1] = 0;
    }
    __syncwarp();
}

// shared-memory caps of k_pe_seed (one warp; it keeps no matches)
constexpr PeCaps PE_LIGHT{64, 256, 256 + NBHD - 1, 64, 0, 320, PE_KMAX};
// caps of the paired middle tiers (global scratch): genome-scale indexes put
// about three entries in a bucket and a few hundred keys in a mate's map.
// The first holds the common pair with small tables (the value-table sweeps
// of a pair cost in proportion to vcap), the second the rest.
constexpr PeCaps PE_MID_S{256, 1024, 1024 + NBHD - 1 + 64, 256, 0, 2048, PE_KMAX};
constexpr PeCaps PE_MID{1024, 4096, 4096 + NBHD - 1 + 64, 256, 0, 4096, PE_KMAX};

__device__ __forceinline__ uint32_t vt_hash(uint32_t k, uint32_t mask) { return (k * 0x9E3779B1u) >> 8 & mask; }

// Lane-0 state of one pair and orientation.
struct PeState {
    uint32_t nkeys[2];   // keys held by each value table
    uint32_t n1[2];      // first-mate insertions
    uint32_t n2[2];      // second-mate insertions
    uint32_t nord[2];
    bool over;           // a capacity was exceeded
};

// slot of key in the strand's table when present, else -1
__device__ __forceinline__ int pm_find(const PeMem& s, int dir, uint32_t key)
{
    if (key == EMPTY_KEY) return -1;
    const uint32_t mask = s.c.vcap - 1;
    for (uint32_t h = vt_hash(key, mask);; h = (h + 1) & mask) {
        const uint32_t k = s.vk[dir][h];
        if (k == key) return (s.vv[dir][h] & PV_PRESENT) ? (int)h : -1;
        if (k == EMPTY_KEY) return -1;
    }
}

// operator[]: the key's slot, inserted (and recorded) when absent; -1 when full
__device__ __forceinline__ int pm_at(const PeMem& s, PeState& st, int dir, uint32_t key, int phase)
{
    const uint32_t mask = s.c.vcap - 1;
    uint32_t h = vt_hash(key, mask);
    for (;; h = (h + 1) & mask) {
        const uint32_t k = s.vk[dir][h];
        if (k == key) break;
        if (k == EMPTY_KEY) {
            if (4 * (st.nkeys[dir] + 1) > 3 * s.c.vcap) { st.over = true; return -1; }
            s.vk[dir][h] = key;
            s.vv[dir][h] = 0;
            s.occ[dir][st.nkeys[dir]] = (uint16_t)h;
            st.nkeys[dir]++;
            s.occn[dir] = st.nkeys[dir];
            break;
        }
    }
    if (!(s.vv[dir][h] & PV_PRESENT)) {
        uint32_t& n = phase == 1 ? st.n1[dir] : st.n2[dir];
        if (n >= s.c.icap) { st.over = true; return -1; }
        (phase == 1 ? s.ins1[dir] : s.ins2[dir])[n++] = key;
        s.vv[dir][h] = PV_PRESENT;
    }
    return (int)h;
}

__device__ __forceinline__ bool filtered_has(const PeIndex& px, uint64_t k)
{
    uint64_t lo = 0, hi = px.n_filtered;
    while (lo < hi) {
        const uint64_t mid = (lo + hi) >> 1;
        if (__ldg(px.filtered + mid) < k) lo = mid + 1;
        else hi = mid;
    }
    return lo < px.n_filtered && __ldg(px.filtered + lo) == k;
}

// Warp: per k-mer bucket bounds, C mask and filteredKmers flag of the read in
// rd; returns the summed bucket sizes (the maps' bucket_count * 5).
__device__ uint32_t pe_kmers(const DevIndex& ix, const PeIndex& px, const PeMem& s, const uint8_t* rd, uint32_t len)
{
    constexpr uint32_t FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t nk = len - KMERLEN + 1;
    uint32_t sigma = 0;
    // per-read arrays in the replay area (dead until both mates' maps are
    // built): the hash prefix P[0..len] of seedhash.h, a C bitmap (bit j of
    // Cw: base j is C) and the filteredKmers codes, 16 per word (base j at
    // bits 2(j mod 16) of Kw[j / 16])
    uint64_t* P = (uint64_t*)s.seq;
    uint32_t* Cw = (uint32_t*)(P + 256);
    uint32_t* Kw = Cw + 8;
    {
        uint64_t carry = 0;
        for (uint32_t b = 0; b <= len; b += 32) {
            const uint32_t j = b + lane;
            const uint8_t c = j < len ? rd[j] : (uint8_t)0;
            const uint64_t u = j < len ? sh_u(c, j) : 0ull;
            uint64_t inc = u;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint64_t t = __shfl_up_sync(FULL, inc, d);
                if (lane >= d) inc ^= t;
            }
            if (j <= len) P[j] = carry ^ inc ^ u;
            carry ^= __shfl_sync(FULL, inc, 31);
            const uint32_t cbits = __ballot_sync(FULL, c == 'C');
            uint32_t kw = ((c == 'C' || c == 'T') ? 3u : (c == 'G' ? 2u : 0u)) << (2 * (lane & 15));
#pragma unroll
            for (int d = 1; d < 16; d <<= 1) kw |= __shfl_xor_sync(FULL, kw, d);
            if (b < 256) {
                if (lane == 0) Cw[b >> 5] = cbits;
                if ((lane & 15) == 0) Kw[(b >> 4) + (lane >> 4)] = kw;
            }
        }
    }
    __syncwarp();
    // per k-mer: table index, bucket bounds (all loads of a lane issued before
    // any is used), C mask (base p at bit 31) and the filteredKmers key (the
    // 2-bit codes of bases p + 16 .. p + 31, the first at the top)
    constexpr int KPL = (PE_KMAX + 31) / 32;
    uint32_t b0[KPL], b1[KPL];
#pragma unroll
    for (int jj = 0; jj < KPL; ++jj) {
        const uint32_t p = lane + 32 * jj;
        if (p < nk) {
            const uint32_t key = sh_prefix_hash([&](uint32_t j) { return P[j]; }, p, HTAB_MASK);
            uint32_t slot;
            // {start, size, ...}; a dense record is read once, evict-first, so that
            // the index lines do not push the warps' working memory out of L2
            const uint4 t = ix.rec_hashed ? rec_lookup(ix, key, slot) : __ldcs(ix.rec + 2ull * key);
            b0[jj] = t.x;
            b1[jj] = t.x + t.y;
        }
    }
#pragma unroll
    for (int jj = 0; jj < KPL; ++jj) {
        const uint32_t p = lane + 32 * jj;
        if (p < nk) {
            const uint32_t w = p >> 5;
            s.kcm[p] = __brev(__funnelshift_r(Cw[w], Cw[w + 1], p & 31));
            uint8_t fl = 0;
            if (p > 0 && px.n_filtered) {
                const uint32_t bit = 2 * (p + 16);
                const uint32_t y = __brev(__funnelshift_r(Kw[bit >> 5], Kw[(bit >> 5) + 1], bit & 31));
                const uint32_t kq = ((y >> 1) & 0x55555555u) | ((y << 1) & 0xAAAAAAAAu);
                fl = filtered_has(px, kq) ? 1 : 0;
            }
            s.kfl[p] = fl;
            s.kst[p] = b0[jj];
            s.kln[p] = b1[jj] - b0[jj];
            sigma += b1[jj] - b0[jj];
        }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) sigma += __shfl_xor_sync(0xffffffffu, sigma, d);
    __syncwarp();
    if (sigma > s.c.ecap) return sigma;     // entries are read in place
    // stage the entries and T masks of all buckets (loads of a lane overlap)
    {
        const uint32_t per = (nk + 31) / 32;
        const uint32_t b = min(nk, lane * per), e = min(nk, b + per);
        uint32_t loc = 0;
        for (uint32_t p = b; p < e; ++p) loc += s.kln[p];
        uint32_t inc = loc;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, d);
            if (lane >= d) inc += v;
        }
        uint32_t run = inc - loc;
        for (uint32_t p = b; p < e; ++p) {
            s.kpre[p] = run;
            for (uint32_t j = 0; j < s.kln[p]; ++j) s.gk[run + j] = (uint8_t)p;
            run += s.kln[p];
        }
    }
    __syncwarp();
    for (uint32_t base = 0; base < sigma; base += 256) {
        uint32_t ev[8], tv[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = base + lane + 32 * j;
            if (i < sigma) {
                const uint32_t p = s.gk[i];
                const uint32_t src = s.kst[p] + (i - s.kpre[p]);
                ev[j] = __ldcs(ix.entry + src);   // read once: evict-first
                tv[j] = __ldcs(px.tmask + src);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const uint32_t i = base + lane + 32 * j;
            if (i < sigma) { s.ge[i] = ev[j]; s.gt[i] = tv[j]; }
        }
    }
    __syncwarp();
    return sigma;
}

// Iteration order of a map that received seq[0..n) by insertion into
// bucket_count buckets; false when the replay exceeds a cap.
__device__ bool pe_replay(const PeMem& s, const uint32_t* seq, uint32_t n, uint32_t bucket_count, uint32_t* out,
                          uint32_t& nout)
{
    SeedMem sm{};
    sm.ins = (uint32_t*)seq;
    sm.slot = s.slot;
    sm.stk = s.stk;
    sm.ovf = s.ovf;
    sm.slot_cap = s.c.slot_cap;
    sm.stk_cap = 2 * s.c.icap;
    sm.ovf_cap = s.c.ovf_cap;
    MapSim m;
    sim_init(m, bucket_count);
    m.nb = 0; m.novf = 0; m.sp = 0;
    if (m.size > s.c.slot_cap) return false;
    for (uint32_t b = 0; b < m.size; ++b) s.slot[b] = EMPTY_KEY;
    for (uint32_t x = 0; x < n; ++x) {
        if (m.sp >= sm.stk_cap) return false;
        s.stk[m.sp++] = x;
        while (m.sp > 0)
            if (!sim_step(m, sm)) return false;
    }
    nout = 0;
    for (uint32_t b = 0; b < m.size; ++b)
        if (s.slot[b] != EMPTY_KEY) out[nout++] = seq[s.slot[b]];
    for (uint32_t i = 0; i < m.novf; ++i) out[nout++] = seq[s.ovf[i]];
    return true;
}

// The same replay run by the whole warp (every lane calls; nout and the
// return value are warp-uniform): insertions batched as in the single-end
// seeding (sim_insert_batch_w), the iteration order taken with ballots.
__device__ bool pe_replay_w(const PeMem& s, const uint32_t* seq, uint32_t n, uint32_t bucket_count, uint32_t* out,
                            uint32_t& nout)
{
    constexpr uint32_t FULL = 0xffffffffu;
    const uint32_t lane = threadIdx.x & 31;
    SeedMem sm{};
    sm.ins = (uint32_t*)seq;
    sm.slot = s.slot;
    sm.stk = s.stk;
    sm.ovf = s.ovf;
    sm.slot_cap = s.c.slot_cap;
    sm.stk_cap = 2 * s.c.icap;
    sm.ovf_cap = s.c.ovf_cap;
    MapSim m;
    sim_init(m, bucket_count);
    m.nb = 0; m.novf = 0; m.sp = 0;
    if (m.size > s.c.slot_cap) return false;
    for (uint32_t b = lane; b < m.size; b += 32) s.slot[b] = EMPTY_KEY;
    __syncwarp();
    for (uint32_t b0 = 0; b0 < n; b0 += 32) {
        const unsigned todo = __ballot_sync(FULL, b0 + lane < n);
        if (!sim_insert_batch_w(m, sm, b0, todo)) return false;
    }
    uint32_t no = 0;
    for (uint32_t b0 = 0; b0 < m.size + m.novf; b0 += 32) {
        const uint32_t b = b0 + lane;
        uint32_t x = EMPTY_KEY;
        if (b < m.size) x = s.slot[b];
        else if (b < m.size + m.novf) x = s.ovf[b - m.size];
        const unsigned bm = __ballot_sync(FULL, x != EMPTY_KEY);
        if (x != EMPTY_KEY) out[no + __popc(bm & ((1u << lane) - 1))] = seq[x];
        no += __popc(bm);
    }
    __syncwarp();
    nout = no;
    return true;
}

// ---------------------------------------------------------------------------
// std::sort of libstdc++ (introsort with median-of-three pivot, heap sort past
// the depth limit, final insertion sort with a 16-element threshold) with
// comp(a, b) = count(a) > count(b) (CompiMetaFirst / CompiMetaSecond,
// ReadQueue.h:340-353).  The sort is not stable, so its exact steps decide the
// order of equal counts.
// ---------------------------------------------------------------------------
struct PeCmp {
    int second;
    __device__ __forceinline__ bool operator()(const uint2& a, const uint2& b) const
    {
        return second ? pv_c2(a.y) > pv_c2(b.y) : pv_c1(a.y) > pv_c1(b.y);
    }
};

__device__ inline void ps_swap(uint2* a, uint2* b) { const uint2 t = *a; *a = *b; *b = t; }

__device__ inline void ps_insertion(uint2* f, uint2* l, PeCmp cmp)
{
    if (f == l) return;
    for (uint2* i = f + 1; i != l; ++i) {
        const uint2 val = *i;
        if (cmp(val, *f)) {
            for (uint2* j = i; j != f; --j) *j = *(j - 1);
            *f = val;
        } else {
            uint2* last = i;
            uint2* next = i - 1;
            while (cmp(val, *next)) { *last = *next; last = next; --next; }
            *last = val;
        }
    }
}

__device__ inline void ps_unguarded_insertion(uint2* f, uint2* l, PeCmp cmp)
{
    for (uint2* i = f; i != l; ++i) {
        const uint2 val = *i;
        uint2* last = i;
        uint2* next = i - 1;
        while (cmp(val, *next)) { *last = *next; last = next; --next; }
        *last = val;
    }
}

__device__ inline void ps_adjust_heap(uint2* f, long hole, long len, uint2 val, PeCmp cmp)
{
    const long top = hole;
    long child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (cmp(f[child], f[child - 1])) --child;
        f[hole] = f[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        f[hole] = f[child - 1];
        hole = child - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && cmp(f[parent], val)) {
        f[hole] = f[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    f[hole] = val;
}

__device__ inline void ps_heap_select_sort(uint2* f, uint2* m, uint2* l, PeCmp cmp)
{
    // make_heap on [f, m)
    const long len = m - f;
    if (len >= 2) {
        for (long parent = (len - 2) / 2;; --parent) {
            ps_adjust_heap(f, parent, len, f[parent], cmp);
            if (parent == 0) break;
        }
    }
    for (uint2* i = m; i < l; ++i)
        if (cmp(*i, *f)) {
            const uint2 val = *i;
            *i = *f;
            ps_adjust_heap(f, 0, len, val, cmp);
        }
    // sort_heap
    for (uint2* e = m; e - f > 1;) {
        --e;
        const uint2 val = *e;
        *e = *f;
        ps_adjust_heap(f, 0, e - f, val, cmp);
    }
}

__device__ inline void ps_median_first(uint2* r, uint2* a, uint2* b, uint2* c, PeCmp cmp)
{
    if (cmp(*a, *b)) {
        if (cmp(*b, *c)) ps_swap(r, b);
        else if (cmp(*a, *c)) ps_swap(r, c);
        else ps_swap(r, a);
    } else if (cmp(*a, *c)) ps_swap(r, a);
    else if (cmp(*b, *c)) ps_swap(r, c);
    else ps_swap(r, b);
}

__device__ inline uint2* ps_partition(uint2* f, uint2* l, uint2* pivot, PeCmp cmp)
{
    while (true) {
        while (cmp(*f, *pivot)) ++f;
        --l;
        while (cmp(*pivot, *l)) --l;
        if (!(f < l)) return f;
        ps_swap(f, l);
        ++f;
    }
}

// introsort loop with an explicit stack (the recursion goes right, the loop left)
__device__ inline void ps_introsort(uint2* f, uint2* l, long depth, PeCmp cmp)
{
    struct Frame { uint2* f; uint2* l; long depth; };
    Frame stk[64];
    int sp = 0;
    stk[sp++] = {f, l, depth};
    while (sp > 0) {
        Frame fr = stk[--sp];
        uint2* a = fr.f;
        uint2* b = fr.l;
        long d = fr.depth;
        while (b - a > 16) {
            if (d == 0) { ps_heap_select_sort(a, b, b, cmp); break; }
            --d;
            uint2* mid = a + (b - a) / 2;
            ps_median_first(a, a + 1, mid, b - 1, cmp);
            uint2* cut = ps_partition(a + 1, b, a, cmp);
            if (sp < 64) stk[sp++] = {cut, b, d};
            b = cut;
        }
    }
}

__device__ inline void pe_sort(uint2* f, long n, PeCmp cmp)
{
    if (n <= 1) return;
    long lg = 0;
    while ((1l << (lg + 1)) <= n) ++lg;
    ps_introsort(f, f + n, 2 * lg, cmp);
    if (n > 16) {
        ps_insertion(f, f + 16, cmp);
        ps_unguarded_insertion(f + 16, f + n, cmp);
    } else {
        ps_insertion(f, f + n, cmp);
    }
}

// ---------------------------------------------------------------------------
// Lane-parallel map counting of the first mate from the staged bucket entries
// (getSeedRefsFirstRead).
//
// A bucket entry survives when the T-mask filter keeps it and it is not a
// repeat of the previous surviving entry of its bucket.  An op may insert its
// key when its k-mer index p has p == 0 or p - 1 < maxQPos, a prefix of the
// ops (they come in k-mer order), so a key's first surviving op decides:
// the key is inserted there when that op may insert, and then every one of
// its ops counts; otherwise none does.  Counts commute, so only the
// first-touch order needs the ops in order: chunks of 32 ops in order, equal
// keys of a chunk grouped with __match_any_sync, new keys appended with
// ballots.  The second mate, whose inserts also need a map key within
// contextWLen windows, is pe_count_par2.  Scratch bits of a value during the
// passes: bit 30 the key was seen, bits 18-29 its op count.
// ---------------------------------------------------------------------------
constexpr uint32_t PV_SEEN = 1u << 30;
constexpr uint32_t PV_RAW_SHIFT = 18;
constexpr uint32_t PV_RAW_MASK = 0xfffu << PV_RAW_SHIFT;

__device__ void pe_survivors(const PeMem& s, uint32_t nk)
{
    const int lane = threadIdx.x & 31;
    for (uint32_t p = lane; p < nk; p += 32) {
        const uint32_t b0 = s.kpre[p], n = s.kln[p], cm = s.kcm[p];
        const bool filt = s.kfl[p] != 0;
        bool have = false;
        uint32_t last = 0;
        for (uint32_t i = b0; i < b0 + n; ++i) {
            uint8_t keep = 0;
            if (!filt && !(cm & SEEDBITS & s.gt[i])) {
                const uint32_t e = s.ge[i];           // window | forward << 31: equal iff same window and strand
                if (!(have && e == last)) keep = 1;
                have = true;
                last = e;
            }
            s.sv[i] = keep;
        }
    }
    __syncwarp();
}

// All lanes.  Returns 1 done, 0 not applicable (second mate, a neighbour
// created by the mate itself would be needed), -1 over the table capacity.
__device__ int pe_count_par(const PeIndex& px, const PeMem& s, PeState& st, uint32_t len, uint32_t sigma)
{
    const int lane = threadIdx.x & 31;
    const uint32_t nk = len - KMERLEN + 1;
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    pe_survivors(s, nk);
    uint32_t nkeys[2] = {__shfl_sync(0xffffffffu, st.nkeys[0], 0), __shfl_sync(0xffffffffu, st.nkeys[1], 0)};
    uint32_t nins[2] = {0, 0};
    uint32_t* ins[2] = {s.ins1[0], s.ins1[1]};
    const uint32_t mask = s.c.vcap - 1;
    bool over = false;
    for (uint32_t base = 0; base < sigma && !over; base += 32) {
        if (4 * (nkeys[0] + 32) > 3 * s.c.vcap || 4 * (nkeys[1] + 32) > 3 * s.c.vcap) { over = true; break; }
        const uint32_t i = base + lane;
        const bool live = i < sigma && s.sv[i];
        const uint32_t e = live ? s.ge[i] : 0u;
        const int dir = (int)(e >> 31);
        const uint32_t id = e & 0x7fffffffu;
        const uint32_t p = live ? s.gk[i] : 0u;
        const bool may = live && (p == 0 || p - 1 < maxQPos);
        const unsigned vm = __ballot_sync(0xffffffffu, live);
        const unsigned grp = __match_any_sync(0xffffffffu, live ? e : EMPTY_KEY) & vm;
        const bool leader = live && (__ffs(grp) - 1) == lane;
        bool fresh = false, added = false;
        uint32_t hs = 0;
        if (leader) {
            uint32_t h = vt_hash(id, mask);
            for (;; h = (h + 1) & mask) {
                const uint32_t k = s.vk[dir][h];
                if (k == id) break;
                if (k == EMPTY_KEY) {
                    const uint32_t old = atomicCAS(&s.vk[dir][h], EMPTY_KEY, id);
                    if (old == EMPTY_KEY) { added = true; break; }
                    if (old == id) break;
                }
            }
            hs = h;
            uint32_t v = s.vv[dir][h];
            if (!(v & PV_SEEN)) {
                v |= PV_SEEN;
                if (!(v & PV_PRESENT) && may) { v |= PV_PRESENT; fresh = true; }
            }
            if (v & PV_PRESENT) v += (uint32_t)__popc(grp) << PV_RAW_SHIFT;
            s.vv[dir][h] = v;
        }
        for (int d = 0; d < 2; ++d) {
            const unsigned na = __ballot_sync(0xffffffffu, added && dir == d);
            if (added && dir == d) s.occ[d][nkeys[d] + __popc(na & ((1u << lane) - 1))] = (uint16_t)hs;
            nkeys[d] += __popc(na);
            if (lane == 0) s.occn[d] = nkeys[d];
            const unsigned bm = __ballot_sync(0xffffffffu, fresh && dir == d);
            if (fresh && dir == d) {
                const uint32_t at = nins[d] + __popc(bm & ((1u << lane) - 1));
                if (at < s.c.icap) ins[d][at] = id;
            }
            nins[d] += __popc(bm);
        }
        if (nins[0] > s.c.icap || nins[1] > s.c.icap) over = true;
        __syncwarp();
    }
    if (over) return -1;
    // fold the op counts into count1 / count2 (8-bit wrap) and clear the scratch bits
    for (int dir = 0; dir < 2; ++dir)
        for (uint32_t x = lane; x < nkeys[dir]; x += 32) {
            const uint32_t h = s.occ[dir][x];
            const uint32_t v = s.vv[dir][h];
            const uint32_t raw = ((v & PV_RAW_MASK) >> PV_RAW_SHIFT) & 0xffu;
            const uint32_t base_v = v & ~(PV_RAW_MASK | PV_SEEN);
            s.vv[dir][h] = (v & PV_PRESENT) ? ((base_v & ~0xffu) | raw) : base_v;
        }
    __syncwarp();
    for (int d = 0; d < 2; ++d) {
        st.nkeys[d] = nkeys[d];
        st.n1[d] = nins[d];
    }
    return 1;
}

// Lane-parallel counting of the second mate, exact for any op order
// (getSeedRefsSecondRead).  An op may insert its absent key K when its k-mer
// index allows it (p == 0 or p - 1 < maxQPos) and a key within ctx windows is
// in the map at that moment: one kept from the first mate, or one the second
// mate inserted at an earlier op.  So the op at which K is inserted is the
// least solution of
//     at(K) = min { i : op i has key K and may insert, and K has a kept key
//                   within ctx windows or some K' within ctx has at(K') < i },
// found by atomicMin passes over the ops until none changes (the chains of
// keys that give each other context are short).  K then counts its ops from
// at(K) on, a kept key all of its ops, and the inserted keys enter ins2 in
// the order of at().  at[] lives in the k-mer area (dead between pe_kmers and
// the replay), one word per value-table slot.  Returns 1, or -1 when a
// capacity is exceeded.
__device__ __forceinline__ int pm_slot(const PeMem& s, int dir, uint32_t key)
{
    const uint32_t mask = s.c.vcap - 1;
    for (uint32_t h = vt_hash(key, mask);; h = (h + 1) & mask) {
        const uint32_t k = s.vk[dir][h];
        if (k == key) return (int)h;
        if (k == EMPTY_KEY) return -1;
    }
}

__device__ int pe_count_par2(const PeIndex& px, const PeMem& s, PeState& st, uint32_t len, uint32_t sigma)
{
    constexpr uint32_t FULL = 0xffffffffu, INF = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const uint32_t nk = len - KMERLEN + 1;
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    const int ctx = (int)px.ctx;
    const uint32_t mask = s.c.vcap - 1;
    pe_survivors(s, nk);
    uint32_t* at[2] = {s.seq, s.seq + s.c.vcap};
    for (uint32_t h = lane; h < s.c.vcap; h += 32) at[0][h] = at[1][h] = INF;
    uint32_t nkeys[2] = {__shfl_sync(FULL, st.nkeys[0], 0), __shfl_sync(FULL, st.nkeys[1], 0)};
    __syncwarp();
    // A: table slots for the keys of ops that may insert; an absent key with a
    //    kept key within ctx windows is inserted by its first such op
    for (uint32_t base = 0; base < sigma; base += 32) {
        if (4 * (nkeys[0] + 32) > 3 * s.c.vcap || 4 * (nkeys[1] + 32) > 3 * s.c.vcap) return -1;
        const uint32_t i = base + lane;
        const bool live = i < sigma && (s.sv[i] & 1);
        const uint32_t p = live ? s.gk[i] : 0u;
        const bool may = live && (p == 0 || p - 1 < maxQPos);
        const uint32_t e = may ? s.ge[i] : 0u;
        const int dir = (int)(e >> 31);
        const uint32_t id = e & 0x7fffffffu;
        bool added = false;
        uint32_t hs = 0;
        if (may) {
            uint32_t h = vt_hash(id, mask);
            for (;; h = (h + 1) & mask) {
                const uint32_t k = s.vk[dir][h];
                if (k == id) break;
                if (k == EMPTY_KEY) {
                    const uint32_t old = atomicCAS(&s.vk[dir][h], EMPTY_KEY, id);
                    if (old == EMPTY_KEY) { added = true; break; }
                    if (old == id) break;
                }
            }
            hs = h;
            if (!(s.vv[dir][h] & PV_PRESENT)) {
                bool kept = false;
                for (int c = -ctx; c <= ctx && !kept; ++c)
                    if (c != 0) kept = pm_find(s, dir, id + (uint32_t)c) >= 0;
                if (kept) atomicMin(&at[dir][h], i);
            }
        }
        for (int d = 0; d < 2; ++d) {
            const unsigned na = __ballot_sync(FULL, added && dir == d);
            if (added && dir == d) s.occ[d][nkeys[d] + __popc(na & ((1u << lane) - 1))] = (uint16_t)hs;
            nkeys[d] += __popc(na);
            if (lane == 0) s.occn[d] = nkeys[d];
        }
        __syncwarp();
    }
    // B: context from keys the second mate inserts earlier, to the fixed point
    // (without one after 64 passes the pair goes to the per-pair path)
    bool settled = false;
    for (int round = 0; round < 64 && !settled; ++round) {
        bool changed = false;
        for (uint32_t i = lane; i < sigma; i += 32) {
            if (!(s.sv[i] & 1)) continue;
            const uint32_t p = s.gk[i];
            if (!(p == 0 || p - 1 < maxQPos)) continue;
            const uint32_t e = s.ge[i];
            const int dir = (int)(e >> 31);
            const uint32_t id = e & 0x7fffffffu;
            const int h = pm_slot(s, dir, id);
            if (h < 0 || (s.vv[dir][h] & PV_PRESENT) || at[dir][h] <= i) continue;
            for (int c = -ctx; c <= ctx; ++c) {
                if (c == 0) continue;
                const int h2 = pm_slot(s, dir, id + (uint32_t)c);
                if (h2 >= 0 && at[dir][h2] < i) {
                    if (atomicMin(&at[dir][h], i) > i) changed = true;
                    break;
                }
            }
        }
        __syncwarp();
        settled = !__any_sync(FULL, changed);
    }
    if (!settled) return -1;
    // C: counts (raw, folded below), then the inserts in op order
    for (uint32_t i = lane; i < sigma; i += 32) {
        if (!(s.sv[i] & 1)) continue;
        const uint32_t e = s.ge[i];
        const int dir = (int)(e >> 31);
        const int h = pm_slot(s, dir, e & 0x7fffffffu);
        if (h < 0) continue;
        if ((s.vv[dir][h] & PV_PRESENT) || at[dir][h] <= i) atomicAdd(&s.vv[dir][h], 1u << PV_RAW_SHIFT);
    }
    __syncwarp();
    uint32_t nins[2] = {0, 0};
    bool over = false;
    for (uint32_t base = 0; base < sigma; base += 32) {
        const uint32_t i = base + lane;
        bool fresh = false;
        int dir = 0;
        uint32_t id = 0;
        if (i < sigma && (s.sv[i] & 1)) {
            const uint32_t e = s.ge[i];
            dir = (int)(e >> 31);
            id = e & 0x7fffffffu;
            const int h = pm_slot(s, dir, id);
            fresh = h >= 0 && at[dir][h] == i;
        }
        for (int d = 0; d < 2; ++d) {
            const unsigned bm = __ballot_sync(FULL, fresh && dir == d);
            if (fresh && dir == d) {
                const uint32_t a = nins[d] + __popc(bm & ((1u << lane) - 1));
                if (a < s.c.icap) s.ins2[d][a] = id;
            }
            nins[d] += __popc(bm);
        }
        if (nins[0] > s.c.icap || nins[1] > s.c.icap) over = true;
    }
    __syncwarp();
    if (over) return -1;
    for (uint32_t i = lane; i < sigma; i += 32) {   // the inserted keys become present
        if (!(s.sv[i] & 1)) continue;
        const uint32_t e = s.ge[i];
        const int dir = (int)(e >> 31);
        const int h = pm_slot(s, dir, e & 0x7fffffffu);
        if (h >= 0 && at[dir][h] == i) atomicOr(&s.vv[dir][h], PV_PRESENT);
    }
    __syncwarp();
    // fold the op counts into count2 (8-bit wrap) and clear the scratch bits
    for (int dir = 0; dir < 2; ++dir)
        for (uint32_t x = lane; x < nkeys[dir]; x += 32) {
            const uint32_t h = s.occ[dir][x];
            const uint32_t v = s.vv[dir][h];
            const uint32_t raw = ((v & PV_RAW_MASK) >> PV_RAW_SHIFT) & 0xffu;
            const uint32_t base_v = v & ~(PV_RAW_MASK | PV_SEEN);
            s.vv[dir][h] = (base_v & PV_PRESENT) ? ((base_v & ~0xff00u) | (raw << 8)) : base_v;
        }
    __syncwarp();
    for (int d = 0; d < 2; ++d) {
        st.nkeys[d] = nkeys[d];
        st.n2[d] = nins[d];
    }
    return 1;
}

// ---------------------------------------------------------------------------
// lane 0: map operations of one mate (getSeedRefsFirstRead / SecondRead)
// ---------------------------------------------------------------------------
__device__ void pe_count_first(const DevIndex& ix, const PeIndex& px, const PeMem& s, PeState& st, uint32_t len,
                               bool staged)
{
    const uint32_t nk = len - KMERLEN + 1;
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    for (uint32_t p = 0; p < nk && !st.over; ++p) {
        if (s.kfl[p]) continue;
        const uint32_t n = s.kln[p], cm = s.kcm[p];
        const uint32_t b0 = staged ? s.kpre[p] : s.kst[p];
        const uint32_t* E = staged ? s.ge : ix.entry;
        const uint32_t* TM = staged ? s.gt : px.tmask;
        bool have = false;
        uint32_t lastId = 0, lastFwd = 0;
        for (uint32_t i = b0; i < b0 + n; ++i) {
            if (cm & SEEDBITS & TM[i]) continue;
            const uint32_t e = E[i];
            const uint32_t id = e & 0x7fffffffu, fwd = e >> 31;
            if (have && id == lastId && fwd == lastFwd) continue;
            have = true; lastId = id; lastFwd = fwd;
            int h;
            if (p == 0 || p - 1 < maxQPos) {
                h = pm_at(s, st, (int)fwd, id, 1);
                if (h < 0) return;
            } else {
                h = pm_find(s, (int)fwd, id);
            }
            if (h >= 0) {
                const uint32_t v = s.vv[fwd][h];
                s.vv[fwd][h] = (v & ~0xffu) | ((pv_c1(v) + 1) & 0xffu);
            }
        }
    }
}

__device__ void pe_count_second(const DevIndex& ix, const PeIndex& px, const PeMem& s, PeState& st, uint32_t len,
                                bool staged)
{
    const uint32_t nk = len - KMERLEN + 1;
    const uint32_t maxQPos = len - KMERLEN + 1 - QTHRESH;
    const int ctx = (int)px.ctx;
    for (uint32_t p = 0; p < nk && !st.over; ++p) {
        if (s.kfl[p]) continue;
        const uint32_t n = s.kln[p], cm = s.kcm[p];
        const uint32_t b0 = staged ? s.kpre[p] : s.kst[p];
        const uint32_t* E = staged ? s.ge : ix.entry;
        const uint32_t* TM = staged ? s.gt : px.tmask;
        bool have = false;
        uint32_t lastId = 0, lastFwd = 0;
        for (uint32_t i = b0; i < b0 + n; ++i) {
            if (cm & SEEDBITS & TM[i]) continue;
            const uint32_t e = E[i];
            const uint32_t id = e & 0x7fffffffu, fwd = e >> 31;
            if (have && id == lastId && fwd == lastFwd) continue;
            have = true; lastId = id; lastFwd = fwd;
            int h = -1;
            if (p == 0 || p - 1 < maxQPos) {
                for (int c = -ctx; c <= ctx; ++c) {
                    if (pm_find(s, (int)fwd, id + (uint32_t)c) >= 0) {
                        h = pm_at(s, st, (int)fwd, id, 2);
                        if (h < 0) return;
                        break;
                    }
                }
            } else {
                h = pm_find(s, (int)fwd, id);
            }
            if (h >= 0) {
                const uint32_t v = s.vv[fwd][h];
                s.vv[fwd][h] = (v & ~0xff00u) | (((pv_c2(v) + 1) & 0xffu) << 8);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// lane 0: one query walk (saQuerySeedSetRefFirst / Second)
// ---------------------------------------------------------------------------
template <int W>
__device__ __noinline__ void pe_walk(const DevIndex& ix, const PeIndex& px, const PeMem& s, PeState& st,
                                     const ChunkBufs& cb, uint32_t r_idx, int orient, int second, uint64_t* hits,
                                     uint32_t& nh)
{
    const uint64_t off0 = cb.offs[r_idx];
    const uint32_t len = (uint32_t)(cb.offs[r_idx + 1] - off0);
    const char* raw = cb.seqs + off0;
    EditScan<W> sa;
    sa.load(raw, len, orient);
    PieceKeys pk;
    pk.load(raw, len, orient);
    const PeCmp cmp{second};
    uint32_t nl[2];
    for (int dir = 0; dir < 2; ++dir) {
        nl[dir] = st.nord[dir];
        for (uint32_t q = 0; q < nl[dir]; ++q) {
            const uint32_t key = s.ord[dir][q];
            const int h = pm_find(s, dir, key);
            s.list[dir][q] = make_uint2(key, h >= 0 ? s.vv[dir][h] : 0u);
        }
        pe_sort(s.list[dir], (long)nl[dir], cmp);
    }
    int order2[2] = {0, 1};
    int nwalk = 0;
    if (nl[1] > 0) {
        if (nl[0] > 0) {
            // both walks compare the heads' count1 (ReadQueue.cpp:2185, 2265)
            if (pv_c1(s.list[1][0].y) > pv_c1(s.list[0][0].y)) { order2[0] = 1; order2[1] = 0; }
            nwalk = 2;
        } else {
            order2[0] = 1;
            nwalk = 1;
        }
    } else if (nl[0] > 0) {
        order2[0] = 0;
        nwalk = 1;
    }
    int32_t bmCount = 0;
    uint32_t prevChr = 0;
    uint64_t prevOff = 0xffffffffffffffffull;
    const int ctx = (int)px.ctx;
    for (int wk = 0; wk < nwalk; ++wk) {
        const int dir = order2[wk];
        if (wk == 1) { prevChr = 0; prevOff = 0xffffffffffffffffull; }
        for (uint32_t q = 0; q < nl[dir]; ++q) {
            const uint2 e = s.list[dir][q];
            const int32_t cnt = (int32_t)(second ? pv_c2(e.y) : pv_c1(e.y));
            const int32_t thr = bmCount - (int32_t)KMERDIST > (int32_t)QTHRESH ? bmCount - (int32_t)KMERDIST : (int32_t)QTHRESH;
            if (cnt < thr) break;
            if (!(e.y & (second ? PV_F3 : PV_F2))) continue;
            const uint32_t w = e.x;
            const uint4 wi = ix.win[w];
            const uint32_t sp = wi.x, ch = wi.y;
            uint32_t n = 0, last = 0;
            scan_window<W>(ix, sa, w, dir, [&](uint32_t off, int err) {
                if (!(n == 0 && (uint64_t)off + sp == prevOff && ch == prevChr)) {
                    if (nh >= s.c.hcap) st.over = true;
                    else hits[nh++] = mk_match(off, (uint32_t)err, (uint64_t)dir, w);
                }
                last = off;
                ++n;
            }, pk.key, pk.valid, pk.q, pk.start, second && dir == 0);
            if (st.over) return;
            if (n > 0) {
                if (cnt > bmCount) bmCount = cnt;
                if (!second) {
                    int h = pm_find(s, dir, w);
                    if (h >= 0) s.vv[dir][h] |= PV_F3;
                    for (int c = 1; c <= ctx; ++c) {
                        h = pm_find(s, dir, w + (uint32_t)c);
                        if (h >= 0) s.vv[dir][h] |= PV_F3;
                        h = pm_find(s, dir, w - (uint32_t)c);
                        if (h >= 0) s.vv[dir][h] |= PV_F3;
                    }
                }
                prevChr = ch;
                prevOff = (uint64_t)sp + last;
            } else {
                prevChr = 0;
                prevOff = 0xffffffffffffffffull;
            }
        }
    }
}

template <int WMAX>
__device__ __forceinline__ void pe_walk_any(const DevIndex& ix, const PeIndex& px, const PeMem& s, PeState& st,
                                            const ChunkBufs& cb, uint32_t r_idx, int orient, int second,
                                            uint64_t* hits, uint32_t& nh)
{
    const uint32_t len = (uint32_t)(cb.offs[r_idx + 1] - cb.offs[r_idx]);
    const int w = (int)(len / 64 + 1);
    if (w == 1 || WMAX == 1) pe_walk<1>(ix, px, s, st, cb, r_idx, orient, second, hits, nh);
    else if (w == 2 || WMAX == 2) pe_walk<(WMAX >= 2 ? 2 : 1)>(ix, px, s, st, cb, r_idx, orient, second, hits, nh);
    else if (w == 3 || WMAX == 3) pe_walk<(WMAX >= 3 ? 3 : 1)>(ix, px, s, st, cb, r_idx, orient, second, hits, nh);
    else pe_walk<(WMAX >= 4 ? 4 : 1)>(ix, px, s, st, cb, r_idx, orient, second, hits, nh);
}

// ---------------------------------------------------------------------------
// one pair (warp); returns false when a cap was exceeded before any output
// ---------------------------------------------------------------------------
__device__ __forceinline__ int pe_extract(const DevIndex& ix, const PeIndex& px, uint64_t m1, uint64_t m2)
{
    const uint4 w1 = ix.win[(uint32_t)(m1 >> 32)], w2 = ix.win[(uint32_t)(m2 >> 32)];
    if (w1.y != w2.y) return -1;
    const uint32_t p1 = w1.x + (uint32_t)(m1 & 0xffffu), p2 = w2.x + (uint32_t)(m2 & 0xffffu);
    const uint32_t d = p2 > p1 ? p2 - p1 : p1 - p2;
    if (d <= px.maxdist) return (int)(((m1 >> 16) & 0xffu) + ((m2 >> 16) & 0xffu));
    return -1;
}

__device__ __forceinline__ void pe_meth(const DevIndex& ix, const ChunkBufs& cb, uint32_t idx, int orient, uint64_t mat)
{
    if (ix.win[(uint32_t)(mat >> 32)].z == CPGDUMMY) return;
    if (((mat >> 16) & 0xffu) == 0) {
        meth_exact(ix, cb, idx, orient, mat);
    } else {
        const uint32_t slot = (uint32_t)atomicAdd(cb.ctr + CTR_DP, 1ull);
        cb.dp_list[slot] = idx;
        cb.dp_mat[slot] = mat;
        cb.dp_orient[slot] = (uint8_t)orient;
    }
}

// Writes the oriented mate into rd: orient 0 as read, 1 reverse complement.
__device__ __forceinline__ void pe_orient(uint8_t* rd, const char* raw, uint32_t len, int orient)
{
    const int lane = threadIdx.x & 31;
    for (uint32_t p = lane; p < len; p += 32) rd[p] = oriented_char(raw, len, orient, p);
}

// The pair choice of matchPairedReads (ReadQueue.cpp:1300-1638): the best
// summed error count over the matches of both orientations within the pair
// distance (extractPairedMatch), non-unique on a tie; CpG calls of a chosen
// pair; counters; the mates' outputs.
__device__ void pe_choose(const DevIndex& ix, const PeIndex& px, const ChunkBufs& cb, uint32_t i1, uint32_t i2,
                          const uint64_t* m1F, uint32_t n1F, const uint64_t* m2R, uint32_t n2R, const uint64_t* m1R,
                          uint32_t n1R, const uint64_t* m2F, uint32_t n2F)
{
    const uint32_t nh[4] = {n1F, n2R, n1R, n2F};
    uint64_t mat1 = 0, mat2 = 0;
    bool ok = false;
    if ((nh[0] == 0 && nh[2] == 0) || (nh[1] == 0 && nh[3] == 0)) {
        atomicAdd(cb.ctr + CTR_UNSUCC, 2ull);
    } else {
        const int WORST = 2 * (int)(MISCOUNT + ADDMIS) + 1;
        int best = WORST;
        bool nonUnique = false, orig = true;
        uint64_t b1 = 0, b2 = 0;
        if (cb.orient_mask & 1u)
            for (uint32_t a = 0; a < nh[0]; ++a)
                for (uint32_t b = 0; b < nh[1]; ++b) {
                    const int e = pe_extract(ix, px, m1F[a], m2R[b]);
                    if (e < 0) continue;
                    if (e == best) nonUnique = true;
                    else if (e < best) { best = e; b1 = m1F[a]; b2 = m2R[b]; nonUnique = false; }
                }
        if (cb.orient_mask & 2u)
            for (uint32_t a = 0; a < nh[2]; ++a)
                for (uint32_t b = 0; b < nh[3]; ++b) {
                    const int e = pe_extract(ix, px, m1R[a], m2F[b]);
                    if (e < 0) continue;
                    if (e == best) nonUnique = true;
                    else if (e < best) { best = e; b1 = m1R[a]; b2 = m2F[b]; orig = false; nonUnique = false; }
                }
        if (best == WORST) {
            atomicAdd(cb.ctr + CTR_UNSUCC, 2ull);
        } else if (nonUnique) {
            atomicAdd(cb.ctr + CTR_NONU, 2ull);
        } else {
            ok = true;
            mat1 = b1;
            mat2 = b2;
            if (cb.stranded) atomicAdd(cb.ctr + (orig ? CTR_R1F : CTR_R1R), 1ull);
            pe_meth(ix, cb, i1, orig ? 0 : 1, b1);
            pe_meth(ix, cb, i2, orig ? 1 : 0, b2);
            const bool d1 = ix.win[(uint32_t)(b1 >> 32)].z == CPGDUMMY, d2 = ix.win[(uint32_t)(b2 >> 32)].z == CPGDUMMY;
            if (d1 && d2) atomicAdd(cb.ctr + CTR_TOOSHORT, 2ull);
            else if (d1 || d2) { atomicAdd(cb.ctr + CTR_TOOSHORT, 1ull); atomicAdd(cb.ctr + CTR_SUCC, 1ull); }
            else { atomicAdd(cb.ctr + CTR_PAIRED, 1ull); atomicAdd(cb.ctr + CTR_SUCC, 2ull); }
        }
    }
    cb.mats[i1] = ok ? mat1 : 0;
    cb.mats[i2] = ok ? mat2 : 0;
    cb.invalid[i1] = ok ? 0 : 1;
    cb.invalid[i2] = ok ? 0 : 1;
}

// One orientation of a pair, all lanes: both maps, the f2 flags, hasCpG and
// the final iteration orders (s.ord, st.nord).  Returns 1 when there is
// something to walk, 0 when not, -1 when a capacity was exceeded.
__device__ int pe_maps(const DevIndex& ix, const PeIndex& px, const ChunkBufs& cb, const PeMem& s, uint32_t i1,
                       uint32_t i2, uint32_t n1, uint32_t n2, int o, PeState& st)
{
    const int lane = threadIdx.x & 31;
    st = PeState{};
    // first = mate 1 (o = 0) or its reverse complement; second = the other strand of mate 2
    pe_orient(s.rd[0], cb.seqs + cb.offs[i1], n1, o);
    pe_orient(s.rd[1], cb.seqs + cb.offs[i2], n2, 1 - o);
    __syncwarp();
    for (int dir = 0; dir < 2; ++dir) {   // the slots the previous pair occupied
        const uint32_t no = s.occn[dir];
        for (uint32_t x = lane; x < no; x += 32) {
            const uint32_t h = s.occ[dir][x];
            s.vk[dir][h] = EMPTY_KEY;
            s.vv[dir][h] = 0;
        }
    }
    __syncwarp();
    if (lane == 0) {
        s.occn[0] = 0;
        s.occn[1] = 0;
    }
    __syncwarp();
    const uint32_t sigma = pe_kmers(ix, px, s, s.rd[0], n1);
    if (sigma <= s.c.ecap) {
        if (pe_count_par(px, s, st, n1, sigma) < 0) return -1;
    } else if (lane == 0) {
        pe_count_first(ix, px, s, st, n1, false);
    }
    if (__shfl_sync(0xffffffffu, st.over, 0)) return -1;
    __syncwarp();
    // rebuild: keep count1 >= QTHRESH (order-independent)
    for (int dir = 0; dir < 2; ++dir)
        for (uint32_t x = lane; x < s.occn[dir]; x += 32) {
            const uint32_t h = s.occ[dir][x];
            const uint32_t v = s.vv[dir][h];
            if (!(v & PV_PRESENT)) continue;
            s.vv[dir][h] = pv_c1(v) < QTHRESH ? 0u : (PV_PRESENT | pv_c1(v));
        }
    __syncwarp();
    bool any = false;
    for (int dir = 0; dir < 2; ++dir) {
        const uint32_t n1d = __shfl_sync(0xffffffffu, st.n1[dir], 0);   // lane 0's, after any ordered counting
        for (uint32_t x = lane; x < n1d && !any; x += 32) any = pm_find(s, dir, s.ins1[dir][x]) >= 0;
    }
    if (!__any_sync(0xffffffffu, any)) return 0;
    __syncwarp();
    const uint32_t sigma2 = pe_kmers(ix, px, s, s.rd[1], n2);
    int par2 = 0;
    // the lane-parallel count keeps two vcap-slot arrays in regions 11 .. 16
    if (sigma2 <= s.c.ecap && 2 * s.c.vcap * 4 <= s.area) par2 = pe_count_par2(px, s, st, n2, sigma2);
    if (par2 < 0) return -1;
    if (par2 == 0 && lane == 0) pe_count_second(ix, px, s, st, n2, sigma2 <= s.c.ecap);
    if (__shfl_sync(0xffffffffu, st.over, 0)) return -1;
    __syncwarp();
    // f2 flags (order-independent: flags are only set) and hasCpG, lanes over the table slots
    {
        const int ctx = (int)px.ctx;
        for (int dir = 0; dir < 2; ++dir)
            for (uint32_t x = lane; x < s.occn[dir]; x += 32) {
                const uint32_t hh = s.occ[dir][x];
                const uint32_t v = s.vv[dir][hh];
                const uint32_t key = s.vk[dir][hh];
                if (key == EMPTY_KEY || !(v & PV_PRESENT) || pv_c2(v) < QTHRESH) continue;
                atomicOr(&s.vv[dir][hh], PV_F2);
                for (int c = 1; c <= ctx; ++c) {
                    int h2 = pm_find(s, dir, key + (uint32_t)c);
                    if (h2 >= 0) atomicOr(&s.vv[dir][h2], PV_F2);
                    h2 = pm_find(s, dir, key - (uint32_t)c);
                    if (h2 >= 0) atomicOr(&s.vv[dir][h2], PV_F2);
                }
            }
    }
    __syncwarp();
    bool mine = false;
    for (int dir = 0; dir < 2; ++dir)
        for (uint32_t x = lane; x < s.occn[dir]; x += 32) {
            const uint32_t hh = s.occ[dir][x];
            const uint32_t v = s.vv[dir][hh];
            const uint32_t key = s.vk[dir][hh];
            mine |= key != EMPTY_KEY && (v & PV_PRESENT) && (v & PV_F2) && ix.win[key].z != CPGDUMMY;
        }
    if (!__any_sync(0xffffffffu, mine)) return 0;
    // Final iteration orders: the replay of the first map, its kept keys, then the second
    // mate's insertions.  The walks scan only keys with count >= QTHRESH (count1 in the
    // first, count2 in the second), and a strand map with at most one such key in both
    // counts puts it first after either sort whatever the order of the others, so then
    // no replay is needed: the kept keys in first-touch order, then the second mate's
    // insertions, taken lane-parallel with ballots.  (The insertion counts of lane 0,
    // which ran any ordered counting, hold for the warp.)
    constexpr uint32_t FULL = 0xffffffffu;
    uint32_t n1d[2], n2d[2];
    for (int dir = 0; dir < 2; ++dir) {
        n1d[dir] = __shfl_sync(FULL, st.n1[dir], 0);
        n2d[dir] = __shfl_sync(FULL, st.n2[dir], 0);
    }
    bool need = false;
    for (int dir = 0; dir < 2; ++dir) {
        uint32_t c1 = 0, c2 = 0;
        for (uint32_t x = lane; x < n1d[dir]; x += 32) {
            const int h = pm_find(s, dir, s.ins1[dir][x]);
            if (h >= 0) { c1 += pv_c1(s.vv[dir][h]) >= QTHRESH; c2 += pv_c2(s.vv[dir][h]) >= QTHRESH; }
        }
        for (uint32_t x = lane; x < n2d[dir]; x += 32) {
            const int h = pm_find(s, dir, s.ins2[dir][x]);
            if (h >= 0) c2 += pv_c2(s.vv[dir][h]) >= QTHRESH;
        }
        c1 = __reduce_add_sync(FULL, c1);
        c2 = __reduce_add_sync(FULL, c2);
        need |= c1 > 1 || c2 > 1;
    }
    if (!need) {
        for (int dir = 0; dir < 2; ++dir) {
            uint32_t ns = 0;
            for (uint32_t b0 = 0; b0 < n1d[dir]; b0 += 32) {
                const uint32_t x = b0 + lane;
                bool keep = false;
                uint32_t key = 0;
                if (x < n1d[dir]) {
                    key = s.ins1[dir][x];
                    const int h = pm_find(s, dir, key);
                    keep = h >= 0 && pv_c1(s.vv[dir][h]) >= QTHRESH;
                }
                const uint32_t bm = __ballot_sync(FULL, keep);
                if (keep) s.ord[dir][ns + __popc(bm & ((1u << lane) - 1))] = key;
                ns += __popc(bm);
            }
            for (uint32_t x = lane; x < n2d[dir]; x += 32) s.ord[dir][ns + x] = s.ins2[dir][x];
            st.nord[dir] = ns + n2d[dir];
        }
        __syncwarp();
        return 1;
    }
    // a strand map with two or more keys to scan: replay its insertions (the warp)
    bool over = false;
    for (int dir = 0; dir < 2 && !over; ++dir) {
        uint32_t nt = 0;
        if (!pe_replay_w(s, s.ins1[dir], n1d[dir], sigma / 5, s.ord[dir], nt)) { over = true; break; }
        // kept keys are present with count1 >= QTHRESH; keys the second mate re-inserted
        // after the rebuild dropped them come later, from ins2
        uint32_t ns = 0;
        for (uint32_t b0 = 0; b0 < nt; b0 += 32) {
            const uint32_t q = b0 + lane;
            bool keep = false;
            uint32_t key = 0;
            if (q < nt) {
                key = s.ord[dir][q];
                const int h = pm_find(s, dir, key);
                keep = h >= 0 && pv_c1(s.vv[dir][h]) >= QTHRESH;
            }
            const unsigned bm = __ballot_sync(FULL, keep);
            if (keep) s.seq[ns + __popc(bm & ((1u << lane) - 1))] = key;
            ns += __popc(bm);
        }
        for (uint32_t x = lane; x < n2d[dir]; x += 32) s.seq[ns + x] = s.ins2[dir][x];
        ns += n2d[dir];
        __syncwarp();
        uint32_t no = 0;
        if (!pe_replay_w(s, s.seq, ns, 20, s.ord[dir], no)) { over = true; break; }
        if (lane == 0) st.nord[dir] = no;
    }
    if (over) {
        if (lane == 0) st.over = true;
        return -1;
    }
    __syncwarp();
    return 1;
}

template <int WMAX>
__device__ bool pe_pair(const DevIndex& ix, const PeIndex& px, const ChunkBufs& cb, const PeMem& s, uint32_t r)
{
    const int lane = threadIdx.x & 31;
    const uint32_t n = cb.n;                 // pairs; mate 2 of pair r is read n + r
    const uint32_t i1 = r, i2 = n + r;
    const uint32_t n1 = (uint32_t)(cb.offs[i1 + 1] - cb.offs[i1]);
    const uint32_t n2 = (uint32_t)(cb.offs[i2 + 1] - cb.offs[i2]);
    uint32_t nh[4] = {0, 0, 0, 0};
    // mates were validated by k_pe_prep: rflags bit0 length, bit1 non-ACGT
    const uint8_t f1 = cb.rflags[i1], f2 = cb.rflags[i2];
    if ((f1 | f2) & 3u) return true;     // counted and written by k_pe_prep
    for (int o = 0; o < 2; ++o) {
        if (!((cb.orient_mask >> o) & 1u)) continue;
        PeState st;
        const int m = pe_maps(ix, px, cb, s, i1, i2, n1, n2, o, st);
        if (m < 0) return false;
        if (m == 0) continue;
        if (lane == 0) {
            uint64_t* ha = s.hits[o == 0 ? 0 : 2];
            uint64_t* hb = s.hits[o == 0 ? 1 : 3];
            pe_walk_any<WMAX>(ix, px, s, st, cb, i1, o, 0, ha, nh[o == 0 ? 0 : 2]);
            if (!st.over && nh[o == 0 ? 0 : 2] > 0)
                pe_walk_any<WMAX>(ix, px, s, st, cb, i2, 1 - o, 1, hb, nh[o == 0 ? 1 : 3]);
        }
        if (__shfl_sync(0xffffffffu, st.over, 0)) return false;
        __syncwarp();
    }
    if (lane == 0) pe_choose(ix, px, cb, i1, i2, s.hits[0], nh[0], s.hits[1], nh[1], s.hits[2], nh[2], s.hits[3], nh[3]);
    __syncwarp();
    return true;
}

// Mate checks of every pair (matchPairedReads, ReadQueue.cpp:968-1080): a mate
// shorter than ceil(0.75 * READLEN) or with a letter other than ACGT is
// invalid.  Pairs with an invalid mate are finished here: tooShort grows by 1
// for a short mate and by 2 more for any invalid pair (the reference's
// counting).  Sets CTR_WMASK bit W for the automaton width of valid pairs.
__global__ void k_pe_prep(ChunkBufs cb, uint32_t readlen)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= cb.n) return;
    const float minlen = ceilf((float)readlen * 0.75f);
    uint32_t wmax = 0;
    uint8_t f[2];
    for (int m = 0; m < 2; ++m) {
        const uint32_t i = m == 0 ? r : cb.n + r;
        const uint64_t o0 = cb.offs[i];
        const uint32_t len = (uint32_t)(cb.offs[i + 1] - o0);
        uint8_t fl = 0;
        if ((float)len < minlen) fl |= 1;
        if (len > FAME_MAX_READ_LEN) fl |= 4;
        for (uint32_t p = 0; p < len && !(fl & 2); ++p) {
            const char c = cb.seqs[o0 + p];
            if (c != 'A' && c != 'C' && c != 'G' && c != 'T') fl |= 2;
        }
        f[m] = fl;
        cb.rflags[i] = fl;
        wmax = max(wmax, len / 64 + 1);
    }
    const uint32_t i2 = cb.n + r;
    // a mate longer than the widest automaton fails the whole call on the host
    if ((f[0] | f[1]) & 4) atomicAdd(cb.ctr + CTR_TOO_LONG, 1ull);
    if ((f[0] | f[1]) & 7) {
        unsigned long long ts = 0;
        if ((f[0] | f[1]) & 1) ts += 1;
        ts += 2;
        atomicAdd(cb.ctr + CTR_TOOSHORT, ts);
        cb.mats[r] = 0;
        cb.mats[i2] = 0;
        cb.invalid[r] = (f[0] & 7) ? 1 : 0;
        cb.invalid[i2] = (f[1] & 7) ? 1 : 0;
        return;
    }
    atomicOr(cb.ctr + CTR_WMASK, 1ull << wmax);
}

// Pairs the pipelined path hands over: the whole per-pair path (pe_pair) with
// large capacities in global scratch.
__global__ void k_pe_heavy(DevIndex ix, PeIndex px, ChunkBufs cb, uint8_t* scratch, uint64_t warp_bytes, PeCaps caps)
{
    const int lane = threadIdx.x & 31;
    const uint32_t wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    const PeMem s = pe_mem(scratch + (uint64_t)wid * warp_bytes, caps);
    const uint32_t nheavy = (uint32_t)cb.ctr[CTR_HEAVY];
    for (uint32_t k = wid; k < nheavy; k += nw) {
        if (k == wid) pe_tables_reset(s);   // the warp's first pair
        const uint32_t r = cb.heavy[k];
        if (!pe_pair<4>(ix, px, cb, s, r)) {
            if (lane == 0) atomicAdd(cb.ctr + CTR_ERRFLAG, 1ull);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Pipelined paired path.  The walks' window scans leave the pair's warp and
// run like the single-end scans, one thread per candidate window:
//   A  k_pe_seed   warp per pair: both orientations' maps (pe_maps), the walk
//                  lists sorted as the walks sort them and cut to the keys whose
//                  count reaches QTHRESH, and the first walk's candidates
//                  (f2-flagged keys; the walk's dynamic threshold
//                  max(bmCount - KMERDIST, QTHRESH) only removes keys, so these
//                  are a superset of what it scans)
//   B  k_shiftand  the first walk's candidates (pattern: the first mate)
//   C  k_pe_walk1  thread per pair orientation: the first walk over the scan
//                  results, its matches, the f3 flags (windows within
//                  contextWLen of a window with hits) and the second walk's
//                  candidates (f3-flagged keys)
//   D  k_shiftand  the second walk's candidates (the second mate, reverse
//                  windows from startPos - 1)
//   E  k_pe_finish thread per pair: the second walks, the pair choice, CpG calls
// A pair that exceeds a list or match capacity, or whose window has more hit
// runs than the scan keeps, is handed whole to k_pe_heavy (the full per-pair
// path above); nothing of it is written before that.
// ---------------------------------------------------------------------------
constexpr int PE_CAPL = 8;    // keys of one walk list and strand
constexpr int PE_HCAP = 32;   // matches of one mate and orientation
constexpr uint32_t PT_NONE = 0, PT_WALK = 1, PT_FALLBACK = 2;
constexpr uint32_t NO_CAND = 0xffffffffu;

struct PeTaskRec {            // one pair orientation
    uint32_t state;
    uint32_t m1n;             // matches of the first walk
    uint8_t n1[2], n2[2];     // keys of the walk lists per strand
    uint32_t pad;
    uint4 w1[2][PE_CAPL];     // {key, count1 | count2 << 8 | f2 << 16, candidate, -}
    uint4 w2[2][PE_CAPL];     // {key, count1 | count2 << 8, candidate, f3}
    uint64_t m1[PE_HCAP];
};

// Stage A, lane 0: the walk lists of one orientation and its first-walk candidates.
// lane 0: sort one strand list and keep its keys with count >= QTHRESH
__device__ bool pe_list_cut(const PeMem& s, PeTaskRec& t, int dir, uint32_t nl, int second, const PeCmp& cmp)
{
    pe_sort(s.list[dir], (long)nl, cmp);
    uint32_t k = 0;
    for (uint32_t q = 0; q < nl; ++q) {
        const uint32_t v = s.list[dir][q].y;
        if ((second ? pv_c2(v) : pv_c1(v)) < QTHRESH) break;   // counts sorted descending
        if (k >= (uint32_t)PE_CAPL) return false;
        const uint32_t cnts = pv_c1(v) | (pv_c2(v) << 8);
        if (second) t.w2[dir][k] = make_uint4(s.list[dir][q].x, cnts, NO_CAND, 0);
        else t.w1[dir][k] = make_uint4(s.list[dir][q].x, cnts | ((v & PV_F2) ? 1u << 16 : 0u), NO_CAND, 0);
        ++k;
    }
    if (second) t.n2[dir] = (uint8_t)k;
    else t.n1[dir] = (uint8_t)k;
    return true;
}

// lane 0: the first walk's f2-flagged keys become scan candidates
__device__ void pe_first_candidates(const ChunkBufs& cb, PeTaskRec& t, uint32_t i1, int o)
{
    for (int dir = 0; dir < 2; ++dir)
        for (uint32_t k = 0; k < t.n1[dir]; ++k) {
            if (!((t.w1[dir][k].y >> 16) & 1u)) continue;
            const uint32_t ci = (uint32_t)atomicAdd(cb.ctr + CTR_CAND, 1ull);
            if (ci < cb.cand_cap) {
                cb.cand[ci] = t.w1[dir][k].x | ((uint32_t)dir << 31);
                cb.cand_task[ci] = (i1 << 1) | (uint32_t)o;
                cb.cand_flags[ci] = 0;
            }
            t.w1[dir][k].z = ci;
        }
}

// The walk lists of one pair orientation (all lanes call it; lane 0's result):
// each strand's keys in iteration order with their values, sorted by count1
// (first walk) or count2 (second walk) with the libstdc++ introsort on lane 0,
// cut at QTHRESH.
__device__ bool pe_lists(const PeMem& s, const PeState& st, const ChunkBufs& cb, PeTaskRec& t, uint32_t i1, int o)
{
    const int lane = threadIdx.x & 31;
    bool ok = true;
    for (int second = 0; second < 2; ++second) {
        const PeCmp cmp{second};
        for (int dir = 0; dir < 2; ++dir) {
            const uint32_t nl = __shfl_sync(0xffffffffu, st.nord[dir], 0);
            for (uint32_t q = lane; q < nl; q += 32) {
                const uint32_t key = s.ord[dir][q];
                const int h = pm_find(s, dir, key);
                s.list[dir][q] = make_uint2(key, h >= 0 ? s.vv[dir][h] : 0u);
            }
            __syncwarp();
            if (lane == 0 && ok) ok = pe_list_cut(s, t, dir, nl, second, cmp);
            __syncwarp();
        }
    }
    if (!__shfl_sync(0xffffffffu, ok ? 1 : 0, 0)) return false;
    if (lane == 0) pe_first_candidates(cb, t, i1, o);
    __syncwarp();
    return true;
}

// Stage A of pair r, both orientations: maps, walk lists and the first walk's
// candidates.  Returns true when a capacity of `caps` is exceeded (the pair
// must then be done by another tier; what was written for it is reset or
// overwritten there).  All lanes of the warp call it.
__device__ bool pe_seed_pair(const DevIndex& ix, const PeIndex& px, const ChunkBufs& cb, PeTaskRec* recs,
                             const PeMem& s, const PeCaps& caps, uint32_t r)
{
    const int lane = threadIdx.x & 31;
    const uint32_t n = cb.n;
    const uint32_t i1 = r, i2 = n + r;
    const uint32_t n1 = (uint32_t)(cb.offs[i1 + 1] - cb.offs[i1]);
    const uint32_t n2 = (uint32_t)(cb.offs[i2 + 1] - cb.offs[i2]);
    bool fb = n1 > caps.kmax + KMERLEN - 1 || n2 > caps.kmax + KMERLEN - 1;   // over the k-mer arrays
    for (int o = 0; o < 2 && !fb; ++o) {
        if (!((cb.orient_mask >> o) & 1u)) continue;
        PeState st;
        const int m = pe_maps(ix, px, cb, s, i1, i2, n1, n2, o, st);
        if (m < 0) { fb = true; break; }
        if (m == 0) continue;
        PeTaskRec& t = recs[2 * r + o];
        const bool ok = pe_lists(s, st, cb, t, i1, o);
        if (lane == 0) t.state = ok ? PT_WALK : PT_FALLBACK;
        fb = !ok;
        __syncwarp();
    }
    return fb;
}

__device__ __forceinline__ void pe_rec_reset(PeTaskRec* recs, uint32_t r)
{
    for (int o = 0; o < 2; ++o) {
        recs[2 * r + o].state = PT_NONE;
        recs[2 * r + o].m1n = 0;
        recs[2 * r + o].n1[0] = recs[2 * r + o].n1[1] = 0;
        recs[2 * r + o].n2[0] = recs[2 * r + o].n2[1] = 0;
    }
}

// Stage A in shared memory, warp per pair.  A pair over the shared-memory caps
// goes to the paired middle tier's list (cb.heavy2, counter CTR_HEAVY2); with
// route_mid every valid pair goes there at once (genome-scale indexes, where
// nearly every pair is over these caps and the attempt would only repeat its
// bucket reads).
__global__ void k_pe_seed(DevIndex ix, PeIndex px, ChunkBufs cb, PeTaskRec* recs, uint32_t warp_bytes, PeCaps caps,
                          int route_mid)
{
    extern __shared__ __align__(16) uint8_t smem[];
    const int lane = threadIdx.x & 31;
    const uint32_t wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const uint32_t nw = gridDim.x * (blockDim.x >> 5);
    const PeMem s = pe_mem(smem + (threadIdx.x >> 5) * warp_bytes, caps);
    const uint32_t n = cb.n;
    if (!route_mid && wid < n) pe_tables_reset(s);
    for (uint32_t r = wid; r < n; r += nw) {
        if (lane == 0) pe_rec_reset(recs, r);
        if ((cb.rflags[r] | cb.rflags[n + r]) & 7u) continue;   // k_pe_prep finished the pair
        const bool over = route_mid ? true : pe_seed_pair(ix, px, cb, recs, s, caps, r);
        if (over && lane == 0) {
            pe_rec_reset(recs, r);
            cb.heavy2[(uint32_t)atomicAdd(cb.ctr + CTR_HEAVY2, 1ull)] = r;
        }
        __syncwarp();
    }
}

// Stage A of a paired middle tier: the pairs of `list` (its length in counter
// ctr_in) with the caps of a genome-scale index, working memory in global
// scratch (warp_bytes per warp), warp per pair, pairs taken from a work queue
// (counter ctr_q).  A pair over these caps goes to `spill` (counter
// ctr_spill) for the next tier, or, without one, is marked for the per-pair
// path (k_pe_heavy).
__global__ void k_pe_seed_mid(DevIndex ix, PeIndex px, ChunkBufs cb, PeTaskRec* recs, uint8_t* scratch,
                              uint64_t warp_bytes, PeCaps caps, const uint32_t* list, int ctr_in, int ctr_q,
                              uint32_t* spill, int ctr_spill)
{
    const int lane = threadIdx.x & 31;
    const uint32_t wid = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const PeMem s = pe_mem(scratch + (uint64_t)wid * warp_bytes, caps);
    const uint32_t npairs = (uint32_t)cb.ctr[ctr_in];
    bool first = true;
    while (true) {
        uint32_t k = 0;
        if (lane == 0) k = (uint32_t)atomicAdd(cb.ctr + ctr_q, 1ull);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= npairs) break;
        if (first) pe_tables_reset(s);   // the warp's first pair
        first = false;
        const uint32_t r = list[k];
        const bool over = pe_seed_pair(ix, px, cb, recs, s, caps, r);
        if (over && lane == 0) {
            if (spill) {
                pe_rec_reset(recs, r);
                spill[(uint32_t)atomicAdd(cb.ctr + ctr_spill, 1ull)] = r;
            } else {
                recs[2 * r].state = PT_FALLBACK;
                recs[2 * r + 1].state = PT_FALLBACK;
            }
        }
        __syncwarp();
    }
}

// Walk order of two strand lists: the heads' count1 decide when both have keys
// to scan (ReadQueue.cpp:2185, 2265); with one list empty the order changes nothing.
__device__ __forceinline__ void pe_walk_order(uint32_t n0, uint32_t n1, uint32_t head0_c1, uint32_t head1_c1, int* order)
{
    order[0] = 0;
    order[1] = 1;
    if (n0 > 0 && n1 > 0 && head1_c1 > head0_c1) { order[0] = 1; order[1] = 0; }
}

// Stage C: the first walk of one pair orientation.
__global__ void k_pe_walk1(DevIndex ix, PeIndex px, ChunkBufs cb, PeTaskRec* recs)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 2 * cb.n) return;
    PeTaskRec& rec = recs[t];
    if (rec.state != PT_WALK) return;
    const uint32_t r = t >> 1;
    const int o = (int)(t & 1);
    int order[2];
    pe_walk_order(rec.n1[0], rec.n1[1], rec.w1[0][0].y & 0xffu, rec.w1[1][0].y & 0xffu, order);
    int32_t bmCount = 0;
    uint32_t prevChr = 0;
    uint64_t prevOff = 0xffffffffffffffffull;
    uint32_t m1n = 0;
    uint32_t hitwin[2][PE_CAPL];
    uint32_t nhw[2] = {0, 0};
    for (int wk = 0; wk < 2; ++wk) {
        const int dir = order[wk];
        if (wk == 1) { prevChr = 0; prevOff = 0xffffffffffffffffull; }
        for (uint32_t k = 0; k < rec.n1[dir]; ++k) {
            const uint4 e = rec.w1[dir][k];
            const int32_t cnt = (int32_t)(e.y & 0xffu);
            const int32_t thr = bmCount - (int32_t)KMERDIST > (int32_t)QTHRESH ? bmCount - (int32_t)KMERDIST : (int32_t)QTHRESH;
            if (cnt < thr) break;
            if (!((e.y >> 16) & 1u)) continue;
            const uint32_t c = e.z, w = e.x;
            const uint32_t nh = cb.hit_n[c];
            if (nh > (uint32_t)HIT_CAP) { rec.state = PT_FALLBACK; return; }
            const uint4 wi = ix.win[w];
            const uint32_t sp = wi.x, ch = wi.y;
            uint32_t last = 0;
            for (uint32_t i = 0; i < nh; ++i) {
                const uint32_t h = cb.hits[(uint64_t)c * HIT_CAP + i];
                const uint32_t off = h >> 8, err = h & 0xffu;
                if (!(i == 0 && (uint64_t)off + sp == prevOff && ch == prevChr)) {
                    if (m1n >= (uint32_t)PE_HCAP) { rec.state = PT_FALLBACK; return; }
                    rec.m1[m1n++] = mk_match(off, err, (uint64_t)dir, w);
                }
                last = off;
            }
            if (nh > 0) {
                if (cnt > bmCount) bmCount = cnt;
                hitwin[dir][nhw[dir]++] = w;
                prevChr = ch;
                prevOff = (uint64_t)sp + last;
            } else {
                prevChr = 0;
                prevOff = 0xffffffffffffffffull;
            }
        }
    }
    rec.m1n = m1n;
    if (m1n == 0) return;
    // f3: the first walk flags each window with hits and its neighbours within contextWLen
    const uint32_t ctx = px.ctx;
    for (int dir = 0; dir < 2; ++dir)
        for (uint32_t k = 0; k < rec.n2[dir]; ++k) {
            const uint32_t key = rec.w2[dir][k].x;
            bool f3 = false;
            for (uint32_t h = 0; h < nhw[dir] && !f3; ++h)
                for (uint32_t c = 0; c <= ctx && !f3; ++c)
                    f3 = key == hitwin[dir][h] + c || key == hitwin[dir][h] - c;
            rec.w2[dir][k].w = f3 ? 1u : 0u;
            if (!f3) continue;
            const uint32_t ci = (uint32_t)atomicAdd(cb.ctr + CTR_CAND, 1ull);
            if (ci < cb.cand_cap) {
                cb.cand[ci] = key | ((uint32_t)dir << 31);
                cb.cand_task[ci] = ((cb.n + r) << 1) | (uint32_t)(1 - o);
                cb.cand_flags[ci] = dir == 0 ? 1 : 0;                        // matchRevSecond's unguarded start
            }
            rec.w2[dir][k].z = ci;
        }
}

// Stage E: the second walks of both orientations and the pair choice.
__global__ void k_pe_finish(DevIndex ix, PeIndex px, ChunkBufs cb, PeTaskRec* recs)
{
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = cb.n;
    if (r >= n) return;
    if ((cb.rflags[r] | cb.rflags[n + r]) & 7u) return;       // k_pe_prep finished the pair
    if (recs[2 * r].state == PT_FALLBACK || recs[2 * r + 1].state == PT_FALLBACK) {
        const uint32_t k = (uint32_t)atomicAdd(cb.ctr + CTR_HEAVY, 1ull);
        cb.heavy[k] = r;
        return;
    }
    uint64_t m2[2][PE_HCAP];
    uint32_t n2c[2] = {0, 0};
    for (int o = 0; o < 2; ++o) {
        const PeTaskRec& rec = recs[2 * r + o];
        if (rec.state != PT_WALK || rec.m1n == 0) continue;
        int order[2];
        pe_walk_order(rec.n2[0], rec.n2[1], rec.w2[0][0].y & 0xffu, rec.w2[1][0].y & 0xffu, order);
        int32_t bmCount = 0;
        uint32_t prevChr = 0;
        uint64_t prevOff = 0xffffffffffffffffull;
        for (int wk = 0; wk < 2; ++wk) {
            const int dir = order[wk];
            if (wk == 1) { prevChr = 0; prevOff = 0xffffffffffffffffull; }
            for (uint32_t k = 0; k < rec.n2[dir]; ++k) {
                const uint4 e = rec.w2[dir][k];
                const int32_t cnt = (int32_t)((e.y >> 8) & 0xffu);
                const int32_t thr = bmCount - (int32_t)KMERDIST > (int32_t)QTHRESH ? bmCount - (int32_t)KMERDIST : (int32_t)QTHRESH;
                if (cnt < thr) break;
                if (!e.w) continue;
                const uint32_t c = e.z, w = e.x;
                const uint32_t nh = cb.hit_n[c];
                const uint4 wi = ix.win[w];
                const uint32_t sp = wi.x, ch = wi.y;
                if (nh > (uint32_t)HIT_CAP) goto fallback;
                uint32_t last = 0;
                for (uint32_t i = 0; i < nh; ++i) {
                    const uint32_t h = cb.hits[(uint64_t)c * HIT_CAP + i];
                    const uint32_t off = h >> 8, err = h & 0xffu;
                    if (!(i == 0 && (uint64_t)off + sp == prevOff && ch == prevChr)) {
                        if (n2c[o] >= (uint32_t)PE_HCAP) goto fallback;
                        m2[o][n2c[o]++] = mk_match(off, err, (uint64_t)dir, w);
                    }
                    last = off;
                }
                if (nh > 0) {
                    if (cnt > bmCount) bmCount = cnt;
                    prevChr = ch;
                    prevOff = (uint64_t)sp + last;
                } else {
                    prevChr = 0;
                    prevOff = 0xffffffffffffffffull;
                }
            }
        }
    }
    {
        const PeTaskRec& a = recs[2 * r];
        const PeTaskRec& b = recs[2 * r + 1];
        pe_choose(ix, px, cb, r, n + r, a.m1, a.state == PT_WALK ? a.m1n : 0, m2[0], n2c[0], b.m1,
                  b.state == PT_WALK ? b.m1n : 0, m2[1], n2c[1]);
    }
    return;
fallback:
    {
        const uint32_t k = (uint32_t)atomicAdd(cb.ctr + CTR_HEAVY, 1ull);
        cb.heavy[k] = r;
    }
}

}  // namespace fame
