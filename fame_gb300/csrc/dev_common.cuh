// Device-side data layout and helpers shared by the matching kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "fame_const.h"

namespace fame {

// The index as it lives in HBM (read-only for the whole context lifetime).
//   rec    : per bucket 32 bytes {start offset (tabIndex), size, its first
//            REC_INLINE entries}, HTABSIZE records: one aligned sector gives a
//            k-mer's bounds and, for buckets of up to REC_INLINE entries (at
//            genome scale nearly every bucket a read's k-mer lands in), all
//            of its entries
//   entry  : one uint32 per k-mer entry: window id | forward-strand << 31
//            (kmerTableSmall.meta with strandTable folded into bit 31; the
//            start-CpG bit the reference reserves there is never set by the
//            window index and is rejected on upload)
//   gpack  : genome, 2 bits per base (A0 C1 G2 T3), 16 bases per word,
//            chromosomes concatenated at 32-base aligned offsets
//   gnmask : one bit per base, set for N
//   win    : {startPos, chrom, startInd, endInd} per window (metaWindows)
constexpr uint32_t REC_INLINE = 6;   // bucket entries held in a dense bucket record
constexpr uint32_t EMPTY_REC_KEY = 0xffffffffu;   // key word of an empty hashed slot

struct DevIndex {
    uint32_t readlen;
    uint32_t n_chrom;
    // bucket records, 32 bytes each, in one of two layouts:
    //  dense (rec_hashed == 0): record k of bucket k, rec[2k] = {start, size,
    //    e0, e1}, rec[2k + 1] = {e2, e3, e4, e5} (the bucket's first
    //    REC_INLINE entries, 0 past its size);
    //  hashed (rec_hashed == 1, small genomes): the non-empty buckets only,
    //    open addressing with linear probing over rec_mask + 1 slots from
    //    rec_slot(k), rec[2h] = {start, size, e0, e1}, rec[2h + 1] = {e2, e3,
    //    e4, k} (five entries inline), an empty slot holding EMPTY_REC_KEY
    //    in its key word.
    // Either way one aligned sector holds a lookup for most buckets.
    const uint4* rec;
    uint32_t rec_mask;
    uint32_t rec_hashed;
    const uint32_t* entry;
    const uint32_t* gpack;
    const uint32_t* gnmask;
    const uint64_t* chrom_off;
    const uint64_t* chrom_len;
    const uint4* win;
    const uint32_t* cpg_pos;
    const uint8_t* cpg_chrom;
    uint64_t n_cpg;
    uint64_t n_win;
};

// Home slot of bucket k in the hashed record layout.
__host__ __device__ __forceinline__ uint32_t rec_slot(uint32_t k, uint32_t mask)
{
    return (k * 0x9E3779B1u) & mask;
}

// Record slot of bucket k and its first half {start, size, e0, e1} (zero for
// an empty bucket); the second half is at rec[2 * slot + 1].
__device__ __forceinline__ uint4 rec_lookup(const DevIndex& ix, uint32_t k, uint32_t& slot)
{
    if (!ix.rec_hashed) {
        slot = k;
        return __ldg(ix.rec + 2ull * k);
    }
    // at most half the slots are used, so a probe ends at the key or at an
    // empty slot well before it has seen the whole table
    uint32_t h = rec_slot(k, ix.rec_mask);
    for (uint32_t i = 0; i <= ix.rec_mask; ++i) {
        const uint32_t sk = __ldg(&ix.rec[2ull * h + 1].w);   // same sector as the first half
        if (sk == k) {
            slot = h;
            return __ldg(ix.rec + 2ull * h);
        }
        if (sk == EMPTY_REC_KEY) break;
        h = (h + 1) & ix.rec_mask;
    }
    slot = h;
    return make_uint4(0, 0, 0, 0);
}

// Per-chunk buffers.
struct ChunkBufs {
    const char* seqs;        // reads back to back
    const uint64_t* offs;    // n + 1
    uint32_t n;
    uint32_t orient_mask;    // bit0 forward read, bit1 reverse complement
    uint32_t stranded;       // count r1 votes (getStranded)
    uint8_t* rflags;         // per read: bit0 too short, bit1 has N, bit2 too long
    uint4* task_cand;        // per task (read*2 + orient): {cand offset, n forward-map, n reverse-map, -}
    uint32_t* cand;          // candidate windows (entry encoding), in iteration order
    uint32_t* cand_task;     // task of each candidate
    uint32_t cand_cap;
    uint32_t* hits;          // HIT_CAP per candidate: offset << 8 | errors
    uint32_t* hit_n;         // number of hits of each candidate (may exceed HIT_CAP)
    uint64_t* mats;
    uint8_t* invalid;
    uint32_t* dp_list;       // reads that need the banded DP: read
    uint64_t* dp_mat;        // their match
    uint8_t* dp_orient;
    uint32_t* meth;          // 4 x n_cpg counters (uint16 semantics after the fact)
    unsigned long long* ctr; // device counters, see CTR_*
    uint32_t* heavy;         // seeding tasks for the middle tiers; the tiers' lists alternate between
    uint32_t* heavy2;        // heavy and heavy2 (pairs: heavy = per-pair path, heavy2 = paired middle tier)
    uint8_t* cand_flags;     // per candidate, bit 0: scan from startPos - 1 even at 0 (paired second mate); may be null
    uint32_t cand_first;     // first candidate the Shift-And launch scans
};

enum {
    CTR_CAND = 0,       // candidates allocated
    CTR_HEAVY,          // heavy tasks
    CTR_DP,             // DP reads
    CTR_SUCC,
    CTR_NONU,
    CTR_UNSUCC,
    CTR_R1F,
    CTR_R1R,
    CTR_INV_LEN,
    CTR_INV_N,
    CTR_GATHER_BYTES,
    CTR_SCANS,
    CTR_TOO_LONG,
    CTR_ERRFLAG,        // a device-side capacity check failed
    CTR_WMASK,          // bit W set when a valid read needs a W-word automaton
    CTR_PAIRED,         // pairs with both mates in CpG windows
    CTR_TOOSHORT,       // the paired path's tooShort count
    CTR_CAND_USED,      // candidate slots holding a candidate (CTR_CAND counts reserved ones)
    CTR_HEAVY2,         // seeding tasks handed on by the first middle tier (pairs: pairs for the paired middle tier)
    CTR_HEAVY3,         // seeding tasks handed on by the second middle tier
    CTR_HEAVY4,         // seeding tasks handed on by the global-memory tier to the large-capacity one
    CTR_QMID,           // work-queue position of the first middle seeding tier (pairs: of the paired middle tier)
    CTR_QMID2,          // work-queue position of the second middle seeding tier
    CTR_REPLAY,         // seeding tasks whose candidate order needed the map replay
    CTR_N
};

constexpr int HIT_CAP = 6;

// A count argument with this value is read from the chunk's device counters
// instead (launches that run without a host round trip).
constexpr uint32_t FROM_DEVICE = 0xffffffffu;
// cand_task value of a reserved candidate slot that holds no candidate
constexpr uint32_t CAND_HOLE = 0xffffffffu;

// The candidate buffer overflowed: the chunk's later stages do nothing and the
// host reruns it with a larger buffer.
// The later stages of a chunk stop when its candidate buffer overflowed (the
// host reruns the chunk with a larger one) or the chunk already failed (a read
// over FAME_MAX_READ_LEN, a capacity error): nothing is tallied then.
__device__ __forceinline__ bool cand_overflow(const ChunkBufs& cb)
{
    return cb.ctr[CTR_CAND] > cb.cand_cap || cb.ctr[CTR_TOO_LONG] || cb.ctr[CTR_ERRFLAG];
}

__device__ __forceinline__ uint64_t rotl64(uint64_t v, unsigned s)
{
    s &= 63u;
    return s ? (v << s) | (v >> (64 - s)) : v;
}

// msTab value of a read byte (spaced_nthash/nthash.hpp:88-121)
__device__ __forceinline__ uint64_t nt_val(uint8_t c)
{
    switch (c) {
        case 'A': case 'a': case 4: return NT_SEED_A;
        case 'C': case 'c': case 'T': case 't': case 1: case 7: return NT_SEED_T;
        case 'G': case 'g': case 3: return NT_SEED_G;
        default: return 0;
    }
}

// reverse complement byte as matchReads builds revSeq (ReadQueue.cpp:448-484):
// other letters leave the zero the string was resized with.
__device__ __forceinline__ uint8_t rc_byte(uint8_t c)
{
    switch (c) {
        case 'A': return 'T';
        case 'C': return 'G';
        case 'G': return 'C';
        case 'T': return 'A';
        default: return 0;
    }
}

// Base of the packed genome: 0..3 for ACGT, 4 for N, 5 outside the chromosome.
__device__ __forceinline__ int gbase(const DevIndex& ix, uint32_t chrom, int64_t pos)
{
    if (pos < 0 || (uint64_t)pos >= ix.chrom_len[chrom]) return 5;
    const uint64_t g = ix.chrom_off[chrom] + (uint64_t)pos;
    if ((__ldg(ix.gnmask + (g >> 5)) >> (g & 31)) & 1u) return 4;
    return (int)((__ldg(ix.gpack + (g >> 4)) >> (2 * (g & 15))) & 3u);
}

__device__ __forceinline__ uint8_t base_char(int b)
{
    return b == 0 ? 'A' : b == 1 ? 'C' : b == 2 ? 'G' : b == 3 ? 'T' : b == 4 ? 'N' : 0;
}

}  // namespace fame
