/* Test infrastructure only (parity checker): a plain-C restatement of FAME's
 * single-end read-matching path.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg use it; the product never links it.
 *
 * Parity is pinned against the compiled reference (oracle/build_ref.sh) on
 * seeded synthetic inputs (tests/golden/) and against the LevenshtDP known-
 * answer tests of the reference (LevenshtDP_unittest.cpp).
 */
#ifndef FAME_ORACLE_H
#define FAME_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Loaded-index view (RefGenome members after load(), RefGenome.h:193-227) with
 * the hash-table offsets stored sparsely: only non-empty buckets, sorted by key. */
typedef struct {
    uint32_t readlen;            /* MyConst::READLEN the index was built for (CONST.h:35) */
    uint32_t n_chrom;
    const uint8_t* const* chrom_seq;
    const uint64_t* chrom_len;
    uint64_t n_cpg;
    const uint8_t* cpg_chrom;
    const uint32_t* cpg_pos;
    uint64_t n_bucket;
    const uint32_t* bucket_key;
    const uint64_t* bucket_start;
    const uint32_t* bucket_len;
    uint64_t n_kmer;
    const uint32_t* kmer_meta;
    const uint8_t* strand;
    uint64_t n_win;
    const uint32_t* win_start;
    const uint8_t* win_chrom;
    const uint32_t* win_sind;
    const uint32_t* win_eind;
} orc_index;

/* Paired-end extras: T masks (kmerTableSmall.tmask), filteredKmers (sorted) and
 * MyConst::MAXPDIST (CONST.h:42). */
typedef struct {
    const uint32_t* kmer_tmask;
    uint64_t n_filtered;
    const uint64_t* filtered;
    uint32_t maxpdist;
} orc_pe_extra;

/* ---- index build (RefReader_istr.h:48-113, RefGenome.cpp:26-74) ---------- */
typedef struct orc_built orc_built;
orc_built* orc_build(uint32_t readlen, uint32_t n_chrom, const uint8_t* const* raw_seq, const uint64_t* raw_len,
                     int noloss);
/* sizes: [n_cpg, n_cpg_start, n_bucket, n_kmer, n_win, n_filtered] */
void orc_built_sizes(const orc_built* b, uint64_t* sizes);
void orc_built_copy(const orc_built* b, uint8_t* cpg_chrom, uint32_t* cpg_pos, uint8_t* cpgs_chrom,
                    uint32_t* cpgs_pos, uint32_t* bucket_key, uint64_t* bucket_start, uint32_t* bucket_len,
                    uint32_t* kmer_meta, uint32_t* kmer_tmask, uint8_t* strand, uint32_t* win_start,
                    uint8_t* win_chrom, uint32_t* win_sind, uint32_t* win_eind, uint64_t* filtered,
                    uint8_t* const* chrom_seq_out);
void orc_built_free(orc_built* b);

/* ---- single-end matching (ReadQueue.cpp:404-933, main.cpp:363-399) ------- */
/* counters: [succ, nonunique, unsucc, r1Fwd, r1Rev, matchR1Fwd] */
int orc_match_se(const orc_index* ix, const uint8_t* seqs, const uint64_t* offs, uint32_t n,
                 uint32_t chunk, int both_strands, uint64_t* mats, uint8_t* invalid, uint16_t* meth,
                 uint64_t* counters);

/* getSeedRefs + hopscotch iteration order for one sequence (ReadQueue.cpp:2325-2461);
 * n_out = [n_fwd, n_rev, buckets_fwd, buckets_rev] */
int orc_seed_order(const orc_index* ix, const uint8_t* seq, uint32_t len, uint32_t cap,
                   uint32_t* out_keys, uint32_t* out_counts, uint64_t* n_out);

/* Banded DP (LevenshtDP.h) with storage as BandedMatrix.h; comp: 0 equality,
 * 1 CompiFwd, 2 CompiRev, 3 plain complement.  colPat = col + col_end.
 * Returns alignment length; trace codes 0 MATCHING 1 MISMATCH 2 INSERTION 3 DELETION. */
int orc_lev(int band, const uint8_t* row, uint32_t row_len, const uint8_t* col, int64_t col_len,
            int64_t col_end, int rev, int comp, uint8_t* trace, uint32_t cap, uint32_t* dist);

/* ShiftAnd<6> on a text (ShiftAnd.h:130-255); same conventions as the reference
 * driver: rev scans text[len-1] .. text[0] with offsets relative to text-1. */
int orc_shiftand(const uint8_t* pat, uint32_t pat_len, const uint8_t* text, uint32_t text_len, int rev,
                 uint64_t* offs, uint8_t* errs, uint32_t cap);

/* One matchReads call with explicit flags; meth accumulates (uint16 wrap).
 * counters: [succ, nonunique, unsucc, r1Fwd, r1Rev] of this call. */
int orc_match_chunk(const orc_index* ix, const uint8_t* seqs, const uint64_t* offs, uint32_t n, int get_stranded,
                    int both_strands, int match_r1_fwd, uint64_t* mats, uint8_t* invalid, uint16_t* meth,
                    uint64_t* counters);

/* Paired-end matching (matchPairedReads, ReadQueue.cpp:935-1655) with the loop
 * of queryRoutinePaired (main.cpp:400-441).  counters: [succ, nonunique,
 * unsucc, succPaired, tooShort, r1Fwd, r1Rev, matchR1Fwd] */
int orc_match_pe(const orc_index* ix, const orc_pe_extra* px, const uint8_t* s1, const uint64_t* o1, const uint8_t* s2,
                 const uint64_t* o2, uint32_t n, uint32_t chunk, int both_strands, uint64_t* mats1, uint64_t* mats2,
                 uint8_t* inv1, uint8_t* inv2, uint16_t* meth, uint64_t* counters);

/* libstdc++ std::sort of (key, count) by count descending; keys out in order. */
int orc_sort_desc(const uint32_t* keys, const uint8_t* counts, uint32_t n, uint32_t* out);

/* Hopscotch insertion model on an explicit key sequence; returns iteration order. */
int orc_hopscotch(const uint32_t* keys, uint32_t n, uint32_t bucket_count, uint32_t* order, uint64_t* final_buckets);

#ifdef __cplusplus
}
#endif
#endif
