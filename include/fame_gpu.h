/* fame_gpu.h — C ABI of the GB300 read-matching library for FAME.
 *
 * The library replaces the body of FAME's single-end matching stage
 * (ReadQueue::matchReads, ReadQueue.cpp:404-933, and everything it calls:
 * getSeedRefs 2325-2461, saQuerySeedSetRef 1928-2160, ShiftAnd.h,
 * computeMethLvl 3278-3947, LevenshtDP.h) with CUDA kernels for sm_103a.
 * FAME's host (CLI, parseChunk, decideStrand, printMethylationLevels, the
 * --load_index reader) stays as it is and calls these functions.
 *
 * Conventions: plain C types, host pointers unless a name ends in _dev,
 * every function returns FAME_OK (0) or a negative FAME_ERR_* code and never
 * exits; fame_gpu_last_error() returns a message for the last failure.
 * One fame_gpu context is used by one host thread at a time.
 */
#ifndef FAME_GPU_H
#define FAME_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    FAME_OK = 0,
    FAME_ERR_ARG = -1,        /* bad argument (null pointer, size)              */
    FAME_ERR_CUDA = -2,       /* CUDA runtime failure (message has the detail)  */
    FAME_ERR_NOMEM = -3,      /* device or host allocation failed               */
    FAME_ERR_INDEX = -4,      /* index tables inconsistent or unsupported       */
    FAME_ERR_READ = -5,       /* a read is longer than FAME_MAX_READ_LEN        */
    FAME_ERR_IO = -6,         /* index file missing, truncated or mismatched    */
    FAME_ERR_TIMEOUT = -7,    /* a bounded device wait gave up                  */
    FAME_ERR_BUSY = -8        /* serving queue full / admission refused         */
};

/* Longest read the kernels accept (the reference has no limit; FAME's
 * CONST.h READLEN is 100 or 150 for the workloads it is run on). */
#define FAME_MAX_READ_LEN 255

/* Match flags of fame_gpu_match_reads, the three inputs of the orientation
 * choice at ReadQueue.cpp:529 and :591. */
#define FAME_GET_STRANDED 1u  /* matchReads(..., getStranded = true): both orientations, count r1 votes */
#define FAME_BOTH_STRANDS 2u  /* bothStrandsFlag (--unord_reads)                                      */
#define FAME_MATCH_R1_FWD 4u  /* matchR1Fwd after decideStrand (ReadQueue.cpp:376-400)               */

/* Layout-compatible with the reference's structs (structs.h:40-72, 118-125). */
typedef struct { uint8_t chrom; uint32_t pos; } fame_cpg;                            /* struct CpG   */
typedef struct { uint32_t start_pos; uint8_t chrom; uint32_t start_ind; uint32_t end_ind; } fame_window; /* metaWindow */
typedef struct { uint32_t meta; uint32_t tmask; } fame_kmer;                        /* KMER_S::kmer */

/* A loaded index: the public members of RefGenome after load()
 * (RefGenome.h:193-227, RefGenome.cpp:230-387), as host pointers the caller
 * keeps alive for the duration of fame_gpu_open.  Exactly one of tab_index
 * (the reference's uint64 offsets) or tab_index32 must be given; both hold
 * 2^30 + 1 entries.  strand_bits is strandTable packed LSB first, the layout
 * of the <index>_strands side file (RefGenome.cpp:392-433). */
typedef struct {
    uint32_t readlen;                 /* MyConst::READLEN of the index (CONST.h:35) */
    uint32_t n_chrom;
    const char* const* chrom_seq;     /* fullSeq[c].data()                          */
    const uint64_t* chrom_len;
    const char* const* chrom_name;    /* chrMap (may be NULL)                       */
    uint64_t n_cpg;
    const fame_cpg* cpg;              /* cpgTable                                   */
    const uint64_t* tab_index;        /* tabIndex (uint64)                          */
    const uint32_t* tab_index32;      /* or the same offsets as uint32              */
    uint64_t n_kmer;
    const fame_kmer* kmer;            /* kmerTableSmall                             */
    const uint8_t* strand_bits;       /* strandTable                                */
    uint64_t n_win;
    const fame_window* win;           /* metaWindows                                */
    uint64_t n_filtered;
    const uint64_t* filtered;         /* filteredKmers (paired path only)           */
} fame_index_view;

/* Per-call statistics: the counters matchReads updates (ReadQueue.cpp:408-416,
 * 926-932) plus the strand votes of the first chunk (r1FwdMatches/r1RevMatches). */
typedef struct {
    uint64_t succ;
    uint64_t nonunique;
    uint64_t unsucc;
    uint64_t r1_fwd;
    uint64_t r1_rev;
    uint64_t invalid_len;     /* reads rejected by the length gate (ReadQueue.cpp:430) */
    uint64_t invalid_n;       /* reads rejected for an N (ReadQueue.cpp:487)            */
    uint64_t gather_bytes;    /* algorithmic index-gather bytes of the call             */
    uint64_t windows_scanned; /* Shift-And window scans of the call                     */
    uint64_t dp_reads;        /* reads aligned with the banded DP                       */
    uint64_t heavy_tasks;     /* (read, orientation) seedings run with the large-capacity
                                 scratch (buckets beyond the shared-memory caps)         */
    uint64_t reruns;          /* chunk passes repeated after the candidate buffer grew  */
} fame_counters;

typedef struct fame_gpu fame_gpu;

/* ---- host-side index (the --load_index format and the index build) ---- */
typedef struct fame_host_index fame_host_index;

/* Read <path> and <path>_strands as written by RefGenome::save
 * (RefGenome.cpp:83-228); the header constants must equal the library's
 * (RefGenome.cpp:239-280 exits on a mismatch, this returns FAME_ERR_IO). */
int fame_index_read(const char* path, fame_host_index** out);

/* Build the index from chromosome sequences the way readReference +
 * RefGenome(cpgTab, ...) do (RefReader_istr.h:48-113, RefGenome.cpp:26-74,
 * 532-759, 1787-1989, 2191-2352), on n_threads host threads (0 = all). */
int fame_index_build(uint32_t readlen, uint32_t n_chrom, const char* const* seq, const uint64_t* len,
                     const char* const* names, int noloss, int n_threads, fame_host_index** out);

/* The same index, identical table for table, built on the GPU `device`
 * (window hashing, bucket fill, bucket order, both filters, compaction and
 * T masks on the device; the tables come back to host memory).  Needs at
 * its peak about 16 bytes of device memory per k-mer entry before the
 * filters, plus 8 GiB of bucket arrays, the genome (a byte per base) and up
 * to 2 GiB of sort scratch: about 66 GB for a 3 Gbp genome.  FAME_ERR_NOMEM
 * when they do not fit, FAME_ERR_CUDA without a usable device. */
int fame_index_build_gpu(uint32_t readlen, uint32_t n_chrom, const char* const* seq, const uint64_t* len,
                         const char* const* names, int noloss, int device, fame_host_index** out);

/* Write the index in the --load_index format to <path> and <path>_strands
 * (RefGenome::save, RefGenome.cpp:83-228): the reference's file for the same
 * index byte for byte, except the struct padding bytes (uninitialised there,
 * zero here).  The filtered k-mers and the chromosome names come in the
 * iteration order of the reference's unordered containers (libstdc++), i.e.
 * as received from the build or from the file read.  The tabIndex section
 * alone is 8 GiB (HTABSIZE + 1 offsets). */
int fame_index_write(const fame_host_index* ix, const char* path);

/* Borrow a view of a host index (valid until fame_index_free). */
int fame_index_view_of(const fame_host_index* ix, fame_index_view* view);
void fame_index_free(fame_host_index* ix);
/* cpgStartTable (CpGs too close to a chromosome start to be reported,
 * RefReader_istr.h:66-76); returns the count, copies up to cap entries. */
uint64_t fame_index_cpg_start(const fame_host_index* ix, fame_cpg* out, uint64_t cap);
/* filteredKmers in the order the reference's unordered_set received them
 * (RefGenome.cpp:2330; the index writer derives the set's iteration order,
 * RefGenome.cpp:434-443, from it); returns the count, copies up to cap
 * entries. */
uint64_t fame_index_filtered_order(const fame_host_index* ix, uint64_t* out, uint64_t cap);

/* ---- device context ----------------------------------------------------- */
/* Copy the index into HBM on `device` (resident until fame_gpu_close).
 * Replaces the index load of main.cpp (RefGenome::load / the index read) as
 * far as the matching path is concerned: the tables stay on the device. */
int fame_gpu_open(const fame_index_view* ix, int device, fame_gpu** out);

/* Layout of the device's bucket records (no counterpart in the reference;
 * results do not depend on it).  Each record holds a bucket's tabIndex start,
 * its size and its first entries in one 32-byte sector. */
#define FAME_REC_AUTO   0  /* hashed when the non-empty buckets are at most HTABSIZE / 4 */
#define FAME_REC_DENSE  1  /* one record per bucket: 32 GiB whatever the genome */
#define FAME_REC_HASHED 2  /* the non-empty buckets only, 2 to 4 slots each */
/* fame_gpu_open with a chosen record layout (FAME_ERR_INDEX when hashed is
 * asked for and more than HTABSIZE / 2 buckets are non-empty). */
int fame_gpu_open_layout(const fame_index_view* ix, int device, int layout, fame_gpu** out);
/* The context's record layout (FAME_REC_DENSE or FAME_REC_HASHED), its record
 * count and the index's non-empty buckets (either pointer may be NULL). */
int fame_gpu_rec_layout(const fame_gpu* g, uint64_t* slots, uint64_t* nonempty);
int fame_gpu_close(fame_gpu* g);
const char* fame_gpu_last_error(const fame_gpu* g);

/* ReadQueue::matchReads for one chunk of reads: seqs holds the sequences back
 * to back, read i is seqs[offs[i] .. offs[i+1]).  Per read it writes the match
 * (MATCH::match encoding, structs.h:154-192; 0 when invalid) and the invalid
 * flag (Read::isInvalid), accumulates the CpG tallies in device memory and
 * adds to *cnt.  Synchronous. */
int fame_gpu_match_reads(fame_gpu* g, const char* seqs, const uint64_t* offs, uint32_t n, uint32_t flags,
                         uint64_t* mats, uint8_t* invalid, fame_counters* cnt);

/* The same with the reads, offsets and outputs already in device memory
 * (allocated by fame_gpu_alloc or by the caller). */
int fame_gpu_match_reads_dev(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, uint32_t n,
                             uint32_t flags, uint64_t* mats_dev, uint8_t* invalid_dev, fame_counters* cnt);

/* Counters of the paired path (matchPairedReads' statistics): mates counted as
 * the reference counts them (a uniquely paired pair adds 2 to succ). */
typedef struct {
    uint64_t succ;        /* successfully matched mates                          */
    uint64_t nonunique;   /* mates of pairs with two equally good pairings       */
    uint64_t unsucc;      /* mates of pairs without a pairing                    */
    uint64_t paired;      /* pairs with both mates in windows holding CpGs       */
    uint64_t too_short;   /* tooShort: short or invalid mates, mates without CpG windows */
    uint64_t r1_fwd;      /* getStranded votes: the first mate matched forward   */
    uint64_t r1_rev;
    uint64_t dp_reads;    /* mates whose CpG calls needed the banded DP          */
    uint64_t heavy_pairs; /* pairs run with the large-capacity scratch           */
} fame_pair_counters;

/* Paired-end matching of one chunk of n read pairs, replacing the body of
 * ReadQueue::matchPairedReads (ReadQueue.cpp:940-1658; called per chunk by
 * queryRoutinePaired, main.cpp:400-441).  Mate 1 of pair i is
 * seqs1[offs1[i] .. offs1[i+1]), mate 2 likewise in seqs2; flags as for
 * fame_gpu_match_reads (FAME_GET_STRANDED on the first chunk unless
 * FAME_BOTH_STRANDS; FAME_MATCH_R1_FWD after decideStrand).  maxpdist is the
 * MAXPDIST the reference is compiled with (CONST.h:42): it sets the mate
 * context (contextWLen = floor(maxpdist / 2048) + 1 windows) and the pairing
 * distance (maxpdist + READLEN, extractPairedMatch, ReadQueue.cpp:3255-3275).
 * Outputs per pair: the MATCH::match of each mate (0 when invalid) and the
 * isInvalid flags; CpG calls of uniquely paired mates go to the tallies.
 * Mates longer than FAME_MAX_READ_LEN give FAME_ERR_READ. */
int fame_gpu_match_pairs(fame_gpu* g, const char* seqs1, const uint64_t* offs1, const char* seqs2,
                         const uint64_t* offs2, uint32_t n, uint32_t flags, uint32_t maxpdist, uint64_t* mats1,
                         uint64_t* mats2, uint8_t* invalid1, uint8_t* invalid2, fame_pair_counters* cnt);

/* The same with the mates already in device memory, concatenated: mate 1 of
 * pair i is read i and mate 2 is read n + i of (seqs_dev, offs_dev[2n + 1]);
 * mats_dev and invalid_dev hold 2n entries in that order. */
int fame_gpu_match_pairs_dev(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, uint32_t n, uint32_t flags,
                             uint32_t maxpdist, uint64_t* mats_dev, uint8_t* invalid_dev, fame_pair_counters* cnt);

/* Copy out the methylation tallies as methLevels (ReadQueue.h:354-367): four
 * uint16 per CpG in cpgTable order {methFwd, unmethFwd, methRev, unmethRev}
 * with the reference's 16-bit wrap-around; reset != 0 zeroes them afterwards
 * (printSCMethylationLevels, ReadQueue.cpp:1894-1921). */
int fame_gpu_tallies(fame_gpu* g, uint16_t* meth, int reset);

/* ---- FASTQ chunks (host) ---------------------------------------------------
 * parseChunk / parseChunkGZ (ReadQueue.cpp:218-373): four lines per record,
 * the sequence is the second, nothing validated.  fame_fastq_read packs the
 * sequences of up to max_reads records back to back into seqs (seq_cap bytes;
 * FAME_ERR_ARG when they do not fit) with offsets offs[n + 1], and returns the
 * record count in *n (0 at the end of the input); parsing is spread over
 * n_threads host threads (<= 0: up to 16).  A plain regular file is mapped
 * and parsed in place (it must not shrink while open); gzip input and pipes
 * are read through a buffer.  Different readers may be used from different
 * threads at the same time. */
typedef struct fame_fastq fame_fastq;
int fame_fastq_open(const char* path, int is_gz, int n_threads, fame_fastq** out);
/* fame_fastq_open, with gzip input written as BGZF (the blocked gzip of
 * bgzip: members of at most 64 KiB whose headers and trailers give their
 * sizes) inflated on GPU `device`, one warp per member, the CRC-32 and size
 * of every member checked (a bad member fails the read with FAME_ERR_IO);
 * other gzip input is inflated by zlib as with fame_fastq_open (one stream
 * cannot be split).  device < 0 is fame_fastq_open.  FAME_ERR_CUDA when the
 * input is BGZF and the device cannot be used. */
int fame_fastq_open_dev(const char* path, int is_gz, int n_threads, int device, fame_fastq** out);
/* 1 when the reader inflates its input on a GPU (BGZF), else 0. */
int fame_fastq_gpu_inflate(const fame_fastq* f);
int fame_fastq_read(fame_fastq* f, uint32_t max_reads, char* seqs, uint64_t seq_cap, uint64_t* offs, uint32_t* n);
int fame_fastq_close(fame_fastq* f);

/* ---- Report writers (host; byte-identical to the reference's output) ------
 * fame_report_cpg writes <path> as printMethylationLevels writes
 * <basename>_cpg.tsv (ReadQueue.cpp:1860-1893): per CpG in cpgTable order
 * "chrom\tpos+READLEN-2\tmethFwd\tunmethFwd\tmethRev\tunmethRev\n";
 * meth holds 4 uint16 per CpG (fame_gpu_tallies).  n_threads <= 0: all cores.
 * fame_report_sc_header starts a single-cell matrix file (the two header rows
 * of the single-cell ReadQueue); fame_report_sc_rows appends one cell's four
 * rows (printSCMethylationLevels, ReadQueue.cpp:1894-1921, including its
 * fourth row label "unmethFwd"). */
int fame_report_cpg(const fame_index_view* v, const uint16_t* meth, const char* path, int n_threads);
int fame_report_sc_header(const fame_index_view* v, const char* path);
int fame_report_sc_rows(const fame_index_view* v, const char* sc_id, const uint16_t* meth, const char* path,
                        int n_threads);

/* ---- Batched and serving form (no counterpart in the reference) ---------
 * A queue of chunk slots on one context.  Each slot owns device buffers for
 * one chunk of up to max_reads reads / max_bytes bases, page-locked staging
 * and a CUDA stream, and runs the chunk pipeline as a captured CUDA graph
 * with no host round trip inside; chunks in different slots overlap on the
 * GPU.  One queue per context (at most 8 slots); its calls and the plain
 * match calls come from one host thread.  Results equal those of
 * fame_gpu_match_reads for the same chunk and flags. */
typedef struct fame_queue fame_queue;
int fame_queue_open(fame_gpu* g, uint32_t slots, uint32_t max_reads, uint64_t max_bytes, fame_queue** out);
/* Copies one chunk into a free slot and starts it; returns the slot.
 * meth_dev: the tally array the chunk adds to (from fame_gpu_tally_alloc,
 * e.g. one job's), NULL for the context's own.  FAME_ERR_BUSY when every
 * slot holds an uncollected chunk. */
int fame_queue_submit(fame_queue* q, const char* seqs, const uint64_t* offs, uint32_t n, uint32_t flags,
                      uint32_t* meth_dev, int* slot);
/* 1 when the slot's chunk has finished, 0 while it runs. */
int fame_queue_ready(fame_queue* q, int slot);
/* Waits up to timeout_ms for the slot's chunk: FAME_OK when it has finished
 * (or the slot holds none), FAME_ERR_TIMEOUT when the time ran out first (the
 * chunk keeps running; wait again or collect later). */
int fame_queue_wait(fame_queue* q, int slot, uint32_t timeout_ms);
/* Waits for the slot's chunk and copies out its results (NULL to skip). */
int fame_queue_collect(fame_queue* q, int slot, uint64_t* mats, uint8_t* invalid, fame_counters* cnt);
/* Kernels launched through the queue so far. */
uint64_t fame_queue_launches(const fame_queue* q);
int fame_queue_close(fame_queue* q);
/* Zero-copy submission: stage reserves a free slot and returns its
 * page-locked staging (room for max_reads reads, offs[0..n] from 0, and
 * max_bytes bases); the caller writes a chunk there (e.g. with
 * fame_fastq_read) and starts it with submit_staged (n = 0 returns the slot
 * unused).  FAME_ERR_BUSY when no slot is free. */
int fame_queue_stage(fame_queue* q, int* slot, char** seqs, uint64_t** offs, uint32_t* max_reads, uint64_t* max_bytes);
int fame_queue_submit_staged(fame_queue* q, int slot, uint32_t n, uint32_t flags, uint32_t* meth_dev);

/* ---- FASTQ file to tallies: queryRoutine (main.cpp:363-399) -------------
 * parseChunk / parseChunkGZ (ReadQueue.cpp:218-373) and matchReads over a
 * whole file, chunks of `chunk` records (0: CHUNKSIZE, 300,000): the first matched alone
 * with the strand vote unless flags has FAME_BOTH_STRANDS, then the others
 * with the decided orientation (decideStrand, ReadQueue.cpp:376-400), parsed
 * by n_threads host threads straight into the staging of a queue of `slots`
 * (2..8) chunk slots while earlier chunks run on the GPU.  Tallies add to
 * meth_dev (NULL: the context's array); cnt receives the summed counters and
 * n_reads the records read.  Opens its own queue: FAME_ERR_BUSY when the
 * context already has one. */
int fame_match_fastq(fame_gpu* g, const char* path, int is_gz, uint32_t flags, uint32_t chunk, uint32_t slots,
                     int n_threads, uint32_t* meth_dev, fame_counters* cnt, uint64_t* n_reads);
/* queryRoutinePaired (main.cpp:400-441) over two mate FASTQ files: chunks of
 * `chunk` pairs (0: CHUNKSIZE) read from both files (FAME_ERR_IO when they
 * hold different numbers of records), the first matched with the strand vote
 * unless flags has FAME_BOTH_STRANDS, each through fame_gpu_match_pairs while
 * a host thread parses the next chunk of both files into page-locked
 * buffers.  maxpdist as for fame_gpu_match_pairs; tallies add to the
 * context's array; cnt receives the summed counters and n_pairs the pairs
 * read. */
int fame_match_fastq_paired(fame_gpu* g, const char* path1, const char* path2, int is_gz, uint32_t flags,
                            uint32_t maxpdist, uint32_t chunk, int n_threads, fame_pair_counters* cnt,
                            uint64_t* n_pairs);
/* Separate tally arrays (4 x n_cpg uint32 in device memory, zeroed), e.g. one
 * per single-cell job of a serving loop; read returns them as methLevels
 * (uint16 wrap), reset zeroes them. */
int fame_gpu_tally_alloc(fame_gpu* g, uint32_t** meth_dev);
int fame_gpu_tally_read(fame_gpu* g, const uint32_t* meth_dev, uint16_t* meth, int reset);
int fame_gpu_tally_free(fame_gpu* g, uint32_t* meth_dev);
/* Free and total device memory (admission control of a serving loop). */
int fame_gpu_mem_info(fame_gpu* g, uint64_t* free_bytes, uint64_t* total_bytes);

/* Device memory helpers for the _dev entry points, and page-locked host
 * buffers (a host that parses its chunks straight into these gets the fast
 * host-to-device copy path).  Host buffers are placed on the host NUMA node
 * nearest the device when the process may use it (else ordinary page-locked
 * memory); free them with fame_gpu_host_free on the same context. */
int fame_gpu_alloc(fame_gpu* g, size_t bytes, void** ptr_dev);
int fame_gpu_free(fame_gpu* g, void* ptr_dev);
int fame_gpu_memcpy(fame_gpu* g, void* dst, const void* src, size_t bytes, int kind /* 1 H2D, 2 D2H, 3 D2D */);
int fame_gpu_host_alloc(fame_gpu* g, size_t bytes, void** ptr);
int fame_gpu_host_free(fame_gpu* g, void* ptr);
/* Where host memory lies, for copy-rate diagnostics: the NUMA node holding
 * the page at ptr (-1 when unknown), and the host node nearest the device
 * (-1 when the device reports none).  A page-locked buffer whose pages the
 * kernel placed on another node (the near node was short of memory) copies
 * over the CPU-to-CPU link, at a fraction of the near node's rate. */
int fame_host_page_node(const void* ptr);
int fame_gpu_host_node(fame_gpu* g);
/* The CUDA stream (cudaStream_t) all work of the context runs on. */
int fame_gpu_stream(fame_gpu* g, void** stream);

/* Per-stage device time of the last single-end match call, in milliseconds,
 * measured with CUDA events on the library's stream when enabled.  Stages:
 * 0 read prep, 1 light seeding (or routing to the middle tiers), 2 Shift-And,
 * 3 select + exact CpG calls, 4 banded DP + CpG calls, 5 the other seeding
 * tiers, split into 6 the smaller shared-memory middle tier, 7 the larger one
 * and 8 the global-memory tiers.  Returns the number of stages (FAME_STAGES). */
#define FAME_STAGES 9
int fame_gpu_set_timing(fame_gpu* g, int enable);
int fame_gpu_stage_times(fame_gpu* g, float* ms, int n);
/* The same for the last paired-end call: 0 mate checks, 1 seeding in shared
 * memory, 2 the paired middle tier, 3 first-mate window scans, 4 first walks,
 * 5 second-mate window scans, 6 second walks and the pair choice, 7 the
 * per-pair path and the banded DP.  Returns FAME_PAIR_STAGES. */
#define FAME_PAIR_STAGES 8
int fame_gpu_pair_stage_times(fame_gpu* g, float* ms, int n);
/* Seeding tasks that entered each tier after the light one in the last
 * single-end chunk: out[0] the smaller shared-memory middle tier (up to 511
 * gathered bucket entries), out[1] the larger one (up to 1023), out[2] the
 * global-memory tier, out[3] the large-capacity tier; out[4] the tasks (of
 * any tier) whose candidate order needed the replay of the map's insertions
 * (a strand map with two or more candidates).  No counterpart in the
 * reference (diagnostics). */
int fame_gpu_seed_tier_counts(const fame_gpu* g, uint64_t* out);
/* Test hook (no counterpart in the reference): replays, on the device, the
 * insertion of keys[0..n) (distinct, bit 31 clear, n <= 65536) into a
 * tsl::hopscotch_map made with bucket_count buckets -- the replay the seeding
 * kernels use to order a read's candidate windows -- and writes the map's
 * iteration order to order[] and its final bucket count.  Returns the number
 * of keys written, or an error code.  Allocates device memory. */
int fame_gpu_map_order_probe(fame_gpu* g, const uint32_t* keys, uint32_t n, uint32_t bucket_count, uint32_t* order,
                             uint64_t* final_buckets);
/* Number of kernel launches of the last match call. */
int fame_gpu_last_launches(const fame_gpu* g);
/* Device bytes held by the resident index tables of the context. */
uint64_t fame_gpu_index_bytes(const fame_gpu* g);
/* How reads are seeded (no counterpart in the reference; results do not
 * depend on it).  Each tier is one warp per (read, orientation) task; a task
 * over a tier's capacity moves on to the next.  Bit 0: 0 = the light tier
 * first (small shared-memory working space, up to 128 gathered bucket
 * entries); 1 = every read starts in the middle tiers (genome-scale indexes).
 * The middle tiers keep the whole working set in shared memory and take
 * their tasks from device work queues: one for up to 511 gathered entries
 * (12 warps per SM), then one for up to 1023; bit 1 = 1 skips the first.
 * After them come a global-memory tier (up to 4096) and a large-capacity one
 * sized by the index's largest bucket.  fame_gpu_open sets bit 0 when the
 * index holds more entries than buckets.  mode < 0 returns the current mode.
 * Waits for the context's queue and drops its captured graphs. */
int fame_gpu_set_seed_tier(fame_gpu* g, int mode);

/* Autotuner of the launch shapes (no counterpart in the reference): runs the
 * chunk (n reads already in device memory, as for fame_gpu_match_reads_dev,
 * with these flags) a few times per stage with different shapes (the seeding
 * modes of fame_gpu_set_seed_tier, the window-scan and banded-DP grids),
 * checks that every shape gives the same per-read results, keeps the fastest
 * shape per stage and, when json_path is given, writes the choice and every
 * trial's stage times there (CUDA events: read prep, light seeding, window
 * scans, selection, DP, other seeding tiers).  The context's tallies are not
 * touched.  The shapes apply to the plain calls and to the queue alike; the
 * queue's captured graphs are dropped.  Allocates and frees device memory. */
int fame_gpu_autotune(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, uint32_t n, uint32_t flags,
                      const char* json_path);
/* Applies the shapes of a file written by fame_gpu_autotune (FAME_ERR_IO when
 * the file cannot be read or holds no valid shape). */
int fame_gpu_load_tuning(fame_gpu* g, const char* json_path);

/* CpG calls that allocate no device memory.  No counterpart in the reference:
 * it is for callers that cannot allocate while they run (a serving loop that
 * must not stall its other streams on the device-wide synchronisation of
 * cudaFree, or code that only receives buffers from an allocator it does not
 * own).  For each read i < n with invalid_dev[i] == 0 it does what
 * computeMethLvl does for the match mats_dev[i] (exact-hit lookup, or the
 * banded DP and alignment walk), with the read as given (orient 0) or its
 * reverse complement (orient 1), and writes four uint32 counters per CpG
 * {methFwd, unmethFwd, methRev, unmethRev} to meth_dev (zeroed first; the low
 * 16 bits are methLevels).  All pointers are device memory owned by the
 * caller; g only supplies the resident index and its stream.
 * Scratch: one static device array of about 10.5 MB per GPU that loads the
 * library (held until exit), shared by every call: calls that overlap on the
 * GPU race (one context's calls run in order on its stream; calls from two
 * contexts on one device must not overlap).  fame_gpu_open resolves the
 * array's device address for its context, so no call here resolves anything.
 * Reads longer than FAME_MAX_READ_LEN give FAME_ERR_READ; a match naming no
 * window of the index gives FAME_ERR_ARG; fame_gpu_last_error has the detail. */
int fame_gpu_call_cpgs_noalloc(fame_gpu* g, const char* seqs_dev, const uint64_t* offs_dev, const uint64_t* mats_dev,
                               const uint8_t* invalid_dev, uint32_t n, int orient, uint32_t* meth_dev);

#ifdef __cplusplus
}
#endif
#endif /* FAME_GPU_H */
