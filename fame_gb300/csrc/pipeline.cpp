// FASTQ files to CpG tallies: queryRoutine (main.cpp:363-399) and
// queryRoutinePaired (main.cpp:400-441) with parseChunk
// (ReadQueue.cpp:218-373) overlapped with the matching.  Chunks of CHUNKSIZE
// (or the caller's count of) records; the first chunk is matched with the
// strand vote (getStranded) unless both strands are queried and decides
// matchR1Fwd for the rest as decideStrand (ReadQueue.cpp:376-400) does.  The
// parse of a chunk never waits for that decision: only the later chunks'
// flags depend on it.  Tallies go to the context's array (single-end: or
// meth_dev); counters are summed over the chunks.  Results do not depend on
// the overlap: every read (pair) is matched alone and tallies and counters
// are sums.
//
// Single-end: the native reader parses straight into a free slot of a
// batched queue (its page-locked staging), so the host parses chunk i + 1
// while the GPU matches chunks i, i - 1, ...
// Paired-end: two page-locked chunk buffers per mate file; a host thread
// parses the next chunk of both files (one reader thread each) into one
// while fame_gpu_match_pairs runs on the other.
#include <cstdint>
#include <deque>
#include <thread>
#include <vector>

#include "../../include/fame_gpu.h"
#include "internal.h"

namespace {

constexpr uint32_t CHUNKSIZE = 300000;   // CONST.h:69

struct Closer {
    fame_fastq* f = nullptr;
    fame_queue* q = nullptr;
    ~Closer()
    {
        if (q) fame_queue_close(q);
        if (f) fame_fastq_close(f);
    }
};

// Parses the next chunk into a staged slot; n = 0 at the end of the input
// (the slot is then submitted empty, which records nothing).
int parse_into_slot(fame_gpu* g, fame_queue* q, fame_fastq* f, uint32_t chunk, int* slot, uint32_t* n)
{
    char* seqs = nullptr;
    uint64_t* offs = nullptr;
    uint32_t max_reads = 0;
    uint64_t max_bytes = 0;
    int rc = fame_queue_stage(q, slot, &seqs, &offs, &max_reads, &max_bytes);
    if (rc) return rc;
    rc = fame_fastq_read(f, chunk < max_reads ? chunk : max_reads, seqs, max_bytes, offs, n);
    if (rc) {
        fame_queue_submit_staged(q, *slot, 0, 0, nullptr);   // give the slot back
        return fame_gpu_fail(g, rc, rc == FAME_ERR_ARG ? "FASTQ chunk larger than the slot (reads over 255 bases)"
                                                        : "FASTQ read failed");
    }
    return FAME_OK;
}

}  // namespace

extern "C" int fame_match_fastq(fame_gpu* g, const char* path, int is_gz, uint32_t flags, uint32_t chunk,
                                uint32_t slots, int n_threads, uint32_t* meth_dev, fame_counters* cnt,
                                uint64_t* n_reads)
{
    if (!g || !path || !cnt) return FAME_ERR_ARG;
    if (chunk == 0) chunk = CHUNKSIZE;
    if (slots < 2) slots = 2;
    if (slots > 8) slots = 8;
    *cnt = fame_counters{};
    if (n_reads) *n_reads = 0;
    Closer c;
    // BGZF input inflated on the context's GPU
    int rc = fame_fastq_open_dev(path, is_gz, n_threads, fame_gpu_device_of(g), &c.f);
    if (rc) return fame_gpu_fail(g, rc, "cannot open the FASTQ file");
    rc = fame_queue_open(g, slots, chunk, (uint64_t)chunk * FAME_MAX_READ_LEN, &c.q);
    if (rc) return rc;
    const bool both = (flags & FAME_BOTH_STRANDS) != 0;
    bool match_r1_fwd = true;
    uint64_t total = 0;
    int slot = -1;
    uint32_t n = 0;
    bool staged = false;   // (slot, n) holds a parsed chunk not yet submitted
    if (!both) {
        // chunk 0 with the strand vote; chunk 1 is parsed while it runs
        int s0 = -1;
        uint32_t n0 = 0;
        if ((rc = parse_into_slot(g, c.q, c.f, chunk, &s0, &n0))) return rc;
        if ((rc = fame_queue_submit_staged(c.q, s0, n0, FAME_GET_STRANDED | FAME_MATCH_R1_FWD, meth_dev))) return rc;
        if (n0 == chunk) {
            if ((rc = parse_into_slot(g, c.q, c.f, chunk, &slot, &n))) return rc;
            staged = true;
        }
        if ((rc = fame_queue_collect(c.q, s0, nullptr, nullptr, cnt))) return rc;
        total += n0;
        match_r1_fwd = cnt->r1_fwd > cnt->r1_rev;
        if (n0 < chunk) {
            if (n_reads) *n_reads = total;
            return FAME_OK;
        }
    }
    const uint32_t later = (both ? FAME_BOTH_STRANDS : 0u) | (match_r1_fwd ? FAME_MATCH_R1_FWD : 0u);
    std::deque<int> inflight;
    for (;;) {
        if (!staged) {
            if (inflight.size() == slots) {   // every slot busy: the oldest chunk finishes first
                if ((rc = fame_queue_collect(c.q, inflight.front(), nullptr, nullptr, cnt))) return rc;
                inflight.pop_front();
            }
            if ((rc = parse_into_slot(g, c.q, c.f, chunk, &slot, &n))) return rc;
        }
        staged = false;
        if ((rc = fame_queue_submit_staged(c.q, slot, n, later, meth_dev))) return rc;
        if (n == 0) {
            if ((rc = fame_queue_collect(c.q, slot, nullptr, nullptr, cnt))) return rc;
            break;
        }
        inflight.push_back(slot);
        total += n;
        if (n < chunk) break;
    }
    while (!inflight.empty()) {
        if ((rc = fame_queue_collect(c.q, inflight.front(), nullptr, nullptr, cnt))) return rc;
        inflight.pop_front();
    }
    if (n_reads) *n_reads = total;
    return FAME_OK;
}

namespace {

struct PairFiles {
    fame_gpu* g = nullptr;
    fame_fastq* f[2] = {nullptr, nullptr};
    std::vector<void*> host;
    ~PairFiles()
    {
        for (fame_fastq* x : f)
            if (x) fame_fastq_close(x);
        for (void* p : host) fame_gpu_host_free(g, p);
    }
    void* alloc(size_t bytes)
    {
        void* p = nullptr;
        if (fame_gpu_host_alloc(g, bytes, &p) != FAME_OK) return nullptr;
        host.push_back(p);
        return p;
    }
};

struct PairChunk {
    char* s[2] = {nullptr, nullptr};
    uint64_t* o[2] = {nullptr, nullptr};
    uint32_t n = 0;
};

// The next chunk of both mate files (parseChunk of the two-file ReadQueue),
// the two files read at the same time (each reader has its own threads; for
// gzip input each file is inflated on its own thread).  Returns a FAME code
// and, on failure, the reason in *why (the caller's thread records it in the
// context).
int parse_pairs(PairFiles& pf, PairChunk& c, uint32_t chunk, uint64_t cap, const char** why)
{
    uint32_t n[2] = {0, 0};
    int rcm[2] = {FAME_OK, FAME_OK};
    std::thread second([&] { rcm[1] = fame_fastq_read(pf.f[1], chunk, c.s[1], cap, c.o[1], &n[1]); });
    rcm[0] = fame_fastq_read(pf.f[0], chunk, c.s[0], cap, c.o[0], &n[0]);
    second.join();
    for (int rc : rcm) {
        if (rc) {
            *why = rc == FAME_ERR_ARG ? "FASTQ chunk larger than the buffer (reads over 255 bases)" : "FASTQ read failed";
            return rc;
        }
    }
    if (n[0] != n[1]) {
        *why = "the mate files hold different numbers of records";
        return FAME_ERR_IO;
    }
    c.n = n[0];
    return FAME_OK;
}

}  // namespace

extern "C" int fame_match_fastq_paired(fame_gpu* g, const char* path1, const char* path2, int is_gz, uint32_t flags,
                                       uint32_t maxpdist, uint32_t chunk, int n_threads, fame_pair_counters* cnt,
                                       uint64_t* n_pairs)
{
    if (!g || !path1 || !path2 || !cnt) return FAME_ERR_ARG;
    if (chunk == 0) chunk = CHUNKSIZE;
    *cnt = fame_pair_counters{};
    if (n_pairs) *n_pairs = 0;
    PairFiles pf;
    pf.g = g;
    int rc;
    if ((rc = fame_fastq_open_dev(path1, is_gz, n_threads, fame_gpu_device_of(g), &pf.f[0])) ||
        (rc = fame_fastq_open_dev(path2, is_gz, n_threads, fame_gpu_device_of(g), &pf.f[1])))
        return fame_gpu_fail(g, rc, "cannot open the mate FASTQ files");
    const uint64_t cap = (uint64_t)chunk * FAME_MAX_READ_LEN;
    PairChunk buf[2];
    for (auto& b : buf)
        for (int m = 0; m < 2; ++m) {
            b.s[m] = (char*)pf.alloc(cap);
            b.o[m] = (uint64_t*)pf.alloc((chunk + 1ull) * sizeof(uint64_t));
            if (!b.s[m] || !b.o[m]) return fame_gpu_fail(g, FAME_ERR_NOMEM, "page-locked chunk buffers");
        }
    uint64_t* mats[2] = {(uint64_t*)pf.alloc(chunk * 8ull), (uint64_t*)pf.alloc(chunk * 8ull)};
    uint8_t* inv[2] = {(uint8_t*)pf.alloc(chunk), (uint8_t*)pf.alloc(chunk)};
    if (!mats[0] || !mats[1] || !inv[0] || !inv[1]) return fame_gpu_fail(g, FAME_ERR_NOMEM, "page-locked results");
    const char* why = nullptr;
    if ((rc = parse_pairs(pf, buf[0], chunk, cap, &why))) return fame_gpu_fail(g, rc, why);
    const bool both = (flags & FAME_BOTH_STRANDS) != 0;
    bool stranded = !both;   // the chunk in hand is chunk 0 of a strand vote
    bool match_r1_fwd = true;
    uint64_t total = 0;
    int cur = 0;
    for (;;) {
        PairChunk& c = buf[cur];
        const bool more = c.n == chunk;   // a full chunk: the input may go on
        int prc = FAME_OK;
        const char* pwhy = nullptr;
        std::thread th;
        if (more) th = std::thread([&] { prc = parse_pairs(pf, buf[cur ^ 1], chunk, cap, &pwhy); });
        const uint32_t fl = stranded ? (FAME_GET_STRANDED | FAME_MATCH_R1_FWD)
                                     : (both ? FAME_BOTH_STRANDS : 0u) | (match_r1_fwd ? FAME_MATCH_R1_FWD : 0u);
        rc = c.n ? fame_gpu_match_pairs(g, c.s[0], c.o[0], c.s[1], c.o[1], c.n, fl, maxpdist, mats[0], mats[1], inv[0],
                                        inv[1], cnt)
                 : FAME_OK;
        if (th.joinable()) th.join();
        if (rc) return rc;
        total += c.n;
        if (stranded) {
            match_r1_fwd = cnt->r1_fwd > cnt->r1_rev;
            stranded = false;
        }
        if (!more) break;
        if (prc) return fame_gpu_fail(g, prc, pwhy);
        cur ^= 1;
    }
    if (n_pairs) *n_pairs = total;
    return FAME_OK;
}
